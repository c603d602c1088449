// fvm_df.cuh -- double-float arithmetic for the FP64-bound stencils of the mixed path.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers (about 48 significant
// bits, relative rounding error near 2^-46 per operation).  GB300 issues FP64 at a
// small fraction of its FP32 rate (an FMA chain measured 0.50 T FMA/s in FP64 against
// 2.9 T double-float FMA/s built from FP32 instructions), so the stencils of the SGS
// model, DIF, NL and P_SOURCE, which are bound by FP64 issue in FP64, run several
// times faster in double-float.  The arrays stay FP64 in memory: a load splits the
// double with integer and FP32 instructions and a store joins the pair with one
// FP64 add.
//
// Algorithms: Knuth's TwoSum and Dekker's FastTwoSum for error-free sums, the
// FMA-based TwoProduct for error-free products (Dekker 1971; Knuth, TAOCP vol. 2,
// 4.2.2), division as the FP32 quotient plus one remainder correction, the square
// root as one Newton correction of the FP32 root (Karp and Markstein 1997).  The round-to-nearest intrinsics keep the compiler from contracting
// the error-free transformations into fused multiply-adds.
#pragma once
#include <cstdint>

namespace fvm {

struct dd {
    float hi, lo;
    dd() = default;
    __device__ __forceinline__ constexpr dd(float h, float l) : hi(h), lo(l) {}
    // from an FP64 value: split on the integer pipe (see dd_split)
    __device__ __forceinline__ dd(double x);
    __device__ __forceinline__ dd(int x) : hi((float)x), lo(0.0f) {}   // small integer constants
};

// Split a double into hi + lo without a conversion instruction (on GB300 the
// conversions issue on the FP64 pipe): hi is the double truncated to 24 bits
// (exponent rebiased 1023 -> 127, top 23 fraction bits), lo the next 23 fraction
// bits times 2^(e - 1069), formed as (1.m) s - s with s a power of two in one
// exact FP32 fused multiply-add.  Relative error below 2^-46.  |x| below 2^-74 keeps
// only hi (zero below 2^-126); |x| at or above 2^128 gives inf, NaN stays NaN.
__device__ __forceinline__ dd dd_split(double x)
{
    const uint32_t hw = (uint32_t)__double2hiint(x), lw = (uint32_t)__double2loint(x);
    const uint32_t sign = hw & 0x80000000u, ah = hw & 0x7fffffffu, e = ah >> 20;
    uint32_t hb = __funnelshift_r(lw, ah - (896u << 20), 29);   // valid for 897 <= e <= 1150
    const float one_m = __uint_as_float(0x3f800000u | ((lw >> 6) & 0x7fffffu));
    const float sc = __uint_as_float((e - 919u) << 23);         // 2^(e - 1046), valid for e >= 920
    uint32_t lb = __float_as_uint(__fmaf_rn(one_m, sc, -sc));
    if (e < 949u) lb = 0u;
    if (e < 897u) hb = 0u;
    if (e > 1150u) {
        hb = (e == 2047u && ((ah & 0xfffffu) | lw) != 0u) ? 0x7fc00000u : 0x7f800000u;
        lb = 0u;
    }
    return dd(__uint_as_float(hb | sign), __uint_as_float(lb | sign));
}
__device__ __forceinline__ dd::dd(double x) : dd(dd_split(x)) {}

// Exact FP32 -> FP64 with integer instructions: normal numbers, inf and NaN keep
// their value, zero and subnormals give a signed zero.
__device__ __forceinline__ double f2d_int(float f)
{
    const uint32_t u = __float_as_uint(f), ex = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    const uint32_t dex = ex == 0xffu ? 0x7ffu : ex + 896u;
    const uint32_t hi = (u & 0x80000000u) | (ex == 0u ? 0u : ((dex << 20) | (m >> 3)));
    const uint32_t lo = ex == 0u ? 0u : (m << 29);
    return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ double dd_join(dd a) { return f2d_int(a.hi) + f2d_int(a.lo); }

__device__ __forceinline__ dd fast_two_sum(float a, float b)   // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return dd(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dd operator+(dd a, dd b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));   // TwoSum error
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s, e);
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);   // TwoProduct error
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
// a / b: the FP32 quotient of the leading parts, corrected once by the remainder
// a - q b formed in double-float (long division in two digits).
__device__ __forceinline__ dd operator/(dd a, dd b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const dd r = a - b * dd(q1, 0.0f);
    return fast_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ dd fma(dd a, dd b, dd c) { return a * b + c; }
// exact scaling by a power of two (no overflow or underflow at the magnitudes used)
__device__ __forceinline__ dd scale2(dd a, float p2) { return dd(__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)); }
__device__ __forceinline__ double scale2(double a, float p2) { return a * (double)p2; }
__device__ __forceinline__ dd sqrt(dd a)
{
    if (!(a.hi > 0.0f)) return dd(sqrtf(a.hi), 0.0f);   // zero, negative or NaN
    const float y = __fsqrt_rn(a.hi);
    const float p = __fmul_rn(y, y);
    const float pe = __fmaf_rn(y, y, -p);                                   // y^2 = p + pe exactly
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);    // a - y^2
    return fast_two_sum(y, __fmul_rn(r, __fdiv_rn(0.5f, y)));
}

// Arithmetic-type helpers for kernels templated over double / dd.
template <class T>
__device__ __forceinline__ T ld(double x);
template <>
__device__ __forceinline__ double ld<double>(double x) { return x; }
template <>
__device__ __forceinline__ dd ld<dd>(double x) { return dd_split(x); }
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(dd x) { return dd_join(x); }

}  // namespace fvm
