// fvm_ops.cuh -- cell operators of the reference step routines, shared by the
// FP64 and mixed-precision translation units.
#pragma once

#include "fvm_internal.cuh"

namespace fvm {

// ---------------------------------------------------------------------------------
// Cell operators (shared by the per-routine and the fused kernels)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double nl_at(const Dev &d, const double *in, int i, int j)
{   // NL (nl.f90:21-27)
    int c = IDX(i, j);
    double t1 = (d.UE[c] * 0.5) * (in[c] + in[IDX(i + 1, j)]);
    double t2 = (d.UW[c] * 0.5) * (in[c] + in[IDX(i - 1, j)]);
    double t3 = (d.VN[c] * 0.5) * (in[c] + in[IDX(i, j + 1)]);
    double t4 = (d.VS[c] * 0.5) * (in[c] + in[IDX(i, j - 1)]);
    return ((t1 - t2) + t3) - t4;
}

// Cross-derivative term 0.25*sum(+-K*(diagonal differences)) with K = coefficient
// array evaluated at the four face neighbours (dif_diagonal.f90:13-23 with K=J*Q12;
// iter_u.f90:31-41 with K=J*xix*etx and K=J*xiy*ety).
__device__ __forceinline__ double cross_at(const Dev &d, const double *K, const double *f, int i, int j)
{
    double fne = f[IDX(i + 1, j + 1)], fse = f[IDX(i + 1, j - 1)];
    double fnw = f[IDX(i - 1, j + 1)], fsw = f[IDX(i - 1, j - 1)];
    double t1 = K[IDX(i + 1, j)] * (fne - fse);
    double t2 = K[IDX(i - 1, j)] * (fnw - fsw);
    double t3 = K[IDX(i, j + 1)] * (fne - fnw);
    double t4 = K[IDX(i, j - 1)] * (fse - fsw);
    return 0.25 * (((t1 - t2) + t3) - t4);
}

// Cross term that DIF adds to cell (i,j).  DIF adds the whole array DD(0:NI,0:NJ)
// to an expression over the section (1:NI-1,1:NJ-1) (dif.f90:15-23); compiled
// code pairs the two element by element by position, so cell (i,j) receives the
// term of cell (i-1,j-1), and zero on row 1 / column 1 (DD's row 0 and column 0
// are never written).  dd_pos = 0 gives the cell's own term.
__device__ __forceinline__ double dif_cross(const Dev &d, const double *in, int i, int j)
{
    if (!d.dd_pos) return cross_at(d, d.JQ12, in, i, j);
    return (i > 1 && j > 1) ? cross_at(d, d.JQ12, in, i - 1, j - 1) : 0.0;
}

__device__ __forceinline__ double dif_at(const Dev &d, const double *in, int i, int j)
{   // DIF (dif.f90:13-23)
    int c = IDX(i, j);
    double dd = dif_cross(d, in, i, j);
    double p = in[c];
    double a = d.DE[c] * (in[IDX(i + 1, j)] - p);
    double b = d.DW[c] * (in[IDX(i - 1, j)] - p);
    double e = d.DN[c] * (in[IDX(i, j + 1)] - p);
    double f = d.DS[c] * (in[IDX(i, j - 1)] - p);
    return (((a + b) + e) + f) + dd;
}

__device__ __forceinline__ void psource_at(const Dev &d, int i, int j, double &su, double &sv)
{   // P_SOURCE (p_source.f90:9-27); P ghost values are read as stored
    const double *J = d.DJAC, *P = d.P;
    int e = IDX(i + 1, j), w = IDX(i - 1, j), nn = IDX(i, j + 1), s = IDX(i, j - 1);
    double a = ((((J[e] * d.XIX[e]) * P[e] - (J[w] * d.XIX[w]) * P[w]) + (J[nn] * d.ETX[nn]) * P[nn]) - (J[s] * d.ETX[s]) * P[s]);
    double b = ((((J[e] * d.XIY[e]) * P[e] - (J[w] * d.XIY[w]) * P[w]) + (J[nn] * d.ETY[nn]) * P[nn]) - (J[s] * d.ETY[s]) * P[s]);
    su = -(0.5 * a);
    sv = -(0.5 * b);
}

__device__ __forceinline__ double u1_at(const Dev &d, int c) { return d.XIX[c] * d.U[c] + d.XIY[c] * d.V[c]; }
__device__ __forceinline__ double u2_at(const Dev &d, int c) { return d.ETX[c] * d.U[c] + d.ETY[c] * d.V[c]; }

// Predictor right-hand side of the first AF factor (iter_u.f90:31-46) with the
// wall/far-field folding of BCU (bcu.f90:15, 35).
__device__ __forceinline__ double af_su1_at(const Dev &d, int kind, const double *phi, const double *phin,
                                            const double *nl, const double *nlm1, const double *dif,
                                            const double *src, int i, int j)
{
    int c = IDX(i, j);
    const bool tk = (kind == FVM_FIELD_T);
    const double rek = tk ? d.pe : d.re;
    const double *JDT = tk ? d.PJDT : d.RJDT;
    double s = (JDT[c] * phin[c] - (3.0 * rek) * nl[c]) + rek * nlm1[c];
    s = s + dif[c];
    if (!tk) s = s + (2.0 * rek) * src[c];
    s = s + cross_at(d, d.JXE, phi, i, j);
    const Coef &cf = tk ? d.cTX : d.cUX;
    if (i == 1) {
        double w = (kind == FVM_FIELD_U) ? d.UFW[j] : (kind == FVM_FIELD_V ? d.VFW[j] : d.TFW[j]);
        s = s + (2.0 * cf.awall[j]) * w;
    }
    if (i == d.NI - 1) {
        double f = (kind == FVM_FIELD_U) ? d.FFU[j] : (kind == FVM_FIELD_V ? d.FFV[j] : d.FFT[j]);
        s = s + (2.0 * cf.afar[j]) * f;
    }
    return s;
}

struct FieldRefs {
    double *phi, *phin, *nl, *nlm1, *dif, *src, *su;
    const double *wallF, *farF;
};

__device__ __forceinline__ FieldRefs field_refs(const Dev &d, int kind)
{
    if (kind == FVM_FIELD_U) return {d.U, d.U_N, d.NLX, d.NLX_NM1, d.DIFX, d.S_U, d.SU, d.UFW, d.FFU};
    if (kind == FVM_FIELD_V) return {d.V, d.V_N, d.NLY, d.NLY_NM1, d.DIFY, d.S_V, d.SUV, d.VFW, d.FFV};
    return {d.T, d.T_N, d.ADV, d.ADV_NM1, d.DIFT, nullptr, d.SUT, d.TFW, d.FFT};
}


enum { BCK_DIRICHLET = 0, BCK_POISSON = 1 };

// Ghost values of radial row j computed from the interior of src and written into
// dst (the BC call that precedes a sweep in the reference: BCU before
// iter_u.f90:50, BCP before iter_p.f90:34): dst(0,j), dst(NI,j) and, for
// j = 1 / NJ-1, the branch-cut row NJ / 0 with its corners.
template <int BCK>
__device__ void refresh_row_ghosts(const Dev &d, const double *src, double *dst, int j, const double *wallF,
                                   const double *farF, int lane)
{
    const int NI = d.NI, NJ = d.NJ;
    double g0, gn;
    if (BCK == BCK_POISSON) {
        g0 = src[IDX(1, j)];
        gn = (3.0 * src[IDX(NI - 1, j)] - 3.0 * src[IDX(NI - 2, j)]) + src[IDX(NI - 3, j)];
    } else {
        g0 = (-src[IDX(1, j)]) + 2.0 * wallF[j];
        gn = (-src[IDX(NI - 1, j)]) + 2.0 * farF[j];
    }
    int rowdst = (j == 1) ? NJ : ((j == NJ - 1) ? 0 : -1);
    if (rowdst >= 0) {
        for (int i = 1 + lane; i <= NI - 1; i += WARP) dst[IDX(i, rowdst)] = src[IDX(i, j)];
    }
    if (lane == 0) {
        dst[IDX(0, j)] = g0;
        dst[IDX(NI, j)] = gn;
        if (rowdst >= 0) {
            dst[IDX(0, rowdst)] = g0;
            dst[IDX(NI, rowdst)] = gn;
        }
    }
}

// Lagged Poisson cross term (dif_diagonal.f90:13-23) from the gathered weights.
__device__ __forceinline__ double dd_p(const Dev &d, const double *P, int i, int j)
{
    int c = IDX(i, j);
    return ((d.CNE[c] * P[IDX(i + 1, j + 1)] + d.CSE[c] * P[IDX(i + 1, j - 1)]) + d.CNW[c] * P[IDX(i - 1, j + 1)])
           + d.CSW[c] * P[IDX(i - 1, j - 1)];
}

// Cross term that ITER_P subtracts from the source of cell (i,j): the same
// positional pairing as DIF (iter_p.f90:27-30), cell (i-1,j-1) or zero.
__device__ __forceinline__ double dd_src(const Dev &d, const double *P, int i, int j)
{
    if (!d.dd_pos) return dd_p(d, P, i, j);
    return (i > 1 && j > 1) ? dd_p(d, P, i - 1, j - 1) : 0.0;
}

// Cross-warp part of a block sum: lane 0 of every warp holds its warp's sums; warp 0
// folds them in a fixed order (the block's sums end on thread 0).
__device__ __forceinline__ void block_fold2(double &a, double &b, double *sh)
{
    const int wid = threadIdx.x / WARP, lane = threadIdx.x & 31, nw = blockDim.x / WARP;
    __syncthreads();
    if (lane == 0) { sh[2 * wid] = a; sh[2 * wid + 1] = b; }
    __syncthreads();
    if (wid == 0) {
        a = lane < nw ? sh[2 * lane] : 0.0;
        b = lane < nw ? sh[2 * lane + 1] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
    }
}

// Deterministic block sum of two values (fixed shuffle tree, then warp 0).
__device__ __forceinline__ void block_sum2(double &a, double &b, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    block_fold2(a, b, sh);
}

// Publish thread 0's block sums and, in the last block to arrive (of nblk blocks),
// reduce all partials in a fixed order.  Returns true in the last block (sums in
// a, b on thread 0).
__device__ __forceinline__ bool grid_publish2(const Dev &d, double &a, double &b, double *sh, bool &last, int nblk)
{
    if (threadIdx.x == 0) {
        d.partial[2 * blockIdx.x] = a;
        d.partial[2 * blockIdx.x + 1] = b;
        __threadfence();
        const unsigned nb = (unsigned)nblk;
        unsigned t = atomicInc(&d.pctl->ticket, nb - 1);
        last = (t == nb - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    // partial k in thread k mod blockDim, in increasing k; four loads in flight per
    // thread (L2 only: the partials were written by other SMs)
    a = 0.0;
    b = 0.0;
    const double2 *pp = reinterpret_cast<const double2 *>(d.partial);
    for (int k0 = threadIdx.x; k0 < nblk; k0 += 4 * blockDim.x) {
        double2 x[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int k = k0 + r * (int)blockDim.x;
            x[r] = k < nblk ? __ldcg(pp + k) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            if (k0 + r * (int)blockDim.x < nblk) {
                a += x[r].x;
                b += x[r].y;
            }
        }
    }
    block_sum2(a, b, sh);
    return true;
}

// Grid sum of two FP64 values per thread (see grid_publish2).
__device__ __forceinline__ bool grid_sum2(const Dev &d, double &a, double &b, double *sh, bool &last, int nblk)
{
    block_sum2(a, b, sh);
    return grid_publish2(d, a, b, sh, last, nblk);
}

// Block sum of two FP32 values per thread: summed in FP32 within the warp (fixed
// tree), in FP64 from there on (sums on thread 0).  For norms that only need a few
// digits.
__device__ __forceinline__ void block_sum2f(float af, float bf, double &a, double &b, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        af += __shfl_down_sync(0xffffffffu, af, o);
        bf += __shfl_down_sync(0xffffffffu, bf, o);
    }
    a = (double)af;
    b = (double)bf;
    block_fold2(a, b, sh);
}

// Grid sum of two FP32 values per thread (block_sum2f, then grid_publish2).
__device__ __forceinline__ bool grid_sum2f(const Dev &d, float af, float bf, double &a, double &b, double *sh,
                                           bool &last, int nblk)
{
    block_sum2f(af, bf, a, b, sh);
    return grid_publish2(d, a, b, sh, last, nblk);
}

// The sums grid_publish2's last block forms, formed by any block of at least 256
// threads from partials another kernel left: thread k < 256 adds partials k, k+256,
// ... in increasing order, threads from 256 on contribute zero (which leaves the
// shuffle trees' sums unchanged), then block_sum2.  Same bits as grid_publish2 with
// 256-thread blocks.
__device__ __forceinline__ void sum_partials256(const double *partial, int nblk, double &a, double &b, double *sh)
{
    a = 0.0;
    b = 0.0;
    if (threadIdx.x < 256) {
        const double2 *pp = reinterpret_cast<const double2 *>(partial);
        for (int k0 = threadIdx.x; k0 < nblk; k0 += 4 * 256) {
            double2 x[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int k = k0 + r * 256;
                x[r] = k < nblk ? __ldcg(pp + k) : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int r = 0; r < 4; r++) {
                if (k0 + r * 256 < nblk) {
                    a += x[r].x;
                    b += x[r].y;
                }
            }
        }
    }
    block_sum2(a, b, sh);
}

// A case's Poisson iteration has ended (converged or capped).  Inside a batch the
// case leaves the count of running cases; the device-side loop ends with the last.
// Once per loop body (case 0, first thread of the residual kernel): a batch's
// device-side loop ends after max_bodies bodies whatever the cases report, so a
// lost completion count cannot keep the GPU looping.
template <int HAS_COND>
__device__ __forceinline__ void batch_body_guard(const Dev &d, cudaGraphConditionalHandle cond)
{
    if (!d.bctl || d.case_id != 0 || blockIdx.x != 0 || threadIdx.x != 0) return;
    const int b = d.bctl->bodies + 1;
    d.bctl->bodies = b;
    if (b > d.bctl->max_bodies) {
        d.bctl->overrun = 1;
        if (HAS_COND) cudaGraphSetConditional(cond, 0);
    }
}

template <int HAS_COND>
__device__ __forceinline__ void poisson_finished(const Dev &d, cudaGraphConditionalHandle cond)
{
    bool last = true;
    if (d.bctl) last = atomicSub(&d.bctl->remaining, 1) == 1;
    if (HAS_COND && last) cudaGraphSetConditional(cond, 0);
}

// Line system, coefficients, right-hand side, field and boundary values of one
// predictor factor of a field (dir 0: radial lines of the first factor, 1:
// circumferential lines of the second).
struct PredLine {
    LineSys s;
    Coef cf;
    const double *SU;
    double *phi;
    const double *wallF, *farF;
};

__device__ __forceinline__ PredLine pred_line(const Dev &d, int field, int dir)
{
    const bool tk = field == FVM_FIELD_T;
    PredLine L;
    L.s = dir == 0 ? (tk ? d.sTX : d.sUX) : (tk ? d.sTY : d.sUY);
    L.cf = dir == 0 ? (tk ? d.cTX : d.cUX) : (tk ? d.cTY : d.cUY);
    L.phi = field == FVM_FIELD_U ? d.U : (field == FVM_FIELD_V ? d.V : d.T);
    L.SU = field == FVM_FIELD_U ? d.SU : (field == FVM_FIELD_V ? d.SUV : d.SUT);
    L.wallF = field == FVM_FIELD_U ? d.UFW : (field == FVM_FIELD_V ? d.VFW : d.TFW);
    L.farF = field == FVM_FIELD_U ? d.FFU : (field == FVM_FIELD_V ? d.FFV : d.FFT);
    return L;
}

// Five-point Poisson residual (iter_p.f90:42-44) of P with the line neighbours
// read through periodic wrap; AE(NI-1)=0 and AW(1)=0 are folded in the coefficients.
__device__ __forceinline__ double pres_at(const Dev &d, const double *P, double su, int i, int j)
{
    const Coef &cf = d.cP;
    int c = IDX(i, j);
    return ((((cf.AE[c] * P[IDX(i + 1, j)] + cf.AW[c] * P[IDX(i - 1, j)]) + cf.AN[c] * P[IDX(i, jwrap(d, j + 1))])
             + cf.AS[c] * P[IDX(i, jwrap(d, j - 1))]) + su) - cf.AP[c] * P[c];
}

}  // namespace fvm
