"""The conversions of the double-float arithmetic (fvm_gb300/csrc/fvm_df.cuh)
restated with numpy bit operations, to check the exponent offsets and the special
cases of the device formulas on the CPU: the split of a double into hi + lo FP32
values without a conversion instruction (hi the truncation to 24 bits, lo the next
23 fraction bits as (1.m) s - s with s = 2^(e - 1046)), and the exact FP32 -> FP64
conversion with integer operations.  The device code itself is checked end to end
by the mixed-path GPU tests (the SGS model and full steps against the oracle)."""
import numpy as np


def split(x):
    """dd_split of fvm_df.cuh on an array of doubles: (hi, lo) float32 arrays."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    b = x.view(np.uint64)
    hw = (b >> np.uint64(32)).astype(np.uint32)
    lw = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    sign = hw & np.uint32(0x80000000)
    ah = hw & np.uint32(0x7FFFFFFF)
    e = ah >> np.uint32(20)
    # __funnelshift_r(lw, ah - (896 << 20), 29): low word of ((hi:lo) >> 29)
    hi_word = (ah - np.uint32(896 << 20)).astype(np.uint64)
    hb = (((hi_word << np.uint64(32)) | lw.astype(np.uint64)) >> np.uint64(29)).astype(np.uint32)
    one_m = (np.uint32(0x3F800000) | ((lw >> np.uint32(6)) & np.uint32(0x7FFFFF))).view(np.float32)
    sc = ((e - np.uint32(919)) << np.uint32(23)).astype(np.uint32).view(np.float32)
    with np.errstate(all="ignore"):
        # fmaf(one_m, sc, -sc): exact in float64 and representable in float32
        lo_val = (one_m.astype(np.float64) * sc.astype(np.float64) - sc.astype(np.float64)).astype(np.float32)
    lb = lo_val.view(np.uint32).copy()
    lb[e < 949] = 0
    hb = hb.copy()
    hb[e < 897] = 0
    big = e > 1150
    nan = (e == 2047) & (((ah & np.uint32(0xFFFFF)) | lw) != 0)
    hb[big] = np.where(nan[big], np.uint32(0x7FC00000), np.uint32(0x7F800000))
    lb[big] = 0
    return (hb | sign).view(np.float32), (lb | sign).view(np.float32)


def f2d_int(f):
    """f2d_int of fvm_df.cuh: float32 -> float64 bits with integer operations."""
    u = np.ascontiguousarray(f, dtype=np.float32).view(np.uint32)
    ex = (u >> np.uint32(23)) & np.uint32(0xFF)
    m = u & np.uint32(0x7FFFFF)
    dex = np.where(ex == 0xFF, np.uint32(0x7FF), ex + np.uint32(896)).astype(np.uint32)
    s = u & np.uint32(0x80000000)
    hi = np.where(ex == 0, s, s | (dex << np.uint32(20)) | (m >> np.uint32(3))).astype(np.uint64)
    lo = np.where(ex == 0, np.uint32(0), m << np.uint32(29)).astype(np.uint64)
    return ((hi << np.uint64(32)) | lo).view(np.float64)


def test_split_reconstructs_to_46_bits_over_the_handled_range():
    rng = np.random.default_rng(11)
    n = 200000
    exps = rng.integers(-74, 127, n)
    mant = rng.uniform(1.0, 2.0, n)
    x = np.ldexp(mant, exps) * rng.choice([-1.0, 1.0], n)
    hi, lo = split(x)
    back = hi.astype(np.float64) + lo.astype(np.float64)
    assert np.all(np.abs(back - x) <= np.ldexp(np.abs(x), -46))
    # hi is the truncation: same sign, not larger in magnitude, within 2^-23
    assert np.all(np.sign(hi) == np.sign(x))
    assert np.all(np.abs(hi.astype(np.float64)) <= np.abs(x))
    assert np.all(np.abs(x - hi) <= np.ldexp(np.abs(x), -23))


def test_split_special_magnitudes():
    x = np.array([0.0, -0.0, 1.0, -2.5, 2.0 ** -74, 2.0 ** -80, 3.0 * 2.0 ** -120, 1e-40, 1e-300, 2.0 ** 127 * 1.5,
                  1e39, -1e300, np.inf, -np.inf, np.nan])
    hi, lo = split(x)
    assert hi[0] == 0.0 and lo[0] == 0.0 and hi[1] == 0.0
    assert (hi[2], lo[2]) == (1.0, 0.0) and (hi[3], lo[3]) == (-2.5, 0.0)
    assert hi[4] == np.float32(2.0 ** -74)
    # below 2^-74 only hi (exact here), below 2^-126 zero
    assert hi[5] == np.float32(2.0 ** -80) and lo[5] == 0.0
    assert hi[6] == np.float32(3.0 * 2.0 ** -120) and lo[6] == 0.0
    assert hi[7] == 0.0 and hi[8] == 0.0
    assert hi[9] == np.float32(2.0 ** 127 * 1.5)
    assert np.isposinf(hi[10]) and np.isneginf(hi[11]) and np.isposinf(hi[12]) and np.isneginf(hi[13])
    assert np.isnan(hi[14])


def test_integer_float_to_double_is_exact():
    rng = np.random.default_rng(12)
    f = (rng.standard_normal(100000) * np.exp(rng.uniform(-80, 80, 100000))).astype(np.float32)
    f = f[np.isfinite(f) & (np.abs(f) >= np.finfo(np.float32).tiny)]
    assert np.array_equal(f2d_int(f), f.astype(np.float64))
    special = np.array([0.0, -0.0, np.inf, -np.inf, 1e-42], dtype=np.float32)   # 1e-42 is subnormal
    d = f2d_int(special)
    assert d[0] == 0.0 and np.signbit(d[1]) and np.isposinf(d[2]) and np.isneginf(d[3]) and d[4] == 0.0
    assert np.isnan(f2d_int(np.array([np.nan], dtype=np.float32)))[0]
