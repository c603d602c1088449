"""Accuracy of the mixed path's double-float Poisson residual, restated on the CPU.

k_mres (fvm_gb300/csrc/fvm_mixed.cu) evaluates r = (DIVDT - DD(P)) + A5(P) - AP P
with every FP64 operand split into an FP32 pair (dd_split) and the operators of
fvm_df.cuh: TwoSum-based addition and FMA-based TwoProduct, renormalised after each
operation.  Here the same operations run in numpy float32 (round to nearest; the
fused multiply-add of TwoProduct restated in float64, where the float32 product is
exact), on random stencil data with the magnitudes of the benchmark's pressure
equation, and the result is compared with the FP64 residual of the same formula:
the difference stays within 2^-44 of the sum of the terms' magnitudes, far below
any Poisson tolerance (the scaled residual is that sum's fraction).
"""
import numpy as np

from tests.test_doublefloat_split import split

F = np.float32


def fma32(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def fast_two_sum(a, b):
    s = (a + b).astype(F)
    return s, (b - (s - a)).astype(F)


def dd_add(a, b):
    s = (a[0] + b[0]).astype(F)
    v = (s - a[0]).astype(F)
    e = ((a[0] - (s - v)) + (b[0] - v)).astype(F)
    e = (e + (a[1] + b[1])).astype(F)
    return fast_two_sum(s, e)


def dd_neg(a):
    return (-a[0], -a[1])


def dd_mul(a, b):
    p = (a[0] * b[0]).astype(F)
    e = fma32(a[0], b[0], -p)
    e = fma32(a[0], b[1], e)
    e = fma32(a[1], b[0], e)
    return fast_two_sum(p, e)


def test_double_float_residual_is_within_2_pow_minus_44_of_fp64():
    rng = np.random.default_rng(5)
    n = 100000
    # coefficients and pressures of the benchmark's magnitudes: couplings O(1-10),
    # AP their sum, cross weights O(0.1), P O(1) with smooth-field cancellation
    ae, aw, an, as_ = (rng.uniform(0.5, 8.0, n) for _ in range(4))
    ap = ae + aw + an + as_ + rng.uniform(0.0, 1e-3, n)
    cw = [rng.uniform(-0.2, 0.2, n) for _ in range(4)]
    p0 = rng.uniform(-1.0, 1.0, n)
    pn = [p0 + rng.normal(0.0, 1e-3, n) for _ in range(8)]   # neighbours close to the centre
    divdt = rng.normal(0.0, 1e-2, n)

    cross64 = ((cw[0] * pn[4] + cw[1] * pn[5]) + cw[2] * pn[6]) + cw[3] * pn[7]
    r64 = ((((ae * pn[0] + aw * pn[1]) + an * pn[2]) + as_ * pn[3]) + (divdt - cross64)) - ap * p0

    S = lambda x: split(x)
    cross = dd_add(dd_add(dd_add(dd_mul(S(cw[0]), S(pn[4])), dd_mul(S(cw[1]), S(pn[5]))),
                          dd_mul(S(cw[2]), S(pn[6]))), dd_mul(S(cw[3]), S(pn[7])))
    su = dd_add(S(divdt), dd_neg(cross))
    app = dd_mul(S(ap), S(p0))
    r = dd_add(dd_add(dd_add(dd_add(dd_add(dd_mul(S(ae), S(pn[0])), dd_mul(S(aw), S(pn[1]))),
                                    dd_mul(S(an), S(pn[2]))), dd_mul(S(as_), S(pn[3]))), su), dd_neg(app))
    rdf = r[0].astype(np.float64) + r[1].astype(np.float64)

    terms = (np.abs(ae * pn[0]) + np.abs(aw * pn[1]) + np.abs(an * pn[2]) + np.abs(as_ * pn[3])
             + np.abs(divdt) + sum(np.abs(c * q) for c, q in zip(cw, pn[4:])) + np.abs(ap * p0))
    err = np.abs(rdf - r64)
    assert np.all(err <= np.ldexp(terms, -44)), float((err / terms).max())
    # the residual itself is small against its terms (the cancellation the FP64
    # residual guards against): the double-float one keeps ~1e-8 of it or better
    assert np.median(np.abs(r64) / terms) < 1e-2
    assert np.median(err / np.maximum(np.abs(r64), 1e-300)) < 1e-8
