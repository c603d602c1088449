"""CPU tests of the 3-D LES restatement: geometry invariants of the extruded
O-grid, the test filter, and the two line orders tracking each other."""
import math

import numpy as np
import pytest

import oracle
from fvm_gb300.grid import o_grid_3d, perturbation_3d, read_grid_file_3d, write_grid_file_3d


def _oracle(order=oracle.O3_GPU, skew=0.0, les=True, **kw):
    g = o_grid_3d(16, 12, 8, lz=math.pi, dr1=0.01, skew=skew)
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=3900.0, dt=0.002, order=order, resimax=1e-10, nswpp=4000,
                        use_les=les, ref_a=math.pi, **kw)
    o.set_grid(g)
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, 0.05, 1)
    o.init(du, dv, dw)
    return g, o


def test_jacobian_sums_to_the_annulus_volume():
    g, o = _oracle()
    J = o.array("DJAC")[1:g.nk, 1:g.nj, 1:g.ni]
    assert (J > 0).all()
    # cell volumes of the 16-sided polygonal annulus times the span, within the
    # accuracy of the centred metric differences on this coarse grid
    poly = 0.5 * 16 * math.sin(2 * math.pi / 16) * (50.0 ** 2 - 0.5 ** 2) * math.pi
    assert abs(J.sum() / poly - 1.0) < 0.15


def test_polar_grid_is_orthogonal_and_spanwise_uniform():
    g, o = _oracle()
    # xi is radial, zeta is spanwise: no xi or eta dependence of z and vice versa
    assert np.max(np.abs(o.array("XIZ")[1:g.nk, 1:g.nj, 1:g.ni])) < 1e-12
    assert np.max(np.abs(o.array("ZTX")[1:g.nk, 1:g.nj, 1:g.ni])) < 1e-12
    zt = o.array("ZTZ")[1:g.nk, 1:g.nj, 1:g.ni]
    assert np.allclose(zt, (g.nk - 1) / math.pi, rtol=1e-9)     # 1 / (dz per index)


def test_grid_file_round_trip(tmp_path):
    g = o_grid_3d(8, 6, 4, lz=1.5)
    path = tmp_path / "g.dat"
    write_grid_file_3d(str(path), g)
    h = read_grid_file_3d(str(path), g.ni, g.nj, g.nk)
    assert np.array_equal(h.xg, g.xg) and np.array_equal(h.zg, g.zg)


def test_orders_track_each_other():
    _, a = _oracle(oracle.O3_FAITHFUL, skew=0.3)
    _, b = _oracle(oracle.O3_GPU, skew=0.3)
    a.step(3)
    b.step(3)
    for nm in ("U", "V", "W"):
        x, y = a.array(nm), b.array(nm)
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 2e-2, nm
    assert abs(a.coeffs()["cd"] - b.coeffs()["cd"]) < 0.05 * abs(b.coeffs()["cd"])


def test_dynamic_coefficient_is_positive_and_small():
    _, o = _oracle(skew=0.2)
    o.step(2)
    c = o.coeffs()
    assert 0.0 < c["cs2"] < 0.1 and np.isfinite(c["ct2"])
