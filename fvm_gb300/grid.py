"""O-grid generator and the reference's grid-file format.

The reference reads node coordinates from ``NNNxMMM.dat`` (one ``XG YG`` pair
per line, I fastest, I = 1..NI radial from the wall, J = 1..NJ circumferential;
cylinder/cylinder_v3.0.3_AF_original 4step_face_nl/grid.f90:28-43) but ships no
grid file, so the cases are generated here: a circle of diameter 1 (wall radius
0.5), geometric radial stretching from a given first spacing to a given outer
radius, uniform spacing in theta with J increasing counter-clockwise from the
downstream axis (theta = 0 at J = 1, so the branch cut lies on the wake
centreline as the reference's base-pressure probe PG(1,1) assumes,
calccoef.f90:43-45).  Node J = NJ coincides exactly with node J = 1.

Arrays use the reference storage: (NI+1)*(NJ+1) doubles, element (i, j) at
i + (NI+1)*j; as numpy arrays they are shaped (NJ+1, NI+1) so that a[j, i] is
the reference's (I, J).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def stretch_ratio(n_cells: int, dr1: float, r_in: float, r_out: float) -> float:
    """Geometric ratio q with r_in + dr1*(q**n - 1)/(q - 1) = r_out (bisection)."""
    span = r_out - r_in
    if n_cells * dr1 >= span:
        raise ValueError("first spacing too large for the requested outer radius")

    def reach(q: float) -> float:
        if abs(q - 1.0) < 1e-15:
            return n_cells * dr1
        return dr1 * (q ** n_cells - 1.0) / (q - 1.0)

    lo, hi = 1.0, 2.0
    while reach(hi) < span:
        hi *= 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if reach(mid) < span:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


@dataclass
class OGrid:
    ni: int              # reference NI (radial node count)
    nj: int              # reference NJ (circumferential node count, NJ = 1 + cells)
    xg: np.ndarray       # (NJ+1, NI+1) node x, valid for i=1..NI, j=1..NJ
    yg: np.ndarray
    ratio: float         # radial stretching ratio
    r: np.ndarray        # node radii r[1..NI] (index 0 unused)

    @property
    def cells(self) -> int:
        return (self.ni - 1) * (self.nj - 1)

    def flat(self):
        """Node arrays flattened in the reference storage order."""
        return np.ascontiguousarray(self.xg).ravel(), np.ascontiguousarray(self.yg).ravel()


def o_grid(n_theta: int, n_r: int, r_in: float = 0.5, r_out: float = 50.0,
           dr1: float = 0.005, skew: float = 0.0) -> OGrid:
    """Generate an O-grid with n_theta x n_r cells.

    skew (in units of one theta spacing) rotates each node ring by
    skew*dtheta*sin(pi*(r - r_in)/(r_out - r_in)); 0 gives the orthogonal polar
    grid, non-zero values make the cross-derivative (Q12) terms non-trivial for
    tests.
    """
    if n_theta < 4 or n_r < 4:
        raise ValueError("grid too small")
    ni, nj = n_r + 1, n_theta + 1
    q = stretch_ratio(n_r, dr1, r_in, r_out)
    r = np.zeros(ni + 1)
    r[1] = r_in
    for i in range(1, ni):
        r[i + 1] = r[i] + dr1 * q ** (i - 1)
    dth = 2.0 * math.pi / n_theta
    xg = np.zeros((nj + 1, ni + 1))
    yg = np.zeros((nj + 1, ni + 1))
    for i in range(1, ni + 1):
        rot = skew * dth * math.sin(math.pi * (r[i] - r_in) / (r_out - r_in))
        for j in range(1, nj):
            th = (j - 1) * dth + rot
            xg[j, i] = r[i] * math.cos(th)
            yg[j, i] = r[i] * math.sin(th)
        xg[nj, i] = xg[1, i]
        yg[nj, i] = yg[1, i]
    return OGrid(ni=ni, nj=nj, xg=xg, yg=yg, ratio=q, r=r)


def write_grid_file(path: str, g: OGrid) -> None:
    """Write the reference's NNNxMMM.dat format (grid.f90:35-43)."""
    with open(path, "w") as f:
        for j in range(1, g.nj + 1):
            for i in range(1, g.ni + 1):
                f.write(f"{float(g.xg[j, i])!r} {float(g.yg[j, i])!r}\n")


def read_grid_file(path: str, ni: int, nj: int) -> OGrid:
    """Read a NNNxMMM.dat grid file (I fastest, list-directed pairs)."""
    vals = np.loadtxt(path).reshape(nj, ni, 2)
    xg = np.zeros((nj + 1, ni + 1))
    yg = np.zeros((nj + 1, ni + 1))
    xg[1:, 1:] = vals[:, :, 0]
    yg[1:, 1:] = vals[:, :, 1]
    r = np.zeros(ni + 1)
    r[1:] = np.hypot(xg[1, 1:], yg[1, 1:])
    return OGrid(ni=ni, nj=nj, xg=xg, yg=yg, ratio=float("nan"), r=r)


def grid_file_name(ni: int, nj: int) -> str:
    """The reference's file name 'NNNxMMM.dat' (grid.f90:28-32)."""
    return f"{ni:03d}x{nj:03d}.dat"


def perturbation(ni: int, nj: int, amp: float, seed: int):
    """Seeded uniform(-amp, amp) perturbations of U and V on the interior cells,
    returned as full (NJ+1, NI+1) arrays (zero on ghost cells).  Both the GPU
    path and the CPU restatement read these same host arrays."""
    rng = np.random.default_rng(seed)
    du = np.zeros((nj + 1, ni + 1))
    dv = np.zeros((nj + 1, ni + 1))
    du[1:nj, 1:ni] = amp * rng.uniform(-1.0, 1.0, size=(nj - 1, ni - 1))
    dv[1:nj, 1:ni] = amp * rng.uniform(-1.0, 1.0, size=(nj - 1, ni - 1))
    return du, dv


class OGrid3D:
    """Extruded O-grid: node arrays shaped (NK+1, NJ+1, NI+1), node (i,j,k) at
    [k, j, i] for i=1..NI, j=1..NJ, k=1..NK (index 0 unused), i.e. the reference
    storage (0:NI,0:NJ,0:NK) in Fortran order when flattened."""

    def __init__(self, ni, nj, nk, xg, yg, zg, lz):
        self.ni, self.nj, self.nk = ni, nj, nk
        self.xg, self.yg, self.zg = xg, yg, zg
        self.lz = lz

    @property
    def cells(self) -> int:
        return (self.ni - 1) * (self.nj - 1) * (self.nk - 1)

    @property
    def shape(self):
        return (self.nk + 1, self.nj + 1, self.ni + 1)


def o_grid_3d(n_theta: int, n_r: int, n_z: int, lz: float = math.pi, r_in: float = 0.5, r_out: float = 50.0,
              dr1: float = 0.001, skew: float = 0.0) -> OGrid3D:
    """The 2-D O-grid law extruded over n_z spanwise cells of length lz (z of node
    k is lz*(k-1)/n_z, as the reference's grid generator lays out the span)."""
    g = o_grid(n_theta, n_r, r_in=r_in, r_out=r_out, dr1=dr1, skew=skew)
    nk = n_z + 1
    shape = (nk + 1, g.nj + 1, g.ni + 1)
    xg, yg, zg = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    for k in range(1, nk + 1):
        xg[k] = g.xg
        yg[k] = g.yg
        zg[k, 1:, 1:] = lz * (k - 1) / n_z
    return OGrid3D(g.ni, g.nj, nk, xg, yg, zg, lz)


def write_grid_file_3d(path: str, g: OGrid3D) -> None:
    """The reference's NNNxMMMxKKK.dat format (grid.f90:52-66): one x y z triple
    per record, I fastest, then J, then K."""
    with open(path, "w") as f:
        for k in range(1, g.nk + 1):
            for j in range(1, g.nj + 1):
                for i in range(1, g.ni + 1):
                    f.write(f"{float(g.xg[k, j, i])!r} {float(g.yg[k, j, i])!r} {float(g.zg[k, j, i])!r}\n")


def read_grid_file_3d(path: str, ni: int, nj: int, nk: int, lz: float = float("nan")) -> OGrid3D:
    vals = np.loadtxt(path).reshape(nk, nj, ni, 3)
    shape = (nk + 1, nj + 1, ni + 1)
    xg, yg, zg = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    xg[1:, 1:, 1:] = vals[..., 0]
    yg[1:, 1:, 1:] = vals[..., 1]
    zg[1:, 1:, 1:] = vals[..., 2]
    return OGrid3D(ni, nj, nk, xg, yg, zg, lz)


def grid_file_name_3d(ni: int, nj: int, nk: int) -> str:
    """'NNNxMMMxKKK.dat' (grid.f90:46-50)."""
    return f"{ni:03d}x{nj:03d}x{nk:03d}.dat"


def perturbation_3d(ni: int, nj: int, nk: int, amp: float, seed: int):
    """Seeded uniform(-amp, amp) perturbations of U, V, W on the interior cells
    (full (NK+1, NJ+1, NI+1) arrays, zero on ghost cells)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(3):
        a = np.zeros((nk + 1, nj + 1, ni + 1))
        a[1:nk, 1:nj, 1:ni] = amp * rng.uniform(-1.0, 1.0, size=(nk - 1, nj - 1, ni - 1))
        out.append(a)
    return tuple(out)
