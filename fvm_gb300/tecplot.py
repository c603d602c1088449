"""Tecplot ASCII files in the layouts the reference writes, for viewing a run the
way the reference's output is viewed.  Host-side only: the arrays come from
`Context.get` / `post_final` (2-D) or `Context3.get` / `post_get` (3-D).

2-D (R2D): the cell-centre file of WRITEDATA (writedata.f90:56-70, `NNNN_CENT.PLT`)
and the time-averaged field of POST_PROCESS (post_process.f90:38-48,
`TIME-AVERAGED FIELD.PLT`): x, y, u, v, P, vorticity, T for J = 0..NJ, I = 0..NI.

3-D (RLES, post_process.f90:120-278): the averaged field (`Avrg000.PLT`: x, y, z, p,
u, v, w, T), the rms field (`Urms000.PLT`) and the Reynolds stresses
(`Strs000.PLT`: uu, uv, uw, vv, vw, ww) at the grid nodes I = 1..NI, J = 1..NJ,
K = 1..NK as the mean of the 8 cells around each node, and the wall file
(`Surf000.PLT`: x, y, z, theta, Cf, Cp, Nu at the wall cells).

Arrays: a[j, i] (2-D), a[k, j, i] (3-D), as elsewhere in this package.
"""
from __future__ import annotations

import numpy as np


def _d169(x: float) -> str:
    """Fortran D16.9: 0.ddddddddD+xx right-justified in 16 columns."""
    x = float(x)
    if x == 0.0:
        return "0.000000000D+00".rjust(16)
    s = f"{abs(x):.8e}"
    digits, e = s.split("e")
    mant = "0." + digits.replace(".", "")
    exp = int(e) + 1
    es = f"D{'+' if exp >= 0 else '-'}{abs(exp):02d}" if abs(exp) <= 99 else f"{'+' if exp >= 0 else '-'}{abs(exp):03d}"
    return (("-" if x < 0 else "") + mant + es).rjust(16)


def _row(values) -> str:
    return "".join(" " + _d169(v) for v in values)


def _ld(x) -> str:
    """A list-directed real (17 significant digits)."""
    return f"{float(x):.17G}"


def write_cell_file_2d(path, x, y, u, v, p, vor, t, rtime, re, pr):
    """The cell-centre file of writedata.f90:56-70."""
    nj1, ni1 = np.asarray(u).shape
    lines = [f' TITLE="RE {_ld(re)} PR {_ld(pr)}"', " variables=x,y,u,v,P,Vorticity,T",
             f' ZONE T="WHOLE", I={ni1:6d}, j={nj1:6d}, SOLUTIONTIME={rtime:10.4f}']
    cols = [np.asarray(a, dtype=np.float64) for a in (x, y, u, v, p, vor, t)]
    for j in range(nj1):
        for i in range(ni1):
            lines.append(" " + " ".join(_ld(a[j, i]) for a in cols))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_averaged_file_2d(path, x, y, avg: dict, rtime):
    """TIME-AVERAGED FIELD.PLT of post_process.f90:38-48 from post_final()'s fields."""
    nj1, ni1 = np.asarray(avg["U"]).shape
    lines = [' title=""', " variables=x,y,u,v,P,Vorticity,T", f' zone t="{_ld(rtime)}",i={ni1},j={nj1}']
    cols = [np.asarray(a, dtype=np.float64) for a in (x, y, avg["U"], avg["V"], avg["P"], avg["VOR"], avg["T"])]
    for j in range(nj1):
        for i in range(ni1):
            lines.append(" " + " ".join(_ld(a[j, i]) for a in cols))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def nodal(a):
    """Node values of a cell array: 0.125 x the 8 cells around node (i, j, k),
    i = 1..NI, j = 1..NJ, k = 1..NK (post_process.f90:120-132), shaped (NK, NJ, NI)."""
    a = np.asarray(a, dtype=np.float64)
    c = a[1:, 1:, 1:]
    return 0.125 * (((((((c + a[1:, :-1, 1:]) + a[1:, 1:, :-1]) + a[1:, :-1, :-1]) + a[:-1, 1:, 1:]) +
                      a[:-1, :-1, 1:]) + a[:-1, 1:, :-1]) + a[:-1, :-1, :-1])


def _write_nodal_3d(path, xg, yg, zg, cols, names, rtime, re, pr):
    nk1, nj1, ni1 = np.asarray(xg).shape
    ni, nj, nk = ni1 - 1, nj1 - 1, nk1 - 1
    lines = [f' TITLE="RE {_ld(re)} PR {_ld(pr)}"', " variables=" + ",".join(names),
             f' ZONE T="WHOLE", I={ni:6d}, J={nj:6d}, K={nk:6d}, SOLUTIONTIME={rtime:10.4f}']
    nod = [nodal(a) for a in cols]
    for k in range(1, nk + 1):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                lines.append(_row([xg[k, j, i], yg[k, j, i], zg[k, j, i]] + [a[k - 1, j - 1, i - 1] for a in nod]))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_averaged_files_3d(prefix, g, post: dict, rtime, re, pr):
    """Avrg000.PLT, Urms000.PLT and Strs000.PLT (post_process.f90:133-240) from the
    arrays of `Context3.post_get` (keys as its names).  prefix: a directory."""
    import os
    _write_nodal_3d(os.path.join(prefix, "Avrg000.PLT"), g.xg, g.yg, g.zg,
                    [post[k] for k in ("P_AVG", "U_AVG", "V_AVG", "W_AVG", "T_AVG")],
                    ["x", "y", "z", "p", "u", "v", "w", "T"], rtime, re, pr)
    _write_nodal_3d(os.path.join(prefix, "Urms000.PLT"), g.xg, g.yg, g.zg,
                    [post[k] for k in ("U_RMS", "V_RMS", "W_RMS")], ["x", "y", "z", "u_rms", "v_rms", "w_rms"],
                    rtime, re, pr)
    _write_nodal_3d(os.path.join(prefix, "Strs000.PLT"), g.xg, g.yg, g.zg,
                    [post[k] for k in ("UU", "UV", "UW", "VV", "VW", "WW")],
                    ["x", "y", "z", "uu", "uv", "uw", "vv", "vw", "ww"], rtime, re, pr)


def write_wall_file_3d(path, x, y, z, theta, cf, cp, nu):
    """Surf000.PLT (post_process.f90:256-278): the wall cells (1, j, k),
    j = 1..NJ-1, k = 1..NK-1; cf, cp, nu shaped (NK+1, NJ+1) as post_get returns."""
    nk1, nj1 = np.asarray(cf).shape
    lines = [' TITLE="SURFACE COEF."', ' variables="x","y","z","Theta","Cf","Cp","Nu"',
             f' ZONE T="POST", I={1:6d}, j={nj1 - 2:6d}, k={nk1 - 2:6d}']
    for k in range(1, nk1 - 1):
        for j in range(1, nj1 - 1):
            lines.append(_row([x[k, j, 1], y[k, j, 1], z[k, j, 1], theta[k, j, 1], cf[k, j], cp[k, j], nu[k, j]]))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_rows(path, skip=3):
    """The numeric rows of a file written above (D exponents read as E)."""
    rows = []
    with open(path) as fh:
        for q, line in enumerate(fh):
            if q < skip:
                continue
            rows.append([float(t.replace("D", "E")) for t in line.split()])
    return np.array(rows)
