"""Restart files in the reference's formats, so that a run can be handed between
this solver and the reference's Fortran programs.

2-D (R2D/writedata.f90:77-90, read by R2D/init.f90:46-60): list-directed records
    RE, PR, DTIME, VEL_ROT
    RTIME, NITER_TIME
    then for J = 0..NJ, I = 0..NI (I fastest):
    NLX, NLY, ADV
    U, V, P, T

3-D (RLES/writedata.f90:191-215, read by RLES/init.f90:183-205), one file per
rank (RESTART000.DAT for the single rank that owns the whole domain), fixed
format (TR1, E24.16) per field:
    RE, PE, DTIME, RTIME (E24.16), NITER_TIME (I16)
    then for K = 0..NK, J = 0..NJ, I = 0..NI:
    NLX, NLY, NLZ, ADV
    U, V, W, P, T

Arrays use this package's numpy layout: a[j, i] (2-D) and a[k, j, i] (3-D) is
the reference's (I, J[, K]).  E24.16 keeps 16 significant digits, as the
reference writes them; the 2-D writer uses 17, which list-directed input reads
back exactly.
"""
from __future__ import annotations

import math
import re

import numpy as np

STATE_2D = ("NLX", "NLY", "ADV", "U", "V", "P", "T")
STATE_3D = ("NLX", "NLY", "NLZ", "ADV", "U", "V", "W", "P", "T")

_REPEAT = re.compile(r"^(\d+)\*(.*)$")


def _tokens(text: str):
    """Values of list-directed input: separated by blanks, commas or line ends,
    with the r*c repeat form and D exponents."""
    for tok in re.split(r"[\s,]+", text.strip()):
        if not tok:
            continue
        m = _REPEAT.match(tok)
        if m:
            for _ in range(int(m.group(1))):
                yield m.group(2)
        else:
            yield tok


def _num(tok: str) -> float:
    t = tok.upper().replace("D", "E")
    # Ew.d output drops the E when the exponent has three digits: 0.1234-301
    m = re.match(r"^([+-]?\d*\.\d*)([+-]\d{3})$", t)
    if m:
        t = m.group(1) + "E" + m.group(2)
    return float(t)


def format_e(x: float, w: int = 24, d: int = 16) -> str:
    """Fortran Ew.d edit descriptor: 0.ddd...E+xx, right-justified in w columns;
    a three-digit exponent is written without the E (+xxx)."""
    x = float(x)
    if not math.isfinite(x):
        s = "NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")
        return s.rjust(w)
    if x == 0.0:
        mant, exp = "0." + "0" * d, 0
        sign = "-" if math.copysign(1.0, x) < 0 else ""
    else:
        sign = "-" if x < 0 else ""
        a = abs(x)
        # d significant digits, mantissa in [0.1, 1)
        s = f"{a:.{d - 1}e}"
        digits, e = s.split("e")
        digits = digits.replace(".", "")
        exp = int(e) + 1
        mant = "0." + digits
    if abs(exp) <= 99:
        es = f"E{'+' if exp >= 0 else '-'}{abs(exp):02d}"
    else:
        es = f"{'+' if exp >= 0 else '-'}{abs(exp):03d}"
    out = sign + mant + es
    if len(out) > w:
        return "*" * w
    return out.rjust(w)


def write_restart_2d(path, state: dict, re: float, pr: float, dt: float, vel_rot: float, rtime: float,
                     niter_time: int):
    """RESTART.DAT of writedata.f90:77-90 from arrays shaped (NJ+1, NI+1)."""
    a = {nm: np.asarray(state[nm], dtype=np.float64) for nm in STATE_2D}
    nj1, ni1 = a["U"].shape

    def f(x):
        return f"{x:.17E}"

    lines = [f" {f(re)} {f(pr)} {f(dt)} {f(vel_rot)}", f" {f(rtime)} {int(niter_time)}"]
    for j in range(nj1):
        for i in range(ni1):
            lines.append(f" {f(a['NLX'][j, i])} {f(a['NLY'][j, i])} {f(a['ADV'][j, i])}")
            lines.append(f" {f(a['U'][j, i])} {f(a['V'][j, i])} {f(a['P'][j, i])} {f(a['T'][j, i])}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_restart_2d(path, ni: int, nj: int):
    """Reads RESTART.DAT as init.f90:46-60 does.  Returns (header, state) with
    header = dict(re, pr, dt, vel_rot, rtime, niter_time) and state arrays
    shaped (NJ+1, NI+1)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    if len(lines) < 2:
        raise ValueError("restart file too short")
    # each READ starts a new record: two header records, then 2 records per cell
    h1 = [_num(t) for t in _tokens(lines[0])][:4]
    h2 = list(_tokens(lines[1]))[:2]
    header = dict(re=h1[0], pr=h1[1], dt=h1[2], vel_rot=h1[3], rtime=_num(h2[0]), niter_time=int(_num(h2[1])))
    n = (ni + 1) * (nj + 1)
    recs = lines[2:]
    if len(recs) < 2 * n:
        raise ValueError(f"restart file has {len(recs)} cell records, expected {2 * n}")
    out = {nm: np.zeros((nj + 1, ni + 1)) for nm in STATE_2D}
    for q in range(n):
        j, i = divmod(q, ni + 1)
        a = [_num(t) for t in _tokens(recs[2 * q])][:3]
        b = [_num(t) for t in _tokens(recs[2 * q + 1])][:4]
        out["NLX"][j, i], out["NLY"][j, i], out["ADV"][j, i] = a
        out["U"][j, i], out["V"][j, i], out["P"][j, i], out["T"][j, i] = b
    return header, out


def write_restart_3d(path, state: dict, re: float, pe: float, dt: float, rtime: float, niter_time: int):
    """RESTART000.DAT of RLES/writedata.f90:191-215 from arrays shaped
    (NK+1, NJ+1, NI+1), in the reference's fixed format."""
    a = {nm: np.asarray(state[nm], dtype=np.float64) for nm in STATE_3D}
    nk1, nj1, ni1 = a["U"].shape
    lines = ["".join(" " + format_e(x) for x in (re, pe, dt, rtime)) + " " + f"{int(niter_time):16d}"]
    for k in range(nk1):
        for j in range(nj1):
            for i in range(ni1):
                lines.append("".join(" " + format_e(a[nm][k, j, i]) for nm in ("NLX", "NLY", "NLZ", "ADV")))
                lines.append("".join(" " + format_e(a[nm][k, j, i]) for nm in ("U", "V", "W", "P", "T")))
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def _fixed_fields(line: str, count: int, w: int = 24):
    """TR1 then Ew.d fields: column 1 skipped, then `count` fields of w columns."""
    vals = []
    for q in range(count):
        s = line[1 + q * (w + 1): 1 + q * (w + 1) + w]
        vals.append(s.strip())
    return vals


def read_restart_3d(path, ni: int, nj: int, nk: int):
    """Reads RESTART000.DAT as RLES/init.f90:183-205 does (fixed columns).
    Returns (header, state): header = dict(re, pe, dt, rtime, niter_time), state
    arrays shaped (NK+1, NJ+1, NI+1)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    h = _fixed_fields(lines[0], 4)
    niter = lines[0][1 + 4 * 25:1 + 4 * 25 + 16].strip()
    header = dict(re=_num(h[0]), pe=_num(h[1]), dt=_num(h[2]), rtime=_num(h[3]), niter_time=int(niter))
    n = (ni + 1) * (nj + 1) * (nk + 1)
    recs = lines[1:]
    if len(recs) < 2 * n:
        raise ValueError(f"restart file has {len(recs)} cell records, expected {2 * n}")
    shape = (nk + 1, nj + 1, ni + 1)
    out = {nm: np.zeros(shape) for nm in STATE_3D}
    for q in range(n):
        k, r = divmod(q, (nj + 1) * (ni + 1))
        j, i = divmod(r, ni + 1)
        a = [_num(t) for t in _fixed_fields(recs[2 * q], 4)]
        b = [_num(t) for t in _fixed_fields(recs[2 * q + 1], 5)]
        for nm, v in zip(("NLX", "NLY", "NLZ", "ADV"), a):
            out[nm][k, j, i] = v
        for nm, v in zip(("U", "V", "W", "P", "T"), b):
            out[nm][k, j, i] = v
    return header, out
