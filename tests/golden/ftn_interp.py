"""Executes the reference's own Fortran 90 sources (the R2D snapshot) in Python.

No Fortran compiler exists on either machine of this project, so the golden
fixtures are produced by translating the reference's source files, statement by
statement, into Python/numpy and running them.  Only the subset of Fortran the
R2D snapshot uses is supported: modules with PARAMETER and array declarations,
subroutines with explicit-shape dummy arrays and SAVE'd locals, DO loops, block and
logical IF, backward GOTO loops, whole-array and array-section expressions,
CALL, and list-directed I/O (grid file in, NU_CD_CL.PLT out; everything else is
discarded).

Semantics kept from compiled Fortran:
  * arrays are column-major with their declared lower bounds; SAVE'd locals and
    module arrays start at zero and keep their values between calls;
  * array expressions are evaluated elementwise by position: an operand whose
    extent differs from the assignment's section is read from its own lower bound
    onwards (what compiled code does for a non-conforming whole-array operand);
  * a logical IF condition may be an integer (non-zero is true);
  * DO variables hold start + trips*step after the loop;
  * x**2.0 is x*x and x**0.5 is sqrt(x); integer division truncates.

This module is test infrastructure: it reads the reference tree given to it and
is only used by make_golden.py in the environment where that tree exists.
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

# ---------------------------------------------------------------------------------
# source handling
# ---------------------------------------------------------------------------------


def strip_comment(line: str) -> str:
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in ("'", '"'):
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def logical_lines(text: str):
    """Free-form source -> (label, statement) with continuations joined."""
    res, buf = [], None
    for raw in text.replace("\t", " ").split("\n"):
        s = strip_comment(raw).rstrip()
        if not s.strip():
            continue
        st = s.strip()
        if buf is not None:
            if st.startswith("&"):
                st = st[1:]
            st = buf + " " + st
            buf = None
        if st.endswith("&"):
            buf = st[:-1]
            continue
        m = re.match(r"^(\d+)\s+(.*)$", st)
        label = None
        if m:
            label, st = int(m.group(1)), m.group(2)
        res.append((label, st.strip()))
    return res


# ---------------------------------------------------------------------------------
# expression parsing
# ---------------------------------------------------------------------------------
TOKEN = re.compile(r"""
    (?P<num>(\d+\.(?!(and|or|not|eq|ne|lt|le|gt|ge|true|false)\.)\d*|\.\d+|\d+)([dDeE][+-]?\d+)?)
  | (?P<dot>\.(and|or|not|eq|ne|lt|le|gt|ge|true|false)\.)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<name>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op>\*\*|//|==|/=|<=|>=|[-+*/(),:<>=])
  | (?P<ws>\s+)
""", re.X | re.I)


def tokenize(s: str):
    toks, pos = [], 0
    while pos < len(s):
        m = TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[pos:pos + 20]!r} in {s!r}")
        pos = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        v = m.group(k)
        if k == "num":
            toks.append(("num", v))
        elif k == "dot":
            toks.append(("op", "." + v.lower().strip(".") + "."))
        else:
            toks.append((k, v))
    return toks


class P:
    """Recursive-descent parser producing a small tuple AST."""

    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        return self.t[self.i + k] if self.i + k < len(self.t) else (None, None)

    def take(self, v=None):
        tok = self.peek()
        if v is not None and tok[1] != v and (tok[1] or "").upper() != v.upper():
            raise SyntaxError(f"expected {v} got {tok}")
        self.i += 1
        return tok

    def expr(self):
        return self.or_()

    def or_(self):
        a = self.and_()
        while self.peek()[1] == ".or.":
            self.take()
            a = ("or", a, self.and_())
        return a

    def and_(self):
        a = self.not_()
        while self.peek()[1] == ".and.":
            self.take()
            a = ("and", a, self.not_())
        return a

    def not_(self):
        if self.peek()[1] == ".not.":
            self.take()
            return ("not", self.not_())
        return self.rel()

    REL = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
           "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}

    def rel(self):
        a = self.add()
        op = self.peek()[1]
        if op in self.REL:
            self.take()
            a = ("rel", self.REL[op], a, self.add())
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.mul()
            if op == "-":
                a = ("neg", a)
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.unary_pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = ("bin", op, a, self.unary_pow())
        return a

    def unary_pow(self):
        # a sign directly after an operator (e.g. "VEL_ROT * -SIN(x)") binds to the power
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = self.power()
            return ("neg", a) if op == "-" else a
        return self.power()

    def power(self):
        a = self.primary()
        if self.peek()[1] == "**":
            self.take()
            return ("pow", a, self.unary_pow())
        return a

    def primary(self):
        k, v = self.peek()
        if k == "num":
            self.take()
            return ("num", v)
        if k == "str":
            self.take()
            return ("str", v[1:-1])
        if v in (".true.", ".false."):
            self.take()
            return ("num", "1" if v == ".true." else "0")
        if v == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return e
        if k == "name":
            self.take()
            name = v.upper()
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.subscript())
                        if self.peek()[1] == ",":
                            self.take()
                            continue
                        break
                self.take(")")
                return ("call", name, args)
            return ("name", name)
        raise SyntaxError(f"unexpected {k} {v}")

    def subscript(self):
        # index, section lo:hi, or keyword argument NAME=expr
        if self.peek()[0] == "name" and self.peek(1)[1] == "=" and self.peek(2)[1] != "=":
            key = self.take()[1].upper()
            self.take("=")
            return ("kw", key, self.expr())
        lo = hi = None
        if self.peek()[1] != ":":
            lo = self.expr()
        if self.peek()[1] == ":":
            self.take()
            if self.peek()[1] not in (",", ")"):
                hi = self.expr()
            return ("sec", lo, hi)
        return lo


def parse_expr(s: str):
    p = P(tokenize(s))
    e = p.expr()
    if p.i != len(p.t):
        raise SyntaxError(f"trailing tokens in {s!r}: {p.t[p.i:]}")
    return e


# ---------------------------------------------------------------------------------
# runtime values
# ---------------------------------------------------------------------------------
class FArray:
    def __init__(self, lows, highs, kind="real"):
        self.low = list(lows)
        shape = [h - l + 1 for l, h in zip(lows, highs)]
        self.a = np.zeros(shape, dtype=np.float64 if kind == "real" else np.int64, order="F")

    def idx(self, subs):
        return tuple(s - l for s, l in zip(subs, self.low))

    def read(self, subs):
        """Element read with compiled-code semantics outside the bounds: the
        column-major offset is used while it stays inside the array's storage,
        otherwise the value is zero (R2D reads outside U_N only in the far-field
        formula at the ghost rows J=0 and J=NJ, whose results are overwritten)."""
        ix = self.idx(subs)
        if all(0 <= k < n for k, n in zip(ix, self.a.shape)):
            return self.a[ix].item()
        off, mul = 0, 1
        for k, n in zip(ix, self.a.shape):
            off += k * mul
            mul *= n
        self.oob_reads = getattr(self, "oob_reads", 0) + 1
        if 0 <= off < self.a.size:
            return self.a.reshape(-1, order="F")[off].item()
        return 0.0

    def sl(self, specs):
        out = []
        for d, sp in enumerate(specs):
            if isinstance(sp, tuple):
                lo, hi = sp
                lo = self.low[d] if lo is None else lo
                hi = self.low[d] + self.a.shape[d] - 1 if hi is None else hi
                out.append(slice(lo - self.low[d], hi - self.low[d] + 1))
            else:
                out.append(sp - self.low[d])
        return tuple(out)


def conform(x, shape):
    """Positional view of x on `shape` (truncated from its own lower bound)."""
    if not isinstance(x, np.ndarray) or x.shape == shape:
        return x
    if x.ndim != len(shape):
        raise ValueError(f"rank mismatch {x.shape} vs {shape}")
    return x[tuple(slice(0, n) for n in shape)]


def binop(op, a, b):
    if isinstance(a, np.ndarray) and isinstance(b, np.ndarray) and a.shape != b.shape:
        shape = tuple(min(p, q) for p, q in zip(a.shape, b.shape))
        a, b = conform(a, shape), conform(b, shape)
    if op == "+":
        return a + b
    if op == "-":
        return a - b
    if op == "*":
        return a * b
    if op == "/":
        if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
            q = abs(int(a)) // abs(int(b))
            return q if (a >= 0) == (b >= 0) else -q
        if not isinstance(a, np.ndarray) and not isinstance(b, np.ndarray) and b == 0:
            with np.errstate(divide="ignore", invalid="ignore"):   # IEEE: inf or NaN, as compiled code
                return float(np.float64(a) / np.float64(b))
        return a / b
    raise ValueError(op)


def power(a, b):
    if isinstance(b, float) and b == 2.0 or isinstance(b, (int, np.integer)) and b == 2:
        return a * a
    if isinstance(b, float) and b == 0.5:
        return np.sqrt(a) if isinstance(a, np.ndarray) else math.sqrt(a)
    return a ** b


def _m(f_scalar, f_array):
    return lambda x: f_array(x) if isinstance(x, np.ndarray) else f_scalar(x)


INTRINSICS = {
    "SIN": _m(math.sin, np.sin), "DSIN": _m(math.sin, np.sin), "COS": _m(math.cos, np.cos),
    "DCOS": _m(math.cos, np.cos), "DATAN": _m(math.atan, np.arctan), "ATAN": _m(math.atan, np.arctan),
    "DASIN": _m(math.asin, np.arcsin), "ASIN": _m(math.asin, np.arcsin), "DACOS": _m(math.acos, np.arccos),
    "ACOS": _m(math.acos, np.arccos), "ABS": _m(abs, np.abs), "DABS": _m(abs, np.abs),
    "SQRT": _m(math.sqrt, np.sqrt), "DSQRT": _m(math.sqrt, np.sqrt),
    "DMAX1": lambda *a: max(a), "MAX": lambda *a: max(a), "MIN": lambda *a: min(a),
    "INT4": lambda x: int(x), "INT": lambda x: int(x), "DBLE": lambda x: float(x),
    "MOD": lambda a, b: int(math.fmod(a, b)),
}


def literal(v: str):
    s = v.lower()
    if any(c in s for c in ".de"):
        return float(s.replace("d", "e"))
    return int(s)


# ---------------------------------------------------------------------------------
# program model
# ---------------------------------------------------------------------------------
class Var:
    def __init__(self, kind, dims=None, param=False):
        self.kind, self.dims, self.param = kind, dims, param


class Machine:
    """Holds module variables, subroutines and I/O streams of one run."""

    def __init__(self, overrides=None):
        self.g = {}            # global (module) values
        self.gtypes = {}       # global declarations
        self.subs = {}         # name -> (args, body, decls)
        self.saved = {}        # per-subroutine SAVE'd locals
        self.overrides = {k.upper(): v for k, v in (overrides or {}).items()}
        self.stdin = []
        self.unit_in = {}      # unit -> list of values
        self.unit_out = {}     # unit -> list of records
        self.units_open = {}
        self.archive = []      # (unit, file name, records) of files a later OPEN replaced
        self.drop_oob_writes = False   # skip (and log) scalar writes past an array's bounds
        self.oob_log = []
        self.g.update(MPI_CONSTANTS)

    # -- declarations -----------------------------------------------------------
    def declare(self, st, scope, types, env):
        up = st.upper()
        kind = "int" if up.startswith("INTEGER") else ("real" if up.startswith("DOUBLE") else
                                                      ("logical" if up.startswith("LOGICAL") else "char"))
        if "::" in st:
            attrs, ents = st.split("::", 1)
        else:
            attrs, ents = st.split(None, 1) if kind != "real" else ("DOUBLE PRECISION", st[len("DOUBLE PRECISION"):])
        attrs_u = attrs.upper()
        is_param = "PARAMETER" in attrs_u
        alloc = "ALLOCATABLE" in attrs_u
        for ent in split_top(ents):
            ent = ent.strip()
            m = re.match(r"^([A-Za-z_][A-Za-z0-9_]*)\s*(\((.*)\))?\s*(=\s*(.*))?$", ent, re.S)
            if not m:
                raise SyntaxError(ent)
            name = m.group(1).upper()
            dims = m.group(3)
            init = m.group(5)
            if dims and not alloc:
                bounds = []
                for dspec in split_top(dims):
                    if ":" in dspec:
                        lo, hi = dspec.split(":", 1)
                        bounds.append((lo, hi))
                    else:
                        bounds.append(("1", dspec))
                types[name] = Var(kind, bounds)
                if scope == "module" or env is not None:
                    self._alloc(name, bounds, kind, env)
            else:
                types[name] = Var(kind, "alloc" if alloc else None, is_param)
                if init is not None:
                    val = self.eval(parse_expr(init), env)
                    if name in self.overrides:
                        val = self.overrides[name]
                    if kind == "int":
                        val = int(val)
                    (env if env is not None else self.g)[name] = val
                elif alloc:
                    (env if env is not None else self.g)[name] = None
                elif name not in (env if env is not None else self.g):
                    (env if env is not None else self.g)[name] = 0 if kind in ("int", "logical") else (
                        0.0 if kind == "real" else "")

    def _alloc(self, name, bounds, kind, env):
        lows, highs = [], []
        for lo, hi in bounds:
            lows.append(int(self.eval(parse_expr(lo), env)))
            highs.append(int(self.eval(parse_expr(hi), env)))
        (env if env is not None else self.g)[name] = FArray(lows, highs, "real" if kind == "real" else "int")

    # -- evaluation ---------------------------------------------------------------
    def lookup(self, name, env):
        if env is not None and name in env:
            return env[name]
        if name in self.g:
            return self.g[name]
        raise NameError(name)

    def eval(self, e, env):
        t = e[0]
        if t == "num":
            return literal(e[1])
        if t == "str":
            return e[1]
        if t == "name":
            v = self.lookup(e[1], env)
            return v.a if isinstance(v, FArray) else v
        if t == "neg":
            return -self.eval(e[1], env)
        if t == "bin":
            return binop(e[1], self.eval(e[2], env), self.eval(e[3], env))
        if t == "pow":
            return power(self.eval(e[1], env), self.eval(e[2], env))
        if t == "rel":
            a, b = self.eval(e[2], env), self.eval(e[3], env)
            return {"==": a == b, "!=": a != b, "<": a < b, "<=": a <= b, ">": a > b, ">=": a >= b}[e[1]]
        if t == "and":
            return bool(self.eval(e[1], env)) and bool(self.eval(e[2], env))
        if t == "or":
            return bool(self.eval(e[1], env)) or bool(self.eval(e[2], env))
        if t == "not":
            return not bool(self.eval(e[1], env))
        if t == "call":
            name, args = e[1], e[2]
            holder = env if (env is not None and name in env) else self.g
            if name in holder and isinstance(holder[name], FArray):
                arr = holder[name]
                specs = [self._spec(a, env) for a in args]
                if any(isinstance(s, tuple) for s in specs):
                    return arr.a[arr.sl(specs)]
                return arr.read(specs)
            if name in INTRINSICS:
                return INTRINSICS[name](*[self.eval(a, env) for a in args])
            raise NameError(f"unknown function or array {name}")
        raise ValueError(t)

    def _spec(self, a, env):
        if isinstance(a, tuple) and a[0] == "sec":
            lo = None if a[1] is None else int(self.eval(a[1], env))
            hi = None if a[2] is None else int(self.eval(a[2], env))
            return (lo, hi)
        return int(self.eval(a, env))

    def assign(self, lhs, value, env):
        if lhs[0] == "name":
            name = lhs[1]
            holder = env if (env is not None and name in env) else self.g
            cur = holder.get(name)
            if isinstance(cur, FArray):
                cur.a[...] = conform(value, cur.a.shape) if isinstance(value, np.ndarray) else value
                return
            decl = self._decl(name, env)
            if decl is not None and decl.kind == "int":
                value = int(value)
            holder[name] = value
            return
        if lhs[0] == "call":
            name, args = lhs[1], lhs[2]
            holder = env if (env is not None and name in env) else self.g
            arr = holder[name]
            if isinstance(arr, str):    # character substring: internal write, ignored
                return
            specs = [self._spec(a, env) for a in args]
            if any(isinstance(s, tuple) for s in specs):
                view = arr.a[arr.sl(specs)]
                view[...] = conform(value, view.shape) if isinstance(value, np.ndarray) else value
            else:
                ix = arr.idx(specs)
                if self.drop_oob_writes and any(q < 0 or q >= n for q, n in zip(ix, arr.a.shape)):
                    # an element past the array (undefined in the compiled program): recorded, not written
                    self.oob_log.append((name, tuple(specs)))
                    return
                arr.a[ix] = value
            return
        raise ValueError(lhs)

    def _decl(self, name, env):
        d = None
        if env is not None and "__types__" in env:
            d = env["__types__"].get(name)
        return d if d is not None else self.gtypes.get(name)


def split_top(s: str):
    """Split on commas at parenthesis depth 0."""
    out, depth, cur = [], 0, []
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    if cur:
        out.append("".join(cur))
    return out


# ---------------------------------------------------------------------------------
# statement compilation
# ---------------------------------------------------------------------------------
DECL = re.compile(r"^(INTEGER|DOUBLE\s+PRECISION|LOGICAL|CHARACTER)\b", re.I)
IGNORE = re.compile(r"^(IMPLICIT|SAVE|USE|PRINT|FORMAT|CLOSE|PAUSE|DEALLOCATE|INCLUDE|CONTINUE)\b", re.I)

# MPI for a single rank with periodic Cartesian neighbours: every neighbour is the
# rank itself, SENDRECV copies the send buffer into the receive buffer, ALLREDUCE
# copies its argument.  Handle and datatype constants are plain integers.
MPI_CONSTANTS = {"MPI_DOUBLE_PRECISION": 1, "MPI_SUM": 1, "MPI_MAX": 2, "MPI_MIN": 3, "MPI_COMM_WORLD": 0,
                 "MPI_STATUS_SIZE": 6, "MPI_INTEGER": 2}


def parse_block(lines, i, enders):
    """Parse statements from lines[i] until a line matching one of enders.
    Returns (stmts, index of ender)."""
    out = []
    while i < len(lines):
        label, st = lines[i]
        up = st.upper()
        if any(re.match(e, up) for e in enders):
            return out, i
        if re.match(r"^DO\s+\w+\s*=", up):
            m = re.match(r"^DO\s+(\w+)\s*=\s*(.*)$", st, re.I)
            parts = split_top(m.group(2))
            body, j = parse_block(lines, i + 1, [r"^END\s*DO\b"])
            out.append(("do", label, m.group(1).upper(), [parse_expr(p) for p in parts], body))
            i = j + 1
            continue
        m = re.match(r"^IF\s*\((.*)\)\s*THEN$", st, re.I)
        if m:
            branches = []
            cond = parse_expr(m.group(1))
            body, j = parse_block(lines, i + 1, [r"^ELSE\s*IF\b", r"^ELSE$", r"^END\s*IF\b"])
            branches.append((cond, body))
            while True:
                _, stj = lines[j]
                uj = stj.upper()
                mm = re.match(r"^ELSE\s*IF\s*\((.*)\)\s*THEN$", stj, re.I)
                if mm:
                    cond = parse_expr(mm.group(1))
                    body, j = parse_block(lines, j + 1, [r"^ELSE\s*IF\b", r"^ELSE$", r"^END\s*IF\b"])
                    branches.append((cond, body))
                    continue
                if re.match(r"^ELSE$", uj):
                    body, j = parse_block(lines, j + 1, [r"^END\s*IF\b"])
                    branches.append((None, body))
                    continue
                break
            out.append(("if", label, branches))
            i = j + 1
            continue
        m = re.match(r"^IF\s*\(", st, re.I)
        if m:
            # logical IF: find the matching parenthesis
            depth, k = 0, st.index("(")
            for k in range(st.index("("), len(st)):
                if st[k] == "(":
                    depth += 1
                elif st[k] == ")":
                    depth -= 1
                    if depth == 0:
                        break
            cond = parse_expr(st[st.index("(") + 1:k])
            inner, _ = parse_block([(None, st[k + 1:].strip())], 0, [])
            out.append(("lif", label, cond, inner))
            i += 1
            continue
        out.append(simple_stmt(label, st))
        i += 1
    return out, i


def io_parts(st, kw):
    """Split 'KW(control) items' with quote- and parenthesis-aware matching."""
    i = st.index("(", len(kw) - 1)
    depth, q = 0, None
    for k in range(i, len(st)):
        ch = st[k]
        if q:
            if ch == q:
                q = None
            continue
        if ch in ("'", '"'):
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return st[i + 1:k], st[k + 1:].strip()
    raise SyntaxError(st)


def split_top_q(s: str):
    """split_top that also ignores commas inside quotes."""
    out, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in ("'", '"'):
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    if cur:
        out.append("".join(cur))
    return out


def simple_stmt(label, st):
    up = st.upper()
    if DECL.match(st):
        return ("decl", label, st)
    if IGNORE.match(st):
        return ("nop", label)
    m = re.match(r"^GO\s*TO\s+(\d+)$", st, re.I)
    if m:
        return ("goto", label, int(m.group(1)))
    m = re.match(r"^CALL\s+(\w+)\s*(\((.*)\))?$", st, re.I)
    if m:
        args = [parse_expr(a) for a in split_top(m.group(3))] if m.group(3) else []
        return ("call", label, m.group(1).upper(), args)
    m = re.match(r"^ALLOCATE\s*\((.*)\)$", st, re.I)
    if m:
        return ("allocate", label, [a for a in split_top(m.group(1)) if "STAT" not in a.upper()])
    if re.match(r"^READ\s*\(", st, re.I):
        ctl, items = io_parts(st, "READ(")
        unit = split_top_q(ctl)[0].strip()
        return ("read", label, unit, [parse_expr(a) for a in split_top(items)] if items else [])
    m = re.match(r"^OPEN\s*\((.*)\)$", st, re.I)
    if m:
        return ("open", label, m.group(1))
    if re.match(r"^WRITE\s*\(", st, re.I):
        ctl, items = io_parts(st, "WRITE(")
        unit = split_top_q(ctl)[0].strip()
        return ("write", label, unit, [parse_expr(a) for a in split_top_q(items)] if items else [])
    m = re.match(r"^([A-Za-z_]\w*(\s*\(.*?\))?)\s*=(?!=)\s*(.*)$", st, re.S)
    if m and not up.startswith(("IF", "DO ")):
        lhs = P(tokenize(m.group(1)))
        lhs_e = lhs.primary()
        return ("assign", label, lhs_e, parse_expr(m.group(3)))
    raise SyntaxError(f"unsupported statement: {st}")


class Routine:
    def __init__(self, name, args, body):
        self.name, self.args, self.body = name, args, body


def load_program(src_dir, files, overrides=None):
    """Parse the given source files into a Machine with modules evaluated."""
    M = Machine(overrides)
    for f in files:
        lines = logical_lines(open(os.path.join(src_dir, f), encoding="latin-1").read())
        i = 0
        while i < len(lines):
            label, st = lines[i]
            up = st.upper()
            if up.startswith("MODULE"):
                body, j = parse_block(lines, i + 1, [r"^END\s*MODULE\b"])
                for s in body:
                    if s[0] == "decl":
                        M.declare(s[2], "module", M.gtypes, None)
                i = j + 1
                continue
            m = re.match(r"^SUBROUTINE\s+(\w+)\s*(\((.*)\))?", st, re.I)
            if m:
                args = [a.strip().upper() for a in m.group(3).split(",")] if m.group(3) else []
                body, j = parse_block(lines, i + 1, [r"^END\s*SUBROUTINE\b"])
                M.subs[m.group(1).upper()] = Routine(m.group(1).upper(), args, body)
                i = j + 1
                continue
            m = re.match(r"^PROGRAM\s+(\w+)", st, re.I)
            if m:
                body, j = parse_block(lines, i + 1, [r"^END\s*PROGRAM\b"])
                M.subs["__MAIN__"] = Routine("__MAIN__", [], body)
                i = j + 1
                continue
            i += 1
    return M


class GotoSignal(Exception):
    def __init__(self, label):
        self.label = label


def run_stmts(M, stmts, env):
    """Execute statements; a GOTO to a label inside `stmts` restarts from it."""
    labels = {s[1]: k for k, s in enumerate(stmts) if s[1] is not None}
    k = 0
    while k < len(stmts):
        try:
            exec_stmt(M, stmts[k], env)
            k += 1
        except GotoSignal as g:
            if g.label in labels:
                k = labels[g.label]
            else:
                raise


def exec_stmt(M, s, env):
    t = s[0]
    if t in ("nop", "decl"):
        return
    if t == "assign":
        M.assign(s[2], M.eval(s[3], env), env)
    elif t == "do":
        _, _, var, parts, body = s
        start = int(M.eval(parts[0], env))
        stop = int(M.eval(parts[1], env))
        step = int(M.eval(parts[2], env)) if len(parts) > 2 else 1
        trips = max(0, (stop - start + step) // step)
        holder = env if (env is not None and var in env) else M.g
        v = start
        for _ in range(trips):
            holder[var] = v
            run_stmts(M, body, env)
            v = holder[var] + step
        holder[var] = start + trips * step
    elif t == "if":
        for cond, body in s[2]:
            if cond is None or bool(M.eval(cond, env)):
                run_stmts(M, body, env)
                break
    elif t == "lif":
        if bool(M.eval(s[2], env)):
            for inner in s[3]:
                exec_stmt(M, inner, env)
    elif t == "goto":
        raise GotoSignal(s[2])
    elif t == "call":
        call(M, s[2], s[3], env)
    elif t == "allocate":
        for a in s[2]:
            e = parse_expr(a)
            name = e[1]
            bounds = []
            for sub in e[2]:
                if sub[0] == "sec":
                    bounds.append((M.eval(sub[1], env), M.eval(sub[2], env)))
                else:
                    bounds.append((1, M.eval(sub, env)))
            M.g[name] = FArray([b[0] for b in bounds], [b[1] for b in bounds])
    elif t == "read":
        unit = s[2]
        for tgt in s[3]:
            if unit == "*":
                val = M.stdin.pop(0)
            else:
                val = M.unit_in[int(unit)].pop(0)
            M.assign(tgt, val, env)
    elif t == "open":
        m = re.match(r"^\s*(?:UNIT\s*=\s*)?([^,]+)", s[2], re.I)
        unit = unit_number(M, m.group(1), env)
        fm = re.search(r"FILE\s*=\s*(?:'([^']*)'|(\w+))", s[2], re.I)
        fname = None
        if fm:
            fname = fm.group(1) if fm.group(1) is not None else str(M.eval(parse_expr(fm.group(2)), env)).strip()
        if re.search(r"ACCESS\s*=\s*'APPEND'", s[2], re.I):
            M.unit_out.setdefault(unit, [])
        else:   # a sequential file opened without APPEND is written from its start
            if M.unit_out.get(unit):   # keep what the unit's previous file received
                M.archive.append((unit, M.units_open.get(unit), M.unit_out[unit]))
            M.unit_out[unit] = []
        M.units_open[unit] = fname
    elif t == "write":
        unit = unit_number(M, s[2], env)
        if unit is None:   # list-directed output to the screen, or an internal write
            return
        vals = [M.eval(e, env) for e in s[3]]
        M.unit_out.setdefault(unit, []).append(vals)


def unit_number(M, text, env):
    """The unit of an OPEN/WRITE: a literal or an integer expression such as
    1000+RANK; None for '*' and for internal writes to character variables."""
    t = text.strip()
    if t == "*":
        return None
    if t.isdigit():
        return int(t)
    if "(" in t or "'" in t:
        return None
    try:
        v = M.eval(parse_expr(t), env)
    except Exception:
        return None
    return int(v) if isinstance(v, (int, np.integer)) else None


def call(M, name, args, env):
    if name == "CPU_TIME":
        M.assign(args[0], 0.0, env)
        return
    if name.startswith("MPI_") and name not in M.subs:
        if name in ("MPI_COMM_RANK",):
            M.assign(args[1], 0, env)
        elif name == "MPI_COMM_SIZE":
            M.assign(args[1], 1, env)
        elif name == "MPI_CART_CREATE":
            M.assign(args[5], 0, env)
        elif name == "MPI_CART_COORDS":
            arr = M.eval(args[3], env)
            M.assign(args[3], np.zeros_like(np.asarray(arr)) if isinstance(arr, np.ndarray) else 0, env)
        elif name == "MPI_CART_SHIFT":
            M.assign(args[3], 0, env)
            M.assign(args[4], 0, env)
        elif name == "MPI_SENDRECV":
            val = M.eval(args[0], env)
            M.assign(args[5], np.array(val, copy=True) if isinstance(val, np.ndarray) else val, env)
        elif name == "MPI_ALLREDUCE":
            M.assign(args[1], M.eval(args[0], env), env)
        return
    r = M.subs[name]
    local = M.saved.setdefault(name, {"__types__": {}})
    # bind dummies: arrays by reference with the dummy's declared bounds
    bindings = {}
    for dummy, actual in zip(r.args, args):
        if actual[0] == "name":
            holder = env if (env is not None and actual[1] in env) else M.g
            bindings[dummy] = holder.get(actual[1])
        else:
            bindings[dummy] = M.eval(actual, env)
    # declarations (first call builds SAVE'd locals; dummies re-bound every call)
    for s in r.body:
        if s[0] != "decl":
            continue
        st = s[2]
        names = decl_names(st)
        if any(n in r.args for n in names):
            for n in names:
                if n not in r.args:
                    continue
                actual = bindings[n]
                if isinstance(actual, FArray):
                    dims = decl_dims(st, n)
                    lows = [int(M.eval(parse_expr(lo), local)) for lo, hi in dims]
                    highs = [int(M.eval(parse_expr(hi), local)) for lo, hi in dims]
                    shape = tuple(h - l + 1 for l, h in zip(lows, highs))
                    if shape != actual.a.shape:
                        raise ValueError(f"{name}: dummy {n} shape {shape} != actual {actual.a.shape}")
                    view = FArray.__new__(FArray)
                    view.low, view.a = lows, actual.a
                    local[n] = view
                else:
                    local[n] = actual
                local["__types__"][n] = Var("real" if "DOUBLE" in st.upper() else "int")
        elif "__init_done__" not in local:
            M.declare(st, "local", local["__types__"], local)
    local["__init_done__"] = True
    run_stmts(M, r.body, local)


def decl_names(st):
    ents = st.split("::", 1)[1] if "::" in st else st.split(None, 2)[-1]
    return [re.match(r"\s*([A-Za-z_]\w*)", e).group(1).upper() for e in split_top(ents)]


def decl_dims(st, name):
    ents = st.split("::", 1)[1]
    for e in split_top(ents):
        m = re.match(r"\s*([A-Za-z_]\w*)\s*\((.*)\)\s*$", e)
        if m and m.group(1).upper() == name:
            return [tuple(d.split(":", 1)) if ":" in d else ("1", d) for d in split_top(m.group(2))]
    raise KeyError(name)
