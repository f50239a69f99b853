"""Test helpers for the PC tree propagators.

* `compile_shim(dir)` builds tests/cpp/pc_fzn_shim.cpp (the FlatZinc front end
  of include/pirgpu_fzn_pc.hpp) and returns a factory of `FznModel`s.
* `OracleModel` / `GpuModel` apply what each FlatZinc tell added (new
  variables, store meets, formulas) to the CPU oracle or to the engine, and
  run deduce_and_test's steps (tests/pc_test.cpp:85-105).
* `random_formulas` builds seeded random formula sets over a store.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INF = 2**31 - 1
MINF = -2**31


class FznModel:
    """One model of the shim; compile() returns what a tell added."""

    def __init__(self, lib):
        self.lib = lib
        self.h = lib.pcfzn_new()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.pcfzn_free(self.h)
            self.h = None

    def compile(self, text):
        buf = ctypes.create_string_buffer(1 << 22)
        rc = self.lib.pcfzn_compile(self.h, text.encode(), buf, len(buf))
        if rc:
            raise ValueError(buf.value.decode())
        lines = buf.value.decode().splitlines()
        nv0, nv, nm, nn, npr = map(int, lines[0].split())
        p = 1
        newvars = [tuple(map(int, l.split()[:2])) for l in lines[p:p + nv - nv0]]
        names = [l.split()[2] for l in lines[p:p + nv - nv0]]
        p += nv - nv0
        meets = [tuple(map(int, l.split())) for l in lines[p:p + nm]]
        p += nm
        tape = np.array([list(map(int, l.split())) for l in lines[p:p + nn]], np.int32).reshape(-1, 4)
        p += nn
        roots = np.array([int(l) for l in lines[p:p + npr]], np.int32)
        return dict(nvars0=nv0, newvars=newvars, names=names, meets=meets, tape=tape, roots=roots)


def compile_shim(outdir):
    out = os.path.join(str(outdir), "libpcfzn_shim.so")
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "pc_fzn_shim.cpp"), "-o", out],
                   check=True, capture_output=True, text=True)
    lib = ctypes.CDLL(out)
    lib.pcfzn_new.restype = ctypes.c_void_p
    lib.pcfzn_free.argtypes = [ctypes.c_void_p]
    lib.pcfzn_compile.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
    lib.pcfzn_compile.restype = ctypes.c_int
    return lambda: FznModel(lib)


def offset_tape(tape, base):
    """Node indices of a tape shifted by `base` (the fields that are indices)."""
    t = np.array(tape, np.int32).reshape(-1, 4).copy()
    k = t[:, 0]
    refs_a = ~np.isin(k, [0, 1, 16, 17, 18, 19, 31, 32, 33, 34, 35, 36])  # data in a: leaves and store items
    refs_b = ((k >= 5) & (k <= 13)) | ((k >= 20) & (k <= 28))
    t[refs_a, 1] += base
    t[refs_b, 2] += base
    return t


class OracleModel:
    """The reference's PC on the CPU oracle: store, tape, propagators."""

    def __init__(self, O):
        self.O = O
        self.store = np.zeros((0, 2), np.int32)
        self.tape = np.zeros((0, 4), np.int32)
        self.roots = np.zeros(0, np.int32)
        self.failed = False

    def apply(self, delta):
        if delta["newvars"]:
            self.store = np.concatenate([self.store, np.array(delta["newvars"], np.int32)]).astype(np.int32)
        for v, l, u in delta["meets"]:
            self.store[v, 0] = max(self.store[v, 0], l)
            self.store[v, 1] = min(self.store[v, 1], u)
        base = len(self.tape)
        self.tape = np.concatenate([self.tape, offset_tape(delta["tape"], base)]).astype(np.int32)
        roots = np.concatenate([self.roots, delta["roots"] + base]).astype(np.int32)
        self.roots = self.O.pc_order(self.tape, roots)
        self.store = np.ascontiguousarray(self.store)
        self.failed = self.failed or bool(np.any((self.store[:, 0] > self.store[:, 1]) |
                                                 (self.store[:, 0] == INF) | (self.store[:, 1] == MINF)))

    def num_deductions(self):
        return len(self.roots)

    def bounds(self, n):
        return [tuple(int(v) for v in self.store[i]) for i in range(n)]

    def fixpoint(self):
        if self.failed:
            return self.O.FAILED, False
        rc, info = self.O.pc_fixpoint(self.tape, self.roots, self.store)
        self.failed = rc == self.O.FAILED
        return rc, info["has_changed"]

    def is_extractable(self):
        return (not self.failed) and all(self.O.pc_ask(self.tape, r, self.store) for r in self.roots)


class GpuModel:
    """The same steps through the engine's C ABI."""

    def __init__(self, ctx_factory):
        self.ctx = ctx_factory()
        self.nvars = 0

    def apply(self, delta):
        if delta["newvars"]:
            if self.nvars:
                lb, ub = self.ctx.read_store()
            else:
                lb, ub = np.zeros(0, np.int32), np.zeros(0, np.int32)
            nv = np.array(delta["newvars"], np.int32).reshape(-1, 2)
            self.ctx.load_store(np.concatenate([lb, nv[:, 0]]), np.concatenate([ub, nv[:, 1]]))
            self.nvars = len(lb) + len(nv)
        for v, l, u in delta["meets"]:
            self.ctx.embed(v, l, u)
        if len(delta["roots"]) or len(delta["tape"]):
            self.ctx.pc_tell(delta["tape"], delta["roots"])

    def num_deductions(self):
        return self.ctx.pc_num_deductions()

    def bounds(self, n):
        lb, ub = self.ctx.read_store()
        return [(int(lb[i]), int(ub[i])) for i in range(n)]

    def fixpoint(self):
        rc, st = self.ctx.pc_fixpoint()
        return rc, st["narrowed"] > 0

    def is_extractable(self):
        return self.ctx.pc_is_extractable()


def run_case(make_fzn, model, case, check_changed=True):
    """Runs every step of one pc_kat_cases case on `model`; returns the list
    of mismatches (empty when the case passes)."""
    from golden import pc_kat_cases as K
    name, line, text, steps = case
    fz = make_fzn()
    bad = []
    for k, (tell, num, before, after, ua, changed) in enumerate(steps):
        d = fz.compile(text if k == 0 else tell)
        model.apply(d)
        n = len(before)
        if model.num_deductions() != num:
            bad.append((k, "num_deductions", model.num_deductions(), num))
        if model.bounds(n) != [tuple(b) for b in before]:
            bad.append((k, "before", model.bounds(n), before))
        rc, ch = model.fixpoint()
        if after == K.BOT:
            if rc != 1:
                bad.append((k, "status", rc, "FAILED"))
            continue
        if rc != 0:
            bad.append((k, "status", rc, "OK"))
        if check_changed and ch != changed:
            bad.append((k, "has_changed", ch, changed))
        if model.bounds(n) != [tuple(b) for b in after]:
            bad.append((k, "after", model.bounds(n), after))
        if model.is_extractable() != ua:
            bad.append((k, "is_extractable", model.is_extractable(), ua))
    return bad


# ----------------------------------------------------------------- random --
def random_formulas(rng, nvars, nprops, depth=3, kinds="all", positive_mul=True):
    """A tape of `nprops` random formulas over `nvars` variables: comparisons
    of random terms (sums, differences, products by constants, min / max,
    |t|, -t, divisions by positive constants, n-ary sums), combined by the
    connectives and reified into 0/1 variables.  Returns (pc.Tape, store)."""
    import pc as P
    t = P.Tape()
    lo = rng.integers(-50, 30, nvars)
    hi = lo + rng.integers(0, 80, nvars)
    store = np.stack([lo, hi], 1).astype(np.int32)
    nbool = max(1, nvars // 4)
    store[:nbool] = [0, 1]

    def term(d):
        r = rng.random()
        if d <= 0 or r < 0.3:
            if rng.random() < 0.15:
                c = int(rng.integers(-5, 6))
                return t.constant(c)
            return t.var(int(rng.integers(nbool, nvars)))
        r = rng.random()
        if r < 0.25:
            return t.add(term(d - 1), term(d - 1))
        if r < 0.4:
            return t.sub(term(d - 1), term(d - 1))
        if r < 0.5:
            return t.mul(t.constant(int(rng.integers(1, 5)) * (1 if positive_mul else int(rng.choice([-1, 1])))),
                         term(d - 1))
        if r < 0.58:
            return t.min(term(d - 1), term(d - 1))
        if r < 0.66:
            return t.max(term(d - 1), term(d - 1))
        if r < 0.72:
            return t.abs(term(d - 1))
        if r < 0.78:
            return t.neg(term(d - 1))
        if r < 0.86:
            if kinds == "planted":
                return t.add(term(d - 1), term(d - 1))
            op = [P.TDIV, P.FDIV, P.CDIV, P.EDIV][int(rng.integers(0, 4))]
            if kinds == "all" and rng.random() < 0.3:  # a divisor that is itself a term
                return t.binary(op, term(d - 1), term(d - 1))
            return t.binary(op, term(d - 1), t.constant(int(rng.integers(1, 6))))
        if r < 0.94:
            if kinds == "all" and rng.random() < 0.2:
                return t.nmul([term(d - 1) for _ in range(int(rng.integers(2, 4)))])
            if kinds == "all" and rng.random() < 0.2:
                return t.mul(term(d - 1), term(d - 1))
            return t.nadd([term(d - 1) for _ in range(int(rng.integers(2, 5)))])
        return t.formula(atom(d - 1))

    def atom(d):
        r = rng.random()
        a, b = term(d), term(d)
        if r < 0.45:
            return t.leq(a, b)
        if r < 0.6:
            return t.gt(a, b)
        if r < 0.8:
            return t.eq(a, b)
        return t.neq(a, b)

    def formula(d):
        r = rng.random()
        if d <= 0 or r < 0.5:
            if rng.random() < 0.15:
                bv = int(rng.integers(0, nbool))
                return t.pvar(bv) if rng.random() < 0.5 else t.nvar(bv)
            return atom(max(d, 1))
        f, g = formula(d - 1), formula(d - 1)
        k = [P.AND, P.OR, P.EQUIV, P.IMPLY, P.XOR][int(rng.integers(0, 4 if kinds == "planted" else 5))]
        return t._add(k, f, g)

    for _ in range(nprops):
        r = rng.random()
        b = int(rng.integers(0, nbool))
        if r < 0.45:  # a reified formula: b <=> f
            t.prop(t.equiv(t.pvar(b), formula(depth - 1)))
        elif r < 0.8:  # a guarded one: b => f
            t.prop(t.imply(t.pvar(b), formula(depth - 1)))
        elif r < 0.9:  # a disjunction
            t.prop(t.disj(formula(depth - 1), formula(depth - 1)))
        else:
            t.prop(formula(depth))
    return t, store


# ----------------------------------------------------------------- planted --
def _eval(tape, n, s):
    """Value of node n under the assignment s: an int for a term, a bool for a
    formula, None where a division by zero leaves it undefined."""
    import pc as P
    k, a, b, _ = (int(x) for x in tape[n])
    if k == P.VAR:
        return int(s[a])
    if k == P.CONST:
        return a
    if k == P.PVAR:
        return s[a] != 0
    if k == P.NVAR:
        return s[a] == 0
    if k in (P.TRUE, P.FALSE):
        return k == P.TRUE
    if k in (P.NADD, P.NMUL):
        vals = [_eval(tape, int(tape[a + i][1]), s) for i in range(b)]
        if any(v is None for v in vals):
            return None
        out = 0 if k == P.NADD else 1
        for v in vals:
            out = out + v if k == P.NADD else out * v
        return out
    x = _eval(tape, a, s)
    if x is None:
        return None
    if k == P.FORMULA:
        return int(bool(x))
    if k == P.NEG:
        return -x
    if k == P.ABS:
        return abs(x)
    y = _eval(tape, b, s)
    if y is None:
        return None
    if k == P.ADD: return x + y
    if k == P.SUB: return x - y
    if k == P.MUL: return x * y
    if k == P.MIN: return min(x, y)
    if k == P.MAX: return max(x, y)
    if k == P.LEQ: return x <= y
    if k == P.GT: return x > y
    if k == P.EQ: return x == y
    if k == P.NEQ: return x != y
    if k == P.AND: return x and y
    if k == P.OR: return x or y
    if k == P.EQUIV: return x == y
    if k == P.IMPLY: return (not x) or y
    raise ValueError(k)


def planted_formulas(rng, nvars, nprops, depth=3):
    """Random formulas that a hidden assignment s (inside the initial domains)
    satisfies: each candidate is kept only if it holds under s.  Sound
    propagation keeps s inside every domain, so the fixpoint is not empty.
    Leaves out the two constructs whose reference propagation is not sound:
    xor (ExclusiveDisjunction::nask as written, formula.hpp:552-556, reports
    an entailed xor as disentailed) and division (GroupDiv::left_residual,
    terms.hpp:272-277, bounds the dividend by u * z joined with z.ub - 1).
    Returns (pc.Tape, store, s)."""
    import pc as P
    t0, store = random_formulas(rng, nvars, 0, depth=depth)
    s = rng.integers(store[:, 0], store[:, 1] + 1)
    t = P.Tape()
    kept = tries = 0
    while kept < nprops and tries < 50 * nprops:
        tries += 1
        sub, _ = random_formulas(rng, nvars, 1, depth=depth, kinds="planted")
        tape, roots = sub.arrays()
        if _eval(tape, int(roots[0]), s) is not True:
            continue
        off = len(t.nodes)
        for row in offset_tape(tape, off):
            t.nodes.append(tuple(int(v) for v in row))
        t.roots.append(int(roots[0]) + off)
        kept += 1
    return t, store, s


def ae_tape(shape):
    """The formula of the AbstractElement cases over x = 0, y = 1."""
    import pc as P
    t = P.Tape()
    if shape == "ge_le":  # nbool_equiv(int_ge(x, 5), int_le(y, 5))
        f = t.abstract_element(tell=[(0, 5, INF)], not_tell=[(0, MINF, 4)], ask=[(0, 5, INF)], not_ask=[(0, MINF, 4)])
        g = t.abstract_element(tell=[(1, MINF, 5)], not_tell=[(1, 6, INF)], ask=[(1, MINF, 5)], not_ask=[(1, 6, INF)])
    else:  # nbool_equiv(int_eq(x, 5), int_eq(y, 5))
        f = t.abstract_element(tell=[(0, 5, 5)], ask=[(0, 5, 5)], not_ask_out=[(0, 5, 5)])
        g = t.abstract_element(tell=[(1, 5, 5)], ask=[(1, 5, 5)], not_ask_out=[(1, 5, 5)])
    t.prop(t.equiv(f, g))
    return t.arrays()


def run_ae_case(model_steps, case):
    """model_steps(meets) -> (status, bounds, extractable, changed) after the
    meets and the fixpoint; returns the mismatches of one AE case."""
    from golden import pc_kat_cases as K
    name, line, shape, steps = case
    bad = []
    for k, (meets, before, after, ua, changed) in enumerate(steps):
        rc, b0, b1, ex, ch = model_steps(meets)
        if b0 != [tuple(x) for x in before]:
            bad.append((k, "before", b0, before))
        if after == K.BOT:
            if rc != 1:
                bad.append((k, "status", rc))
            continue
        if rc != 0 or b1 != [tuple(x) for x in after] or ex != ua or ch != changed:
            bad.append((k, rc, b1, after, ex, ua, ch, changed))
    return bad
