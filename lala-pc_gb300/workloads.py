"""Seeded synthetic PIR instances (the benchmark and parity workloads).

Every generator is deterministic across hosts and numpy versions: random
numbers come from a counter-based splitmix64 written here, not from numpy's
generators.  Instances are structure-of-arrays bytecode (op, x, y, z int32)
plus an initial store (lb, ub int32), in the layout the C ABI takes.

Workloads (sizes, bound distribution and operator mix of the benchmark
configurations):

* plain single instance: nvars variables with lb ~ U[-S, 0], ub = lb + U[0, 2S];
  nprops propagators, mix 45% x=y+z, 15% x=y*z, 5% min, 5% max, 10% x=y-z
  (written as ADD y = x + z: PIR has no SUB, pir.hpp:270-273), 20% reified
  x=(y<=z) (x forced to [0,1] at install, pir.hpp:333-335).
* deep chain: x_{i+1} = x_i + c_i over dedicated variables, c_i ~ U[1,5]
  singletons, which changes one bound per round for ~length rounds.
* uneven instances: propagator counts log-uniform, vars = props / 4, the mix
  with 5% truncating division and 5% truncating modulo (q = y tdiv z,
  m = q * z, y = m + x: two fresh variables, three propagators).
* search nodes: k ~ U[1, 64] variables of a base store bisected at
  lb + (ub - lb) / 2 into the lower or upper half.

Two variants of the random part:
* variant="spec": variable indices uniform.  With 20% reified propagators
  whose target must meet [0, 1], these instances are empty at install (the
  failure path), so the fixpoint is trivial;
* variant="planted" (default for benchmarks): a hidden assignment s with
  s_v in [lb_v, ub_v] is drawn first; y and z are uniform and x is drawn
  among the variables whose hidden value equals s_y op s_z, so the hidden
  assignment satisfies every propagator and the fixpoint is never empty.
  The reified targets are drawn from the variables whose domain holds [0, 1]
  and whose hidden value is 0 or 1.
"""
import decimal

import numpy as np

ADD, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, EQ, LEQ = range(10)
INF = 2**31 - 1
MINF = -2**31

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


class Rng:
    """Counter-based splitmix64: stream `key` of seed `seed`."""

    def __init__(self, seed, key=0):
        with np.errstate(over="ignore"):
            self.base = np.uint64((int(seed) * 0x632BE59BD9B4E019 + int(key) * 0x8CB92BA72F3D8DD7
                                   + 0x2545F4914F6CDD1D) & 0xFFFFFFFFFFFFFFFF)
        self.ctr = 0

    def u64(self, n):
        with np.errstate(over="ignore"):
            i = np.arange(self.ctr, self.ctr + n, dtype=np.uint64)
            self.ctr += n
            z = self.base + (i + np.uint64(1)) * _GAMMA
            z = (z ^ (z >> np.uint64(30))) * _C1
            z = (z ^ (z >> np.uint64(27))) * _C2
            return z ^ (z >> np.uint64(31))

    def integers(self, lo, hi, n):
        """n integers uniform in [lo, hi] (inclusive); lo/hi may be arrays."""
        lo = np.asarray(lo, np.int64)
        hi = np.asarray(hi, np.int64)
        span = (hi - lo + 1).astype(np.uint64)
        return lo + (self.u64(n) % span).astype(np.int64)

    def random(self, n):
        return (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


class Instance:
    """A PIR instance: initial store and bytecode (int32 arrays)."""

    def __init__(self, lb, ub, op, x, y, z, **meta):
        self.lb = np.ascontiguousarray(lb, np.int32)
        self.ub = np.ascontiguousarray(ub, np.int32)
        self.op = np.ascontiguousarray(op, np.int32)
        self.x = np.ascontiguousarray(x, np.int32)
        self.y = np.ascontiguousarray(y, np.int32)
        self.z = np.ascontiguousarray(z, np.int32)
        self.meta = meta

    @property
    def nvars(self):
        return len(self.lb)

    @property
    def nprops(self):
        return len(self.op)

    def store(self):
        return np.ascontiguousarray(np.stack([self.lb, self.ub], 1))


# Operator mix of the plain workloads: (kind, fraction).  "sub" is x = y - z.
MIX_BASE = (("add", .45), ("mul", .15), ("min", .05), ("max", .05), ("sub", .10), ("leq", .20))
MIX_UNEVEN = (("add", .40), ("mul", .15), ("min", .05), ("max", .05), ("sub", .10), ("leq", .15),
              ("tdiv", .05), ("tmod", .05))


def _counts(n, mix):
    """Exact per-kind counts (largest remainder), in mix order."""
    raw = np.array([f for _, f in mix]) * n
    c = np.floor(raw).astype(np.int64)
    rem = n - c.sum()
    order = np.argsort(-(raw - c), kind="stable")
    c[order[:rem]] += 1
    return {k: int(v) for (k, _), v in zip(mix, c)}


def _bounds(rng, nvars, scale):
    lb = rng.integers(-scale, 0, nvars)
    ub = lb + rng.integers(0, 2 * scale, nvars)
    return lb, ub


class _ValueIndex:
    """Variables grouped by hidden value, for drawing x with s_x == v."""

    def __init__(self, s, mask=None):
        idx = np.arange(len(s)) if mask is None else np.nonzero(mask)[0]
        order = np.argsort(s[idx], kind="stable")
        self.vars = idx[order]
        self.vals = s[self.vars]

    def draw(self, rng, v):
        """For each value in v: a uniform variable with that hidden value, or -1."""
        lo = np.searchsorted(self.vals, v, "left")
        hi = np.searchsorted(self.vals, v, "right")
        cnt = hi - lo
        pick = lo + (rng.u64(len(v)) % np.maximum(cnt, 1).astype(np.uint64)).astype(np.int64)
        out = np.where(cnt > 0, self.vars[np.minimum(pick, len(self.vars) - 1)], -1)
        return out


def _planted(rng, kind, count, s, vidx, bidx, nvars, pool=None):
    """`count` propagators of one kind whose hidden values satisfy them.
    Returns arrays (x, y, z) in the x = y op z convention of that kind."""
    xs, ys, zs = [], [], []
    need = count
    tries = 0
    while need > 0:
        tries += 1
        if tries > 400:
            raise RuntimeError("planted generator could not place %s propagators" % kind)
        m = max(4 * need, 1024)
        y = rng.integers(0, nvars - 1, m) if pool is None else pool[rng.integers(0, len(pool) - 1, m)]
        z = rng.integers(0, nvars - 1, m) if pool is None else pool[rng.integers(0, len(pool) - 1, m)]
        sy, sz = s[y], s[z]
        if kind == "add":
            v = sy + sz
        elif kind == "sub":
            v = sy - sz
        elif kind == "mul":
            v = sy * sz
        elif kind == "min":
            v = np.minimum(sy, sz)
        elif kind == "max":
            v = np.maximum(sy, sz)
        elif kind == "leq":
            v = (sy <= sz).astype(np.int64)
        elif kind in ("tdiv", "tmod"):
            ok = sz != 0
            q = np.where(ok, np.trunc(sy / np.where(ok, sz, 1)).astype(np.int64), 0)
            v = q if kind == "tdiv" else sy - q * sz
        else:
            raise ValueError(kind)
        x = (bidx if kind == "leq" else vidx).draw(rng, v)
        good = x >= 0
        if kind in ("tdiv", "tmod"):
            good &= ok
        if kind in ("min", "max"):
            good &= (x != y) & (x != z)
        x, y, z = x[good][:need], y[good][:need], z[good][:need]
        xs.append(x); ys.append(y); zs.append(z)
        need -= len(x)
    return np.concatenate(xs), np.concatenate(ys), np.concatenate(zs)


def plain(nvars, nprops, scale, seed, variant="planted", mix=MIX_BASE, key=0):
    """Random part of the plain / node / uneven workloads."""
    rng = Rng(seed, key)
    lb, ub = _bounds(rng, nvars, scale)
    counts = _counts(nprops, mix)
    ops, X, Y, Z = [], [], [], []
    fresh = [nvars]  # next fresh variable index (modulo decompositions)
    if variant == "spec":
        s = None
        for kind, c in counts.items():
            if c == 0:
                continue
            x = rng.integers(0, nvars - 1, c)
            y = rng.integers(0, nvars - 1, c)
            z = rng.integers(0, nvars - 1, c)
            if kind in ("tdiv", "tmod"):
                # divisor domain built to exclude 0
                zlo = rng.integers(1, scale, c)
                lb[z], ub[z] = zlo, zlo + rng.integers(0, scale, c)
            _emit(kind, x, y, z, ops, X, Y, Z, fresh)
    elif variant == "planted":
        s = rng.integers(lb, ub, nvars)
        # boolean-capable variables: domain holds [0, 1]; hidden value 0 or 1
        boolmask = (lb <= 0) & (ub >= 1) & (rng.random(nvars) < 0.5)
        s = np.where(boolmask, rng.integers(0, 1, nvars), s)
        vidx = _ValueIndex(s)
        bidx = _ValueIndex(s, boolmask)
        for kind, c in counts.items():
            if c == 0:
                continue
            x, y, z = _planted(rng, kind, c, s, vidx, bidx, nvars)
            if kind in ("tdiv", "tmod"):
                # keep the divisor's domain clear of 0 (its hidden value is not 0)
                zpos = s[z] > 0
                lb[z] = np.where(zpos, np.maximum(lb[z], 1), lb[z])
                ub[z] = np.where(~zpos, np.minimum(ub[z], -1), ub[z])
            _emit(kind, x, y, z, ops, X, Y, Z, fresh)
    else:
        raise ValueError(variant)
    nfresh = fresh[0] - nvars
    lb_all = np.concatenate([lb, np.full(nfresh, MINF, np.int64)])
    ub_all = np.concatenate([ub, np.full(nfresh, INF, np.int64)])
    op = np.concatenate(ops) if ops else np.zeros(0, np.int64)
    inst = Instance(lb_all, ub_all, op, np.concatenate(X), np.concatenate(Y), np.concatenate(Z),
                    variant=variant, seed=seed, scale=scale)
    # shuffle propagators (the engines sort by opcode themselves)
    perm = np.argsort(Rng(seed, key + 7).u64(inst.nprops), kind="stable")
    inst.op, inst.x, inst.y, inst.z = (a[perm].copy() for a in (inst.op, inst.x, inst.y, inst.z))
    if s is not None:
        inst.meta["hidden"] = _complete_hidden(s, inst, nvars)
    return inst


def _complete_hidden(s, inst, nvars):
    """Hidden values of the fresh modulo variables (q = y tdiv z, m = q * z)."""
    h = np.concatenate([s, np.zeros(inst.nvars - nvars, np.int64)])
    q = (inst.op == TDIV) & (inst.x >= nvars)
    h[inst.x[q]] = np.trunc(h[inst.y[q]] / h[inst.z[q]]).astype(np.int64)
    m = (inst.op == MUL) & (inst.x >= nvars)
    h[inst.x[m]] = h[inst.y[m]] * h[inst.z[m]]
    return h


def _emit(kind, x, y, z, ops, X, Y, Z, fresh):
    """Bytecode of `count` constraints x = y <kind> z."""
    n = len(x)
    if kind == "sub":     # x = y - z  <=>  y = x + z
        ops.append(np.full(n, ADD)); X.append(y); Y.append(x); Z.append(z)
    elif kind == "tmod":  # x = y tmod z  <=>  q = y tdiv z, m = q * z, y = m + x
        q = np.arange(fresh[0], fresh[0] + n)
        m = np.arange(fresh[0] + n, fresh[0] + 2 * n)
        fresh[0] += 2 * n
        ops += [np.full(n, TDIV), np.full(n, MUL), np.full(n, ADD)]
        X += [q, m, y]
        Y += [y, q, m]
        Z += [z, z, x]
    else:
        code = {"add": ADD, "mul": MUL, "min": MIN, "max": MAX, "leq": LEQ, "tdiv": TDIV}[kind]
        ops.append(np.full(n, code)); X.append(x); Y.append(y); Z.append(z)


def add_chain(inst, length, scale, seed, key=11):
    """Appends x_{i+1} = x_i + c_i over length+1 new variables x_i and length
    constant variables c_i ~ U[1, 5].  x_0 = [0, scale]; the others start at
    [-scale, scale], so the upper bounds ripple back from x_length one link
    per round (and against the propagator order)."""
    if 5 * length >= scale:
        raise ValueError("chain of %d links does not fit in [-%d, %d]" % (length, scale, scale))
    rng = Rng(seed, key)
    n0 = inst.nvars
    xs = np.arange(n0, n0 + length + 1)
    cs = np.arange(n0 + length + 1, n0 + 2 * length + 1)
    c = rng.integers(1, 5, length)
    lb = np.concatenate([inst.lb, np.full(length + 1, -scale), c]).astype(np.int64)
    ub = np.concatenate([inst.ub, np.full(length + 1, scale), c]).astype(np.int64)
    lb[n0] = 0
    op = np.concatenate([inst.op, np.full(length, ADD)])
    x = np.concatenate([inst.x, xs[1:]])
    y = np.concatenate([inst.y, xs[:-1]])
    z = np.concatenate([inst.z, cs])
    out = Instance(lb, ub, op, x, y, z, **inst.meta)
    out.meta["chain"] = (int(n0), int(length))
    if "hidden" in inst.meta:
        # a solution of the chain: x_0 = 0, x_i = prefix sums
        hc = np.concatenate([[0], np.cumsum(c)])
        out.meta["hidden"] = np.concatenate([inst.meta["hidden"], hc, c])
    return out


# ----------------------------------------------------------- workloads -----

def single_small(seed=0, variant="planted"):
    """1,000 vars, 3,000 propagators, bounds scale 1,000."""
    return plain(1000, 3000, 1000, seed, variant)


def single_large(seed=0, variant="planted", nvars=1_000_000, nprops=4_000_000, chain=20_000):
    """1,000,000 vars / 4,000,000 propagators at bounds scale 1e6, plus a
    20,000-link chain."""
    inst = plain(nvars, nprops, 1_000_000, seed, variant)
    return add_chain(inst, chain, 1_000_000, seed) if chain else inst


def nodes(base_vars=100_000, base_props=400_000, nnodes=4096, seed=0, kmax=64, base_store=None,
          scale=1_000_000):
    """Search nodes over a base instance (bounds scale 1e6: at scale 1e3 the
    planted base's fixpoint fixes nearly every variable and leaves nothing to
    branch on): node j bisects k_j ~ U[1, kmax]
    random unfixed variables (lb < ub) of `base_store` (lb, ub arrays; the base
    instance's fixpoint in practice) at mid = lb + (ub - lb) / 2, keeping the
    lower half [lb, mid] or the upper half [mid + 1, ub] by a coin flip.
    Returns (base Instance, off, var, lb, ub) with the tightenings in CSR form."""
    base = plain(base_vars, base_props, scale, seed)
    if base_store is None:
        blb, bub = base.lb.astype(np.int64), base.ub.astype(np.int64)
    else:
        blb, bub = (np.asarray(a, np.int64) for a in base_store)
    free = np.nonzero(blb[:base_vars] < bub[:base_vars])[0]
    if len(free) == 0:
        raise ValueError("every variable of the base store is fixed")
    rng = Rng(seed, 101)
    k = rng.integers(1, kmax, nnodes)
    off = np.concatenate([[0], np.cumsum(k)]).astype(np.int32)
    tot = int(off[-1])
    var = free[rng.integers(0, len(free) - 1, tot)]
    lo, hi = blb[var], bub[var]
    mid = lo + (hi - lo) // 2
    upper = rng.integers(0, 1, tot) == 1
    tl = np.where(upper, mid + 1, lo)
    tu = np.where(upper, hi, mid)
    return base, off, var.astype(np.int32), tl.astype(np.int32), tu.astype(np.int32)


def uneven_sizes(ninst, pmin, pmax, seed):
    """The uneven workload's propagator counts before the modulo decomposition:
    floor(exp(ln pmin + u (ln pmax - ln pmin))), u uniform in [0, 1), in
    decimal arithmetic (software, correctly rounded), so the sizes are the same
    on every machine; numpy's exp / log come from the platform's libm."""
    u = Rng(seed, 202).random(ninst)
    c = decimal.Context(prec=50)
    lo, hi = c.ln(decimal.Decimal(pmin)), c.ln(decimal.Decimal(pmax))
    return np.array([int(c.exp(c.add(lo, c.multiply(decimal.Decimal(float(x)), c.subtract(hi, lo))))
                         .to_integral_value(rounding=decimal.ROUND_FLOOR)) for x in u], np.int64)


def uneven(ninst=512, pmin=1_000, pmax=200_000, seed=0, variant="planted"):
    """Independent instances with log-uniform propagator counts in
    [pmin, pmax], vars = props / 4, the mix with truncating division and
    modulo.  Returns a list of Instances."""
    props = uneven_sizes(ninst, pmin, pmax, seed)
    out = []
    for j, p in enumerate(props):
        nv = max(int(p) // 4, 8)
        out.append(plain(nv, int(p), 1000, seed * 100003 + j, variant, MIX_UNEVEN, key=300 + j))
    return out


def pack(instances):
    """Concatenate instances: returns (prop_off, var_off, op, x, y, z, lb, ub)
    with var indices local to each instance."""
    prop_off = np.zeros(len(instances) + 1, np.int64)
    var_off = np.zeros(len(instances) + 1, np.int64)
    for j, inst in enumerate(instances):
        prop_off[j + 1] = prop_off[j] + inst.nprops
        var_off[j + 1] = var_off[j] + inst.nvars
    cat = lambda f: np.concatenate([getattr(i, f) for i in instances]).astype(np.int32)
    return prop_off, var_off, cat("op"), cat("x"), cat("y"), cat("z"), cat("lb"), cat("ub")


def queens(n):
    """n queens as PIR propagators: q_i in [0, n-1] is the row of the queen in
    column i; for i < j, d_ij = q_i - q_j (ADD q_i = d_ij + q_j) and
    d_ij != 0, d_ij != j - i, d_ij != i - j, each written as the reified
    EQ false = (d_ij == c) with c a singleton.  Variables: q_0..q_{n-1}, then
    the d_ij, the constants -(n-1)..n-1 and false = [0, 0].  Solutions: 1, 0,
    0, 2, 10, 4, 40, 92 for n = 1..8."""
    pairs = [(i, j) for i in range(n) for j in range(i + 1, n)]
    nq, nd = n, len(pairs)
    c0 = nq + nd                      # constant k lives at c0 + k + (n - 1)
    false = c0 + 2 * n - 1
    nvars = false + 1
    lb = np.zeros(nvars, np.int64)
    ub = np.zeros(nvars, np.int64)
    ub[:nq] = n - 1
    lb[nq:c0] = -(n - 1)
    ub[nq:c0] = n - 1
    for k in range(-(n - 1), n):
        lb[c0 + k + n - 1] = ub[c0 + k + n - 1] = k
    op, x, y, z = [], [], [], []
    for t, (i, j) in enumerate(pairs):
        d = nq + t
        op.append(ADD); x.append(i); y.append(d); z.append(j)
        for k in (0, j - i, i - j):
            op.append(EQ); x.append(false); y.append(d); z.append(c0 + k + n - 1)
    return Instance(lb, ub, op, x, y, z, queens=n)


# ----------------------------------------------------------------------- PC --
# Tree propagators for lala-pc's PC domain (tape format of include/pirgpu.h,
# enum pc_kind), built from the constraint shapes of lala-pc's PC tests
# (tests/pc_test.cpp): pseudo-boolean / linear sums (PseudoBoolean*), reified
# differences (ResourceConstraint*, InfiniteDomain*), disjunctive temporal
# constraints (TemporalConstraint*) and max equalities (MaxConstraint*).
PC_MIX = (("linear", .40), ("reified", .30), ("disjunctive", .20), ("max", .10))
_PC = dict(VAR=0, CONST=1, ADD=5, SUB=6, MUL=7, MAX=13, NADD=14, PVAR=16, LEQ=20, EQ=22, OR=25, EQUIV=26, ARG=29)


def pc_mix(nvars=1_000_000, nprops=1_000_000, scale=1000, seed=0, terms=4, key=31):
    """A planted PC instance: a hidden assignment s (s_v in [lb_v, ub_v]) is
    drawn first and every propagator holds under it, so the fixpoint is not
    empty and its rounds narrow domains towards s.  Shapes (nodes per tree):

      linear       sum_k a_k * x_k <= b, `terms` terms, a_k ~ U[1, 5],
                   b = sum a_k s_k + U[0, 10 * terms]      (3*terms + terms + 3)
      reified      r <=> (x - y <= k), r a fresh 0/1 variable,
                   k = s_x - s_y + U[-10, 10]              (7)
      disjunctive  (x + dx <= y) or (y + dy <= x), the disjunct s satisfies
                   with a slack drawn in [0, |s_x - s_y|]  (11)
      max          z = max(x, y), z fresh with domain [-2S, 2S]  (5)

    Returns (tape (n, 4) int32, roots int32, lb int32, ub int32, hidden int64)."""
    rng = Rng(seed, key)
    lb, ub = _bounds(rng, nvars, scale)
    s = rng.integers(lb, ub, nvars)
    counts = _counts(nprops, PC_MIX)
    blocks, roots = [], []
    extra_lb, extra_ub, extra_s = [], [], []
    base = [0]
    nv = [nvars]

    def fresh(lo, hi, val):
        n = len(val)
        idx = np.arange(nv[0], nv[0] + n)
        nv[0] += n
        extra_lb.append(np.broadcast_to(np.asarray(lo, np.int64), (n,)))
        extra_ub.append(np.broadcast_to(np.asarray(hi, np.int64), (n,)))
        extra_s.append(np.asarray(val, np.int64))
        return idx

    def emit(rows, width, root):
        """rows: (count, width, 4) with child fields relative to the tree."""
        c = rows.shape[0]
        start = base[0] + width * np.arange(c)
        rows = rows.copy()
        k = rows[:, :, 0]
        refs_a = ~np.isin(k, [_PC["VAR"], _PC["CONST"], _PC["PVAR"]])
        refs_b = np.isin(k, [_PC["ADD"], _PC["SUB"], _PC["MUL"], _PC["MAX"], _PC["LEQ"], _PC["EQ"], _PC["OR"],
                             _PC["EQUIV"]])
        rows[:, :, 1] += np.where(refs_a, start[:, None], 0)
        rows[:, :, 2] += np.where(refs_b, start[:, None], 0)
        blocks.append(rows.reshape(-1, 4))
        roots.append(start + root)
        base[0] += c * width

    def draw(c):
        return rng.integers(0, nvars - 1, c)

    P = _PC
    c = counts["linear"]
    if c:
        K = terms
        w = 4 * K + 3
        rows = np.zeros((c, w, 4), np.int64)
        xs = np.stack([draw(c) for _ in range(K)], 1)
        a = rng.integers(1, 5, c * K).reshape(c, K)
        for t in range(K):
            rows[:, 3 * t] = np.stack([np.full(c, P["VAR"]), xs[:, t], np.zeros(c), np.zeros(c)], 1)
            rows[:, 3 * t + 1] = np.stack([np.full(c, P["CONST"]), a[:, t], a[:, t], np.zeros(c)], 1)
            rows[:, 3 * t + 2] = [P["MUL"], 3 * t + 1, 3 * t, 0]
            rows[:, 3 * K + t] = [P["ARG"], 3 * t + 2, 0, 0]
        b = (a * s[xs]).sum(1) + rng.integers(0, 10 * K, c)
        rows[:, 4 * K] = [P["NADD"], 3 * K, K, 0]
        rows[:, 4 * K + 1] = np.stack([np.full(c, P["CONST"]), b, b, np.zeros(c)], 1)
        rows[:, 4 * K + 2] = [P["LEQ"], 4 * K, 4 * K + 1, 0]
        emit(rows, w, 4 * K + 2)
    c = counts["reified"]
    if c:
        x, y = draw(c), draw(c)
        k = s[x] - s[y] + rng.integers(-10, 10, c)
        r = fresh(0, 1, (s[x] - s[y] <= k).astype(np.int64))
        rows = np.zeros((c, 7, 4), np.int64)
        rows[:, 0] = np.stack([np.full(c, P["VAR"]), x, np.zeros(c), np.zeros(c)], 1)
        rows[:, 1] = np.stack([np.full(c, P["VAR"]), y, np.zeros(c), np.zeros(c)], 1)
        rows[:, 2] = [P["SUB"], 0, 1, 0]
        rows[:, 3] = np.stack([np.full(c, P["CONST"]), k, k, np.zeros(c)], 1)
        rows[:, 4] = [P["LEQ"], 2, 3, 0]
        rows[:, 5] = np.stack([np.full(c, P["PVAR"]), r, np.zeros(c), np.zeros(c)], 1)
        rows[:, 6] = [P["EQUIV"], 5, 4, 0]
        emit(rows, 7, 6)
    c = counts["disjunctive"]
    if c:
        x, y = draw(c), draw(c)
        gap = np.abs(s[x] - s[y])
        first = s[x] <= s[y]  # x + dx <= y holds for dx <= gap
        d_hold = rng.integers(0, gap, c)
        d_other = rng.integers(1, 20, c)
        dx = np.where(first, d_hold, d_other)
        dy = np.where(first, d_other, d_hold)
        rows = np.zeros((c, 11, 4), np.int64)
        for j, v in ((0, x), (3, y), (5, y), (8, x)):
            rows[:, j] = np.stack([np.full(c, P["VAR"]), v, np.zeros(c), np.zeros(c)], 1)
        rows[:, 1] = np.stack([np.full(c, P["CONST"]), dx, dx, np.zeros(c)], 1)
        rows[:, 6] = np.stack([np.full(c, P["CONST"]), dy, dy, np.zeros(c)], 1)
        rows[:, 2] = [P["ADD"], 0, 1, 0]
        rows[:, 4] = [P["LEQ"], 2, 3, 0]
        rows[:, 7] = [P["ADD"], 5, 6, 0]
        rows[:, 9] = [P["LEQ"], 7, 8, 0]
        rows[:, 10] = [P["OR"], 4, 9, 0]
        emit(rows, 11, 10)
    c = counts["max"]
    if c:
        x, y = draw(c), draw(c)
        z = fresh(-2 * scale, 2 * scale, np.maximum(s[x], s[y]))
        rows = np.zeros((c, 5, 4), np.int64)
        rows[:, 0] = np.stack([np.full(c, P["VAR"]), x, np.zeros(c), np.zeros(c)], 1)
        rows[:, 1] = np.stack([np.full(c, P["VAR"]), y, np.zeros(c), np.zeros(c)], 1)
        rows[:, 2] = [P["MAX"], 0, 1, 0]
        rows[:, 3] = np.stack([np.full(c, P["VAR"]), z, np.zeros(c), np.zeros(c)], 1)
        rows[:, 4] = [P["EQ"], 2, 3, 0]
        emit(rows, 5, 4)
    tape = np.ascontiguousarray(np.concatenate(blocks), np.int32)
    roots = np.ascontiguousarray(np.concatenate(roots), np.int32)
    lb_all = np.concatenate([lb] + extra_lb)
    ub_all = np.concatenate([ub] + extra_ub)
    hidden = np.concatenate([s] + extra_s)
    return tape, roots, np.ascontiguousarray(lb_all, np.int32), np.ascontiguousarray(ub_all, np.int32), hidden
