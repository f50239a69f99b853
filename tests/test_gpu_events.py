"""Event-driven single-instance fixpoint (sched = EVENTS) against the CPU
oracle: bit-exact bounds and the same failure flag, on planted, failing,
chain and uneven (division) instances, with the small-frontier rounds run on
one CTA or on the whole grid."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from golden import kat_cases as K
from kat_runner import GpuEngine, run_case


@pytest.fixture(scope="module")
def P():
    import pirgpu
    return pirgpu


def _both(P, oracle, inst, **kw):
    # the event kernel from the first round unless a test asks for the AC-1 lead
    kw.setdefault("lead", -1)
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS, **kw)
    lb, ub = ctx.read_store()
    s = inst.store()
    orc, info = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
    return rc, np.stack([lb, ub], 1), st, orc, s, info


@pytest.mark.parametrize("local", [0, 1, 1 << 30])
@pytest.mark.parametrize("seed", range(4))
def test_events_small_planted(seed, local, P, oracle):
    import workloads as W
    inst = W.single_small(seed)
    rc, g, st, orc, o, _ = _both(P, oracle, inst, local_frontier=local)
    assert rc == orc
    if orc == oracle.OK:
        np.testing.assert_array_equal(g, o)


@pytest.mark.parametrize("seed", range(3))
def test_events_spec_fails(seed, P, oracle):
    import workloads as W
    inst = W.single_small(seed, variant="spec")
    rc, _, _, orc, _, _ = _both(P, oracle, inst)
    assert rc == orc == oracle.FAILED


@pytest.mark.parametrize("chase", [-1, 0])
@pytest.mark.parametrize("local", [0, 1])
def test_events_chain_and_random(local, chase, P, oracle):
    """100k vars / 400k propagators plus a 3,000-link chain, every propagator
    on its own (no segments): without chasing the deep part takes a round per
    link, mostly small-frontier rounds; with it, a few dozen rounds."""
    import workloads as W
    inst = W.add_chain(W.plain(100_000, 400_000, 10**6, 7), 3000, 10**6, 7)
    rc, g, st, orc, o, info = _both(P, oracle, inst, local_frontier=local, chase=chase, segments=-1)
    assert rc == orc == oracle.OK
    np.testing.assert_array_equal(g, o)
    if chase < 0:
        assert st["rounds"] >= 2500  # about one link per round
        # far fewer executions than AC-1 sweeps of every propagator
        assert st["executions"] < st["rounds"] * inst.nprops // 20
    else:
        assert st["rounds"] < 500
        assert st["executions"] < 20 * inst.nprops


@pytest.mark.parametrize("segments", [0, -1])
@pytest.mark.parametrize("chase", [-1, 0])
@pytest.mark.parametrize("local", [0, 300, 1 << 30])
def test_events_hub_overflow(local, chase, segments, P, oracle):
    """A 300-link chain whose middle variable feeds 3,000 more propagators
    y_j = x_150 + c_j: the round that narrows x_150 lists more propagators
    than a round on one CTA keeps in shared memory (256) and than its dedupe
    set holds (2,048), so both spill to the global list and round stamps."""
    import workloads as W
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    chain = W.add_chain(empty, 300, 10**6, 5)
    n0, k, hub = chain.nvars, 3000, 150
    c = np.random.default_rng(5).integers(1, 6, k)
    ys, cs = np.arange(n0, n0 + k), np.arange(n0 + k, n0 + 2 * k)
    inst = W.Instance(np.concatenate([chain.lb, np.full(k, -10**6), c]),
                      np.concatenate([chain.ub, np.full(k, 10**6), c]),
                      np.concatenate([chain.op, np.full(k, W.ADD)]), np.concatenate([chain.x, ys]),
                      np.concatenate([chain.y, np.full(k, hub)]), np.concatenate([chain.z, cs]))
    rc, g, st, orc, o, info = _both(P, oracle, inst, local_frontier=local, chase=chase, segments=segments)
    assert rc == orc == oracle.OK
    np.testing.assert_array_equal(g, o)
    assert st["certify_narrowed"] == 0
    # (a round may read bounds joined earlier in the same round, so the waves
    # can move faster than one link per round; segments move 64 links a round)
    if segments < 0:
        assert st["rounds"] >= (100 if chase < 0 else 2)
    # x_150 narrows in about 150 rounds, each listing its 3,002 propagators
    # (once each): fewer executions than the oracle's 301 sweeps
    assert st["executions"] < info["execs"]


@pytest.mark.parametrize("chase", [-1, 1, 3, 64, 100_000])  # 100,000: capped at 256
@pytest.mark.parametrize("local", [1, 256, 1 << 30])
def test_events_chase(chase, local, P, oracle):
    """The chase budget (runs of small variables' propagators done at once by
    the narrowing thread; -1: none) changes the rounds, never the fixpoint
    (every propagator on its own, no segments)."""
    import workloads as W
    inst = W.add_chain(W.plain(30_000, 120_000, 10**6, 11), 2000, 10**6, 11)
    rc, g, st, orc, o, _ = _both(P, oracle, inst, local_frontier=local, chase=chase, segments=-1)
    assert rc == orc == oracle.OK
    np.testing.assert_array_equal(g, o)
    if chase < 0:
        assert st["rounds"] >= 1500  # about one link per round
    elif chase >= 64:
        assert st["rounds"] < 1000


def _mixed_chain(L, seed):
    """x_{i+1} = x_i op c_i with op in {+, max, min, *} and c_i in [1, 3],
    each x_{i+1} also reified against a constant (b_i <-> x_{i+1} <= t_i or
    x_{i+1} = t_i); the last link's upper bound is cut so that a wave also
    runs back.  Every variable has at most 3 propagators, so chases run
    through all of it, including reified propagators whose result needs both
    bounds of a variable."""
    import workloads as W
    rng = np.random.default_rng(seed)
    lb, ub, op, X, Y, Z = [], [], [], [], [], []

    def var(lo, hi):
        lb.append(lo)
        ub.append(hi)
        return len(lb) - 1

    x = var(0, 20)
    for _ in range(L):
        c = int(rng.integers(1, 4))
        cv = var(c, c)
        nx = var(-10**6, 10**6)
        op.append([W.ADD, W.MAX, W.MIN, W.MUL][int(rng.integers(0, 4))])
        X.append(nx), Y.append(x), Z.append(cv)
        t = int(rng.integers(0, 40))
        op.append(W.LEQ if rng.integers(0, 2) else W.EQ)
        X.append(var(0, 1)), Y.append(nx), Z.append(var(t, t))
        x = nx
    ub[x] = int(rng.integers(5, 60))
    return W.Instance(lb, ub, op, X, Y, Z)


@pytest.mark.parametrize("segments", [0, -1])
@pytest.mark.parametrize("chase", [-1, 0, 1, 256])
@pytest.mark.parametrize("seed", range(6))
def test_events_chase_mixed_chains(seed, chase, segments, P, oracle):
    inst = _mixed_chain(1500, seed)
    for local in (0, 1 << 30):
        rc, g, st, orc, o, _ = _both(P, oracle, inst, local_frontier=local, chase=chase, segments=segments)
        assert rc == orc
        if orc == oracle.OK:
            np.testing.assert_array_equal(g, o)
            assert st["certify_narrowed"] == 0


def test_events_long_chain_capped_chase(P):
    """A 100,000-link chain x_{i+1} = x_i + c_i with x_0 in [0, 1e6] and every
    x_i in [-1e6, 1e6]: its fixpoint is x_i in [prefix sum, 1e6 - suffix sum].
    An unbounded chase request is capped, so no round outlasts the grid
    barrier's wait limit."""
    import workloads as W
    L = 100_000
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    inst = W.add_chain(empty, L, 10**6, 3)
    c = inst.lb[L + 1:].astype(np.int64)
    want_lb = np.concatenate([[0], np.cumsum(c)])
    want_ub = 10**6 - np.concatenate([np.cumsum(c[::-1])[::-1], [0]])
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS, chase=1 << 30, segments=-1, lead=-1)
    assert rc == P.OK
    lb, ub = ctx.read_store()
    np.testing.assert_array_equal(lb[:L + 1], want_lb)
    np.testing.assert_array_equal(ub[:L + 1], want_ub)
    # capped: far more rounds than the 3 an unbounded chase takes (a chaser
    # that starts late inside what the front already updated can carry it
    # past 256 links in a round, so not L / 256 exactly)
    assert st["rounds"] >= L // 1024
    # as segments of at most 64 links, a warp chasing at most 32 of them per
    # entry: the same store
    ctx.load_store(inst.lb, inst.ub)
    rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS, lead=-1)
    assert rc == P.OK and st["certify_narrowed"] == 0
    lb, ub = ctx.read_store()
    np.testing.assert_array_equal(lb[:L + 1], want_lb)
    np.testing.assert_array_equal(ub[:L + 1], want_ub)
    assert st["rounds"] < L // 64 + 100


@pytest.mark.parametrize("chase", [-1, 0, 2])
@pytest.mark.parametrize("seed", range(3))
def test_events_chase_failures_and_divisions(seed, chase, P, oracle):
    import workloads as W
    for inst in [W.single_small(seed, variant="spec")] + W.uneven(3, 2000, 20_000, seed):
        rc, g, _, orc, o, _ = _both(P, oracle, inst, chase=chase)
        assert rc == orc
        if orc == oracle.OK:
            np.testing.assert_array_equal(g, o)


@pytest.mark.parametrize("seed", range(3))
def test_events_chain_local_everywhere(seed, P, oracle):
    """Every round after the first on one CTA, frontiers of thousands
    included, on the chain-and-random instance."""
    import workloads as W
    inst = W.add_chain(W.plain(20_000, 80_000, 10**6, seed), 1000, 10**6, seed)
    rc, g, st, orc, o, _ = _both(P, oracle, inst, local_frontier=1 << 30)
    assert rc == orc
    if orc == oracle.OK:
        np.testing.assert_array_equal(g, o)


def test_events_uneven_divisions(P, oracle):
    import workloads as W
    for inst in W.uneven(6, 2000, 40_000, 3):
        rc, g, _, orc, o, _ = _both(P, oracle, inst)
        assert rc == orc
        if orc == oracle.OK:
            np.testing.assert_array_equal(g, o)


def test_events_round_cap(P, oracle):
    import workloads as W
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    inst = W.add_chain(empty, 2000, 10**6, 1)
    for local, chase, cap, segs in ((0, -1, 100, -1), (1, -1, 100, -1), (0, 0, 2, -1), (1, 0, 2, -1),
                                    (0, -1, 10, 0), (1, -1, 10, 0)):
        ctx = P.Context(0)
        ctx.load_store(inst.lb, inst.ub)
        ctx.tell(inst.op, inst.x, inst.y, inst.z)
        rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS, max_rounds=cap, local_frontier=local, chase=chase, lead=-1,
                              segments=segs)
        assert rc == P.TIMEOUT and st["rounds"] == cap
        rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS)
        assert rc == P.OK
        lb, ub = ctx.read_store()
        s = inst.store()
        orc, _ = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        np.testing.assert_array_equal(np.stack([lb, ub], 1), s)


@pytest.mark.parametrize("local", [0, 1, 1 << 30])
def test_events_segments_chain_and_random(local, P, oracle):
    """100k vars / 400k propagators plus a 3,000-link chain, the chain run as
    47 segments of at most 64 links: the oracle's fixpoint in far fewer
    rounds than one link per round, and a certifying sweep that finds
    nothing."""
    import workloads as W
    inst = W.add_chain(W.plain(100_000, 400_000, 10**6, 7), 3000, 10**6, 7)
    o = inst.store()
    orc, _ = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, o)
    assert orc == oracle.OK
    for chase in (0, -1):  # without chasing: segment by segment
        ctx = P.Context(0)
        ctx.load_store(inst.lb, inst.ub)
        ctx.tell(inst.op, inst.x, inst.y, inst.z)
        rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS, local_frontier=local, chase=chase, lead=-1)
        assert rc == P.OK
        np.testing.assert_array_equal(np.stack(ctx.read_store(), 1), o)
        assert st["certify_narrowed"] == 0 and st["certify_executions"] > 0
        assert st["rounds"] < (300 if chase == 0 else 3000 // 20)


def _rings(nring, length, seed):
    """nring rings of `length` propagators, x_{i+1} = x_i + 0 or x_{i+1} =
    max(x_i, c_i) (indices mod length; every x_i occurs twice, so each ring
    is one cycle of link variables: all its variables equal, at least the
    largest c_i), with a reified side check on every 7th variable (which
    breaks the path there)."""
    import workloads as W
    rng = np.random.default_rng(seed)
    lb, ub, op, X, Y, Z = [], [], [], [], [], []

    def var(lo, hi):
        lb.append(lo)
        ub.append(hi)
        return len(lb) - 1

    for _ in range(nring):
        xs = [var(-10**5, 10**5) for _ in range(length)]
        lb[xs[0]], ub[xs[0]] = 0, 50
        for i in range(length):
            mx = rng.integers(0, 4) == 0
            c = int(rng.integers(0, 41)) if mx else 0
            op.append(W.MAX if mx else W.ADD)
            X.append(xs[(i + 1) % length]), Y.append(xs[i]), Z.append(var(c, c))
            if i % 7 == 3:
                t = int(rng.integers(0, 80))
                op.append(W.LEQ)
                X.append(var(0, 1)), Y.append(xs[i]), Z.append(var(t, t))
    return W.Instance(lb, ub, op, X, Y, Z)


@pytest.mark.parametrize("seed", range(3))
def test_events_segments_rings_and_failure(seed, P, oracle):
    """Cycles of link variables (cut once each), and a chain whose last link
    is cut below the sum of its increments, so a segment fails."""
    import workloads as W
    inst = _rings(40, 150, seed)
    rc, g, st, orc, o, _ = _both(P, oracle, inst)
    assert rc == orc
    if orc == oracle.OK:
        np.testing.assert_array_equal(g, o)
        assert st["certify_narrowed"] == 0
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    chain = W.add_chain(empty, 500, 10**6, seed)
    chain.lb[0], chain.ub[0] = 0, 0
    chain.ub[500] = 400  # the increments are at least 1 each: x_500 >= 500
    rc, _, _, orc, _, _ = _both(P, oracle, chain)
    assert rc == orc == oracle.FAILED


@pytest.mark.parametrize("case", K.CASES, ids=[c.name for c in K.CASES])
def test_kat_events(case, P):
    class E(GpuEngine):
        pass
    E.sched = P.SCHED_EVENTS
    E.opts = {"lead": -1}
    assert run_case(case, E) == []


@pytest.mark.parametrize("case", K.CASES, ids=[c.name for c in K.CASES])
def test_kat_events_with_lead(case, P):
    class E(GpuEngine):
        pass
    E.sched = P.SCHED_EVENTS
    assert run_case(case, E) == []


@pytest.mark.parametrize("lead", [0, 4, 64])
def test_events_ac1_lead(lead, P, oracle):
    """The event schedule's default start: AC-1 rounds of the persistent
    kernel until a round whose narrowed bounds have not shrunk by an eighth
    against the round `lead` rounds before (0: 8), then the event kernel
    from that store.  A random instance (the lead may reach the fixpoint
    alone, its last round then being the certifying sweep), the same with a
    2,000-link chain, and a 5,000-link chain with little else (the chain's
    steady trickle is handed over instead of taking one AC-1 round per link):
    the oracle's fixpoint every time."""
    import workloads as W
    for inst in (W.plain(20_000, 80_000, 10**6, 21),
                 W.add_chain(W.plain(20_000, 80_000, 10**6, 22), 2000, 10**6, 22),
                 W.add_chain(W.plain(1000, 100, 10**6, 23), 5000, 10**6, 23)):
        rc, store, st, orc, s, info = _both(P, oracle, inst, lead=lead)
        assert rc == orc == P.OK
        np.testing.assert_array_equal(store, s)
        assert st["certify_executions"] > 0 and st["certify_narrowed"] == 0
        assert st["rounds"] < 1000  # never one round per link


@pytest.mark.parametrize("dense", [0, -1, 1, 1000])
def test_events_dense_rounds(dense, P, oracle):
    """Dense rounds (every unit once, AC-1 style, noting the narrowed
    variables) while the narrowed variables' units are at least 1/dense of
    all and getting fewer (0: 1/32; -1: only the first and the certifying
    round; 1: hardly ever; 1000: nearly every round), then event rounds from
    the noted variables: the oracle's fixpoint or failure every time."""
    import workloads as W
    insts = [W.add_chain(W.plain(30_000, 120_000, 10**6, 11), 2000, 10**6, 11), _mixed_chain(800, 3),
             W.single_small(2, variant="spec")] + W.uneven(2, 2000, 20_000, 5)
    for inst in insts:
        for segments in (0, -1):
            rc, g, st, orc, o, _ = _both(P, oracle, inst, dense=dense, segments=segments)
            assert rc == orc
            if orc == oracle.OK:
                np.testing.assert_array_equal(g, o)
                assert st["certify_narrowed"] == 0


def _add_path(n_links, seed, reverse=False, const_first=False, sign=1, first=(0, 10**6), last=None,
              scale=10**6, extra=0):
    """A path of ADD links over fresh variables v_0 .. v_n with a singleton
    constant per link: v_{i+1} = v_i + c_i, written as x = v_{i+1}, y = v_i,
    z = c_i (reverse: x = v_i, y = v_{i+1}, so v_i = v_{i+1} + c_i;
    const_first: the constant as y), c_i = sign * U[1, 4]; optionally a random
    instance of `extra` propagators beside it."""
    import workloads as W
    rng = np.random.default_rng(seed)
    base = W.plain(max(extra // 4, 8), extra, 1000, seed) if extra else None
    n0 = base.nvars if base else 0
    v = n0 + np.arange(n_links + 1)
    cv = n0 + n_links + 1 + np.arange(n_links)
    c = sign * rng.integers(1, 5, n_links)
    lb = np.full(2 * n_links + 1, -scale, np.int64)
    ub = np.full(2 * n_links + 1, scale, np.int64)
    lb[n_links + 1:] = ub[n_links + 1:] = c
    lb[0], ub[0] = first
    if last is not None:
        lb[n_links], ub[n_links] = last
    xo, yo = (v[:-1], v[1:]) if reverse else (v[1:], v[:-1])
    yy, zz = (cv, yo) if const_first else (yo, cv)
    op = np.zeros(n_links, np.int64)
    if base:
        return W.Instance(np.concatenate([base.lb, lb]), np.concatenate([base.ub, ub]),
                          np.concatenate([base.op, op]), np.concatenate([base.x, xo]),
                          np.concatenate([base.y, yy]), np.concatenate([base.z, zz]))
    return W.Instance(lb, ub, op, xo, yy, zz)


@pytest.mark.parametrize("case", ["forward", "reverse", "const_first", "reverse_const_first", "negative",
                                  "infeasible", "huge_bounds", "with_random"])
@pytest.mark.parametrize("lead", [-1, 0])
def test_events_add_paths(case, lead, P, oracle):
    """Paths of ADD links with constants, which the event kernel's segments
    solve in closed form (the difference-constraint closure along the path)
    when their bounds are small, else sweep: the oracle's store and failure
    flag in every orientation, with the constants as either operand,
    negative constants, an infeasible path and bounds beyond 2^28."""
    kw = dict(reverse=case.startswith("reverse"), const_first=case.endswith("const_first"))
    if case == "negative":
        kw["sign"] = -1
    if case == "infeasible":
        kw.update(first=(0, 0), last=(0, 10))  # v_n >= n while v_n <= 10
    if case == "huge_bounds":
        kw.update(scale=1 << 29, first=(0, 1 << 29))
    if case == "with_random":
        kw["extra"] = 8000
    inst = _add_path(3000, 31, **kw)
    rc, store, st, orc, s, info = _both(P, oracle, inst, lead=lead)
    assert rc == orc
    if case == "infeasible":
        assert rc == P.FAILED
    else:
        assert rc == P.OK
        np.testing.assert_array_equal(store, s)
        assert st["certify_narrowed"] == 0
