"""GPU engine (through the C ABI) against the CPU oracle: bit-exact bounds
and identical failure flags."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from golden import kat_cases as K
from kat_runner import GpuEngine, run_case

MODES = {"auto": 0, "persistent": 1, "hostloop": 2, "smem": 3}


@pytest.fixture(scope="module")
def P():
    import pirgpu
    return pirgpu


@pytest.mark.parametrize("mode", ["persistent", "hostloop", "smem"])
@pytest.mark.parametrize("case", K.CASES, ids=[c.name for c in K.CASES])
def test_kat_gpu(case, mode):
    class E(GpuEngine):
        pass
    E.mode = MODES[mode]
    assert run_case(case, E) == []


def _intervals(lo, hi):
    return np.array([(l, u) for l in range(lo, hi + 1) for u in range(l, hi + 1)], np.int32)


@pytest.mark.parametrize("op", range(10))
def test_deduce_batch_exhaustive(op, P, oracle):
    """One propagator over every interval triple of [-6, 6] and random wide /
    extreme intervals: GPU == oracle bit for bit."""
    itv = _intervals(-6, 6)
    k = len(itv)
    idx = np.stack(np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij"), -1).reshape(-1, 3)
    lb = itv[idx, 0]
    ub = itv[idx, 1]
    rng = np.random.default_rng(op)
    edge = np.array([P.MINF, P.MINF + 1, -2**30, -10**6, -1000, -2, -1, 0, 1, 2, 1000, 10**6, 2**30,
                     P.INF - 1, P.INF], np.int64)
    m = 400_000
    a = np.where(rng.random((m, 3)) < .5, rng.choice(edge, (m, 3)), rng.integers(-10**6, 10**6, (m, 3)))
    b = np.where(rng.random((m, 3)) < .5, rng.choice(edge, (m, 3)), a + rng.integers(0, 10**6, (m, 3)))
    rl = np.minimum(a, b).clip(P.MINF, P.INF).astype(np.int32)
    ru = np.maximum(a, b).clip(P.MINF, P.INF).astype(np.int32)
    # inputs must be non-empty stores (an empty input is a failed store already)
    keep = np.all((rl != P.INF) & (ru != P.MINF), axis=1)
    rl, ru = rl[keep], ru[keep]
    lb = np.concatenate([lb, rl])
    ub = np.concatenate([ub, ru])
    ops = np.full(len(lb), op, np.int32)
    ctx = P.Context(0)
    g = ctx.deduce_batch(ops, lb, ub)
    o = oracle.deduce_batch(ops, lb, ub)
    # bounds compared where neither side reports an empty interval; the
    # failure flag itself must agree everywhere
    np.testing.assert_array_equal(g[3], o[3])
    ok = ~o[3]
    np.testing.assert_array_equal(g[0][ok], o[0][ok])
    np.testing.assert_array_equal(g[1][ok], o[1][ok])
    np.testing.assert_array_equal(g[2][ok], o[2][ok])


def _gpu_fixpoint(P, inst, **kw):
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    rc, st = ctx.fixpoint(**kw)
    lb, ub = ctx.read_store()
    return rc, np.stack([lb, ub], 1), st, ctx


def _oracle_fixpoint(oracle, inst):
    s = inst.store()
    rc, info = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
    return rc, s, info


@pytest.mark.parametrize("mode", ["persistent", "hostloop", "smem"])
@pytest.mark.parametrize("seed", range(10))
def test_single_small(seed, mode, P, oracle):
    import workloads as W
    inst = W.single_small(seed)
    rc, s, st, _ = _gpu_fixpoint(P, inst, mode=MODES[mode])
    orc, os_, info = _oracle_fixpoint(oracle, inst)
    assert rc == orc == P.OK
    np.testing.assert_array_equal(s, os_)
    assert st["rounds"] >= 2


@pytest.mark.parametrize("mode", ["persistent", "hostloop", "smem"])
def test_spec_variant_failure(mode, P, oracle):
    import workloads as W
    for seed in range(3):
        inst = W.single_small(seed, variant="spec")
        rc, _, _, ctx = _gpu_fixpoint(P, inst, mode=MODES[mode])
        orc, _, _ = _oracle_fixpoint(oracle, inst)
        assert rc == orc == P.FAILED
        assert ctx.is_bot()


def _failing_late(seed):
    """A planted instance plus one contradicting unary bound: fails after
    some rounds of propagation rather than at install."""
    import workloads as W
    inst = W.plain(3000, 9000, 1000, seed)
    h = inst.meta["hidden"]
    v = int(np.argmax(inst.ub - inst.lb))
    inst.lb[v] = h[v] + 1 if h[v] < inst.ub[v] else inst.lb[v]
    return inst


@pytest.mark.parametrize("mode", ["persistent", "hostloop", "smem"])
@pytest.mark.parametrize("seed", range(6))
def test_failure_flag_matches(seed, mode, P, oracle):
    inst = _failing_late(seed)
    rc, s, _, _ = _gpu_fixpoint(P, inst, mode=MODES[mode])
    orc, os_, _ = _oracle_fixpoint(oracle, inst)
    assert rc == orc
    if rc == P.OK:
        np.testing.assert_array_equal(s, os_)


@pytest.mark.parametrize("mode", ["persistent", "hostloop"])
@pytest.mark.parametrize("kind", ["base", "uneven", "wide"])
def test_medium_instances(kind, mode, P, oracle):
    import workloads as W
    if kind == "base":
        inst = W.add_chain(W.plain(20_000, 80_000, 1000, 5), 150, 1000, 5)
    elif kind == "uneven":
        inst = W.plain(20_000, 80_000, 1000, 6, mix=W.MIX_UNEVEN)
    else:  # bounds at 1e6: products leave int32 and saturate
        inst = W.plain(20_000, 80_000, 1_000_000, 7)
    rc, s, st, _ = _gpu_fixpoint(P, inst, mode=MODES[mode])
    orc, os_, info = _oracle_fixpoint(oracle, inst)
    assert rc == orc == P.OK
    np.testing.assert_array_equal(s, os_)
    h = inst.meta["hidden"]
    assert np.all((s[:, 0] <= h) & (h <= s[:, 1]))
    if kind == "wide":
        assert info["overflows"] > 0  # the saturating path was exercised


def test_round_cap_timeout(P):
    import workloads as W
    inst = W.add_chain(W.plain(2000, 6000, 1000, 1), 150, 1000, 1)
    for mode in (1, 2, 3):
        rc, _, st, _ = _gpu_fixpoint(P, inst, mode=mode, max_rounds=5)
        assert rc == P.TIMEOUT and st["rounds"] == 5


def test_barrier_timeout_is_reported(P):
    """A grid-barrier wait bounded to 1 ns runs out: the kernel returns
    BARRIER_TIMEOUT and the context stays usable."""
    import workloads as W
    inst = W.add_chain(W.plain(1_000_000, 4_000_000, 1000, 2), 150, 1000, 2)
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    snap = ctx.snapshot()
    rc, _ = ctx.fixpoint(mode=P.MODE_PERSISTENT, barrier_timeout_ns=1)
    assert rc == P.BARRIER_TIMEOUT
    ctx.restore(snap)
    rc, _ = ctx.fixpoint(mode=P.MODE_PERSISTENT)
    assert rc == P.OK


def test_bad_arguments(P):
    ctx = P.Context(0)
    ctx.load_store(np.zeros(4, np.int32), np.ones(4, np.int32))
    with pytest.raises(P.PirError) as e:
        ctx.tell([P.ADD], [0], [1], [4])
    assert e.value.code == P.EINVAL
    with pytest.raises(P.PirError):
        ctx.tell([12], [0], [1], [2])
    assert ctx.num_deductions() == 0
    with pytest.raises(P.PirError):
        ctx.embed(7, 0, 0)


def test_snapshot_restore_and_deduce_one(P, oracle):
    import workloads as W
    inst = W.single_small(3)
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    s0 = np.stack(ctx.read_store(), 1)
    snap = ctx.snapshot()
    ctx.fixpoint()
    ctx.restore(snap)
    np.testing.assert_array_equal(np.stack(ctx.read_store(), 1), s0)
    # deduce(i) in engine order against the oracle, for the first 300 propagators
    op, x, y, z = ctx.bytecode()
    s = s0.copy()
    for i in range(300):
        g = ctx.deduce_one(i)
        o, _ = oracle.deduce(int(op[i]), int(x[i]), int(y[i]), int(z[i]), s)
        assert g == o
    np.testing.assert_array_equal(np.stack(ctx.read_store(), 1), s)
    # ask(i) against the oracle
    np.testing.assert_array_equal(ctx.ask_all(), oracle.ask_all(op, x, y, z, s))


def test_engine_order_is_reference_sort(P, oracle):
    import workloads as W
    inst = W.single_small(4)
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    _, perm = oracle.install(inst.op, inst.x, inst.y, inst.z, inst.store())
    for a, b in zip(ctx.bytecode(), (inst.op, inst.x, inst.y, inst.z)):
        np.testing.assert_array_equal(a, b[perm])


@pytest.mark.parametrize("variant", range(1, 11))  # 1..PERSISTENT_VARIANTS
def test_persistent_variants(variant, P, oracle):
    """Every autotuner candidate computes the same fixpoint."""
    import workloads as W
    inst = W.add_chain(W.plain(30_000, 120_000, 1000, 8), 100, 1000, 8)
    rc, s, _, _ = _gpu_fixpoint(P, inst, mode=P.MODE_PERSISTENT, variant=variant)
    orc, os_, _ = _oracle_fixpoint(oracle, inst)
    assert rc == orc == P.OK
    np.testing.assert_array_equal(s, os_)


def test_autotune_keeps_store(P):
    import workloads as W
    inst = W.plain(30_000, 120_000, 1000, 9)
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    before = ctx.read_store()
    v, us = ctx.autotune(8)
    assert 1 <= v <= P.PERSISTENT_VARIANTS and us > 0
    after = ctx.read_store()
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])
