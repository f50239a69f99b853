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


@pytest.mark.parametrize("local", [0, 1])
def test_events_chain_and_random(local, P, oracle):
    """100k vars / 400k propagators plus a 3,000-link chain: the deep part runs
    mostly in small-frontier rounds."""
    import workloads as W
    inst = W.add_chain(W.plain(100_000, 400_000, 10**6, 7), 3000, 10**6, 7)
    rc, g, st, orc, o, info = _both(P, oracle, inst, local_frontier=local)
    assert rc == orc == oracle.OK
    np.testing.assert_array_equal(g, o)
    assert st["rounds"] >= 2900
    # far fewer executions than AC-1 sweeps of every propagator
    assert st["executions"] < st["rounds"] * inst.nprops // 20


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
    for local in (0, 1):
        ctx = P.Context(0)
        ctx.load_store(inst.lb, inst.ub)
        ctx.tell(inst.op, inst.x, inst.y, inst.z)
        rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS, max_rounds=100, local_frontier=local)
        assert rc == P.TIMEOUT and st["rounds"] == 100
        rc, st = ctx.fixpoint(sched=P.SCHED_EVENTS)
        assert rc == P.OK
        lb, ub = ctx.read_store()
        s = inst.store()
        orc, _ = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        np.testing.assert_array_equal(np.stack([lb, ub], 1), s)


@pytest.mark.parametrize("case", K.CASES, ids=[c.name for c in K.CASES])
def test_kat_events(case, P):
    class E(GpuEngine):
        pass
    E.sched = P.SCHED_EVENTS
    assert run_case(case, E) == []
