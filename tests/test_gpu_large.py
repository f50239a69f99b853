"""The benchmark workload at full size: 1,000,000 variables / 4,000,000
propagators (bounds scale 1e6, saturating products) plus a 20,000-link chain.
Its two parts share no variable, so the oracle runs them separately (the
fixpoint of the union is the union of the fixpoints) and the GPU result of the
whole instance, under AC-1 rounds and under the event schedule, must equal
both, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def large(oracle):
    """The instance and the oracle's fixpoint of it (lb, ub per variable)."""
    import workloads as W
    inst = W.single_large(0)
    n0, length = inst.meta["chain"]
    # random part alone
    rnd = W.single_large(0, chain=0)
    s = rnd.store()
    orc, info = oracle.install_and_fixpoint(rnd.op, rnd.x, rnd.y, rnd.z, s)
    assert orc == oracle.OK and info["overflows"] > 0  # the saturating path is exercised
    # chain alone (same generator stream as inside single_large)
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    chain = W.add_chain(empty, length, 1_000_000, 0)
    c = chain.store()
    orc, cinfo = oracle.install_and_fixpoint(chain.op, chain.x, chain.y, chain.z, c)
    assert orc == oracle.OK and cinfo["sweeps"] > 19_000
    lb = np.concatenate([s[:, 0], c[:, 0]])
    ub = np.concatenate([s[:, 1], c[:, 1]])
    assert len(lb) == inst.nvars
    return inst, lb, ub


def _ctx(inst):
    import pirgpu
    ctx = pirgpu.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    return ctx


def _check(ctx, inst, lb, ub):
    glb, gub = ctx.read_store()
    np.testing.assert_array_equal(glb, lb)
    np.testing.assert_array_equal(gub, ub)
    # the planted solution is inside
    h = inst.meta["hidden"]
    assert np.all((glb <= h) & (h <= gub))


def test_single_large_ac1_bit_exact(large):
    import pirgpu
    inst, lb, ub = large
    ctx = _ctx(inst)
    ctx.autotune(8)
    rc, st = ctx.fixpoint()
    assert rc == pirgpu.OK and st["rounds"] > 19_000
    _check(ctx, inst, lb, ub)


@pytest.mark.parametrize("chase,segments", [(0, 0), (0, -1), (-1, -1)])
def test_single_large_events_bit_exact(large, chase, segments):
    """The event schedule at full size (the chain as segments of 64 links, or
    every propagator on its own with and without chasing), ending with its
    certifying sweep of every unit, which must find nothing left."""
    import pirgpu
    inst, lb, ub = large
    ctx = _ctx(inst)
    rc, st = ctx.fixpoint(sched=pirgpu.SCHED_EVENTS, chase=chase, segments=segments, lead=-1)
    assert rc == pirgpu.OK
    _check(ctx, inst, lb, ub)
    n = ctx.num_deductions()
    assert st["certify_executions"] >= n - 20_000 and st["certify_narrowed"] == 0
    assert st["executions"] < 200 * n  # far below the 20,000 AC-1 sweeps
    if chase < 0:
        assert st["rounds"] > 19_000  # one chain link per round
    else:
        assert st["rounds"] < 2_000


def test_single_large_events_default_bit_exact(large):
    """The event schedule as the benchmark runs it: AC-1 rounds first while
    many CTAs still narrow something, then the event kernel on the chain."""
    import pirgpu
    inst, lb, ub = large
    ctx = _ctx(inst)
    ctx.autotune(16)  # the lead runs the tuned variant; the store is put back
    rc, st = ctx.fixpoint(sched=pirgpu.SCHED_EVENTS)
    assert rc == pirgpu.OK
    _check(ctx, inst, lb, ub)
    assert st["certify_executions"] > 0 and st["certify_narrowed"] == 0
    assert st["rounds"] < 2_000


def test_single_large_events_uncertified_agrees(large):
    """certify < 0 skips the final sweep: the same store, n fewer executions."""
    import pirgpu
    inst, lb, ub = large
    ctx = _ctx(inst)
    rc, st = ctx.fixpoint(sched=pirgpu.SCHED_EVENTS, certify=-1, lead=-1)
    assert rc == pirgpu.OK
    assert st["certify_executions"] == 0 and st["certify_narrowed"] == 0
    _check(ctx, inst, lb, ub)
