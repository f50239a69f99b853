"""The batched benchmark workloads at full size, bit for bit against the
oracle run node by node / instance by instance (the per-node loop of
tests/bound_consistency_test.hpp:162-196 around the Gauss-Seidel driver of
tests/pir_test.cpp:60-62):

* search nodes: a 100,000-variable / 400,000-propagator base at its fixpoint
  and 4,096 nodes, each bisecting k ~ U[1, 64] unfixed variables, in one
  launch of the event node kernel (with its certifying sweeps) and of the
  AC-1 node kernel;
* 512 uneven instances, propagators log-uniform in [1e3, 2e5], 5% tdiv and
  5% tmod, in one launch, under AC-1 and under the event-filtered rounds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NODE_CHUNK = 512  # nodes the oracle holds at once (100,000 vars x 8 B x 512 = 410 MB)


@pytest.fixture(scope="module")
def nodes_setup():
    import pirgpu
    import workloads as W
    base = W.plain(100_000, 400_000, 10**6, 0)
    ctx = pirgpu.Context(0)
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    rc, _ = ctx.fixpoint()
    assert rc == pirgpu.OK
    blb, bub = ctx.read_store()
    _, off, var, lb, ub = W.nodes(100_000, 400_000, 4096, 0, 64, base_store=(blb, bub))
    assert len(off) == 4097
    return ctx, (blb, bub), off, var, lb, ub


def _check_nodes(oracle, ctx, base, off, var, lb, ub, status, olb, oub):
    op, x, y, z = ctx.bytecode()
    bs = np.ascontiguousarray(np.stack(base, 1))
    nn = len(off) - 1
    nok = 0
    for j0 in range(0, nn, NODE_CHUNK):
        j1 = min(nn, j0 + NODE_CHUNK)
        o = off[j0:j1 + 1] - off[j0]
        sl = slice(off[j0], off[j1])
        ost, ostore, _ = oracle.fixpoint_nodes(op, x, y, z, bs, o, var[sl], lb[sl], ub[sl])
        np.testing.assert_array_equal(status[j0:j1], ost)
        ok = ost == oracle.OK
        nok += int(ok.sum())
        np.testing.assert_array_equal(olb[j0:j1][ok], ostore[ok, :, 0])
        np.testing.assert_array_equal(oub[j0:j1][ok], ostore[ok, :, 1])
    assert nok > nn // 2


def test_nodes_4096_events_bit_exact(nodes_setup, oracle):
    import pirgpu
    ctx, base, off, var, lb, ub = nodes_setup
    status, olb, oub, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub, sched=pirgpu.SCHED_EVENTS)
    assert st["certify_executions"] > 0 and st["certify_narrowed"] == 0
    _check_nodes(oracle, ctx, base, off, var, lb, ub, status, olb, oub)
    # the context's own store is untouched
    l2, u2 = ctx.read_store()
    np.testing.assert_array_equal(l2, base[0])
    np.testing.assert_array_equal(u2, base[1])


def test_nodes_4096_ac1_bit_exact(nodes_setup, oracle):
    import pirgpu
    ctx, base, off, var, lb, ub = nodes_setup
    status, olb, oub, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub, sched=pirgpu.SCHED_AC1)
    _check_nodes(oracle, ctx, base, off, var, lb, ub, status, olb, oub)


def test_nodes_4096_statuses_without_stores(nodes_setup, oracle):
    """The benchmark's call (no stores downloaded, autotuned variant): the
    same statuses as with stores."""
    import pirgpu
    ctx, base, off, var, lb, ub = nodes_setup
    ctx.autotune_nodes(off, var, lb, ub)
    s1, _, _, r1, st1 = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=pirgpu.SCHED_EVENTS)
    s2, _, _, r2, _ = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=True, sched=pirgpu.SCHED_EVENTS)
    np.testing.assert_array_equal(s1, s2)
    assert st1["certify_narrowed"] == 0


@pytest.mark.parametrize("sched", ("ac1", "events"))
def test_uneven_512_bit_exact(sched, oracle):
    import pirgpu
    import workloads as W
    insts = W.uneven(512, 1000, 200_000, 0)
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    glb, gub = lb.copy(), ub.copy()
    ctx = pirgpu.Context(0)
    status, rounds, ms, st = ctx.fixpoint_instances(
        prop_off, var_off, op, x, y, z, glb, gub,
        sched={"ac1": pirgpu.SCHED_AC1, "events": pirgpu.SCHED_EVENTS}[sched])
    s = np.ascontiguousarray(np.stack([lb, ub], 1))
    ost, _ = oracle.fixpoint_instances(prop_off, var_off, op, x, y, z, s)
    np.testing.assert_array_equal(status, ost)
    assert (ost == oracle.OK).sum() > 400
    for j in np.nonzero(ost == oracle.OK)[0]:
        v0, v1 = var_off[j], var_off[j + 1]
        np.testing.assert_array_equal(glb[v0:v1], s[v0:v1, 0])
        np.testing.assert_array_equal(gub[v0:v1], s[v0:v1, 1])
