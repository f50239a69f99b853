"""Search driver (pir_search) against the CPU reference search built on the
oracle: n-queens (known solution counts) and planted instances; with one node
per launch the nodes, failures and solutions come in the reference's
depth-first order, with batches the solution sets agree."""
import numpy as np
import pytest

from search_ref import cpu_search

pytestmark = pytest.mark.gpu

QUEENS = {4: 2, 5: 10, 6: 4, 7: 40, 8: 92, 10: 724}


@pytest.fixture(scope="module")
def P():
    import pirgpu
    return pirgpu


def _ctx(P, inst):
    ctx = P.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    return ctx


def _reference(oracle, inst, dec, **kw):
    s = inst.store()
    st, perm = oracle.install(inst.op, inst.x, inst.y, inst.z, s)
    assert st == oracle.OK
    return cpu_search(oracle, inst.op[perm], inst.x[perm], inst.y[perm], inst.z[perm], s, dec, **kw)


@pytest.mark.parametrize("n", [4, 5, 6, 7, 8])
def test_queens_depth_first_order(n, P, oracle):
    import workloads as W
    inst = W.queens(n)
    dec = np.arange(n)
    ctx = _ctx(P, inst)
    status, sols, st = ctx.search(dec, max_solutions=1000, batch=1)
    assert status == P.OK and st["solutions"] == QUEENS[n]
    ref, nodes, fails = _reference(oracle, inst, dec)
    np.testing.assert_array_equal(sols, np.array(ref).reshape(-1, n))
    assert st["nodes"] == nodes and st["failures"] == fails
    # every solution is one: no two queens share a row or a diagonal
    for q in sols:
        assert len(set(q)) == n and len({q[i] - i for i in range(n)}) == n and len({q[i] + i for i in range(n)}) == n


@pytest.mark.parametrize("n", [8, 10])
@pytest.mark.parametrize("order", [0, 1])
def test_queens_batched(n, order, P):
    import workloads as W
    inst = W.queens(n)
    ctx = _ctx(P, inst)
    status, sols, st = ctx.search(np.arange(n), max_solutions=1000, order=order)
    assert status == P.OK and st["solutions"] == QUEENS[n]
    assert len({tuple(q) for q in sols}) == QUEENS[n]
    assert st["launches"] < st["nodes"]
    # counting only
    status, none, st2 = ctx.search(np.arange(n), order=order)
    assert st2["solutions"] == QUEENS[n] and len(none) == 0


@pytest.mark.parametrize("order", [0, 1])
def test_planted_solution_sets(order, P, oracle):
    import workloads as W
    inst = W.plain(20, 24, 8, 1)
    dec = np.arange(20)
    ref, _, _ = _reference(oracle, inst, dec, order=order)
    ctx = _ctx(P, inst)
    status, sols, st = ctx.search(dec, max_solutions=len(ref) + 10, order=order)
    assert status == P.OK and st["solutions"] == len(ref)
    assert sorted(map(tuple, sols)) == sorted(map(tuple, ref))
    # the hidden solution is among them
    assert tuple(inst.meta["hidden"][:20]) in set(map(tuple, sols))


def test_limits(P, oracle):
    import workloads as W
    inst = W.queens(8)
    ctx = _ctx(P, inst)
    status, sols, st = ctx.search(np.arange(8), max_solutions=1, batch=1)
    ref, _, _ = _reference(oracle, inst, np.arange(8), max_solutions=1)
    assert status == P.OK and st["solutions"] == 1
    np.testing.assert_array_equal(sols[0], ref[0])
    status, _, st = ctx.search(np.arange(8), max_nodes=50, batch=16)
    assert status == P.TIMEOUT and st["nodes"] == 50


def test_watch_matches_full_stores(P, oracle):
    """pir_fixpoint_nodes_watch reports the same bounds and statuses as the
    full node stores."""
    import workloads as W
    base = W.plain(3000, 12_000, 10**6, 3)
    ctx = _ctx(P, base)
    rc, _ = ctx.fixpoint()
    assert rc == P.OK
    blb, bub = ctx.read_store()
    _, off, var, lb, ub = W.nodes(3000, 12_000, 128, 3, 32, base_store=(blb, bub))
    watch = np.arange(0, 3000, 7)
    s1, wl, wu, _, _ = ctx.fixpoint_nodes_watch(off, var, lb, ub, watch)
    s2, fl, fu, _, _ = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS)
    np.testing.assert_array_equal(s1, s2)
    ok = s1 == P.OK
    np.testing.assert_array_equal(wl[ok], fl[ok][:, watch])
    np.testing.assert_array_equal(wu[ok], fu[ok][:, watch])


def test_bad_arguments_are_rejected(P):
    """Errors come back as EINVAL before anything runs; the context stays usable."""
    import workloads as W
    inst = W.queens(6)
    ctx = _ctx(P, inst)
    for bad in ([0, 1, 10**6], [-1]):
        with pytest.raises(P.PirError, match="EINVAL"):
            ctx.search(bad)
    with pytest.raises(P.PirError, match="EINVAL"):
        ctx.search(np.arange(6), max_nodes=-1)
    with pytest.raises(P.PirError, match="EINVAL"):
        ctx.fixpoint_nodes_watch([0, 1], [0], [0], [1], [10**6])
    with pytest.raises(P.PirError, match="EINVAL"):
        ctx.fixpoint_nodes_watch([0, 1], [10**6], [0], [1], [0])
    with pytest.raises(P.PirError, match="EINVAL"):
        ctx.fixpoint(variant=P.PERSISTENT_VARIANTS + 1, mode=P.MODE_PERSISTENT)
    status, sols, st = ctx.search(np.arange(6), max_solutions=10)
    assert status == P.OK and st["solutions"] == 4
