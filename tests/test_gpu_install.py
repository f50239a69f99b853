"""The install on the device (pir_install.cu): for bytecodes of 65,536
propagators or more, pir_tell sorts the bytecode into the engine order on the
GPU and the event schedules build their variable -> propagator adjacency
there.  The order must be exactly the stable sort by (op, y, x, z) that
lala-pc's CPU install makes (pir.hpp:343-347): checked against numpy's stable
lexsort, with many equal keys (few variables) so that stability shows, across
two tells (the second re-sorts the concatenation), and with variable indices
that need many bits of the key fields.  The adjacency is checked through the
fixpoints of the event schedule against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import pirgpu
    return pirgpu


def _stable_order(op, x, y, z):
    return np.lexsort((z, x, y, op))  # last key first; numpy's lexsort is stable


@pytest.mark.parametrize("nvars", [7, 1000, 3_000_000])
def test_device_install_order(nvars, P):
    rng = np.random.default_rng(nvars % 1000)
    n1, n2 = 70_000, 90_000

    def draw(n):
        op = rng.integers(0, 10, n).astype(np.int32)
        x, y, z = (rng.integers(0, nvars, n).astype(np.int32) for _ in range(3))
        return op, x, y, z

    ctx = P.Context(0)
    lb = np.full(nvars, -10**6, np.int32)
    ub = np.full(nvars, 10**6, np.int32)
    ctx.load_store(lb, ub)
    a = draw(n1)
    ctx.tell(*a)
    got = ctx.bytecode()
    perm = _stable_order(*a)
    for g, w in zip(got, a):
        np.testing.assert_array_equal(g, w[perm])
    b = draw(n2)
    ctx.tell(*b)
    got = ctx.bytecode()
    cat = [np.concatenate([w[perm], v]) for w, v in zip(a, b)]
    perm2 = _stable_order(*cat)
    for g, w in zip(got, cat):
        np.testing.assert_array_equal(g, w[perm2])


def test_device_install_events_and_ac1_agree(P, oracle):
    """A 200,000-propagator instance plus a chain (device sort and device
    adjacency): AC-1 and the event schedule reach the oracle's fixpoint."""
    import workloads as W
    inst = W.add_chain(W.plain(50_000, 200_000, 10**6, 21), 500, 10**6, 21)
    s = inst.store()
    orc, _ = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
    assert orc == oracle.OK
    for sched in (P.SCHED_AC1, P.SCHED_EVENTS):
        ctx = P.Context(0)
        ctx.load_store(inst.lb, inst.ub)
        ctx.tell(inst.op, inst.x, inst.y, inst.z)
        rc, st = ctx.fixpoint(sched=sched)
        assert rc == P.OK
        np.testing.assert_array_equal(np.stack(ctx.read_store(), 1), s)
        if sched == P.SCHED_EVENTS:
            assert st["certify_narrowed"] == 0
