"""The benchmark workload at full size: 1,000,000 variables / 4,000,000
propagators (bounds scale 1e6, saturating products) plus a 20,000-link chain.
Its two parts share no variable, so the oracle runs them separately (the
fixpoint of the union is the union of the fixpoints) and the GPU result of the
whole instance must equal both, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_single_large_bit_exact(oracle):
    import pirgpu
    import workloads as W
    inst = W.single_large(0)
    ctx = pirgpu.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    ctx.autotune(8)
    rc, st = ctx.fixpoint()
    assert rc == pirgpu.OK and st["rounds"] > 19_000
    lb, ub = ctx.read_store()
    n0, length = inst.meta["chain"]
    # random part alone
    rnd = W.single_large(0, chain=0)
    s = rnd.store()
    orc, info = oracle.install_and_fixpoint(rnd.op, rnd.x, rnd.y, rnd.z, s)
    assert orc == oracle.OK and info["overflows"] > 0  # the saturating path is exercised
    np.testing.assert_array_equal(lb[:n0], s[:, 0])
    np.testing.assert_array_equal(ub[:n0], s[:, 1])
    # chain alone (same generator stream as inside single_large)
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    chain = W.add_chain(empty, length, 1_000_000, 0)
    c = chain.store()
    orc, info = oracle.install_and_fixpoint(chain.op, chain.x, chain.y, chain.z, c)
    assert orc == oracle.OK and info["sweeps"] > 19_000
    np.testing.assert_array_equal(lb[n0:], c[:, 0])
    np.testing.assert_array_equal(ub[n0:], c[:, 1])
    # the planted solution is inside
    h = inst.meta["hidden"]
    assert np.all((lb <= h) & (h <= ub))
