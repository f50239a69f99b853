"""Committed golden fixtures (tests/golden/fixpoints_small.npz, made by
tests/golden/make_fixtures.py): the generator is bit-identical on this host,
the oracle reproduces the stored fixpoints, and the GPU engine matches them."""
import numpy as np
import pytest

from golden import make_fixtures as MF


@pytest.fixture(scope="module")
def golden():
    import os
    return dict(np.load(os.path.join(os.path.dirname(MF.__file__), "fixpoints_small.npz")))


def test_generator_is_deterministic(golden):
    for name, inst in MF.cases():
        assert str(golden[name + "_hash"]) == MF.instance_hash(inst), name


def test_oracle_reproduces_fixtures(golden, oracle):
    for name, inst in MF.cases():
        s = inst.store()
        st, info = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        assert st == int(golden[name + "_status"]), name
        if st == oracle.OK:
            np.testing.assert_array_equal(s, golden[name + "_store"])
            assert info["sweeps"] == int(golden[name + "_sweeps"])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2, 3])
def test_gpu_matches_fixtures(golden, mode):
    import pirgpu
    for name, inst in MF.cases():
        ctx = pirgpu.Context(0)
        ctx.load_store(inst.lb, inst.ub)
        ctx.tell(inst.op, inst.x, inst.y, inst.z)
        rc, _ = ctx.fixpoint(mode=mode)
        assert rc == int(golden[name + "_status"]), name
        if rc == pirgpu.OK:
            lb, ub = ctx.read_store()
            np.testing.assert_array_equal(np.stack([lb, ub], 1), golden[name + "_store"])
