"""Exhaustive soundness / completeness properties of the oracle's
propagators, restating tests/bound_consistency_test.hpp with the predicates
of tests/pir_test.cpp:120-171, plus schedule independence and the division
semantics."""
import numpy as np
import pytest

PREDS = ["int_eq_reif", "int_le_reif", "int_plus", "int_min", "int_max", "int_times",
         "int_ediv", "int_tdiv", "int_cdiv", "int_fdiv", "int_emod", "int_tmod",
         "int_cmod", "int_fmod"]
# test_completeness flags of tests/pir_test.cpp:123-136
COMPLETE = {0: True, 1: True, 2: True, 3: True, 4: True}


@pytest.mark.parametrize("pred", range(14), ids=PREDS)
def test_exhaustive_soundness(pred, oracle):
    # tests/pir_test.cpp:122-137 over every sub-interval triple of [-10, 10]^3
    bad, cases, first = oracle.check_exhaustive(pred, -10, 10, COMPLETE.get(pred, False))
    assert cases == 231 ** 3
    assert bad == 0, "first failing case %d" % first


@pytest.mark.parametrize("pred", range(14), ids=PREDS)
def test_listed_soundness(pred, oracle):
    # tests/pir_test.cpp:139-154
    bad, cases, first = oracle.check_listed(pred, COMPLETE.get(pred, False))
    assert cases == 23 ** 3 and bad == 0, first


@pytest.mark.parametrize("pred", range(14), ids=PREDS)
def test_completeness_singletons(pred, oracle):
    # tests/pir_test.cpp:156-171 (with_fixpoint for the modulo decompositions)
    bad, cases, first = oracle.check_completeness(pred, pred >= 10)
    assert cases == 1000 and bad == 0, first


def test_checker_rejects_incomplete_claim(oracle):
    # int_times is sound but not complete: claiming completeness must fail
    bad, _, _ = oracle.check_exhaustive(5, -5, 5, True)
    assert bad > 0


def test_division_semantics(oracle):
    # truncating / floor / ceiling / Euclidean (cuda-battery tdiv, fdiv, cdiv, ediv)
    T, F, C, E = oracle.TDIV, oracle.FDIV, oracle.CDIV, oracle.EDIV
    cases = [(7, 2, 3, 3, 4, 3), (-7, 2, -3, -4, -3, -4), (7, -2, -3, -4, -3, -3),
             (-7, -2, 3, 3, 4, 4), (6, 3, 2, 2, 2, 2), (-6, 3, -2, -2, -2, -2), (0, -5, 0, 0, 0, 0)]
    for a, b, t, f, c, e in cases:
        assert (oracle.div(T, a, b), oracle.div(F, a, b), oracle.div(C, a, b),
                oracle.div(E, a, b)) == (t, f, c, e), (a, b)
        assert 0 <= oracle.mod(0, a, b) < abs(b)


def _planted(seed, nv=300, npr=900):
    import workloads as W
    return W.plain(nv, npr, 1000, seed)


@pytest.mark.parametrize("seed", range(6))
def test_schedule_independence(seed, oracle):
    """Any propagator order reaches the same fixpoint (monotone propagators):
    the reference's sorted order vs random permutations."""
    inst = _planted(seed)
    ref = inst.store()
    st0, _ = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, ref)
    rng = np.random.default_rng(seed)
    for _ in range(5):
        s = inst.store()
        oracle.install(inst.op, inst.x, inst.y, inst.z, s)
        p = rng.permutation(inst.nprops)
        st, _ = oracle.fixpoint(inst.op[p], inst.x[p], inst.y[p], inst.z[p], s)
        assert st == st0
        np.testing.assert_array_equal(s, ref)


@pytest.mark.parametrize("seed", range(4))
def test_planted_solution_survives(seed, oracle):
    """Soundness on whole instances: the hidden assignment satisfies every
    propagator, so it stays inside the fixpoint."""
    import workloads as W
    inst = W.plain(2000, 6000, 1000, seed, mix=W.MIX_UNEVEN)
    s = inst.store()
    st, info = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
    h = inst.meta["hidden"]
    assert st == oracle.OK
    assert np.all((s[:, 0] <= h) & (h <= s[:, 1]))
    assert info["overflows"] == 0


def test_spec_variant_fails_at_install(oracle):
    import workloads as W
    inst = W.single_small(0, variant="spec")
    s = inst.store()
    st, _ = oracle.install_and_fixpoint(inst.op, inst.x, inst.y, inst.z, s)
    assert st == oracle.FAILED
