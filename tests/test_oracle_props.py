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


def _triples(lo, hi):
    itv = np.array([(l, u) for l in range(lo, hi + 1) for u in range(l, hi + 1)], np.int32)
    k = len(itv)
    idx = np.stack(np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij"), -1).reshape(-1, 3)
    return itv[idx, 0], itv[idx, 1]


def _install_invariant(op, lb, ub):
    """Reified targets live in [0, 1] after install (pir.hpp:333-335): keep
    the triples whose x meets [0, 1], with x narrowed to it."""
    if op not in (8, 9):
        return lb, ub
    lb, ub = lb.copy(), ub.copy()
    lb[:, 0] = np.maximum(lb[:, 0], 0)
    ub[:, 0] = np.minimum(ub[:, 0], 1)
    keep = lb[:, 0] <= ub[:, 0]
    return lb[keep], ub[keep]


@pytest.mark.parametrize("op", range(10))
def test_entailed_propagator_narrows_nothing(op, oracle):
    """The premise of dropping propagators entailed at a search node's base
    store: where ask(bytecode) holds (pir.hpp:417-438), deduce(bytecode)
    (pir.hpp:721-817) changes no bound.  Every interval triple of [-5, 5]^3 and
    random wide ones, reified targets within [0, 1] as install leaves them
    (outside it the reified ask reads x <= 0 as false)."""
    lb, ub = _triples(-5, 5)
    rng = np.random.default_rng(100 + op)
    m = 300_000
    a = rng.integers(-10**6, 10**6, (m, 3))
    b = a + rng.integers(0, 3, (m, 3)) * rng.integers(0, 10**3, (m, 3))
    # many singletons so that entailment happens
    b = np.where(rng.random((m, 3)) < .6, a, b)
    a = np.where(rng.random((m, 3)) < .3, rng.integers(-3, 4, (m, 3)), a)
    b = np.maximum(a, np.where(rng.random((m, 3)) < .3, a, b))
    lb = np.concatenate([lb, a.astype(np.int32)])
    ub = np.concatenate([ub, b.astype(np.int32)])
    lb, ub = _install_invariant(op, lb, ub)
    ops = np.full(len(lb), op, np.int32)
    ent = oracle.ask_batch(ops, lb, ub)
    assert ent.sum() > 100
    out_lb, out_ub, changed, failed, _ = oracle.deduce_batch(ops[ent], lb[ent], ub[ent])
    assert not changed.any() and not failed.any()
    np.testing.assert_array_equal(out_lb, lb[ent].reshape(-1, 3))
    np.testing.assert_array_equal(out_ub, ub[ent].reshape(-1, 3))


@pytest.mark.parametrize("op", range(10))
def test_entailment_is_monotone(op, oracle):
    """ask(bytecode) stays true when any of its intervals narrows: a
    propagator entailed at a base store is entailed at every node below it."""
    lb, ub = _install_invariant(op, *_triples(-4, 4))
    ops = np.full(len(lb), op, np.int32)
    ent = oracle.ask_batch(ops, lb, ub)
    lb, ub = lb[ent], ub[ent]
    rng = np.random.default_rng(op)
    for _ in range(4):
        # a random non-empty sub-interval of each interval
        nl = lb + (rng.random(lb.shape) * (ub - lb + 1)).astype(np.int32)
        nu = nl + (rng.random(lb.shape) * (ub - nl + 1)).astype(np.int32)
        assert oracle.ask_batch(ops[:len(nl)], nl, nu).all()


def test_queens_model_counts(oracle):
    """The n-queens PIR model (reified EQ with a false target as !=, ADD for
    differences) has the known solution counts under the CPU reference search."""
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    import workloads as W
    from search_ref import cpu_search
    for n, want in [(1, 1), (2, 0), (3, 0), (4, 2), (5, 10), (6, 4), (7, 40), (8, 92)]:
        inst = W.queens(n)
        s = inst.store()
        st, perm = oracle.install(inst.op, inst.x, inst.y, inst.z, s)
        sols, _, _ = cpu_search(oracle, inst.op[perm], inst.x[perm], inst.y[perm], inst.z[perm], s, np.arange(n))
        assert len(sols) == want


@pytest.mark.parametrize("order", [0, 1])
def test_oracle_search_matches_reference_search(order, oracle):
    """orc_search (the C++ CPU search, the bench's baseline) visits the same
    nodes and finds the same solutions, in the same order, as the Python
    reference search."""
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    import workloads as W
    from search_ref import cpu_search
    cases = [(W.queens(n), np.arange(n)) for n in (5, 6, 8)] + [(W.plain(20, 24, 8, 1), np.arange(20))]
    for inst, dec in cases:
        s = inst.store()
        st, perm = oracle.install(inst.op, inst.x, inst.y, inst.z, s)
        args = (inst.op[perm], inst.x[perm], inst.y[perm], inst.z[perm])
        ref, nodes, fails = cpu_search(oracle, *args, s, dec, order=order)
        rc, sols, info = oracle.search(*args, s, dec, order=order, max_solutions=len(ref) + 1)
        assert rc == oracle.OK and info["nodes"] == nodes and info["failures"] == fails
        np.testing.assert_array_equal(sols, np.array(ref).reshape(-1, len(dec)))
    rc, _, info = oracle.search(*args, s, dec, order=order, max_nodes=10)
    assert rc == oracle.TIMEOUT and info["nodes"] == 10


def test_quotient_extremes_at_sign_analysis_corners():
    """The premise of the device's MUL inverse and division forward: for a
    sign-definite divisor box, the min / max over the four corners of each
    integer division (truncating, floor, ceiling, Euclidean) is the division
    at the corner a sign analysis names; and the narrowing tests
    cdiv(a, b) > n iff a > n b (b > 0) / a < n b (b < 0), fdiv(a, b) < n iff
    a < n b (b > 0) / a > n b (b < 0) are exact."""
    def tdiv(a, b):
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b > 0) else -q

    def fdiv(a, b):
        return a // b

    def cdiv(a, b):
        return -((-a) // b)

    def ediv(a, b):
        q = tdiv(a, b)
        return q - 1 if a - q * b < 0 and b > 0 else (q + 1 if a - q * b < 0 else q)

    R = range(-9, 10)
    for d in (tdiv, fdiv, cdiv, ediv):
        for yl in R:
            for yu in range(yl, 10):
                for zl in R:
                    for zu in range(zl, 10):
                        if not (zl > 0 or zu < 0):
                            continue
                        c = [d(a, b) for a in (yl, yu) for b in (zl, zu)]
                        if zl > 0:
                            lo, hi = d(yl, zu if yl >= 0 else zl), d(yu, zl if yu >= 0 else zu)
                        else:
                            lo, hi = d(yu, zu if yu >= 0 else zl), d(yl, zl if yl >= 0 else zu)
                        assert (lo, hi) == (min(c), max(c))
    vals = list(range(-12, 13)) + [-2**31, -2**31 + 1, 2**31 - 1, -10**6, 10**6]
    for a in vals:
        for b in [v for v in vals if v != 0]:
            for n in vals:
                assert (cdiv(a, b) > n) == ((a > n * b) if b > 0 else (a < n * b))
                assert (fdiv(a, b) < n) == ((a < n * b) if b > 0 else (a > n * b))


def test_idempotent_opcodes(oracle):
    """ADD, MIN, MAX and the reified EQ / LEQ (target inside [0, 1], as install
    leaves it) are idempotent: a second run on the intervals the first left
    narrows nothing.  Checked on every triple of sub-intervals of [-6, 6]
    together with unbounded ends, and on a grid of bounds at the int32
    saturation edges.  The event kernel's segment sweeps rely on it to skip
    re-running such a propagator after its own narrowing (and MUL and the
    divisions are not idempotent, so they are re-run)."""
    import itertools
    INF, MINF = 2**31 - 1, -2**31
    small = [(a, b) for a in range(-6, 7) for b in range(-6, 7) if a <= b]
    small += [(MINF, 3), (-2, INF), (MINF, INF), (0, INF), (MINF, 0)]
    edge = [MINF, MINF + 1, -2**30, -1, 0, 1, 2**30, INF - 1, INF]
    edge = [(a, b) for a in edge for b in edge if a <= b and a != INF and b != MINF]
    for itv in (small, edge):
        itv = np.array(itv, np.int64)
        idx = np.array(list(itertools.product(range(len(itv)), repeat=3)))
        lb = itv[idx][:, :, 0].astype(np.int32)
        ub = itv[idx][:, :, 1].astype(np.int32)
        for op in (0, 6, 7, 8, 9):
            L, U = lb.copy(), ub.copy()
            if op in (8, 9):
                L[:, 0] = np.maximum(L[:, 0], 0)
                U[:, 0] = np.minimum(U[:, 0], 1)
                keep = L[:, 0] <= U[:, 0]
                L, U = L[keep], U[keep]
            ops = np.full(len(L), op, np.int32)
            l1, u1, _, f1, _ = oracle.deduce_batch(ops, L, U)
            _, _, ch2, _, _ = oracle.deduce_batch(ops, l1, u1)
            ok = ~f1 & ~(l1 > u1).any(1) & ~(l1 == INF).any(1) & ~(u1 == MINF).any(1)
            assert not (ok & ch2).any(), op
