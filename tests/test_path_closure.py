"""The closed form the event kernel uses for a path segment of ADD links with
constants: for v_{k+1} = v_k + d_k (d_k the link's constant, negated when
the link is written the other way round), P_0 = 0, P_{k+1} = P_k + d_k,

    lb(v_j) = P_j + max_i (lb(v_i) - P_i),   ub(v_j) = P_j + min_i (ub(v_i) - P_i),

and the path fails when the max exceeds the min.  Checked here against the
oracle's fixpoint of the same propagators (the reference's ADD,
pir.hpp:758-766, run to its fixpoint by Gauss-Seidel sweeps) on random paths
with small finite bounds, in both directions and with the constant as either
operand: the same store, or the same failure."""
import numpy as np
import pytest

ADD = 0


def _path(rng, n, reverse, const_first):
    v = np.arange(n + 1)
    cv = n + 1 + np.arange(n)
    c = rng.integers(-50, 51, n)
    lb = rng.integers(-10_000, 10_000, 2 * n + 1)
    ub = lb + rng.integers(0, 20_000, 2 * n + 1)
    lb[cv] = ub[cv] = c
    xo, yo = (v[:-1], v[1:]) if reverse else (v[1:], v[:-1])
    yy, zz = (cv, yo) if const_first else (yo, cv)
    op = np.full(n, ADD)
    return lb, ub, op, xo, yy, zz, c


def _closure(lb, ub, c, n, reverse):
    d = -c if reverse else c
    P = np.concatenate([[0], np.cumsum(d)])
    lo = P + np.max(lb[:n + 1] - P)
    hi = P + np.min(ub[:n + 1] - P)
    return lo, hi, bool(np.max(lb[:n + 1] - P) > np.min(ub[:n + 1] - P))


@pytest.mark.parametrize("reverse", [False, True])
@pytest.mark.parametrize("const_first", [False, True])
@pytest.mark.parametrize("n", [1, 4, 31, 64])
def test_closure_is_the_fixpoint(n, reverse, const_first, oracle):
    rng = np.random.default_rng(1000 * n + 10 * reverse + const_first)
    feasible = failed = 0
    for trial in range(40):
        lb, ub, op, x, y, z, c = _path(rng, n, reverse, const_first)
        if trial % 2:  # also paths that stay feasible: every variable wide
            lb[:n + 1] = rng.integers(-10_000, 0, n + 1) - 10**6
            ub[:n + 1] = rng.integers(0, 10_000, n + 1) + 10**6
        store = np.ascontiguousarray(np.stack([lb, ub], 1).astype(np.int32))
        rc, _ = oracle.install_and_fixpoint(op, x, y, z, store)
        lo, hi, fails = _closure(lb, ub, c, n, reverse)
        assert (rc == oracle.FAILED) == fails
        if fails:
            failed += 1
            continue
        feasible += 1
        np.testing.assert_array_equal(store[:n + 1, 0], lo)
        np.testing.assert_array_equal(store[:n + 1, 1], hi)
        np.testing.assert_array_equal(store[n + 1:, 0], c)  # the constants narrow nothing
        np.testing.assert_array_equal(store[n + 1:, 1], c)
    assert feasible > 0 and failed > 0
