"""PC tree propagators on the CPU: the oracle (oracle/pc_oracle.cpp) pinned
against the known answers of lala-pc's PC tests (tests/pc_test.cpp,
transcribed in tests/golden/pc_kat_cases.py) through the FlatZinc front end
(include/pirgpu_fzn_pc.hpp), the term tests, properties of the restated
interval arithmetic, and the schedule independence the GPU engine relies on."""
import itertools
import re

import numpy as np
import pytest

import pc as P
import pc_harness as H
from golden import pc_kat_cases as K


@pytest.fixture(scope="module")
def make_fzn(tmp_path_factory):
    return H.compile_shim(tmp_path_factory.mktemp("pcfzn"))


@pytest.mark.parametrize("case", K.CASES, ids=[c[0] for c in K.CASES])
def test_kat_oracle(case, make_fzn, oracle):
    assert H.run_case(make_fzn, H.OracleModel(oracle), case) == []


def test_term_add_binary(oracle):
    """TermTest.AddTermBinary (tests/pc_test.cpp:31-47)."""
    t = P.Tape()
    s = t.add(t.var(0), t.var(1))
    tape, _ = t.arrays()
    st = np.array([[0, 10], [0, 10]], np.int32)
    assert oracle.pc_project(tape, s, st) == (0, 20)
    assert oracle.pc_embed(tape, s, P.MINF, 5, st) == (True, False)
    assert oracle.pc_project(tape, s, st) == (0, 10)


def test_term_add_nary(oracle):
    """TermTest.AddTermNary (tests/pc_test.cpp:49-67)."""
    t = P.Tape()
    s = t.nadd([t.var(0), t.var(1), t.var(2)])
    tape, _ = t.arrays()
    st = np.array([[0, 10]] * 3, np.int32)
    assert oracle.pc_project(tape, s, st) == (0, 30)
    assert oracle.pc_embed(tape, s, P.MINF, 5, st) == (True, False)
    assert oracle.pc_project(tape, s, st) == (0, 15)


def test_front_end_errors(make_fzn):
    fz = make_fzn()
    with pytest.raises(ValueError, match="unsupported constraint"):
        fz.compile("var int: x; constraint no_such_thing(x, x);")
    with pytest.raises(ValueError):
        fz.compile("var int x;")


def test_front_end_shapes(make_fzn):
    """Store parts and formula shapes of the front end (pc.hpp:505-605)."""
    fz = make_fzn()
    d = fz.compile("var 1..10: x; var int: y; constraint int_lt(x, 5); constraint int_ge(7, y);"
                   " constraint int_lin_le([2, 3, 1], [x, y, x], 20); constraint int_lt(x, y);")
    assert d["newvars"] == [(1, 4), (P.MINF, 7)]
    kinds = [int(k) for k in d["tape"][:, 0]]
    roots = [kinds[r] for r in d["roots"]]
    assert roots == [P.LEQ, P.GT]           # the sum <= 20, then y > x
    assert P.NADD in kinds and kinds.count(P.ARG) == 3
    d2 = fz.compile("constraint int_le(x, 3); constraint int_ne(y, 2);")
    assert d2["meets"] == [(0, P.MINF, 3)] and len(d2["roots"]) == 1


def _interval_ref(op, a, b):
    """Brute force over small finite intervals: the hull of the images."""
    xs = range(a[0], a[1] + 1)
    ys = range(b[0], b[1] + 1)
    def q(x, y):
        if op == P.TDIV:
            return int(x / y)
        if op == P.FDIV:
            return x // y
        if op == P.CDIV:
            return -((-x) // y)
        r = x % abs(y)
        return (x - r) // y  # Euclidean
    if op == P.NEG:
        vals = [-x for x in xs]
    elif op == P.ABS:
        vals = [abs(x) for x in xs]
    elif op in (P.TDIV, P.FDIV, P.CDIV, P.EDIV):
        vals = [q(x, y) for x in xs for y in ys if y != 0]
    else:
        f = {P.ADD: lambda x, y: x + y, P.SUB: lambda x, y: x - y, P.MUL: lambda x, y: x * y,
             P.MIN: min, P.MAX: max}[op]
        vals = [f(x, y) for x in xs for y in ys]
    return (min(vals), max(vals)) if vals else None


@pytest.mark.parametrize("op", [P.NEG, P.ABS, P.ADD, P.SUB, P.MUL, P.TDIV, P.FDIV, P.CDIV, P.EDIV, P.MIN, P.MAX])
def test_interval_ops_exact_hull(op, oracle):
    """The restated lala-core interval operators give the exact hull of the
    images on every pair of small intervals (exhaustive over [-4, 4])."""
    ivs = [(l, u) for l in range(-4, 5) for u in range(l, 5)]
    for a, b in itertools.product(ivs, ivs if op not in (P.NEG, P.ABS) else [(0, 0)]):
        want = _interval_ref(op, a, b)
        got = oracle.pc_itv(op, a, b)
        if want is None:
            assert got[0] > got[1], (op, a, b, got)
        else:
            assert got == want, (op, a, b, got, want)


def test_interval_ops_infinite(oracle):
    """Infinite bounds: products and quotients on the extended integers."""
    assert oracle.pc_itv(P.EDIV, (P.MINF, 2), (3, 3)) == (P.MINF, 0)
    assert oracle.pc_itv(P.TDIV, (P.MINF, 2), (2, 2)) == (P.MINF, 1)
    assert oracle.pc_itv(P.TDIV, (5, P.INF), (1, P.INF)) == (0, P.INF)
    assert oracle.pc_itv(P.FDIV, (-7, 7), (P.MINF, -1)) == (-7, 7)
    assert oracle.pc_itv(P.MUL, (0, 0), (P.MINF, P.INF)) == (0, 0)
    assert oracle.pc_itv(P.MUL, (1, P.INF), (-2, -1)) == (P.MINF, -1)
    assert oracle.pc_itv(P.ADD, (P.MINF, 3), (1, 2)) == (P.MINF, 5)
    assert oracle.pc_itv(P.NEG, (P.MINF, 3)) == (-3, P.INF)
    assert oracle.pc_itv(P.ABS, (P.MINF, 3)) == (0, P.INF)


@pytest.mark.parametrize("seed", range(6))
def test_schedule_independence(seed, oracle):
    """The fixpoint does not depend on the propagator order (forward,
    reversed, shuffled Gauss-Seidel sweeps agree), the property that lets the
    GPU run every propagator of a round at once."""
    rng = np.random.default_rng(seed)
    t, store = H.random_formulas(rng, 40, 60, depth=3)
    tape, roots = t.arrays()
    assert oracle.pc_validate(tape, roots, len(store)) >= 1
    order = oracle.pc_order(tape, roots)
    results = []
    for perm in (order, order[::-1].copy(), rng.permutation(order)):
        s = store.copy()
        rc, _ = oracle.pc_fixpoint(tape, np.ascontiguousarray(perm, np.int32), s)
        results.append((rc, s if rc == oracle.OK else None))
    assert len({r[0] for r in results}) == 1
    if results[0][0] == oracle.OK:
        for r in results[1:]:
            np.testing.assert_array_equal(r[1], results[0][1])


def test_validate_rejects(oracle):
    t = P.Tape()
    x = t.var(0)
    t.prop(t.leq(x, t.constant(3)))
    tape, roots = t.arrays()
    assert oracle.pc_validate(tape, roots, 1) == 2
    assert oracle.pc_validate(tape, roots, 0) == -1          # var out of range
    bad = tape.copy()
    bad[2, 1] = 2                                               # child not before parent
    assert oracle.pc_validate(bad, roots, 1) == -3
    assert oracle.pc_validate(tape, np.array([0], np.int32), 1) == -1 - len(tape)  # root is a term


def test_planted_formulas_keep_their_solution(oracle):
    """Soundness on whole sets: formulas that a hidden assignment satisfies
    never lose it (Gauss-Seidel and Jacobi agree)."""
    for seed in range(6):
        rng = np.random.default_rng(400 + seed)
        t, store, hidden = H.planted_formulas(rng, 300, 200, depth=3)
        tape, roots = t.arrays()
        order = oracle.pc_order(tape, roots)
        a, b = store.copy(), store.copy()
        assert oracle.pc_fixpoint(tape, order, a)[0] == oracle.OK
        assert oracle.pc_fixpoint_jacobi(tape, order, b)[0] == oracle.OK
        np.testing.assert_array_equal(a, b)
        assert np.all((hidden >= a[:, 0]) & (hidden <= a[:, 1]))


@pytest.mark.parametrize("case", K.AE_CASES, ids=[c[0] for c in K.AE_CASES])
def test_abstract_element_oracle(case, oracle):
    """tests/pc_test.cpp:714-764 on the oracle."""
    tape, roots = H.ae_tape(case[2])
    store = np.array([[0, 10], [0, 10]], np.int32)
    state = {"failed": False}

    def steps(meets):
        for v, l, u in meets:
            store[v] = [max(store[v, 0], l), min(store[v, 1], u)]
        b0 = [tuple(int(x) for x in r) for r in store]
        rc, info = oracle.pc_fixpoint(tape, roots, store)
        state["failed"] = rc == oracle.FAILED
        ex = rc == oracle.OK and all(oracle.pc_ask(tape, r, store) for r in roots)
        return rc, b0, [tuple(int(x) for x in r) for r in store], ex, info["has_changed"]

    assert H.run_ae_case(steps, case) == []


def _pc_check_by_assignment(make_fzn, oracle, text, users, pred, one_sided=False):
    """Compiled to PC formulas: at every full assignment of the user
    variables the Gauss-Seidel fixpoint fails exactly where the definition
    is false (one_sided: at least there).  Returns the number of assignments
    checked."""
    import itertools
    m = make_fzn()
    d = m.compile(text)
    names = {n: i for i, n in enumerate(d["names"]) if n != "-"}
    store = np.array(d["newvars"], np.int32).reshape(-1, 2)
    for v, l, u in d["meets"]:
        store[v, 0] = max(store[v, 0], l)
        store[v, 1] = min(store[v, 1], u)
    tape, roots = d["tape"], oracle.pc_order(d["tape"], d["roots"])
    dec = [names[u] for u in users]
    decl = dict(zip(d["names"], d["newvars"]))
    n = 0
    for t in itertools.product(*(range(decl[u][0], decl[u][1] + 1) for u in users)):
        s = store.copy()
        inside = all(s[v, 0] <= a <= s[v, 1] for v, a in zip(dec, t))
        for v, a in zip(dec, t):
            s[v] = (a, a)
        if inside and len(roots):
            s = np.ascontiguousarray(s)
            rc, _ = oracle.pc_fixpoint(tape, roots, s)
            ok = rc == oracle.OK
        else:
            ok = inside
        if one_sided:
            assert not ok or pred(*t), (text, t)
        else:
            assert ok == bool(pred(*t)), (text, t)
        n += 1
    return n


@pytest.mark.parametrize("case", __import__("test_fzn").BUILTINS, ids=[c[0] for c in __import__("test_fzn").BUILTINS])
def test_fzn_builtins_by_assignment(case, make_fzn, oracle):
    """The builtins of the PIR front end's enumeration tests, through the PC
    front end (formula trees instead of ternary propagators)."""
    name, text, users, pred = case
    # the reference's GroupDiv::left_residual (terms.hpp:272-277) bounds the
    # dividend by r * y joined with y.ub - 1, which rejects valid assignments
    # of a rounding division (x = -7, y = 2, q = -3 under truncation): there
    # only a violating assignment must fail
    one_sided = bool(re.match(r"int_[tfce]?(div|mod)_", name))
    try:
        n = _pc_check_by_assignment(make_fzn, oracle, text, users.split(), pred, one_sided)
    except ValueError as e:
        if "unsupported" in str(e):
            pytest.skip("not in the PC front end's subset: %s" % e)
        raise
    assert n > 0


def test_fzn_minizinc_output_items(make_fzn, oracle):
    """The PC front end reads what MiniZinc writes around the constraints."""
    m = make_fzn()
    d = m.compile("""
    predicate fzn_all_different_int(array [int] of var int: x);
    var 1..3: x :: output_var;
    var 1..3: y :: output_var;
    array [1..2] of var int: xs :: output_array([1..2]) = [x, y];
    constraint int_lin_eq([1, 1], xs, 6) :: domain;
    solve satisfy;
    """)
    store = np.ascontiguousarray(np.array(d["newvars"], np.int32).reshape(-1, 2))
    rc, _ = oracle.pc_fixpoint(d["tape"], oracle.pc_order(d["tape"], d["roots"]), store)
    names = {n: i for i, n in enumerate(d["names"])}
    assert rc == oracle.OK
    assert tuple(store[names["x"]]) == (3, 3) and tuple(store[names["y"]]) == (3, 3)
