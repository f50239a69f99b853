"""The FlatZinc front end (include/pirgpu_fzn.hpp): models compiled to PIR
propagators reach lala-pc's known bounds for the user variables (the tests
whose generated variables come from lala-core's ternarizer: checked on the
user variables only), and known solutions under search -- on the oracle
without a GPU, and on the GPU engine."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import fzn_models as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def fzn(tmp_path_factory):
    out = tmp_path_factory.mktemp("fzn") / "libfzn_shim.so"
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "fzn_shim.cpp"), "-o", str(out)],
                   check=True, capture_output=True, text=True)
    lib = ctypes.CDLL(str(out))
    lib.fzn_compile.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
    lib.fzn_compile.restype = ctypes.c_int

    def compile_model(text):
        buf = ctypes.create_string_buffer(1 << 22)
        rc = lib.fzn_compile(text.encode(), buf, len(buf))
        if rc:
            raise ValueError(buf.value.decode())
        lines = buf.value.decode().splitlines()
        nv, npr = map(int, lines[0].split())
        dom = np.array([list(map(int, l.split()[:2])) for l in lines[1:1 + nv]], np.int64).reshape(-1, 2)
        names = {l.split()[2]: i for i, l in enumerate(lines[1:1 + nv]) if l.split()[2] != "-"}
        props = np.array([list(map(int, l.split())) for l in lines[1 + nv:1 + nv + npr]], np.int32).reshape(-1, 4)
        return dom.astype(np.int32), props, names
    return compile_model


def _oracle_fix(oracle, dom, props):
    s = np.ascontiguousarray(dom, np.int32)
    rc, _ = oracle.install_and_fixpoint(props[:, 0], props[:, 1], props[:, 2], props[:, 3], s)
    return rc, s


@pytest.mark.parametrize("case", M.KATS, ids=[c[0] for c in M.KATS])
def test_kat_user_bounds_oracle(case, fzn, oracle):
    name, texts, users, expect = case
    for k in range(len(texts)):
        dom, props, names = fzn(" ".join(texts[:k + 1]))
        rc, s = _oracle_fix(oracle, dom, props)
        assert rc == oracle.OK
        got = [tuple(s[names[u]]) for u in users]
        assert got == [tuple(e) for e in expect[k]], (name, k)


def test_minizinc_output_items(fzn, oracle):
    """What MiniZinc writes around the constraints: predicate declarations,
    annotations on variables, arrays, constraints and the solve item."""
    text = """
    predicate fzn_all_different_int(array [int] of var int: x);
    var 1..3: x :: output_var;
    var 1..3: y :: output_var;
    var 2..6: s :: is_defined_var;
    array [1..2] of var int: xs :: output_array([1..2]) = [x, y];
    array [1..2] of int: cs = [1, 1];
    constraint int_lin_eq(cs, xs, 6) :: domain;
    constraint int_plus(x, y, s) :: defines_var(s);
    solve :: int_search(xs, input_order, indomain_min, complete) satisfy;
    """
    dom, props, names = fzn(text)
    rc, s = _oracle_fix(oracle, dom, props)
    assert rc == oracle.OK
    assert tuple(s[names["x"]]) == (3, 3) and tuple(s[names["y"]]) == (3, 3) and tuple(s[names["s"]]) == (6, 6)
    with pytest.raises(ValueError, match="predicate name"):
        fzn("predicate ;")


def test_errors_are_reported(fzn):
    with pytest.raises(ValueError, match="unsupported constraint"):
        fzn("var int: x; constraint no_such_thing(x);")
    with pytest.raises(ValueError, match="unknown identifier"):
        fzn("var int: x; constraint int_le(x, y);")
    with pytest.raises(ValueError, match="FlatZinc"):
        fzn("var int x;")
    # half reification of functions that are not boolean
    with pytest.raises(ValueError, match="not a boolean function"):
        fzn("var 0..3: x; var 0..3: y; var 0..6: z; var bool: r; constraint int_plus_imp(x, y, z, r);")
    with pytest.raises(ValueError, match="not a boolean function"):
        fzn("var 0..3: m; var 0..3: x; var bool: r; constraint array_int_maximum_imp(m, [x], r);")
    with pytest.raises(ValueError, match="empty array"):
        fzn("var 0..3: m; constraint array_int_minimum(m, []);")


def _search_oracle(oracle, dom, props, dec):
    s = np.ascontiguousarray(dom, np.int32)
    st, perm = oracle.install(props[:, 0], props[:, 1], props[:, 2], props[:, 3], s)
    p = props[perm]
    return oracle.search(p[:, 0], p[:, 1], p[:, 2], p[:, 3], s, dec, max_solutions=1000)


def test_send_more_money_oracle(fzn, oracle):
    text, letters = M.send_more_money()
    dom, props, names = fzn(text)
    rc, sols, info = _search_oracle(oracle, dom, props, [names[c] for c in letters])
    assert rc == oracle.OK and info["solutions"] == 1
    assert dict(zip(letters, sols[0])) == dict(S=9, E=5, N=6, D=7, M=1, O=0, R=8, Y=2)


def test_queens_oracle(fzn, oracle):
    text, qs = M.queens(8)
    dom, props, names = fzn(text)
    rc, sols, info = _search_oracle(oracle, dom, props, [names[q] for q in qs])
    assert rc == oracle.OK and info["solutions"] == 92


def test_magic_square_oracle(fzn, oracle):
    text, cells = M.magic_square3()
    dom, props, names = fzn(text)
    rc, sols, info = _search_oracle(oracle, dom, props, [names[c] for c in cells])
    assert rc == oracle.OK and info["solutions"] == 8
    for sol in sols:
        g = np.array(sol).reshape(3, 3)
        assert sorted(sol) == list(range(1, 10))
        assert all(g.sum(0) == 15) and all(g.sum(1) == 15) and np.trace(g) == 15 and np.trace(g[::-1]) == 15


# ------------------------------------------------------------------- GPU ----

def _gpu_ctx(dom, props):
    import pirgpu
    ctx = pirgpu.Context(0)
    ctx.load_store(dom[:, 0], dom[:, 1])
    if len(props):
        ctx.tell(props[:, 0], props[:, 1], props[:, 2], props[:, 3])
    return ctx


@pytest.mark.gpu
@pytest.mark.parametrize("case", M.KATS, ids=[c[0] for c in M.KATS])
def test_kat_user_bounds_gpu(case, fzn):
    import pirgpu
    name, texts, users, expect = case
    for k in range(len(texts)):
        dom, props, names = fzn(" ".join(texts[:k + 1]))
        ctx = _gpu_ctx(dom, props)
        rc, _ = ctx.fixpoint()
        assert rc == pirgpu.OK
        lb, ub = ctx.read_store()
        assert [(lb[names[u]], ub[names[u]]) for u in users] == [tuple(e) for e in expect[k]], (name, k)


@pytest.mark.gpu
def test_send_more_money_and_queens_gpu(fzn):
    import pirgpu
    text, letters = M.send_more_money()
    dom, props, names = fzn(text)
    ctx = _gpu_ctx(dom, props)
    status, sols, st = ctx.search([names[c] for c in letters], max_solutions=10)
    assert status == pirgpu.OK and st["solutions"] == 1
    assert list(sols[0]) == [9, 5, 6, 7, 1, 0, 8, 2]
    text, qs = M.queens(8)
    dom, props, names = fzn(text)
    ctx = _gpu_ctx(dom, props)
    status, sols, st = ctx.search([names[q] for q in qs], max_solutions=100)
    assert st["solutions"] == 92


# -------------------------------------------------- builtins, exhaustively ----

def _tdiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def _cdiv(a, b):
    return -((-a) // b)


def _ediv(a, b):
    return (a - a % abs(b)) // b


_DIVS = {"int_div": _tdiv, "int_tdiv": _tdiv, "int_fdiv": lambda a, b: a // b, "int_cdiv": _cdiv,
         "int_ediv": _ediv}
_MODS = {"int_mod": _tdiv, "int_tmod": _tdiv, "int_fmod": lambda a, b: a // b, "int_cmod": _cdiv,
         "int_emod": _ediv}

BUILTINS = [
    ("array_int_maximum", "var -3..3: m; var -2..2: x; var -2..2: y; var -2..2: z; "
     "constraint array_int_maximum(m, [x, y, z]);", "m x y z", lambda m, x, y, z: m == max(x, y, z)),
    ("array_int_minimum", "var -3..3: m; var -2..2: x; var -2..2: y; var 0..2: z; "
     "constraint array_int_minimum(m, [x, y, z]);", "m x y z", lambda m, x, y, z: m == min(x, y, z)),
    ("array_int_maximum_one", "var -3..3: m; var -2..2: x; constraint array_int_maximum(m, [x]);", "m x",
     lambda m, x: m == x),
    ("bool_lin_eq", "var bool: a; var bool: b; var bool: c; constraint bool_lin_eq([2, 3, -1], [a, b, c], 2);",
     "a b c", lambda a, b, c: 2 * a + 3 * b - c == 2),
    ("bool_lin_le", "var bool: a; var bool: b; var bool: c; constraint bool_lin_le([1, 1, 1], [a, b, c], 1);",
     "a b c", lambda a, b, c: a + b + c <= 1),
    ("array_bool_xor", "var bool: a; var bool: b; var bool: c; var bool: d; "
     "constraint array_bool_xor([a, b, c, d]);", "a b c d", lambda a, b, c, d: (a + b + c + d) % 2 == 1),
    ("int_lin_le_imp", "var -2..2: x; var -2..2: y; var bool: r; constraint int_lin_le_imp([1, 2], [x, y], 1, r);",
     "x y r", lambda x, y, r: not r or x + 2 * y <= 1),
    ("int_lin_ne_reif", "var -2..2: x; var -2..2: y; var bool: r; "
     "constraint int_lin_ne_reif([1, -1], [x, y], 1, r);", "x y r", lambda x, y, r: r == (x - y != 1)),
    ("int_eq_imp", "var -2..2: x; var -2..2: y; var bool: r; constraint int_eq_imp(x, y, r);", "x y r",
     lambda x, y, r: not r or x == y),
    ("int_ne_imp", "var -2..2: x; var -2..2: y; var bool: r; constraint int_ne_imp(x, y, r);", "x y r",
     lambda x, y, r: not r or x != y),
    ("int_lt_imp", "var -2..2: x; var -2..2: y; var bool: r; constraint int_lt_imp(x, y, r);", "x y r",
     lambda x, y, r: not r or x < y),
    ("set_in_imp", "var -3..3: x; var bool: r; constraint set_in_imp(x, {-1, 2}, r);", "x r",
     lambda x, r: not r or x in (-1, 2)),
    ("bool_clause_imp", "var bool: a; var bool: b; var bool: c; var bool: r; "
     "constraint bool_clause_imp([a, b], [c], r);", "a b c r", lambda a, b, c, r: not r or a or b or not c),
    ("int_times", "var -3..3: x; var -3..3: y; var -9..9: z; constraint int_times(x, y, z);", "x y z",
     lambda x, y, z: z == x * y),
    ("int_abs", "var -3..3: x; var -3..3: y; constraint int_abs(x, y);", "x y", lambda x, y: y == abs(x)),
    ("int_max_reif_nested", "var -2..2: x; var -2..2: y; var bool: r; "
     "constraint int_le_reif(int_max(x, y), 1, r);", "x y r", lambda x, y, r: r == (max(x, y) <= 1)),
] + [
    # comparisons, imposed and reified
    ("%s%s" % (f, "_reif" if reif else ""),
     "var -2..2: x; var -2..2: y;%s constraint %s%s(x, y%s);" % (
         " var bool: r;" if reif else "", f, "_reif" if reif else "", ", r" if reif else ""),
     "x y r" if reif else "x y",
     (lambda c, reif: (lambda x, y, r: r == c(x, y)) if reif else (lambda x, y: c(x, y)))(c, reif))
    for f, c in (("int_eq", lambda x, y: x == y), ("int_ne", lambda x, y: x != y), ("int_le", lambda x, y: x <= y),
                 ("int_lt", lambda x, y: x < y), ("int_ge", lambda x, y: x >= y), ("int_gt", lambda x, y: x > y))
    for reif in (False, True)
] + [
    ("%s%s" % (f, "_reif" if reif else ""),
     "var bool: a; var bool: b;%s constraint %s%s(a, b%s);" % (
         " var bool: r;" if reif else "", f, "_reif" if reif else "", ", r" if reif else ""),
     "a b r" if reif else "a b",
     (lambda c, reif: (lambda a, b, r: r == c(a, b)) if reif else (lambda a, b: c(a, b)))(c, reif))
    for f, c in (("bool_eq", lambda a, b: a == b), ("bool_ne", lambda a, b: a != b), ("bool_le", lambda a, b: a <= b),
                 ("bool_lt", lambda a, b: a < b), ("bool_and", lambda a, b: bool(a and b)),
                 ("bool_or", lambda a, b: bool(a or b)), ("bool_xor", lambda a, b: a != b))
    for reif in (False, True)
] + [
    ("all_different_int", "var 1..3: x; var 1..3: y; var 1..4: z; constraint fzn_all_different_int([x, y, z]);",
     "x y z", lambda x, y, z: len({x, y, z}) == 3),
    ("bool_not", "var bool: a; var bool: b; constraint bool_not(a, b);", "a b", lambda a, b: b == 1 - a),
    ("bool2int", "var bool: a; var 0..3: i; constraint bool2int(a, i);", "a i", lambda a, i: i == a),
    ("bool_clause", "var bool: a; var bool: b; var bool: c; constraint bool_clause([a, b], [c]);", "a b c",
     lambda a, b, c: bool(a or b or not c)),
    ("bool_clause_reif", "var bool: a; var bool: b; var bool: r; constraint bool_clause_reif([a], [b], r);",
     "a b r", lambda a, b, r: r == bool(a or not b)),
    ("array_bool_and_reif", "var bool: a; var bool: b; var bool: c; var bool: r; "
     "constraint array_bool_and([a, b, c], r);", "a b c r", lambda a, b, c, r: r == bool(a and b and c)),
    ("array_bool_or", "var bool: a; var bool: b; var bool: c; constraint array_bool_or([a, b, c], true);",
     "a b c", lambda a, b, c: bool(a or b or c)),
    ("set_in", "var -3..3: x; constraint set_in(x, {-2, 0, 3});", "x", lambda x: x in (-2, 0, 3)),
    ("set_in_range_reif", "var -3..3: x; var bool: r; constraint set_in_reif(x, -1..1, r);", "x r",
     lambda x, r: r == (-1 <= x <= 1)),
    ("array_int_element", "var 1..4: i; var -5..5: x; constraint array_int_element(i, [3, -1, 4, 1], x);", "i x",
     lambda i, x: x == [3, -1, 4, 1][i - 1]),
    ("array_var_int_element", "var 1..3: i; var 0..2: a; var 0..2: b; var 0..2: c; var 0..2: x; "
     "constraint array_var_int_element(i, [a, b, c], x);", "i a b c x",
     lambda i, a, b, c, x: x == [a, b, c][i - 1]),
    ("array_var_bool_element", "var 1..2: i; var bool: a; var bool: b; var bool: x; "
     "constraint array_var_bool_element(i, [a, b], x);", "i a b x", lambda i, a, b, x: x == [a, b][i - 1]),
    ("int_lin_eq", "var -2..2: x; var -2..2: y; var -2..2: z; constraint int_lin_eq([2, -3, 1], [x, y, z], 1);",
     "x y z", lambda x, y, z: 2 * x - 3 * y + z == 1),
    ("int_lin_lt_reif", "var -2..2: x; var -2..2: y; var bool: r; "
     "constraint int_lin_lt_reif([1, 1], [x, y], 0, r);", "x y r", lambda x, y, r: r == (x + y < 0)),
    ("int_lin_ge", "var -2..2: x; var -2..2: y; constraint int_lin_ge([3, -1], [x, y], 2);", "x y",
     lambda x, y: 3 * x - y >= 2),
    ("int_plus_minus_negate", "var -3..3: x; var -3..3: y; var -6..6: s; var -6..6: d; var -3..3: n; "
     "constraint int_plus(x, y, s); constraint int_minus(x, y, d); constraint int_negate(x, n);",
     "x y s d n", lambda x, y, s, d, n: s == x + y and d == x - y and n == -x),
    ("int_min_max", "var -2..2: x; var -2..2: y; var -2..2: lo; var -2..2: hi; "
     "constraint int_min(x, y, lo); constraint int_max(x, y, hi);", "x y lo hi",
     lambda x, y, lo, hi: lo == min(x, y) and hi == max(x, y)),
] + [
    ("%s_%s" % (f, sign), "var -7..7: x; var %s: y; var -8..8: q; constraint %s(x, y, q);" % (dom, f), "x y q",
     (lambda d: lambda x, y, q: q == d(x, y))(d))
    for f, d in _DIVS.items() for sign, dom in (("pos", "1..3"), ("neg", "-3..-1"))
] + [
    ("%s_%s" % (f, sign), "var -7..7: x; var %s: y; var -3..3: m; constraint %s(x, y, m);" % (dom, f), "x y m",
     (lambda d: lambda x, y, m: m == x - y * d(x, y))(d))
    for f, d in _MODS.items() for sign, dom in (("pos", "1..3"), ("neg", "-3..-1"))
]


@pytest.mark.parametrize("case", BUILTINS, ids=[c[0] for c in BUILTINS])
def test_builtin_solutions_match_brute_force(case, fzn, oracle):
    """Every solution of the compiled model (the oracle's search over the
    user variables) and nothing else satisfies the builtin's definition."""
    import itertools
    name, text, users, pred = case
    users = users.split()
    dom, props, names = fzn(text)
    dec = [names[u] for u in users]
    want = sorted(t for t in itertools.product(*(range(dom[v][0], dom[v][1] + 1) for v in dec)) if pred(*t))
    assert len(props) > 0
    s = np.ascontiguousarray(dom, np.int32)
    _, perm = oracle.install(props[:, 0], props[:, 1], props[:, 2], props[:, 3], s)
    p = props[perm]
    _, sols, _ = oracle.search(p[:, 0], p[:, 1], p[:, 2], p[:, 3], s, dec, max_solutions=100_000)
    got = sorted(tuple(int(v) for v in row) for row in sols)
    assert want and got == want, name


@pytest.mark.gpu
@pytest.mark.parametrize("case", BUILTINS, ids=[c[0] for c in BUILTINS])
def test_builtin_solutions_match_brute_force_gpu(case, fzn):
    import itertools
    import pirgpu
    name, text, users, pred = case
    users = users.split()
    dom, props, names = fzn(text)
    dec = [names[u] for u in users]
    want = sorted(t for t in itertools.product(*(range(dom[v][0], dom[v][1] + 1) for v in dec)) if pred(*t))
    ctx = _gpu_ctx(dom, props)
    status, sols, st = ctx.search(dec, max_solutions=100_000)
    assert status == pirgpu.OK
    got = sorted(tuple(int(v) for v in row) for row in sols)
    assert got == want, name


@pytest.mark.gpu
def test_magic_square_gpu(fzn):
    import pirgpu
    text, cells = M.magic_square3()
    dom, props, names = fzn(text)
    ctx = _gpu_ctx(dom, props)
    status, sols, st = ctx.search([names[c] for c in cells], max_solutions=100)
    assert status == pirgpu.OK and st["solutions"] == 8
    for sol in sols:
        g = np.array(sol).reshape(3, 3)
        assert sorted(sol) == list(range(1, 10)) and all(g.sum(0) == 15) and all(g.sum(1) == 15)
