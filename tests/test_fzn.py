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


def test_errors_are_reported(fzn):
    with pytest.raises(ValueError, match="unsupported constraint"):
        fzn("var int: x; constraint no_such_thing(x);")
    with pytest.raises(ValueError, match="unknown identifier"):
        fzn("var int: x; constraint int_le(x, y);")
    with pytest.raises(ValueError, match="FlatZinc"):
        fzn("var int x;")


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
