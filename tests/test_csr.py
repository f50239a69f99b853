"""The host-threaded builders of the install (pir_csr.h, pir_sort.h): the
event schedules' variable -> propagator adjacency (the arrays of a
sequential counting sort, on random bytecodes with repeated variables), the
PC event schedule's variable -> formula adjacency (a Python walk of every
formula) and the install order of the bytecode (numpy's stable sort by
(op, y, x, z)), for every thread count."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def csr(tmp_path_factory):
    out = tmp_path_factory.mktemp("csr") / "libcsr_shim.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread",
                    os.path.join(ROOT, "tests", "cpp", "csr_shim.cpp"), "-o", str(out)],
                   check=True, capture_output=True, text=True)
    lib = ctypes.CDLL(str(out))
    P = ctypes.POINTER(ctypes.c_int)
    lib.csr_build.argtypes = [ctypes.c_longlong, ctypes.c_int, P, P, P, P, P, ctypes.c_int]
    lib.csr_build.restype = ctypes.c_int
    lib.csr_threads.argtypes = [ctypes.c_longlong, ctypes.c_int, ctypes.c_longlong]
    lib.csr_threads.restype = ctypes.c_int

    def build(nv, x, y, z, threads):
        n = len(x)
        x, y, z = (np.ascontiguousarray(a, np.int32) for a in (x, y, z))
        ptr = np.full(nv + 1, -7, np.int32)
        adj = np.full(3 * n, -7, np.int32)
        p = lambda a: a.ctypes.data_as(P)
        assert lib.csr_build(n, nv, p(x), p(y), p(z), p(ptr), p(adj), threads) == 1
        return ptr, adj
    build.threads = lib.csr_threads
    build.lib = lib
    build.lib_path = out
    return build


def _reference(nv, x, y, z):
    v = np.stack([x, y, z], 1).ravel()           # per propagator: x, y, z
    p = np.repeat(np.arange(len(x), dtype=np.int32), 3)
    order = np.argsort(v, kind="stable")
    ptr = np.concatenate([[0], np.cumsum(np.bincount(v, minlength=nv))]).astype(np.int32)
    return ptr, p[order]


@pytest.mark.parametrize("threads", [1, 2, 3, 7, 16])
@pytest.mark.parametrize("shape", [(0, 1), (1, 1), (5, 3), (1000, 10), (20000, 50000), (300000, 1000)])
def test_adjacency_matches_counting_sort(csr, shape, threads):
    n, nv = shape
    rng = np.random.default_rng(n * 31 + nv)
    x, y, z = (rng.integers(0, nv, n) for _ in range(3))
    y[: n // 4] = x[: n // 4]                    # repeated variables within a propagator
    ptr, adj = csr(nv, x, y, z, threads)
    rptr, radj = _reference(nv, x, y, z)
    np.testing.assert_array_equal(ptr, rptr)
    np.testing.assert_array_equal(adj, radj)


def test_adjacency_rejects_int32_overflow(csr):
    """3 n adjacency entries beyond INT32_MAX (n > 715,827,882 propagators,
    which fit a GB300's memory) would wrap the int32 offsets: the builder
    refuses before touching anything (the bytecode arrays are never read,
    so a fake n with one-element arrays is safe)."""
    P = ctypes.POINTER(ctypes.c_int)
    one = np.zeros(1, np.int32)
    ptr = np.full(2, -7, np.int32)
    adj = np.full(1, -7, np.int32)
    p = lambda a: a.ctypes.data_as(P)
    for n in ((2**31 - 1) // 3 + 1, 2**31, 2**40):
        assert csr.lib.csr_build(n, 1, p(one), p(one), p(one), p(ptr), p(adj), 4) == 0
    assert np.all(ptr == -7) and np.all(adj == -7)


def test_thread_choice(csr):
    assert csr.threads(1000, 8, 0) == 1             # small inputs stay on one thread
    assert csr.threads(1 << 20, 8, 0) == 8
    assert csr.threads(1 << 20, 64, 0) == 16        # capped
    assert 1 <= csr.threads(1 << 20, 0, 0) <= 16
    # per-thread counts of nvars words stay within the 3 n entries
    assert csr.threads(4_000_000, 16, 1_000_000) == 12
    assert csr.threads(4_000_000, 16, 100_000_000) == 1


def _pc_reference(tape, roots, nv):
    """Variable -> formula adjacency by walking every formula in Python."""
    import pc as P
    lists = [[] for _ in range(nv)]
    for i, r in enumerate(roots):
        seen, todo = set(), [int(r)]
        while todo:
            k, a, b, _ = (int(v) for v in tape[todo.pop()])
            if k in (P.VAR, P.PVAR, P.NVAR) or P.TELL <= k <= P.NASK_OUT:
                seen.add(a)
            elif k in (P.AE, P.NADD, P.NMUL):
                todo += list(range(a, a + b))
            elif k in (P.FORMULA, P.NEG, P.ABS, P.ARG):
                todo.append(a)
            elif P.ADD <= k <= P.MAX or P.LEQ <= k <= P.XOR:
                todo += [a, b]
        for v in seen:
            lists[v].append(i)
    ptr = np.concatenate([[0], np.cumsum([len(l) for l in lists])]).astype(np.int32)
    adj = np.array([i for l in lists for i in l], np.int32)
    return ptr, adj


def _pc_tapes():
    import pc as P
    import workloads as W
    tape, roots, lb, _, _ = W.pc_mix(3000, 2000, seed=2)
    yield "pc_mix", tape, roots, len(lb)
    t = P.Tape()
    x = [t.var(v) for v in range(6)]
    t.prop(t.leq(t.nadd([x[0], x[1], x[2], x[0]]), t.constant(5)))
    t.prop(t.disj(t.eq(t.mul(x[3], x[3]), t.constant(4)), t.pvar(5)))
    t.prop(t.abstract_element(tell=[(1, 0, 3)], ask=[(2, 1, 1)], not_ask=[(4, 0, 0)]))
    t.prop(t.true())
    t.prop(t.imply(t.gt(t.abs(x[4]), t.neg(x[1])), t.nvar(0)))
    tape, roots = t.arrays()
    yield "mixed", tape, roots, 8


@pytest.mark.parametrize("threads", [1, 2, 5, 16])
def test_formula_adjacency_matches_reference(csr, threads):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "lala-pc_gb300"))
    lib = ctypes.CDLL(str(csr.lib_path))
    P_ = ctypes.POINTER(ctypes.c_int)
    lib.pc_adjacency.argtypes = [ctypes.c_int, P_, P_, ctypes.c_int, P_, P_, ctypes.c_int, ctypes.c_int]
    lib.pc_adjacency.restype = ctypes.c_int
    for name, tape, roots, nv in _pc_tapes():
        tape = np.ascontiguousarray(tape, np.int32)
        roots = np.ascontiguousarray(roots, np.int32)
        ptr = np.full(nv + 1, -7, np.int32)
        adj = np.full(8 * len(tape) + 1, -7, np.int32)
        p = lambda a: a.ctypes.data_as(P_)
        k = lib.pc_adjacency(len(roots), p(roots), p(tape), nv, p(ptr), p(adj), len(adj), threads)
        rptr, radj = _pc_reference(tape, roots, nv)
        assert k == len(radj), name
        np.testing.assert_array_equal(ptr, rptr, err_msg=name)
        np.testing.assert_array_equal(adj[:k], radj, err_msg=name)


@pytest.mark.parametrize("threads", [1, 2, 3, 8, 16])
@pytest.mark.parametrize("shape", [(0, 1), (1, 1), (4095, 3), (5000, 3), (100_000, 40), (300_000, 1000)])
def test_install_order_is_the_stable_sort(csr, shape, threads):
    """The parallel stable sort gives numpy's stable sort by (op, y, x, z):
    ties keep their input order (small variable ranges make many ties)."""
    lib = ctypes.CDLL(str(csr.lib_path))
    P_ = ctypes.POINTER(ctypes.c_int)
    lib.install_order.argtypes = [ctypes.c_int, P_, P_, P_, P_, P_, ctypes.c_int]
    n, nv = shape
    rng = np.random.default_rng(n + nv)
    op = rng.integers(0, 10, n).astype(np.int32)
    x, y, z = (rng.integers(0, nv, n).astype(np.int32) for _ in range(3))
    perm = np.full(n, -1, np.int32)
    p = lambda a: a.ctypes.data_as(P_)
    lib.install_order(n, p(op), p(x), p(y), p(z), p(perm), threads)
    want = np.lexsort((z, x, y, op))  # lexsort is stable: the last key is the primary one
    np.testing.assert_array_equal(perm, want)
