"""The event schedules' variable -> propagator adjacency (pir_csr.h), built
on the host's threads: the same arrays as a sequential counting sort for
every thread count, on random bytecodes with repeated variables."""
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
    lib.csr_threads.argtypes = [ctypes.c_longlong, ctypes.c_int]
    lib.csr_threads.restype = ctypes.c_int

    def build(nv, x, y, z, threads):
        n = len(x)
        x, y, z = (np.ascontiguousarray(a, np.int32) for a in (x, y, z))
        ptr = np.full(nv + 1, -7, np.int32)
        adj = np.full(3 * n, -7, np.int32)
        p = lambda a: a.ctypes.data_as(P)
        lib.csr_build(n, nv, p(x), p(y), p(z), p(ptr), p(adj), threads)
        return ptr, adj
    build.threads = lib.csr_threads
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


def test_thread_choice(csr):
    assert csr.threads(1000, 8) == 1             # small inputs stay on one thread
    assert csr.threads(1 << 20, 8) == 8
    assert csr.threads(1 << 20, 64) == 16        # capped
    assert 1 <= csr.threads(1 << 20, 0) <= 16
