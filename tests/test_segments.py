"""The path segments of the single-instance event schedule (pir_segments.h),
checked on the host against their definition: a segment is 4 to 64
propagators of a path, consecutive ones sharing a variable that occurs
exactly twice in the whole bytecode (once in each); every propagator is in at
most one segment; the segment's local code names its propagators' variables;
a local variable is marked as a boundary exactly when it also occurs outside
the segment; the use masks list the segment's propagators using each local
variable; and the variable -> unit adjacency lists, for every variable, each
distinct unit (a propagator outside the segments, or a segment) using it."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DTYPES = [np.int32, np.int32, np.int32, np.int32, np.int32, np.uint32, np.uint64, np.int32, np.int32, np.uint32]


@pytest.fixture(scope="module")
def seg(tmp_path_factory):
    out = tmp_path_factory.mktemp("seg") / "libseg_shim.so"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread",
                    os.path.join(ROOT, "tests", "cpp", "csr_shim.cpp"), "-o", str(out)],
                   check=True, capture_output=True, text=True)
    lib = ctypes.CDLL(str(out))
    P = ctypes.POINTER(ctypes.c_int)
    lib.seg_build.argtypes = [ctypes.c_longlong, ctypes.c_int, P, P, P, P, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_longlong)]
    lib.seg_build.restype = ctypes.c_int
    lib.seg_get.argtypes = [ctypes.c_int, ctypes.c_void_p]

    def build(nv, op, x, y, z, threads=4):
        arrs = [np.ascontiguousarray(a, np.int32) for a in (op, x, y, z)]
        sizes = (ctypes.c_longlong * 10)()
        nseg = lib.seg_build(len(arrs[0]), nv, *(a.ctypes.data_as(P) for a in arrs), threads, sizes)
        assert nseg >= 0
        out = []
        for k in range(10):
            a = np.zeros(sizes[k], DTYPES[k])
            if sizes[k]:
                lib.seg_get(k, a.ctypes.data_as(ctypes.c_void_p))
            out.append(a)
        return nseg, out
    return build


def _check(nv, op, x, y, z, nseg, out):
    seg_of, pptr, code, prop, vptr, var, umask, uptr, uadj, in_seg = out
    n = len(op)
    occ = np.bincount(np.concatenate([x, y, z]), minlength=nv)
    users = [set() for _ in range(nv)]
    for p in range(n):
        for v in (x[p], y[p], z[p]):
            users[v].add(p)
    assert len(pptr) == nseg + 1 and len(vptr) == nseg + 1
    covered = set()
    for s in range(nseg):
        props = prop[pptr[s]:pptr[s + 1]]
        assert 4 <= len(props) <= 64
        assert not covered & set(props.tolist())
        covered |= set(props.tolist())
        assert np.all(seg_of[props] == s)
        for a, b in zip(props[:-1], props[1:]):
            link = [v for v in {x[a], y[a], z[a]} & {x[b], y[b], z[b]} if occ[v] == 2]
            assert link, (s, a, b)
        lvars = (var[vptr[s]:vptr[s + 1]] & 0x7FFFFFFF).astype(np.int64)
        bnd = (var[vptr[s]:vptr[s + 1]] >> 31).astype(bool)
        assert len(set(lvars.tolist())) == len(lvars) <= 192
        seg_occ = {}
        for k, p in enumerate(props):
            c = int(code[pptr[s] + k]) & 0xFFFFFFFF
            assert c & 0xFF == op[p]
            sl = [(c >> 8) & 0xFF, (c >> 16) & 0xFF, c >> 24]
            assert [lvars[j] for j in sl] == [x[p], y[p], z[p]]
            for j in sl:
                seg_occ[j] = seg_occ.get(j, 0) + 1
        for j, v in enumerate(lvars):
            assert bnd[j] == (occ[v] > seg_occ[j])
            m = int(umask[vptr[s] + j])
            expect = sum(1 << k for k, p in enumerate(props) if v in (x[p], y[p], z[p]))
            assert m == expect
    assert np.all(seg_of[[p for p in range(n) if p not in covered]] == -1)
    bits = np.unpackbits(in_seg.view(np.uint8), bitorder="little")[:n].astype(bool)
    assert np.array_equal(bits, seg_of >= 0)
    # unit adjacency
    assert len(uptr) == nv + 1
    for v in range(nv):
        units = uadj[uptr[v]:uptr[v + 1]].tolist()
        assert len(units) == len(set(units))
        expect = {(~int(seg_of[p]) if seg_of[p] >= 0 else p) for p in users[v]}
        assert set(units) == expect


def test_chain_is_cut_into_segments(seg):
    """A 1,000-link chain x_{i+1} = x_i + c_i: one path, cut into 16 segments."""
    import workloads as W
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    inst = W.add_chain(empty, 1000, 10**6, 3)
    nseg, out = seg(inst.nvars, inst.op, inst.x, inst.y, inst.z)
    assert nseg == 16
    assert (out[0] >= 0).sum() == 1000
    _check(inst.nvars, inst.op, inst.x, inst.y, inst.z, nseg, out)


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_random_and_chain(seg, threads):
    """A random part (few variables of degree 2) plus a chain and mixed links."""
    import workloads as W
    inst = W.add_chain(W.plain(3_000, 12_000, 1000, 5), 300, 10**4, 5)
    nseg, out = seg(inst.nvars, inst.op, inst.x, inst.y, inst.z, threads)
    assert nseg >= 4
    _check(inst.nvars, inst.op, inst.x, inst.y, inst.z, nseg, out)


def test_cycles_and_double_links(seg):
    """A ring of 10 propagators (every variable of degree 2), a pair sharing
    two link variables, and a propagator using one variable twice."""
    ring = [(0, i, (i + 1) % 10, 10 + i) for i in range(10)]
    pair = [(0, 30, 31, 32), (1, 30, 31, 33)]
    twice = [(0, 40, 40, 41)]
    rows = np.array(ring + pair + twice, np.int32)
    nv = 50
    nseg, out = seg(nv, rows[:, 0], rows[:, 1], rows[:, 2], rows[:, 3])
    assert nseg == 1 and out[1][1] == 10
    _check(nv, rows[:, 0], rows[:, 1], rows[:, 2], rows[:, 3], nseg, out)


def test_no_paths(seg):
    """Every variable occurring three times or more: no segment, and the unit
    adjacency is the propagator adjacency."""
    rng = np.random.default_rng(1)
    n, nv = 4000, 300
    x, y, z = (rng.integers(0, nv, n) for _ in range(3))
    op = rng.integers(0, 10, n)
    nseg, out = seg(nv, op, x, y, z)
    assert nseg == 0
    _check(nv, op, x, y, z, nseg, out)
