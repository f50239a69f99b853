"""pir_fixpoint_static: the fixpoint entry point that allocates no device memory.

It serves callers that own every byte of device memory themselves (a solver
handing the engine slices of its own pool, or a search loop on many streams
that cannot afford cudaMalloc / cudaFree and the device-wide synchronization
they may cause).  Here the test plays such a caller: it allocates the bytecode
and store buffers itself, calls the entry point through the C ABI on two
different instances in a row (the second call must not see anything left in
the shared scratch by the first), and checks each result bit for bit against
the context entry point pir_fixpoint."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class _DeviceBuffers:
    """Caller-owned device memory through libcudart."""

    def __init__(self):
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                self.L = ctypes.CDLL(name)
                break
            except OSError:
                continue
        self.ptrs = []

    def upload(self, a):
        a = np.ascontiguousarray(a)
        p = ctypes.c_void_p()
        assert self.L.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(a.nbytes, 8))) == 0
        self.ptrs.append(p)
        assert self.L.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1) == 0
        return p

    def download(self, p, like):
        out = np.empty_like(like)
        assert self.L.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), p, ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        for p in self.ptrs:
            self.L.cudaFree(p)
        self.ptrs = []


def test_static_entry_point_matches_context_entry_point():
    import pirgpu
    import workloads as W
    L = pirgpu.lib()
    mem = _DeviceBuffers()
    instances = [W.add_chain(W.plain(30_000, 120_000, 1000, 11), 150, 1000, 11),
                 W.plain(20_000, 80_000, 10**6, 12)]
    try:
        for inst in instances:
            ctx = pirgpu.Context(0)
            ctx.load_store(inst.lb, inst.ub)
            ctx.tell(inst.op, inst.x, inst.y, inst.z)
            lb0, ub0 = ctx.read_store()          # installed initial store
            op, x, y, z = ctx.bytecode()
            rc_ref, st_ref = ctx.fixpoint(mode=pirgpu.MODE_PERSISTENT)
            lb_ref, ub_ref = ctx.read_store()
            store = np.ascontiguousarray(np.stack([lb0, ub0], 1).astype(np.int32))
            d = [mem.upload(a) for a in (op, x, y, z)]
            d_store = mem.upload(store)
            opts = pirgpu.make_opts()
            stats = pirgpu.Stats()
            rc = L.pir_fixpoint_static(d[0], d[1], d[2], d[3], len(op), d_store, len(lb0),
                                       ctypes.byref(opts), ctypes.byref(stats), None)
            out = mem.download(d_store, store)
            assert rc == rc_ref == pirgpu.OK
            assert stats.status == pirgpu.OK and stats.rounds >= 2
            assert stats.executions == stats.rounds * len(op)
            np.testing.assert_array_equal(out[:, 0], lb_ref)
            np.testing.assert_array_equal(out[:, 1], ub_ref)
            ctx.close()
    finally:
        mem.free()
