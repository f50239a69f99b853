"""pir_fixpoint_static: the fixpoint entry point that allocates no device memory.

It serves callers that own every byte of device memory themselves (a solver
handing the engine slices of its own pool, or a search loop on many streams
that cannot afford cudaMalloc / cudaFree and the device-wide synchronization
they may cause).  Here the test plays such a caller: it allocates the bytecode
and store buffers itself, calls the entry point through the C ABI on two
different instances in a row (the second call must not see anything left in
the shared scratch by the first), and checks each result bit for bit against
the context entry point pir_fixpoint.  The other tests take each documented
status path through this entry point (invalid bytecode or launch shape, an
empty store before and after propagation, the round cap, the barrier time
limit), check that a valid call after each of them is still right, and that a
call leaves the device's free memory unchanged."""
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

    def free_bytes(self):
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        assert self.L.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
        return free.value


def _installed(inst):
    """The engine's installed form of an instance (bytecode in engine order,
    store after the install meets) and its fixpoint through pir_fixpoint."""
    import pirgpu
    ctx = pirgpu.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    lb0, ub0 = ctx.read_store()
    op, x, y, z = ctx.bytecode()
    rc, st = ctx.fixpoint(mode=pirgpu.MODE_PERSISTENT)
    lb, ub = ctx.read_store()
    ctx.close()
    return (op, x, y, z), np.ascontiguousarray(np.stack([lb0, ub0], 1).astype(np.int32)), rc, st, lb, ub


def _call(mem, code, store, **opts):
    """Uploads the bytecode and the store, calls pir_fixpoint_static on the
    default stream, returns (status, stats, the store after the call)."""
    import pirgpu
    L = pirgpu.lib()
    d = [mem.upload(np.ascontiguousarray(a, np.int32)) for a in code]
    d_store = mem.upload(store)
    o = pirgpu.make_opts(**opts)
    stats = pirgpu.Stats()
    rc = L.pir_fixpoint_static(d[0], d[1], d[2], d[3], len(code[0]), d_store, store.shape[0],
                               ctypes.byref(o), ctypes.byref(stats), None)
    return rc, stats, mem.download(d_store, store)


@pytest.fixture(scope="module")
def mem():
    m = _DeviceBuffers()
    yield m
    m.free()


@pytest.fixture(scope="module")
def plain_case():
    import workloads as W
    return _installed(W.plain(20_000, 80_000, 10**6, 12))


def _still_right(mem, plain_case):
    code, store, rc_ref, _, lb_ref, ub_ref = plain_case
    rc, stats, out = _call(mem, code, store)
    assert rc == rc_ref == 0 and stats.status == 0
    np.testing.assert_array_equal(out[:, 0], lb_ref)
    np.testing.assert_array_equal(out[:, 1], ub_ref)


@pytest.mark.parametrize("what", ["opcode", "negative_opcode", "var_x", "var_z"])
def test_static_rejects_bad_bytecode(mem, plain_case, what):
    """PIR_EINVAL, found on the device before propagating, with the store untouched."""
    import pirgpu
    code, store = [a.copy() for a in plain_case[0]], plain_case[1]
    j = len(code[0]) // 2
    if what == "opcode":
        code[0][j] = 10
    elif what == "negative_opcode":
        code[0][j] = -1
    elif what == "var_x":
        code[1][j] = store.shape[0]
    else:
        code[3][j] = -5
    rc, stats, out = _call(mem, code, store)
    assert rc == pirgpu.EINVAL
    np.testing.assert_array_equal(out, store)
    _still_right(mem, plain_case)


def test_static_rejects_grid_beyond_slots(mem, plain_case):
    """ctas_per_sm beyond what fits an SM or the 1,024 scratch slots: PIR_EINVAL."""
    import pirgpu
    code, store = plain_case[0], plain_case[1]
    rc, _, out = _call(mem, code, store, ctas_per_sm=64)
    assert rc == pirgpu.EINVAL
    np.testing.assert_array_equal(out, store)
    _still_right(mem, plain_case)


def test_static_failed_before_propagation(mem, plain_case):
    """A store that is already empty: PIR_FAILED without propagating."""
    import pirgpu
    code, store = plain_case[0], plain_case[1].copy()
    store[7] = (5, 4)
    rc, stats, out = _call(mem, code, store)
    assert rc == pirgpu.FAILED and stats.status == pirgpu.FAILED and stats.rounds == 0
    np.testing.assert_array_equal(out, store)
    _still_right(mem, plain_case)


def test_static_failed_by_propagation(mem, plain_case):
    """x = y + z with x = [10, 10], y, z in [0, 1]: the first round empties x."""
    import pirgpu
    code = (np.array([pirgpu.ADD], np.int32), np.array([0], np.int32), np.array([1], np.int32),
            np.array([2], np.int32))
    store = np.array([[10, 10], [0, 1], [0, 1]], np.int32)
    rc, stats, _ = _call(mem, code, store)
    assert rc == pirgpu.FAILED and stats.status == pirgpu.FAILED and stats.rounds >= 1
    _still_right(mem, plain_case)


def test_static_round_cap(mem, plain_case):
    """A 200-link chain needs far more than 3 rounds: PIR_TIMEOUT after exactly 3."""
    import pirgpu
    import workloads as W
    code, store, rc_ref, st_ref, _, _ = _installed(W.add_chain(W.plain(2_000, 8_000, 1000, 4), 200, 10**4, 4))
    assert rc_ref == pirgpu.OK and st_ref["rounds"] > 10
    rc, stats, _ = _call(mem, code, store, max_rounds=3)
    assert rc == pirgpu.TIMEOUT and stats.status == pirgpu.TIMEOUT and stats.rounds == 3
    _still_right(mem, plain_case)


def test_static_barrier_time_limit(mem, plain_case):
    """A 1 ns limit on each grid-barrier wait: the kernel's bounded waits give
    up, every CTA leaves, and the call returns PIR_BARRIER_TIMEOUT."""
    import pirgpu
    code, store = plain_case[0], plain_case[1]
    rc, stats, _ = _call(mem, code, store, barrier_timeout_ns=1)
    assert rc == pirgpu.BARRIER_TIMEOUT and stats.status == pirgpu.BARRIER_TIMEOUT
    _still_right(mem, plain_case)


def test_static_allocates_nothing(mem, plain_case):
    """Device free memory is the same before and after a call (the first call
    on the device, which may load the module, has already run), and the
    narrowing count covers every bound the fixpoint moved."""
    import pirgpu
    code, store, _, _, lb_ref, ub_ref = plain_case
    L = pirgpu.lib()
    d = [mem.upload(np.ascontiguousarray(a, np.int32)) for a in code]
    d_store = mem.upload(store)
    o = pirgpu.make_opts()
    stats = pirgpu.Stats()
    assert L.pir_fixpoint_static(d[0], d[1], d[2], d[3], len(code[0]), d_store, store.shape[0],
                                 ctypes.byref(o), ctypes.byref(stats), None) == pirgpu.OK
    d_store2 = mem.upload(store)
    before = mem.free_bytes()
    assert L.pir_fixpoint_static(d[0], d[1], d[2], d[3], len(code[0]), d_store2, store.shape[0],
                                 ctypes.byref(o), ctypes.byref(stats), None) == pirgpu.OK
    after = mem.free_bytes()
    assert before == after
    out = mem.download(d_store2, store)
    np.testing.assert_array_equal(out[:, 0], lb_ref)
    moved = int((out[:, 0] != store[:, 0]).sum() + (out[:, 1] != store[:, 1]).sum())
    assert moved > 0 and stats.narrowed >= moved


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
