"""ctypes binding of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It wraps oracle/_build/liboracle.so (a C++ restatement of
lala-pc include/lala/pir.hpp:326-817 and of the Gauss-Seidel loop of
tests/pir_test.cpp:60-62).  Stores are int32 arrays of shape (nvars, 2):
column 0 = lb, column 1 = ub.
"""
import ctypes
import os

import numpy as np

from . import build as _build

ADD, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, EQ, LEQ = range(10)
OK, FAILED, TIMEOUT, EINVAL = range(4)
PREDS = ["int_eq_reif", "int_le_reif", "int_plus", "int_min", "int_max", "int_times",
         "int_ediv", "int_tdiv", "int_cdiv", "int_fdiv", "int_emod", "int_tmod",
         "int_cmod", "int_fmod"]

_lib = None
_I32P = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        i32, i64 = ctypes.c_int32, ctypes.c_int64
        L.orc_install.argtypes = [i32, _I32P, _I32P, _I32P, _I32P, i32, _I32P, _I32P]
        L.orc_fixpoint.argtypes = [i32, _I32P, _I32P, _I32P, _I32P, i32, _I32P, i64, _I64P]
        L.orc_sweeps.argtypes = [i32, _I32P, _I32P, _I32P, _I32P, _I32P, i64, _I64P]
        L.orc_deduce.argtypes = [i32, i32, i32, i32, _I32P, ctypes.POINTER(ctypes.c_int)]
        L.orc_ask.argtypes = [i32, i32, i32, i32, _I32P]
        _U8P = ctypes.POINTER(ctypes.c_uint8)
        L.orc_search.argtypes = [i32, _I32P, _I32P, _I32P, _I32P, i32, _I32P, i32, _I32P, i32, i64, i64,
                                 _I32P, _I64P]
        L.orc_search.restype = ctypes.c_int
        L.orc_ask_batch.argtypes = [i64, _I32P, _I32P, _I32P, _U8P]
        L.orc_ask_batch.restype = None
        L.orc_deduce_batch.argtypes = [i64, _I32P, _I32P, _I32P, _I32P, _I32P, _U8P, _U8P, _I64P]
        L.orc_deduce_batch.restype = None
        L.orc_store_is_bot.argtypes = [i32, _I32P]
        L.orc_fixpoint_nodes.argtypes = [i32, _I32P, _I32P, _I32P, _I32P, i32, _I32P, i32,
                                         _I32P, _I32P, _I32P, _I32P, i64, i32, _I32P, _I32P,
                                         _I64P]
        L.orc_fixpoint_instances.argtypes = [i32, _I64P, _I64P, _I32P, _I32P, _I32P, _I32P,
                                             _I32P, i64, i32, i32, _I32P, _I64P]
        for f in ("orc_check_exhaustive",):
            getattr(L, f).argtypes = [i32, i32, i32, i32, _I64P]
            getattr(L, f).restype = i64
        L.orc_check_listed.argtypes = [i32, i32, _I64P]
        L.orc_check_listed.restype = i64
        L.orc_check_completeness.argtypes = [i32, i32, _I64P]
        L.orc_check_completeness.restype = i64
        L.orc_build_pred.argtypes = [i32, _I32P, _I32P, _I32P, _I32P, _I32P]
        L.orc_build_pred.restype = i32
        L.orc_div.argtypes = [i32, i64, i64]
        L.orc_div.restype = i64
        L.orc_mod.argtypes = [i32, i64, i64]
        L.orc_mod.restype = i64
        T4 = [_I32P, _I32P, _I32P, _I32P]
        L.orc_pc_validate.argtypes = [i32] + T4 + [i32, _I32P, i32]
        L.orc_pc_validate.restype = i32
        L.orc_pc_order.argtypes = [i32] + T4 + [i32, _I32P, _I32P]
        L.orc_pc_order.restype = None
        L.orc_pc_deduce.argtypes = T4 + [i32, _I32P, _I32P, _I64P]
        L.orc_pc_deduce.restype = i32
        L.orc_pc_ask.argtypes = T4 + [i32, _I32P, i32]
        L.orc_pc_ask.restype = i32
        L.orc_pc_project.argtypes = T4 + [i32, _I32P, _I32P, _I32P]
        L.orc_pc_project.restype = None
        L.orc_pc_embed.argtypes = T4 + [i32, i32, i32, _I32P, _I32P]
        L.orc_pc_embed.restype = i32
        L.orc_pc_fixpoint.argtypes = [i32] + T4 + [i32, _I32P, i32, _I32P, i64, _I64P]
        L.orc_pc_fixpoint.restype = i32
        L.orc_pc_fixpoint_jacobi.argtypes = [i32] + T4 + [i32, _I32P, i32, _I32P, i64, _I64P]
        L.orc_pc_fixpoint_jacobi.restype = i32
        L.orc_pc_itv.argtypes = [i32, i32, i32, i32, i32, _I32P, _I32P]
        L.orc_pc_itv.restype = None
        _lib = L
    return _lib


def _p32(a):
    return a.ctypes.data_as(_I32P)


def _p64(a):
    return a.ctypes.data_as(_I64P)


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def install(op, x, y, z, store):
    """PIR::deduce(tell) (pir.hpp:326-352): meets reified x with [0,1] in
    `store` (in place) and returns (status, perm) with perm the CPU sort."""
    op, x, y, z = map(_c32, (op, x, y, z))
    assert store.dtype == np.int32 and store.flags.c_contiguous
    perm = np.empty(len(op), np.int32)
    st = lib().orc_install(len(op), _p32(op), _p32(x), _p32(y), _p32(z), store.shape[0],
                           _p32(store), _p32(perm))
    return st, perm


def fixpoint(op, x, y, z, store, max_sweeps=1 << 40):
    """Gauss-Seidel fixpoint in the given order; `store` (nvars, 2) is updated
    in place.  Returns (status, dict(sweeps, execs, narrowed, overflows))."""
    op, x, y, z = map(_c32, (op, x, y, z))
    assert store.dtype == np.int32 and store.flags.c_contiguous
    out = np.zeros(4, np.int64)
    st = lib().orc_fixpoint(len(op), _p32(op), _p32(x), _p32(y), _p32(z), store.shape[0],
                            _p32(store), max_sweeps, _p64(out))
    return st, dict(sweeps=int(out[0]), execs=int(out[1]), narrowed=int(out[2]),
                    overflows=int(out[3]))


def sweeps(op, x, y, z, store, count):
    """Exactly `count` Gauss-Seidel sweeps (a bounded sample for timing)."""
    op, x, y, z = map(_c32, (op, x, y, z))
    out = np.zeros(4, np.int64)
    st = lib().orc_sweeps(len(op), _p32(op), _p32(x), _p32(y), _p32(z), _p32(store), count,
                          _p64(out))
    return st, dict(sweeps=int(out[0]), execs=int(out[1]), narrowed=int(out[2]),
                    overflows=int(out[3]))


def install_and_fixpoint(op, x, y, z, store, max_sweeps=1 << 40):
    """Reference order of events: install (meet + CPU sort), then the
    Gauss-Seidel fixpoint over the sorted bytecode."""
    st, perm = install(op, x, y, z, store)
    if st == EINVAL:
        return st, None
    if st == FAILED:
        return FAILED, dict(sweeps=0, execs=0, narrowed=0, overflows=0)
    op, x, y, z = (np.asarray(a, np.int32)[perm] for a in (op, x, y, z))
    return fixpoint(op, x, y, z, store, max_sweeps)


def fixpoint_nodes(op, x, y, z, base_store, off, var, lb, ub, max_sweeps=1 << 40, threads=0):
    """One store per node: base + tightenings, then Gauss-Seidel (host threads)."""
    op, x, y, z, off, var, lb, ub = map(_c32, (op, x, y, z, off, var, lb, ub))
    base_store = _c32(base_store)
    nnodes = len(off) - 1
    nvars = base_store.shape[0]
    out_store = np.empty((nnodes, nvars, 2), np.int32)
    out_status = np.empty(nnodes, np.int32)
    out_stats = np.zeros((nnodes, 4), np.int64)
    lib().orc_fixpoint_nodes(len(op), _p32(op), _p32(x), _p32(y), _p32(z), nvars,
                             _p32(base_store), nnodes, _p32(off), _p32(var), _p32(lb),
                             _p32(ub), max_sweeps, threads, _p32(out_store), _p32(out_status),
                             _p64(out_stats))
    return out_status, out_store, out_stats


def fixpoint_instances(prop_off, var_off, op, x, y, z, store, max_sweeps=1 << 40, threads=0,
                       install=True):
    """Independent instances packed back to back; `store` updated in place.
    With install=True each instance is installed (reified meets, CPU sort) first."""
    prop_off = np.ascontiguousarray(prop_off, np.int64)
    var_off = np.ascontiguousarray(var_off, np.int64)
    op, x, y, z = map(_c32, (op, x, y, z))
    assert store.dtype == np.int32 and store.flags.c_contiguous
    ninst = len(prop_off) - 1
    out_status = np.empty(ninst, np.int32)
    out_stats = np.zeros((ninst, 4), np.int64)
    lib().orc_fixpoint_instances(ninst, _p64(prop_off), _p64(var_off), _p32(op), _p32(x),
                                 _p32(y), _p32(z), _p32(store), max_sweeps, threads,
                                 int(install), _p32(out_status), _p64(out_stats))
    return out_status, out_stats


def deduce(op, x, y, z, store):
    f = ctypes.c_int(0)
    ch = lib().orc_deduce(op, x, y, z, _p32(store), ctypes.byref(f))
    return bool(ch), bool(f.value)


def deduce_batch(op, in_lb, in_ub):
    """deduce(bytecode) of op[k] over private intervals in_lb/in_ub[k, 0:3]."""
    op = _c32(op)
    in_lb, in_ub = _c32(in_lb).reshape(-1, 3), _c32(in_ub).reshape(-1, 3)
    n = len(op)
    out_lb = np.empty((n, 3), np.int32)
    out_ub = np.empty((n, 3), np.int32)
    ch = np.empty(n, np.uint8)
    f = np.empty(n, np.uint8)
    ovf = np.zeros(1, np.int64)
    u8 = ctypes.POINTER(ctypes.c_uint8)
    lib().orc_deduce_batch(n, _p32(op), _p32(in_lb), _p32(in_ub), _p32(out_lb), _p32(out_ub),
                           ch.ctypes.data_as(u8), f.ctypes.data_as(u8), _p64(ovf))
    return out_lb, out_ub, ch.astype(bool), f.astype(bool), int(ovf[0])


def ask(op, x, y, z, store):
    return bool(lib().orc_ask(op, x, y, z, _p32(store)))


def search(op, x, y, z, store, dec, order=0, max_solutions=0, max_nodes=0):
    """Depth-first search from `store` (installed bytecode): (status,
    solutions (rows of decision values, up to max_solutions), dict(nodes,
    failures, solutions))."""
    op, x, y, z, dec = map(_c32, (op, x, y, z, dec))
    store = _c32(store)
    out = np.zeros((max(max_solutions, 1), len(dec)), np.int32)
    st = np.zeros(3, np.int64)
    rc = lib().orc_search(len(op), _p32(op), _p32(x), _p32(y), _p32(z), store.shape[0], _p32(store),
                          len(dec), _p32(dec), order, max_solutions, max_nodes, _p32(out), _p64(st))
    k = int(st[2]) if max_solutions else 0
    return rc, out[:k], dict(nodes=int(st[0]), failures=int(st[1]), solutions=int(st[2]))


def ask_batch(op, in_lb, in_ub):
    """ask(bytecode) of op[k] over private intervals in_lb/in_ub[k, 0:3]."""
    op = _c32(op)
    in_lb, in_ub = _c32(in_lb).reshape(-1, 3), _c32(in_ub).reshape(-1, 3)
    out = np.empty(len(op), np.uint8)
    lib().orc_ask_batch(len(op), _p32(op), _p32(in_lb), _p32(in_ub),
                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return out.astype(bool)


def ask_all(op, x, y, z, store):
    return np.array([ask(int(a), int(b), int(c), int(d), store)
                     for a, b, c, d in zip(op, x, y, z)], dtype=bool)


def store_is_bot(store):
    return bool(lib().orc_store_is_bot(store.shape[0], _p32(_c32(store))))


def check_exhaustive(pred, minval, maxval, completeness):
    out = np.zeros(2, np.int64)
    bad = lib().orc_check_exhaustive(pred, minval, maxval, int(completeness), _p64(out))
    return int(bad), int(out[0]), int(out[1])


def check_listed(pred, completeness):
    out = np.zeros(2, np.int64)
    bad = lib().orc_check_listed(pred, int(completeness), _p64(out))
    return int(bad), int(out[0]), int(out[1])


def check_completeness(pred, with_fixpoint):
    out = np.zeros(2, np.int64)
    bad = lib().orc_check_completeness(pred, int(with_fixpoint), _p64(out))
    return int(bad), int(out[0]), int(out[1])


def build_pred(pred):
    a = [np.zeros(4, np.int32) for _ in range(4)]
    nv = np.zeros(1, np.int32)
    n = lib().orc_build_pred(pred, *(_p32(t) for t in a), _p32(nv))
    return [t[:n].copy() for t in a], int(nv[0])


def div(op, a, b):
    return int(lib().orc_div(op, a, b))


def mod(kind, a, b):
    return int(lib().orc_mod(kind, a, b))


# --------------------------------------------------------------------- PC --
# Tapes are int32 arrays of shape (nnodes, 4): kind, a, b, c per node (the
# node kinds of oracle/pc_oracle.h); a propagator is its root node's index.

def _tape_cols(tape):
    t = np.ascontiguousarray(np.asarray(tape, np.int32).reshape(-1, 4).T)
    return t, [_p32(t[k]) for k in range(4)]


def pc_validate(tape, roots, nvars):
    """Depth of the deepest root (>= 1), or a negative error code."""
    t, cols = _tape_cols(tape)
    roots = _c32(roots)
    return int(lib().orc_pc_validate(t.shape[1], *cols, len(roots), _p32(roots), nvars))


def pc_order(tape, roots):
    """PC::deduce(tell)'s order: roots stably sorted by (kind, length)."""
    t, cols = _tape_cols(tape)
    roots = _c32(roots)
    out = np.empty(len(roots), np.int32)
    lib().orc_pc_order(t.shape[1], *cols, len(roots), _p32(roots), _p32(out))
    return out


def pc_fixpoint(tape, roots, store, max_sweeps=1 << 40):
    """Gauss-Seidel fixpoint of the PC propagators in roots[] order; `store`
    (nvars, 2) int32 is updated in place.  Returns (status, stats dict)."""
    t, cols = _tape_cols(tape)
    roots = _c32(roots)
    assert store.dtype == np.int32 and store.flags.c_contiguous
    out = np.zeros(4, np.int64)
    st = lib().orc_pc_fixpoint(t.shape[1], *cols, len(roots), _p32(roots), store.shape[0], _p32(store),
                               max_sweeps, _p64(out))
    return st, dict(sweeps=int(out[0]), execs=int(out[1]), narrowed=int(out[2]), has_changed=bool(out[3]))


def pc_fixpoint_jacobi(tape, roots, store, max_rounds=1 << 40):
    """The GPU engine's schedule on the CPU: Jacobi rounds (every deduction of
    a round reads the round's initial store).  Returns (status, stats)."""
    t, cols = _tape_cols(tape)
    roots = _c32(roots)
    assert store.dtype == np.int32 and store.flags.c_contiguous
    out = np.zeros(4, np.int64)
    st = lib().orc_pc_fixpoint_jacobi(t.shape[1], *cols, len(roots), _p32(roots), store.shape[0], _p32(store),
                                      max_rounds, _p64(out))
    return st, dict(rounds=int(out[0]), execs=int(out[1]), narrowed=int(out[2]))


def pc_deduce(tape, root, store, failed=False):
    """One deduce of the formula at `root`: (has_changed, failed)."""
    t, cols = _tape_cols(tape)
    f = np.array([int(failed)], np.int32)
    nar = np.zeros(1, np.int64)
    ch = lib().orc_pc_deduce(*cols, int(root), _p32(store), _p32(f), _p64(nar))
    return bool(ch), bool(f[0])


def pc_ask(tape, root, store, failed=False):
    t, cols = _tape_cols(tape)
    return bool(lib().orc_pc_ask(*cols, int(root), _p32(_c32(store)), int(failed)))


def pc_project(tape, node, store):
    t, cols = _tape_cols(tape)
    lo = np.zeros(1, np.int32)
    hi = np.zeros(1, np.int32)
    lib().orc_pc_project(*cols, int(node), _p32(_c32(store)), _p32(lo), _p32(hi))
    return int(lo[0]), int(hi[0])


def pc_embed(tape, node, lb, ub, store):
    t, cols = _tape_cols(tape)
    f = np.zeros(1, np.int32)
    ch = lib().orc_pc_embed(*cols, int(node), int(lb), int(ub), _p32(store), _p32(f))
    return bool(ch), bool(f[0])


def pc_itv(op, a, b=(0, 0)):
    lo = np.zeros(1, np.int32)
    hi = np.zeros(1, np.int32)
    lib().orc_pc_itv(op, a[0], a[1], b[0], b[1], _p32(lo), _p32(hi))
    return int(lo[0]), int(hi[0])
