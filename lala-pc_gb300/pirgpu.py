"""Python binding of the pirgpu C ABI (include/pirgpu.h) via ctypes.

`Context` mirrors the PIR abstract-domain surface of lala-pc
(include/lala/pir.hpp): tell / deduce / ask / embed / snapshot / restore,
plus the batched entry points.  Arrays are numpy int32.  The shared library
must have been built (lala-pc_gb300/build.py); importing this module never
falls back to anything else: a missing library raises ImportError.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpirgpu.so")

ADD, MUL, TDIV, FDIV, CDIV, EDIV, MIN, MAX, EQ, LEQ = range(10)
OK, FAILED, TIMEOUT, BARRIER_TIMEOUT, EINVAL, ECUDA, ENOMEM = range(7)
STATUS = ["OK", "FAILED", "TIMEOUT", "BARRIER_TIMEOUT", "EINVAL", "ECUDA", "ENOMEM"]
MODE_AUTO, MODE_PERSISTENT, MODE_HOSTLOOP, MODE_SMEM = range(4)
SCHED_AC1, SCHED_LEARNED, SCHED_EVENTS = range(3)
PERSISTENT_VARIANTS = 10  # PIR_PERSISTENT_VARIANTS
NODE_VARIANTS = 10  # PIR_NODE_VARIANTS
INF = 2**31 - 1
MINF = -2**31


class PirError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS[code] if 0 <= code < len(STATUS) else code, msg))
        self.code = code


class Opts(ctypes.Structure):
    _fields_ = [("max_rounds", ctypes.c_int64), ("barrier_timeout_ns", ctypes.c_int64),
                ("mode", ctypes.c_int32), ("block", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("sched", ctypes.c_int32),
                ("wake_fraction", ctypes.c_float), ("variant", ctypes.c_int32),
                ("local_frontier", ctypes.c_int32), ("chase", ctypes.c_int32),
                ("certify", ctypes.c_int32), ("segments", ctypes.c_int32), ("dense", ctypes.c_int32),
                ("lead", ctypes.c_int32)]


class SearchOpts(ctypes.Structure):
    _fields_ = [("max_nodes", ctypes.c_int64), ("max_solutions", ctypes.c_int64),
                ("batch", ctypes.c_int32), ("order", ctypes.c_int32), ("reserved", ctypes.c_int32 * 6)]


class SearchStats(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_int64), ("failures", ctypes.c_int64), ("solutions", ctypes.c_int64),
                ("launches", ctypes.c_int64), ("max_depth", ctypes.c_int64), ("device_ms", ctypes.c_float),
                ("status", ctypes.c_int32), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


ORDER_INPUT, ORDER_MIN_DOMAIN = range(2)


class Stats(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_int64), ("executions", ctypes.c_int64),
                ("narrowed", ctypes.c_int64), ("device_ms", ctypes.c_float),
                ("status", ctypes.c_int32), ("certify_executions", ctypes.c_int64),
                ("certify_narrowed", ctypes.c_int64)]

    def asdict(self):
        return dict(rounds=self.rounds, executions=self.executions, narrowed=self.narrowed,
                    device_ms=self.device_ms, status=self.status,
                    certify_executions=self.certify_executions, certify_narrowed=self.certify_narrowed)


_lib = None
_P = ctypes.c_void_p
_I32P = ctypes.POINTER(ctypes.c_int32)
_I64P = ctypes.POINTER(ctypes.c_int64)
_U8P = ctypes.POINTER(ctypes.c_uint8)
_F32P = ctypes.POINTER(ctypes.c_float)

# (name, restype, argtypes) of every entry point of include/pirgpu.h
SIGNATURES = [
    ("pir_ctx_create", ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int]),
    ("pir_ctx_destroy", None, [_P]),
    ("pir_last_error", ctypes.c_char_p, [_P]),
    ("pir_load_store", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P]),
    ("pir_read_store", ctypes.c_int, [_P, _I32P, _I32P]),
    ("pir_project", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P]),
    ("pir_embed", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                 ctypes.POINTER(ctypes.c_int)]),
    ("pir_embed_many", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P,
                                      ctypes.POINTER(ctypes.c_int)]),
    ("pir_tell", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P,
                                ctypes.POINTER(ctypes.c_int)]),
    ("pir_num_deductions", ctypes.c_int64, [_P]),
    ("pir_vars", ctypes.c_int32, [_P]),
    ("pir_get_bytecode", ctypes.c_int, [_P, _I32P, _I32P, _I32P, _I32P]),
    ("pir_fixpoint", ctypes.c_int, [_P, ctypes.POINTER(Opts), ctypes.POINTER(Stats)]),
    ("pir_autotune", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _F32P]),
    ("pir_deduce_one", ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    ("pir_ask", ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    ("pir_ask_all", ctypes.c_int, [_P, _U8P]),
    ("pir_ask_bytecodes", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, _U8P]),
    ("pir_is_bot", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    ("pir_is_top", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    ("pir_is_extractable", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    ("pir_snapshot", ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    ("pir_restore", ctypes.c_int, [_P, _P]),
    ("pir_snapshot_free", None, [_P]),
    ("pir_deduce_batch", ctypes.c_int, [_P, ctypes.c_int64, _I32P, _I32P, _I32P, _I32P, _I32P,
                                        _U8P, _U8P]),
    ("pir_fixpoint_nodes", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P,
                                          ctypes.POINTER(Opts), _I32P, _I32P, _I32P, _I32P,
                                          ctypes.POINTER(Stats)]),
    ("pir_sched_score", ctypes.c_int, [_P, ctypes.c_int32, _F32P, _F32P]),
    ("pir_autotune_nodes", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, _I32P, _F32P]),
    ("pir_fixpoint_nodes_watch", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P,
                                                ctypes.POINTER(Opts), ctypes.c_int32, _I32P, _I32P, _I32P,
                                                _I32P, _I32P, ctypes.POINTER(Stats)]),
    ("pir_search", ctypes.c_int, [_P, ctypes.c_int32, _I32P, ctypes.POINTER(SearchOpts), _I32P,
                                  ctypes.POINTER(SearchStats)]),
    ("pir_nodes_stage", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.POINTER(_I32P)]),
    ("pir_fixpoint_nodes_staged", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                 ctypes.POINTER(Opts), _I32P, _I32P, _I32P, _I32P,
                                                 ctypes.POINTER(Stats)]),
    ("pir_fixpoint_instances", ctypes.c_int, [_P, ctypes.c_int32, _I64P, _I64P, _I32P, _I32P,
                                              _I32P, _I32P, _I32P, _I32P, ctypes.POINTER(Opts),
                                              _I32P, _I32P, _F32P, ctypes.POINTER(Stats)]),
    ("pir_device_info", ctypes.c_int, [_P, _I32P, ctypes.c_char_p, ctypes.c_size_t]),
    ("pir_sched_collect", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P,
                                         ctypes.c_int64, ctypes.c_float, _I64P, _I64P]),
    ("pir_sched_train", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                       ctypes.c_float, _F32P]),
    ("pir_sched_grad", ctypes.c_int, [_P, ctypes.c_int32, _F32P, _F32P, ctypes.c_float, _F32P,
                                      _F32P]),
    ("pir_sched_params", ctypes.c_int, [_P, _F32P, ctypes.c_int32, ctypes.c_int32]),
    ("pir_fixpoint_static", ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int64, _P, ctypes.c_int32,
                                           ctypes.POINTER(Opts), ctypes.POINTER(Stats), _P]),
    ("pc_tell", ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32, _I32P]),
    ("pc_num_deductions", ctypes.c_int64, [_P]),
    ("pc_get_roots", ctypes.c_int, [_P, _I32P]),
    ("pc_tape_size", ctypes.c_int64, [_P]),
    ("pc_get_tape", ctypes.c_int, [_P, _I32P, _I32P, _I32P, _I32P]),
    ("pc_fixpoint", ctypes.c_int, [_P, ctypes.POINTER(Opts), ctypes.POINTER(Stats)]),
    ("pc_deduce_one", ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    ("pc_ask", ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    ("pc_ask_all", ctypes.c_int, [_P, _U8P]),
    ("pc_is_extractable", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
]


def lib():
    """Loads libpirgpu.so (raises ImportError when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libpirgpu.so is not built (%s); run lala-pc_gb300/build.py" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p32(a):
    return a.ctypes.data_as(_I32P)


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def make_opts(mode=MODE_AUTO, max_rounds=0, barrier_timeout_ns=0, block=0, ctas_per_sm=0,
              sched=SCHED_AC1, wake_fraction=0.0, variant=0, local_frontier=0, chase=0, certify=0, segments=0, dense=0,
              lead=0):
    o = Opts()
    o.max_rounds, o.barrier_timeout_ns, o.mode, o.block = max_rounds, barrier_timeout_ns, mode, block
    o.ctas_per_sm, o.sched, o.wake_fraction, o.variant = ctas_per_sm, sched, wake_fraction, variant
    o.local_frontier, o.chase, o.certify, o.segments, o.dense = local_frontier, chase, certify, segments, dense
    o.lead = lead
    return o


class Context:
    """One PIR (store + bytecode) on one GPU."""

    def __init__(self, device=0):
        self._L = lib()
        h = _P()
        rc = self._L.pir_ctx_create(ctypes.byref(h), device)
        if rc != OK:
            raise PirError(rc, "pir_ctx_create(device=%d) failed" % device)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._L.pir_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, allowed=(OK,)):
        if rc not in allowed:
            raise PirError(rc, self._L.pir_last_error(self.h).decode())
        return rc

    # -- store ---------------------------------------------------------
    def load_store(self, lb, ub):
        lb, ub = _c32(lb), _c32(ub)
        assert lb.shape == ub.shape
        self._check(self._L.pir_load_store(self.h, len(lb), _p32(lb), _p32(ub)))

    def read_store(self):
        n = self.vars()
        lb = np.empty(n, np.int32)
        ub = np.empty(n, np.int32)
        self._check(self._L.pir_read_store(self.h, _p32(lb), _p32(ub)))
        return lb, ub

    def project(self, v):
        l, u = ctypes.c_int32(), ctypes.c_int32()
        self._check(self._L.pir_project(self.h, v, ctypes.byref(l), ctypes.byref(u)))
        return l.value, u.value

    def embed(self, v, lb, ub):
        ch = ctypes.c_int(0)
        self._check(self._L.pir_embed(self.h, v, lb, ub, ctypes.byref(ch)))
        return bool(ch.value)

    def embed_many(self, var, lb, ub):
        var, lb, ub = map(_c32, (var, lb, ub))
        ch = ctypes.c_int(0)
        self._check(self._L.pir_embed_many(self.h, len(var), _p32(var), _p32(lb), _p32(ub),
                                           ctypes.byref(ch)))
        return bool(ch.value)

    def vars(self):
        return self._L.pir_vars(self.h)

    # -- bytecode ------------------------------------------------------
    def tell(self, op, x, y, z):
        op, x, y, z = map(_c32, (op, x, y, z))
        ch = ctypes.c_int(0)
        self._check(self._L.pir_tell(self.h, len(op), _p32(op), _p32(x), _p32(y), _p32(z),
                                     ctypes.byref(ch)))
        return bool(ch.value)

    def num_deductions(self):
        return self._L.pir_num_deductions(self.h)

    def bytecode(self):
        n = self.num_deductions()
        arrs = [np.empty(n, np.int32) for _ in range(4)]
        self._check(self._L.pir_get_bytecode(self.h, *map(_p32, arrs)))
        return arrs

    # -- propagation ---------------------------------------------------
    def fixpoint(self, **kw):
        o = make_opts(**kw)
        s = Stats()
        rc = self._L.pir_fixpoint(self.h, ctypes.byref(o), ctypes.byref(s))
        self._check(rc, (OK, FAILED, TIMEOUT, BARRIER_TIMEOUT))
        return rc, s.asdict()

    def autotune(self, rounds=64):
        """Times the persistent-kernel variants; returns (variant, us per round)."""
        v = ctypes.c_int32(0)
        us = ctypes.c_float(0)
        self._check(self._L.pir_autotune(self.h, rounds, ctypes.byref(v), ctypes.byref(us)))
        return v.value, us.value

    def deduce_one(self, i):
        ch = ctypes.c_int(0)
        self._check(self._L.pir_deduce_one(self.h, i, ctypes.byref(ch)))
        return bool(ch.value)

    def ask(self, i):
        e = ctypes.c_int(0)
        self._check(self._L.pir_ask(self.h, i, ctypes.byref(e)))
        return bool(e.value)

    def ask_all(self):
        out = np.zeros(self.num_deductions(), np.uint8)
        self._check(self._L.pir_ask_all(self.h, out.ctypes.data_as(_U8P)))
        return out.astype(bool)

    def ask_bytecodes(self, op, x, y, z):
        """Entailment of the given propagators against the store (ask(ask_type))."""
        op, x, y, z = map(_c32, (op, x, y, z))
        out = np.zeros(len(op), np.uint8)
        self._check(self._L.pir_ask_bytecodes(self.h, len(op), _p32(op), _p32(x), _p32(y), _p32(z),
                                              out.ctypes.data_as(_U8P)))
        return out.astype(bool)

    def _flag(self, fn):
        v = ctypes.c_int(0)
        self._check(fn(self.h, ctypes.byref(v)))
        return bool(v.value)

    def is_bot(self):
        return self._flag(self._L.pir_is_bot)

    def is_top(self):
        return self._flag(self._L.pir_is_top)

    def is_extractable(self):
        return self._flag(self._L.pir_is_extractable)

    def snapshot(self):
        s = _P()
        self._check(self._L.pir_snapshot(self.h, ctypes.byref(s)))
        return Snapshot(self._L, s)

    def restore(self, snap):
        self._check(self._L.pir_restore(self.h, snap.h))

    # -- PC tree propagators (pc.hpp) ----------------------------------
    def pc_tell(self, tape, roots):
        """PC::deduce(tell): appends the formulas of `tape` ((n, 4) int32:
        kind, a, b, c per node; see pc.py) with propagators at `roots`."""
        t = np.ascontiguousarray(np.asarray(tape, np.int32).reshape(-1, 4).T)
        roots = _c32(roots)
        self._check(self._L.pc_tell(self.h, t.shape[1], *(_p32(t[k]) for k in range(4)), len(roots),
                                    _p32(roots)))

    def pc_num_deductions(self):
        return self._L.pc_num_deductions(self.h)

    def pc_roots(self):
        """Root node of every PC propagator, in engine order."""
        out = np.empty(self.pc_num_deductions(), np.int32)
        self._check(self._L.pc_get_roots(self.h, _p32(out)))
        return out

    def pc_tape(self):
        n = self._L.pc_tape_size(self.h)
        cols = [np.empty(n, np.int32) for _ in range(4)]
        self._check(self._L.pc_get_tape(self.h, *map(_p32, cols)))
        return np.stack(cols, axis=1)

    def pc_fixpoint(self, **kw):
        o = make_opts(**kw)
        s = Stats()
        rc = self._L.pc_fixpoint(self.h, ctypes.byref(o), ctypes.byref(s))
        self._check(rc, (OK, FAILED, TIMEOUT, BARRIER_TIMEOUT))
        return rc, s.asdict()

    def pc_deduce_one(self, i):
        ch = ctypes.c_int(0)
        self._check(self._L.pc_deduce_one(self.h, i, ctypes.byref(ch)))
        return bool(ch.value)

    def pc_ask(self, i):
        e = ctypes.c_int(0)
        self._check(self._L.pc_ask(self.h, i, ctypes.byref(e)))
        return bool(e.value)

    def pc_ask_all(self):
        out = np.zeros(self.pc_num_deductions(), np.uint8)
        self._check(self._L.pc_ask_all(self.h, out.ctypes.data_as(_U8P)))
        return out.astype(bool)

    def pc_is_extractable(self):
        return self._flag(self._L.pc_is_extractable)

    # -- batched -------------------------------------------------------
    def deduce_batch(self, op, in_lb, in_ub):
        """deduce(bytecode) of op[k] over the private intervals in_lb/in_ub[k, 0:3]."""
        op = _c32(op)
        in_lb, in_ub = _c32(in_lb).reshape(-1, 3), _c32(in_ub).reshape(-1, 3)
        n = len(op)
        out_lb = np.empty((n, 3), np.int32)
        out_ub = np.empty((n, 3), np.int32)
        ch = np.empty(n, np.uint8)
        f = np.empty(n, np.uint8)
        self._check(self._L.pir_deduce_batch(self.h, n, _p32(op), _p32(in_lb), _p32(in_ub),
                                             _p32(out_lb), _p32(out_ub), ch.ctypes.data_as(_U8P),
                                             f.ctypes.data_as(_U8P)))
        return out_lb, out_ub, ch.astype(bool), f.astype(bool)

    def fixpoint_nodes(self, off, var, lb, ub, want_stores=True, **kw):
        off, var, lb, ub = map(_c32, (off, var, lb, ub))
        nn = len(off) - 1
        nv = self.vars()
        out_lb = np.empty((nn, nv), np.int32) if want_stores else None
        out_ub = np.empty((nn, nv), np.int32) if want_stores else None
        status = np.empty(nn, np.int32)
        rounds = np.empty(nn, np.int32)
        o = make_opts(**kw)
        s = Stats()
        rc = self._L.pir_fixpoint_nodes(self.h, nn, _p32(off), _p32(var), _p32(lb), _p32(ub),
                                        ctypes.byref(o),
                                        _p32(out_lb) if want_stores else None,
                                        _p32(out_ub) if want_stores else None,
                                        _p32(status), _p32(rounds), ctypes.byref(s))
        self._check(rc)
        return status, out_lb, out_ub, rounds, s.asdict()

    def autotune_nodes(self, off, var, lb, ub):
        """Times the event node kernel variants on this batch; returns (variant, ms)."""
        off, var, lb, ub = map(_c32, (off, var, lb, ub))
        v = ctypes.c_int32(0)
        ms = ctypes.c_float(0)
        self._check(self._L.pir_autotune_nodes(self.h, len(off) - 1, _p32(off), _p32(var), _p32(lb), _p32(ub),
                                               ctypes.byref(v), ctypes.byref(ms)))
        return v.value, ms.value

    def sched_score(self, X):
        """Scores of feature rows X (n x 8) by the tensor-core inference MLP."""
        X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
        out = np.empty(len(X), np.float32)
        self._check(self._L.pir_sched_score(self.h, len(X), X.ctypes.data_as(_F32P), out.ctypes.data_as(_F32P)))
        return out

    def fixpoint_nodes_watch(self, off, var, lb, ub, watch, **kw):
        """Per node: status, rounds and the final bounds of the `watch` variables
        (nnodes x nwatch arrays)."""
        off, var, lb, ub, watch = map(_c32, (off, var, lb, ub, watch))
        nn, nw = len(off) - 1, len(watch)
        wl = np.empty((nn, nw), np.int32)
        wu = np.empty((nn, nw), np.int32)
        status = np.empty(nn, np.int32)
        rounds = np.empty(nn, np.int32)
        o = make_opts(**kw)
        s = Stats()
        self._check(self._L.pir_fixpoint_nodes_watch(self.h, nn, _p32(off), _p32(var), _p32(lb), _p32(ub),
                                                     ctypes.byref(o), nw, _p32(watch), _p32(wl), _p32(wu),
                                                     _p32(status), _p32(rounds), ctypes.byref(s)))
        return status, wl, wu, rounds, s.asdict()

    def nodes_stage(self, nnodes, ntight, nwatch):
        """The context's pinned staging of a node batch, as an int32 array:
        watch[nwatch] | off[nnodes + 1] | var | lb | ub (ntight each).  Valid
        until the next nodes_stage call."""
        p = _I32P()
        self._check(self._L.pir_nodes_stage(self.h, nnodes, ntight, nwatch, ctypes.byref(p)))
        return np.ctypeslib.as_array(p, shape=(nwatch + nnodes + 1 + 3 * ntight,))

    def fixpoint_nodes_staged(self, nnodes, ntight, nwatch, **kw):
        """Runs the staged batch as one CUDA graph: (status, watched lb, watched
        ub (nnodes x nwatch), rounds, stats)."""
        status = np.empty(nnodes, np.int32)
        rounds = np.empty(nnodes, np.int32)
        wl = np.empty((nnodes, nwatch), np.int32)
        wu = np.empty((nnodes, nwatch), np.int32)
        o = make_opts(**kw)
        s = Stats()
        self._check(self._L.pir_fixpoint_nodes_staged(self.h, nnodes, ntight, nwatch, ctypes.byref(o),
                                                      _p32(status), _p32(rounds), _p32(wl), _p32(wu),
                                                      ctypes.byref(s)))
        return status, wl, wu, rounds, s.asdict()

    def search(self, dec, max_solutions=0, max_nodes=0, batch=0, order=ORDER_INPUT):
        """Depth-first search over the decision variables `dec`: (status, the
        solutions found (rows of decision values; none kept when max_solutions
        is 0), stats)."""
        dec = _c32(dec)
        o = SearchOpts()
        o.max_nodes, o.max_solutions, o.batch, o.order = max_nodes, max_solutions, batch, order
        out = np.empty((max(max_solutions, 1), len(dec)), np.int32)
        s = SearchStats()
        rc = self._L.pir_search(self.h, len(dec), _p32(dec), ctypes.byref(o), _p32(out), ctypes.byref(s))
        self._check(rc, (OK, TIMEOUT))
        st = s.asdict()
        return st["status"], out[:st["solutions"] if max_solutions else 0], st

    def fixpoint_instances(self, prop_off, var_off, op, x, y, z, lb, ub, **kw):
        """lb/ub are updated in place (int32 contiguous arrays)."""
        prop_off = np.ascontiguousarray(prop_off, np.int64)
        var_off = np.ascontiguousarray(var_off, np.int64)
        op, x, y, z = map(_c32, (op, x, y, z))
        assert lb.dtype == np.int32 and ub.dtype == np.int32
        ni = len(prop_off) - 1
        status = np.empty(ni, np.int32)
        rounds = np.empty(ni, np.int32)
        ms = np.empty(ni, np.float32)
        o = make_opts(**kw)
        s = Stats()
        rc = self._L.pir_fixpoint_instances(self.h, ni, prop_off.ctypes.data_as(_I64P),
                                            var_off.ctypes.data_as(_I64P), _p32(op), _p32(x),
                                            _p32(y), _p32(z), _p32(lb), _p32(ub), ctypes.byref(o),
                                            _p32(status), _p32(rounds), ms.ctypes.data_as(_F32P),
                                            ctypes.byref(s))
        self._check(rc)
        return status, rounds, ms, s.asdict()

    # -- learned scheduler ---------------------------------------------
    NPARAM = 1377

    def sched_collect(self, off, var, lb, ub, max_samples=1_000_000, keep_negative=0.05):
        off, var, lb, ub = map(_c32, (off, var, lb, ub))
        ns, npos = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self._L.pir_sched_collect(self.h, len(off) - 1, _p32(off), _p32(var), _p32(lb),
                                              _p32(ub), max_samples, keep_negative,
                                              ctypes.byref(ns), ctypes.byref(npos)))
        return ns.value, npos.value

    def sched_train(self, epochs=8, batch=8192, lr=3e-3, pos_weight=1.0):
        loss = np.zeros(max(epochs, 1), np.float32)
        self._check(self._L.pir_sched_train(self.h, epochs, batch, lr, pos_weight,
                                            loss.ctypes.data_as(_F32P)))
        return loss[:epochs]

    def sched_grad(self, X, Y, pos_weight=1.0):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        g = np.zeros(self.NPARAM, np.float32)
        loss = ctypes.c_float(0)
        self._check(self._L.pir_sched_grad(self.h, len(Y), X.ctypes.data_as(_F32P),
                                           Y.ctypes.data_as(_F32P), pos_weight,
                                           g.ctypes.data_as(_F32P), ctypes.byref(loss)))
        return g, loss.value

    def sched_params(self, params=None):
        if params is None:
            p = np.zeros(self.NPARAM, np.float32)
            self._check(self._L.pir_sched_params(self.h, p.ctypes.data_as(_F32P), self.NPARAM, 0))
            return p
        p = np.ascontiguousarray(params, np.float32)
        self._check(self._L.pir_sched_params(self.h, p.ctypes.data_as(_F32P), self.NPARAM, 1))

    def device_info(self):
        n = ctypes.c_int32()
        name = ctypes.create_string_buffer(128)
        self._check(self._L.pir_device_info(self.h, ctypes.byref(n), name, 128))
        return n.value, name.value.decode()


class Snapshot:
    def __init__(self, L, h):
        self._L, self.h = L, h

    def __del__(self):
        if getattr(self, "h", None):
            self._L.pir_snapshot_free(self.h)
            self.h = None
