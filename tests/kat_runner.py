"""Runs the known-answer cases of tests/golden/kat_cases.py against an engine.

An engine mirrors the PIR surface used by lala-pc's tests
(tests/pir_test.cpp:31-89): `add_props` (interpret_tell + deduce(tell)),
`embed`, `num_deductions`, `fixpoint` (the Gauss-Seidel driver or the GPU
fixpoint), `read` (operator[]), `ask_all` (ask(i) for every i) and `is_bot`.
"""
import numpy as np

from golden import kat_cases as K


class OracleEngine:
    """The CPU oracle behind the engine interface."""

    def __init__(self, lb, ub):
        from oracle import oracle as O
        self.O = O
        self.store = np.ascontiguousarray(np.stack([lb, ub], 1).astype(np.int32))
        self.props = np.zeros((0, 4), np.int32)
        self.failed = self.O.store_is_bot(self.store)

    def add_props(self, props):
        props = np.asarray(props, np.int32).reshape(-1, 4)
        st, _ = self.O.install(props[:, 0], props[:, 1], props[:, 2], props[:, 3], self.store)
        self.failed |= st == self.O.FAILED
        self.props = np.concatenate([self.props, props])

    def embed(self, v, lb, ub):
        self.store[v, 0] = max(self.store[v, 0], lb)
        self.store[v, 1] = min(self.store[v, 1], ub)
        self.failed |= self.O.store_is_bot(self.store)

    def num_deductions(self):
        return len(self.props)

    def fixpoint(self):
        if self.failed:
            return True
        p = self.props
        _, perm = self.O.install(p[:, 0], p[:, 1], p[:, 2], p[:, 3], self.store.copy())
        q = p[perm]
        st, info = self.O.fixpoint(q[:, 0], q[:, 1], q[:, 2], q[:, 3], self.store)
        self.info = info
        self.failed = st == self.O.FAILED
        return self.failed

    def read(self):
        return self.store.copy()

    def is_bot(self):
        return self.failed

    def ask_all(self):
        p = self.props
        return self.O.ask_all(p[:, 0], p[:, 1], p[:, 2], p[:, 3], self.store)


def _props_idx(m, props):
    return [[op, m.index[x], m.index[y], m.index[z]] for op, x, y, z in props]


def run_case(case, make_engine):
    """Returns a list of mismatch descriptions (empty when the case passes)."""
    errors = []
    m = K.build_case(case)
    eng = make_engine(np.array(m.lb, np.int64), np.array(m.ub, np.int64))
    eng.add_props(_props_idx(m, m.props))
    for si, step in enumerate(case.steps):
        for v, lb, ub in step.bounds:
            eng.embed(m.index[v], lb, ub)
        if step.props:
            eng.add_props(_props_idx(m, step.props))
        tag = "%s step %d" % (case.name, si)
        if eng.num_deductions() != step.num:
            errors.append("%s: num_deductions %d != %d" % (tag, eng.num_deductions(), step.num))
        s = eng.read()
        for i, (lb, ub) in enumerate(step.before):
            if (s[i, 0], s[i, 1]) != (lb, ub):
                errors.append("%s: before var %d = %s, expected %s"
                              % (tag, i, tuple(s[i]), (lb, ub)))
        failed = eng.fixpoint()
        if step.bot:
            if not failed:
                errors.append("%s: expected failure" % tag)
            continue
        if failed:
            errors.append("%s: unexpected failure" % tag)
            continue
        s = eng.read()
        for i, (lb, ub) in enumerate(step.after):
            if (s[i, 0], s[i, 1]) != (lb, ub):
                errors.append("%s: after var %d (%s) = %s, expected %s"
                              % (tag, i, m.names[i], tuple(s[i]), (lb, ub)))
        ua = (not eng.is_bot()) and bool(np.all(eng.ask_all()))
        if ua != step.ua:
            errors.append("%s: extractable %s, expected %s" % (tag, ua, step.ua))
    return errors


class GpuEngine:
    """The CUDA engine through the C ABI behind the engine interface."""

    mode = 0  # pirgpu.MODE_AUTO; set per test
    sched = 0  # pirgpu.SCHED_AC1; set per test
    opts = {}  # further fixpoint options, set per test

    def __init__(self, lb, ub):
        import pirgpu
        self.P = pirgpu
        self.ctx = pirgpu.Context(0)
        self.ctx.load_store(np.asarray(lb, np.int64).astype(np.int32),
                            np.asarray(ub, np.int64).astype(np.int32))

    def add_props(self, props):
        p = np.asarray(props, np.int32).reshape(-1, 4)
        self.ctx.tell(p[:, 0], p[:, 1], p[:, 2], p[:, 3])

    def embed(self, v, lb, ub):
        self.ctx.embed(v, lb, ub)

    def num_deductions(self):
        return self.ctx.num_deductions()

    def fixpoint(self):
        rc, _ = self.ctx.fixpoint(mode=self.mode, sched=self.sched, **self.opts)
        return rc == self.P.FAILED

    def read(self):
        lb, ub = self.ctx.read_store()
        return np.stack([lb, ub], 1)

    def is_bot(self):
        return self.ctx.is_bot()

    def ask_all(self):
        return self.ctx.ask_all()
