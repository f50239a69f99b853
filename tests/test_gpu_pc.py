"""PC tree propagators on the GPU (lala-pc_gb300/csrc/pir_pc.cu) through the C
ABI: the known answers of lala-pc's PC tests, bit-exact parity with the oracle
run in the engine's schedule (Jacobi rounds) on seeded random formula sets --
monotone ones, where every schedule meets, and order-dependent ones alike --
deduce(i) / ask(i) against the reference's sequential semantics, snapshot /
restore, the depth limit and the argument checks."""
import numpy as np
import pytest

import pc as P
import pc_harness as H
import pirgpu
from golden import pc_kat_cases as K

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def make_fzn(tmp_path_factory):
    return H.compile_shim(tmp_path_factory.mktemp("pcfzn_gpu"))


@pytest.mark.parametrize("case", K.CASES, ids=[c[0] for c in K.CASES])
def test_kat_gpu(case, make_fzn, gpu_ctx_factory):
    assert H.run_case(make_fzn, H.GpuModel(gpu_ctx_factory), case) == []


def _ctx(gpu_ctx_factory, tape, roots, store):
    ctx = gpu_ctx_factory()
    ctx.load_store(store[:, 0], store[:, 1])
    ctx.pc_tell(tape, roots)
    return ctx


def _gpu_vs_oracle(ctx, oracle, tape, store, **kw):
    roots = ctx.pc_roots()
    ref = store.copy()
    rc_o, info = oracle.pc_fixpoint_jacobi(ctx.pc_tape(), roots, ref)
    rc, st = ctx.pc_fixpoint(**kw)
    assert rc == rc_o
    if rc == pirgpu.OK:
        lb, ub = ctx.read_store()
        np.testing.assert_array_equal(np.stack([lb, ub], 1), ref)
        assert st["rounds"] == info["rounds"]
        assert st["narrowed"] == info["narrowed"]
    return rc


@pytest.mark.parametrize("seed", range(24))
def test_random_parity_small(seed, gpu_ctx_factory, oracle):
    rng = np.random.default_rng(seed)
    t, store = H.random_formulas(rng, 60, 40, depth=3, positive_mul=seed % 2 == 0)
    tape, roots = t.arrays()
    _gpu_vs_oracle(_ctx(gpu_ctx_factory, tape, roots, store), oracle, tape, store)


@pytest.mark.parametrize("nvars,nprops,depth", [(2000, 1500, 3), (20000, 12000, 4)])
def test_random_parity_large(nvars, nprops, depth, gpu_ctx_factory, oracle):
    """Larger unconstrained sets (these end FAILED: the status is compared)."""
    for seed in range(2):
        rng = np.random.default_rng(100 + seed)
        t, store = H.random_formulas(rng, nvars, nprops, depth=depth)
        tape, roots = t.arrays()
        _gpu_vs_oracle(_ctx(gpu_ctx_factory, tape, roots, store), oracle, tape, store)


@pytest.mark.parametrize("seed", range(4))
def test_planted_parity(seed, gpu_ctx_factory, oracle):
    """Random formulas a hidden assignment satisfies: the fixpoint is not
    empty, equal bit for bit to the oracle's, and the assignment stays inside."""
    rng = np.random.default_rng(300 + seed)
    t, store, hidden = H.planted_formulas(rng, 2000, 1500, depth=3)
    tape, roots = t.arrays()
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    assert _gpu_vs_oracle(ctx, oracle, tape, store) == pirgpu.OK
    lb, ub = ctx.read_store()
    assert np.all((hidden >= lb) & (hidden <= ub))


@pytest.mark.parametrize("n", [50_000, 200_000])
def test_benchmark_mix_parity(n, gpu_ctx_factory, oracle):
    """The benchmark's formula mix (workloads.pc_mix) at 50k and 200k trees:
    bit-exact with the oracle, planted solution inside the fixpoint."""
    import workloads as W
    tape, roots, lb0, ub0, hidden = W.pc_mix(n, n, seed=2)
    store = np.ascontiguousarray(np.stack([lb0, ub0], 1))
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    assert _gpu_vs_oracle(ctx, oracle, tape, store) == pirgpu.OK
    lb, ub = ctx.read_store()
    assert np.all((hidden >= lb) & (hidden <= ub))


def test_monotone_sets_match_gauss_seidel(gpu_ctx_factory, oracle):
    """Where the reference's Gauss-Seidel loop is order-independent (forward,
    reversed and shuffled orders agree), the engine reaches that fixpoint."""
    checked = 0
    for seed in range(40):
        rng = np.random.default_rng(7000 + seed)
        t, store = H.random_formulas(rng, 60, 40, depth=3)
        tape, roots = t.arrays()
        order = oracle.pc_order(tape, roots)
        outs = set()
        for perm in (order, order[::-1].copy(), rng.permutation(order)):
            s = store.copy()
            rc, _ = oracle.pc_fixpoint(tape, np.ascontiguousarray(perm, np.int32), s)
            outs.add((rc, s.tobytes() if rc == oracle.OK else b""))
        if len(outs) != 1:
            continue
        (rc_gs, s_gs), = outs
        ctx = _ctx(gpu_ctx_factory, tape, roots, store)
        rc, _ = ctx.pc_fixpoint()
        assert rc == rc_gs
        if rc == pirgpu.OK:
            lb, ub = ctx.read_store()
            assert np.stack([lb, ub], 1).astype(np.int32).tobytes() == s_gs
        checked += 1
    assert checked >= 30


def test_deduce_one_and_ask_follow_the_reference(gpu_ctx_factory, oracle):
    """deduce(i) reads its own joins (the reference's sequential semantics)
    and returns its has_changed; ask(i) is Formula::ask."""
    rng = np.random.default_rng(11)
    t, store = H.random_formulas(rng, 50, 30, depth=3)
    tape, roots = t.arrays()
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    order = ctx.pc_roots()
    full = ctx.pc_tape()
    ref = store.copy()
    failed = False
    for i, r in enumerate(order):
        if failed:
            break
        ch_o, failed = oracle.pc_deduce(full, r, ref, failed)
        assert ctx.pc_deduce_one(i) == ch_o
        if not failed:
            lb, ub = ctx.read_store()
            np.testing.assert_array_equal(np.stack([lb, ub], 1), ref)
            assert ctx.is_bot() is False
    if not failed:
        asks = ctx.pc_ask_all()
        assert list(asks) == [oracle.pc_ask(full, r, ref) for r in order]
        assert ctx.pc_is_extractable() == all(asks)


def test_order_is_kind_then_length(gpu_ctx_factory, oracle):
    rng = np.random.default_rng(3)
    t, store = H.random_formulas(rng, 40, 50, depth=3)
    tape, roots = t.arrays()
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    np.testing.assert_array_equal(ctx.pc_roots(), oracle.pc_order(tape, roots))
    np.testing.assert_array_equal(ctx.pc_tape(), tape)


def test_snapshot_restore(gpu_ctx_factory):
    t = P.Tape()
    x, y = t.var(0), t.var(1)
    t.prop(t.leq(t.add(x, y), t.constant(5)))
    tape, roots = t.arrays()
    ctx = gpu_ctx_factory()
    ctx.load_store(np.array([0, 0]), np.array([10, 10]))
    ctx.pc_tell(tape, roots)
    snap = ctx.snapshot()
    t2 = P.Tape()
    t2.prop(t2.gt(t2.var(0), t2.constant(3)))
    ctx.pc_tell(*t2.arrays())
    assert ctx.pc_num_deductions() == 2
    assert ctx.pc_fixpoint()[0] == pirgpu.OK
    assert ctx.project(0) == (4, 5) and ctx.project(1) == (0, 1)
    ctx.restore(snap)
    assert ctx.pc_num_deductions() == 1
    assert ctx.project(0) == (0, 10)
    assert ctx.pc_fixpoint()[0] == pirgpu.OK
    assert ctx.project(0) == (0, 5)


def test_deep_trees(gpu_ctx_factory, oracle):
    """A formula of the maximum depth (the call stack sized for it) and one
    level more (rejected)."""
    def chain(depth):
        t = P.Tape()
        s = t.var(0)
        for k in range(depth - 2):
            s = t.add(s, t.var(1 + k % 7))
        t.prop(t.leq(s, t.constant(40)))
        return t.arrays()
    tape, roots = chain(P.MAX_DEPTH)
    assert oracle.pc_validate(tape, roots, 8) == P.MAX_DEPTH
    store = np.array([[0, 10]] * 8, np.int32)
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    _gpu_vs_oracle(ctx, oracle, tape, store)
    tape, roots = chain(P.MAX_DEPTH + 1)
    ctx = gpu_ctx_factory()
    ctx.load_store(store[:, 0], store[:, 1])
    with pytest.raises(pirgpu.PirError, match="depth"):
        ctx.pc_tell(tape, roots)
    assert ctx.pc_num_deductions() == 0


def test_rejects_bad_tapes(gpu_ctx_factory):
    ctx = gpu_ctx_factory()
    ctx.load_store(np.array([0, 0]), np.array([5, 5]))
    t = P.Tape()
    t.prop(t.leq(t.var(0), t.constant(3)))
    good, roots = t.arrays()
    cases = []
    bad = good.copy(); bad[0, 1] = 2; cases.append((bad, roots))        # variable out of range
    bad = good.copy(); bad[2, 1] = 2; cases.append((bad, roots))        # child not before its parent
    bad = good.copy(); bad[2, 0] = 99; cases.append((bad, roots))       # unknown kind
    bad = good.copy(); bad[2, 3] = 1; cases.append((bad, roots))        # reserved field
    cases.append((good, np.array([0], np.int32)))                      # root is a term
    cases.append((good, np.array([3], np.int32)))                      # root outside the tape
    for tape, r in cases:
        with pytest.raises(pirgpu.PirError):
            ctx.pc_tell(tape, r)
        assert ctx.pc_num_deductions() == 0 and len(ctx.pc_tape()) == 0
    ctx.pc_tell(good, roots)
    assert ctx.pc_num_deductions() == 1
    with pytest.raises(pirgpu.PirError):
        ctx.load_store(np.zeros(0, np.int32), np.zeros(0, np.int32))  # smaller than the variables used


def test_round_cap_and_failure(gpu_ctx_factory):
    # x_{k+1} >= x_k + 1 over a chain: one bound moves per round
    t = P.Tape()
    n = 30
    for k in range(n - 1):
        t.prop(t.leq(t.add(t.var(k), t.constant(1)), t.var(k + 1)))
    tape, roots = t.arrays()
    store = np.array([[0, 100]] * n, np.int32)
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    rc, st = ctx.pc_fixpoint(max_rounds=5)
    assert rc == pirgpu.TIMEOUT and st["rounds"] == 5
    rc, st = ctx.pc_fixpoint()
    assert rc == pirgpu.OK and ctx.project(n - 1) == (n - 1, 100)
    t2 = P.Tape()
    t2.prop(t2.gt(t2.var(0), t2.var(n - 1)))  # x0 > x29 contradicts the chain
    ctx.pc_tell(*t2.arrays())
    rc, st = ctx.pc_fixpoint()
    assert rc == pirgpu.FAILED and ctx.is_bot()
    assert ctx.pc_fixpoint()[0] == pirgpu.FAILED


def test_tree_and_shared_node_paths(gpu_ctx_factory, oracle):
    """Propagators whose formula reuses a node (x + x, a shared sub-sum) or
    has more than 24 nodes take the recursive path, small trees the two-pass
    one; all of them in one launch, against the oracle."""
    rng = np.random.default_rng(5)
    t = P.Tape()
    nv = 40
    store = np.stack([rng.integers(-30, 0, nv), rng.integers(0, 40, nv)], 1).astype(np.int32)
    for k in range(30):
        x, y = t.var(k % nv), t.var((k * 7 + 3) % nv)
        if k % 3 == 0:
            s = t.add(x, x)                                   # a node with two parents
            t.prop(t.leq(s, t.var((k + 1) % nv)))
        elif k % 3 == 1:
            terms = [t.mul(t.constant(1 + i % 3), t.var((k + i) % nv)) for i in range(9)]
            t.prop(t.leq(t.nadd(terms), t.constant(int(rng.integers(0, 60)))))   # 30 nodes
        else:
            t.prop(t.disj(t.leq(t.add(x, t.constant(2)), y), t.leq(t.add(y, t.constant(3)), x)))
    tape, roots = t.arrays()
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    _gpu_vs_oracle(ctx, oracle, tape, store)


def _events_vs_full(ctx, snap):
    ctx.restore(snap)
    rc_a, a = ctx.pc_fixpoint()
    sa = np.stack(ctx.read_store(), 1)
    ctx.restore(snap)
    rc_e, e = ctx.pc_fixpoint(sched=pirgpu.SCHED_EVENTS)
    se = np.stack(ctx.read_store(), 1)
    assert rc_a == rc_e
    if rc_a == pirgpu.OK:
        np.testing.assert_array_equal(sa, se)
        assert a["rounds"] == e["rounds"] and a["narrowed"] == e["narrowed"]
        assert e["executions"] <= a["executions"]
    return rc_a, a, e


@pytest.mark.parametrize("kind", ["mix", "planted", "random"])
def test_event_schedule_matches_full_rounds(kind, gpu_ctx_factory, oracle):
    """The event schedule runs only the formulas of the variables narrowed in
    the previous round: the same rounds, stores and narrowing count as full
    Jacobi rounds, fewer executions."""
    import workloads as W
    if kind == "mix":
        tape, roots, lb0, ub0, _ = W.pc_mix(100_000, 100_000, seed=4)
        store = np.ascontiguousarray(np.stack([lb0, ub0], 1))
    elif kind == "planted":
        t, store, _ = H.planted_formulas(np.random.default_rng(9), 2000, 1500, depth=3)
        tape, roots = t.arrays()
    else:
        t, store = H.random_formulas(np.random.default_rng(10), 60, 40, depth=3)
        tape, roots = t.arrays()
    ctx = _ctx(gpu_ctx_factory, tape, roots, store)
    snap = ctx.snapshot()
    rc, a, e = _events_vs_full(ctx, snap)
    if kind == "mix":
        assert rc == pirgpu.OK and e["executions"] < a["executions"]
    # a later tell and a grown store rebuild the adjacency
    t2 = P.Tape()
    t2.prop(t2.leq(t2.var(0), t2.var(len(store))))
    ctx.restore(snap)
    lb, ub = ctx.read_store()
    ctx.load_store(np.append(lb, -5), np.append(ub, 5))
    ctx.pc_tell(*t2.arrays())
    _events_vs_full(ctx, ctx.snapshot())


def test_error_paths_and_edge_cases(gpu_ctx_factory):
    ctx = gpu_ctx_factory()
    ctx.load_store(np.array([0, 0]), np.array([3, 3]))
    # no PC propagators: the fixpoint is trivially OK, the lists empty
    assert ctx.pc_fixpoint()[0] == pirgpu.OK
    assert ctx.pc_num_deductions() == 0 and len(ctx.pc_roots()) == 0
    assert ctx.pc_is_extractable()
    t = P.Tape()
    t.prop(t.leq(t.var(0), t.var(1)))
    ctx.pc_tell(*t.arrays())
    for bad in (-1, 1, 7):
        with pytest.raises(pirgpu.PirError, match="out of range"):
            ctx.pc_deduce_one(bad)
        with pytest.raises(pirgpu.PirError, match="out of range"):
            ctx.pc_ask(bad)
    assert ctx.pc_ask(0) is False      # x <= y over [0, 3] x [0, 3]: not entailed (3 > 0)
    # a store that is empty from the start: every call reports the failure
    ctx.load_store(np.array([2, 0]), np.array([1, 3]))
    assert ctx.is_bot()
    assert ctx.pc_fixpoint()[0] == pirgpu.FAILED
    assert ctx.pc_fixpoint(sched=pirgpu.SCHED_EVENTS)[0] == pirgpu.FAILED
    assert not ctx.pc_is_extractable()
    # True / False formulas: False empties the store, True is entailed
    ctx.load_store(np.array([0, 0]), np.array([3, 3]))
    t2 = P.Tape()
    t2.prop(t2.true())
    ctx.pc_tell(*t2.arrays())
    assert ctx.pc_fixpoint()[0] == pirgpu.OK
    t3 = P.Tape()
    t3.prop(t3.false())
    ctx.pc_tell(*t3.arrays())
    assert ctx.pc_fixpoint()[0] == pirgpu.FAILED and ctx.is_bot()


@pytest.mark.parametrize("case", K.AE_CASES, ids=[c[0] for c in K.AE_CASES])
def test_abstract_element_gpu(case, gpu_ctx_factory):
    """tests/pc_test.cpp:714-764 through the C ABI (both schedules)."""
    for sched in (pirgpu.SCHED_AC1, pirgpu.SCHED_EVENTS):
        tape, roots = H.ae_tape(case[2])
        ctx = _ctx(gpu_ctx_factory, tape, roots, np.array([[0, 10], [0, 10]], np.int32))

        def steps(meets):
            for v, l, u in meets:
                ctx.embed(v, l, u)
            lb, ub = ctx.read_store()
            b0 = [(int(lb[i]), int(ub[i])) for i in range(2)]
            rc, st = ctx.pc_fixpoint(sched=sched)
            lb, ub = ctx.read_store()
            return rc, b0, [(int(lb[i]), int(ub[i])) for i in range(2)], ctx.pc_is_extractable(), st["narrowed"] > 0

        assert H.run_ae_case(steps, case) == []
