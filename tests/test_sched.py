"""The learned propagator scheduler: the CPU reference of its network
(gradients against finite differences), the device training kernels
(gradients against that reference), and the learned fixpoint (bit-exact with
the plain fixpoint, fewer propagator executions once trained)."""
import numpy as np
import pytest


def _params(seed):
    from oracle import mlp_ref as M
    rng = np.random.default_rng(seed)
    p = np.zeros(M.NPARAM, np.float32)
    p[M.OFF_W1:M.OFF_B1] = rng.uniform(-.8, .8, M.NH * M.NF)
    p[M.OFF_B1:M.OFF_W2] = rng.uniform(-.1, .1, M.NH)
    p[M.OFF_W2:M.OFF_B2] = rng.uniform(-.4, .4, M.NH * M.NH)
    p[M.OFF_B2:M.OFF_W3] = rng.uniform(-.1, .1, M.NH)
    p[M.OFF_W3:M.OFF_B3] = rng.uniform(-.4, .4, M.NH)
    p[M.OFF_B3] = -.5
    return p


def _batch(seed, n):
    rng = np.random.default_rng(seed)
    X = rng.random((n, 8)).astype(np.float32)
    X[:, :3] = np.eye(3)[rng.integers(0, 3, n)]
    Y = (rng.random(n) < .3).astype(np.float32)
    return X, Y


def test_reference_gradient_matches_finite_differences():
    from oracle import mlp_ref as M
    p = _params(0).astype(np.float64)
    X, Y = _batch(1, 64)
    loss, g = M.loss_and_grad(p, X, Y, pos_weight=2.0, round_bf16=False)
    eps = 1e-4
    idx = np.random.default_rng(2).choice(M.NPARAM, 60, replace=False)
    for i in idx:
        q = p.copy(); q[i] += eps
        lp, _ = M.loss_and_grad(q.astype(np.float32), X, Y, 2.0, False)
        q[i] -= 2 * eps
        lm, _ = M.loss_and_grad(q.astype(np.float32), X, Y, 2.0, False)
        num = (lp - lm) / (2 * eps)
        # float32 parameters: tolerance for the rounding of p +- eps
        assert abs(num - g[i]) <= 2e-3 + 2e-2 * abs(g[i]), (i, num, g[i])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(3))
def test_device_gradient_matches_reference(seed):
    """pir_sched_grad (the training kernel) == the float64 reference on the
    same BF16-rounded weights; tolerance rtol 1e-3 + atol 1e-6 (FP32
    accumulation over the batch)."""
    import pirgpu
    from oracle import mlp_ref as M
    ctx = pirgpu.Context(0)
    p = _params(seed)
    ctx.sched_params(p)
    X, Y = _batch(seed + 10, 1000)
    g, loss = ctx.sched_grad(X, Y, pos_weight=3.0)
    rl, rg = M.loss_and_grad(p, X, Y, 3.0)
    np.testing.assert_allclose(loss, rl, rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(g, rg, rtol=1e-3, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(3))
def test_inference_scores_match_reference(seed):
    """pir_sched_score (the tensor-core inference path of the learned
    fixpoint: mma with BF16 features, weights and first hidden layer, FP32
    accumulation) against the float64 restatement with the same roundings.
    Tolerance: 1e-3 x (1 + |score|) on 99.5% of the rows; a first-layer value
    that sits on a BF16 rounding boundary may round the other way on the
    device (one BF16 ulp, 2^-8 relative), so every row is within
    3e-2 x (1 + |score|)."""
    import pirgpu
    from oracle import mlp_ref as M
    ctx = pirgpu.Context(0)
    p = _params(seed)
    ctx.sched_params(p)
    X, _ = _batch(seed + 20, 4099)  # not a multiple of 32
    X[:5] = 0.0
    got = ctx.sched_score(X)
    ref = M.forward_inference(p, X)
    err = np.abs(got - ref) / (1 + np.abs(ref))
    assert np.quantile(err, 0.995) < 1e-3
    assert err.max() < 3e-2


def _nodes(P, seed=0, nvars=20_000, nprops=80_000, nnodes=96):
    import workloads as W
    base = W.plain(nvars, nprops, 10**6, seed)
    ctx = P.Context(0)
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    rc, _ = ctx.fixpoint()
    assert rc == P.OK
    blb, bub = ctx.read_store()
    _, off, var, lb, ub = W.nodes(nvars, nprops, nnodes, seed, 64, base_store=(blb, bub))
    return ctx, off, var, lb, ub


def _run_nodes(ctx, off, var, lb, ub, sched, nodes, **kw):
    snap = ctx.snapshot()
    out = []
    for j in nodes:
        ctx.restore(snap)
        ctx.embed_many(var[off[j]:off[j + 1]], lb[off[j]:off[j + 1]], ub[off[j]:off[j + 1]])
        rc, st = ctx.fixpoint(sched=sched, mode=1, **kw)
        l, u = ctx.read_store()
        out.append((rc, l, u, st))
    ctx.restore(snap)
    return out


# the learned rounds on the frontier of the embedded variables (one CTA), and
# the grid kernel that scores every propagator every round
PATHS = {"frontier": 0, "grid": -1}


@pytest.mark.gpu
@pytest.mark.parametrize("path", PATHS)
def test_learned_fixpoint_is_the_plain_fixpoint(path):
    """Untrained (random) weights: the schedule is poor but the certified
    result equals the AC-1 fixpoint bit for bit, failures included."""
    import pirgpu as P
    ctx, off, var, lb, ub = _nodes(P)
    nodes = range(24)
    plain = _run_nodes(ctx, off, var, lb, ub, P.SCHED_AC1, nodes)
    learned = _run_nodes(ctx, off, var, lb, ub, P.SCHED_LEARNED, nodes, wake_fraction=0.05,
                         local_frontier=PATHS[path])
    for (r0, l0, u0, _), (r1, l1, u1, s1) in zip(plain, learned):
        assert r0 == r1
        if r0 == P.OK:
            np.testing.assert_array_equal(l0, l1)
            np.testing.assert_array_equal(u0, u1)
            assert s1["certify_executions"] > 0


@pytest.mark.gpu
def test_learned_frontier_needs_a_fixpoint_before_the_embeddings():
    """The frontier rounds start from the variables embedded since the store
    was last a fixpoint: after a store load (no fixpoint yet) the grid kernel
    runs instead, and the result is the AC-1 fixpoint either way; a fixpoint,
    then embeddings, then the learned fixpoint takes the frontier path, whose
    executions are far fewer than one sweep."""
    import pirgpu as P
    import workloads as W
    base = W.plain(20_000, 80_000, 10**6, 7)
    ctx = P.Context(0)
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    rc, st = ctx.fixpoint(sched=P.SCHED_LEARNED)
    assert rc == P.OK and st["executions"] >= 80_000  # grid kernel: a full certifying sweep at least
    l0, u0 = ctx.read_store()
    ref = P.Context(0)
    ref.load_store(base.lb, base.ub)
    ref.tell(base.op, base.x, base.y, base.z)
    assert ref.fixpoint()[0] == P.OK
    l1, u1 = ref.read_store()
    np.testing.assert_array_equal(l0, l1)
    np.testing.assert_array_equal(u0, u1)
    # branch on a few unfixed variables, as a search node does
    free = np.nonzero(l0 < u0)[0][:8]
    mid = l0[free] + (u0[free] - l0[free]) // 2
    ctx.embed_many(free, l0[free], mid)
    ref.embed_many(free, l1[free], mid)
    rc, st = ctx.fixpoint(sched=P.SCHED_LEARNED)
    rr, _ = ref.fixpoint()
    assert rc == rr
    assert st["executions"] < 80_000
    if rc == P.OK:
        np.testing.assert_array_equal(ctx.read_store()[0], ref.read_store()[0])
        np.testing.assert_array_equal(ctx.read_store()[1], ref.read_store()[1])


@pytest.mark.gpu
@pytest.mark.parametrize("path", PATHS)
def test_training_reduces_executions_and_keeps_the_fixpoint(path):
    """Train on change traces of the plain fixpoint (first 64 nodes), then
    compare on 32 held-out nodes: bit-exact results, and the trained network
    needs at least 2x fewer propagator executions than plain AC-1 rounds."""
    import pirgpu as P
    ctx, off, var, lb, ub = _nodes(P, seed=3, nnodes=96)
    train = 64
    ns, npos = ctx.sched_collect(off[:train + 1], var, lb, ub, max_samples=400_000, keep_negative=0.02)
    assert ns > 1000 and npos > 100
    loss = ctx.sched_train(epochs=6, batch=4096, lr=3e-3, pos_weight=4.0)
    assert loss[-1] < loss[0]
    held = range(train, 96)
    plain = _run_nodes(ctx, off, var, lb, ub, P.SCHED_AC1, held)
    learned = _run_nodes(ctx, off, var, lb, ub, P.SCHED_LEARNED, held, wake_fraction=1 / 32,
                         local_frontier=PATHS[path])
    e0 = e1 = 0
    for (r0, l0, u0, s0), (r1, l1, u1, s1) in zip(plain, learned):
        assert r0 == r1
        if r0 == P.OK:
            np.testing.assert_array_equal(l0, l1)
            np.testing.assert_array_equal(u0, u1)
        e0 += s0["executions"]
        e1 += s1["executions"]
    assert e1 * 2 <= e0, (e0, e1)


@pytest.mark.gpu
@pytest.mark.parametrize("nembed", [10_000, 20_000])
def test_learned_frontier_overflow_hands_over(nembed):
    """Many embedded variables: with 10,000 the frontier outgrows the one-CTA
    lists (65,536 entries) and the grid kernel finishes the run from the
    store reached so far; with 20,000 the embedded variables exceed what the
    host hands over (16,384) and the grid kernel runs from the start.  The
    AC-1 fixpoint either way."""
    import pirgpu as P
    import workloads as W
    base = W.plain(100_000, 400_000, 10**6, 9)
    ctx = P.Context(0)
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    assert ctx.fixpoint()[0] == P.OK
    l0, u0 = ctx.read_store()
    free = np.nonzero(l0 < u0)[0][:nembed]
    assert len(free) == nembed
    # bisect each toward the half holding the planted solution: the node stays feasible
    hidden = base.meta["hidden"][free]
    mid = l0[free] + (u0[free] - l0[free]) // 2
    lo = np.where(hidden <= mid, l0[free], mid + 1)
    hi = np.where(hidden <= mid, mid, u0[free])
    snap = ctx.snapshot()
    out = []
    for sched, kw in ((P.SCHED_AC1, {}), (P.SCHED_LEARNED, {"wake_fraction": 0.25})):
        ctx.restore(snap)
        ctx.embed_many(free, lo, hi)
        rc, st = ctx.fixpoint(sched=sched, mode=1, **kw)
        out.append((rc, ctx.read_store(), st))
    (r0, (a0, b0), s0), (r1, (a1, b1), s1) = out
    assert r0 == r1 == P.OK
    np.testing.assert_array_equal(a0, a1)
    np.testing.assert_array_equal(b0, b1)
    # the grid kernel's full certifying sweep ran
    assert s1["certify_executions"] >= 400_000
