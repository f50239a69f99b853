"""Batched fixpoints (search nodes, uneven instances) against the CPU oracle:
bit-exact stores of the nodes / instances that reach a fixpoint and identical
status flags."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import pirgpu
    return pirgpu


def _uneven_set(seed, n=24, pmin=500, pmax=20_000, spec_every=0):
    import workloads as W
    insts = W.uneven(ninst=n, pmin=pmin, pmax=pmax, seed=seed)
    if spec_every:
        for j in range(0, n, spec_every):
            p = insts[j].nprops
            insts[j] = W.plain(max(p // 4, 8), p, 1000, 1000 + j, variant="spec", mix=W.MIX_UNEVEN)
    return insts


SCHEDS = ("ac1", "events")


def _sched(P, name):
    return {"ac1": P.SCHED_AC1, "events": P.SCHED_EVENTS}[name]


@pytest.mark.parametrize("sched", SCHEDS)
@pytest.mark.parametrize("seed", range(3))
def test_instances_parity(seed, sched, P, oracle):
    import workloads as W
    insts = _uneven_set(seed, spec_every=7)
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    glb, gub = lb.copy(), ub.copy()
    ctx = P.Context(0)
    status, rounds, ms, st = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, glb, gub,
                                                    sched=_sched(P, sched))
    nfail = 0
    for j, inst in enumerate(insts):
        s = inst.store()
        orc, info = oracle.install(inst.op, inst.x, inst.y, inst.z, s)
        if orc != oracle.FAILED:
            orc, info = oracle.fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        assert status[j] == orc, j
        v0, v1 = var_off[j], var_off[j + 1]
        if orc == oracle.OK:
            np.testing.assert_array_equal(glb[v0:v1], s[:, 0])
            np.testing.assert_array_equal(gub[v0:v1], s[:, 1])
        else:
            nfail += 1
    assert nfail >= 3  # the spec-variant instances fail
    assert np.all(ms > 0)
    ac1_execs = int(sum(rounds[j] * insts[j].nprops for j in range(len(insts))))
    if sched == "ac1":
        assert st["executions"] == ac1_execs
    else:  # round 0 runs every propagator, later rounds only those of narrowed variables
        assert sum(i.nprops for i in insts) <= st["executions"] < ac1_execs


@pytest.mark.parametrize("mode", ("auto", "one_cta"))
@pytest.mark.parametrize("sched", SCHEDS)
def test_instances_smem_and_global_paths(sched, mode, P, oracle):
    """Small instances run from shared memory; the largest runs on a cluster
    (auto) or, with the cluster kernel off (one CTA per instance), from the
    global store: all agree with the oracle."""
    import workloads as W
    insts = [W.plain(200, 800, 1000, 1), W.plain(60_000, 240_000, 1000, 2, mix=W.MIX_UNEVEN),
             W.plain(3000, 12_000, 1000, 3, mix=W.MIX_UNEVEN)]
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    ctx = P.Context(0)
    status, rounds, ms, st = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb, ub,
                                                    mode=P.MODE_SMEM if mode == "one_cta" else P.MODE_AUTO,
                                                    sched=_sched(P, sched))
    for j, inst in enumerate(insts):
        s = inst.store()
        oracle.install(inst.op, inst.x, inst.y, inst.z, s)
        orc, _ = oracle.fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        assert status[j] == orc == oracle.OK
        np.testing.assert_array_equal(lb[var_off[j]:var_off[j + 1]], s[:, 0])
        np.testing.assert_array_equal(ub[var_off[j]:var_off[j + 1]], s[:, 1])


@pytest.mark.parametrize("sched", SCHEDS)
def test_instances_round_cap(sched, P):
    import workloads as W
    insts = [W.add_chain(W.plain(2000, 8000, 1000, 4), 100, 1000, 4)]
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    ctx = P.Context(0)
    status, rounds, _, _ = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb, ub, max_rounds=7,
                                                  sched=_sched(P, sched))
    assert status[0] == P.TIMEOUT and rounds[0] == 7


def test_instances_events_fewer_executions(P, oracle):
    """The event-filtered rounds reach the AC-1 rounds' stores and statuses
    (a chain of 190 links forces a long tail of rounds that narrow a few
    variables) with fewer executions; the learned schedule is refused."""
    import workloads as W
    insts = [W.add_chain(W.plain(4000, 16_000, 1000, 11), 190, 1000, 11),
             W.add_chain(W.plain(40_000, 160_000, 1000, 12, mix=W.MIX_UNEVEN), 190, 1000, 12),
             W.plain(900, 3600, 1000, 13, mix=W.MIX_UNEVEN)]
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    ctx = P.Context(0)
    res = {}
    for name in SCHEDS:
        glb, gub = lb.copy(), ub.copy()
        status, rounds, _, st = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, glb, gub,
                                                       sched=_sched(P, name))
        assert np.all(status == P.OK)
        res[name] = (glb, gub, st["executions"])
    np.testing.assert_array_equal(res["ac1"][0], res["events"][0])
    np.testing.assert_array_equal(res["ac1"][1], res["events"][1])
    assert res["events"][2] * 5 < res["ac1"][2]
    with pytest.raises(P.PirError):
        ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb.copy(), ub.copy(), sched=P.SCHED_LEARNED)


def _nodes_setup(P, nvars=5000, nprops=20_000, nnodes=200, kmax=48, seed=0):
    import workloads as W
    base = W.plain(nvars, nprops, 10**6, seed)
    ctx = P.Context(0)
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    rc, _ = ctx.fixpoint()
    assert rc == P.OK
    blb, bub = ctx.read_store()
    _, off, var, lb, ub = W.nodes(nvars, nprops, nnodes, seed, kmax, base_store=(blb, bub))
    return ctx, (blb, bub), off, var, lb, ub


@pytest.mark.parametrize("seed", range(3))
def test_nodes_parity(seed, P, oracle):
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, seed=seed)
    status, olb, oub, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub)
    op, x, y, z = ctx.bytecode()
    base = np.ascontiguousarray(np.stack([blb, bub], 1))
    ostatus, ostore, ostats = oracle.fixpoint_nodes(op, x, y, z, base, off, var, lb, ub)
    np.testing.assert_array_equal(status, ostatus)
    ok = ostatus == oracle.OK
    assert ok.sum() > 0 and (~ok).sum() > 0  # both outcomes are exercised
    np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])
    np.testing.assert_array_equal(oub[ok], ostore[ok, :, 1])
    # the context's own store is untouched
    l2, u2 = ctx.read_store()
    np.testing.assert_array_equal(l2, blb)


def test_nodes_partial_group_and_cap(P, oracle):
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, nnodes=45, seed=5)
    status, olb, oub, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub)
    op, x, y, z = ctx.bytecode()
    base = np.ascontiguousarray(np.stack([blb, bub], 1))
    ostatus, ostore, _ = oracle.fixpoint_nodes(op, x, y, z, base, off, var, lb, ub)
    np.testing.assert_array_equal(status, ostatus)
    ok = ostatus == oracle.OK
    np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])
    capped, _, _, r2, _ = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, max_rounds=1)
    assert np.all((capped != P.OK) | (r2 <= 1))


@pytest.mark.parametrize("seed", range(3))
def test_nodes_events_parity(seed, P, oracle):
    """Event-driven nodes (base at its fixpoint): same statuses and stores as
    the oracle's Gauss-Seidel per node."""
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, seed=seed)
    status, olb, oub, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS)
    op, x, y, z = ctx.bytecode()
    base = np.ascontiguousarray(np.stack([blb, bub], 1))
    ostatus, ostore, ostats = oracle.fixpoint_nodes(op, x, y, z, base, off, var, lb, ub)
    np.testing.assert_array_equal(status, ostatus)
    ok = ostatus == oracle.OK
    assert ok.sum() > 0 and (~ok).sum() > 0
    np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])
    np.testing.assert_array_equal(oub[ok], ostore[ok, :, 1])
    # far fewer executions than AC-1 rounds over the whole bytecode
    assert st["executions"] < 0.5 * (ostats[:, 1].sum())
    # a second launch reuses the scratch (stamps, working stores) correctly
    s2, l2, u2, _, _ = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS)
    np.testing.assert_array_equal(s2, status)
    np.testing.assert_array_equal(l2[ok], olb[ok])


@pytest.mark.parametrize("variant", list(range(1, 11)))
def test_nodes_events_variants(variant, P, oracle):
    """The event node kernel: one node per CTA with 256 threads sized for 2,
    3, 4, 6 and 8 resident CTAs per SM, 128 threads for 8 and 10; one node per
    warp with 8 warps per CTA sized for 2 and 3 CTAs per SM, 4 warps for 6.
    Twice in a row: the second launch finds the scratch as the first left it."""
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, seed=4, nnodes=300)
    status, olb, oub, _, st = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS, variant=variant)
    assert st["certify_narrowed"] == 0
    s2, l2, u2, _, _ = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS, variant=variant)
    np.testing.assert_array_equal(s2, status)
    np.testing.assert_array_equal(l2, olb)
    np.testing.assert_array_equal(u2, oub)
    op, x, y, z = ctx.bytecode()
    base = np.ascontiguousarray(np.stack([blb, bub], 1))
    ostatus, ostore, _ = oracle.fixpoint_nodes(op, x, y, z, base, off, var, lb, ub)
    np.testing.assert_array_equal(status, ostatus)
    ok = ostatus == oracle.OK
    np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])
    np.testing.assert_array_equal(oub[ok], ostore[ok, :, 1])


def test_nodes_autotune(P, oracle):
    """pir_autotune_nodes picks one of the variants and later calls use it."""
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, seed=6, nnodes=256)
    v, ms = ctx.autotune_nodes(off, var, lb, ub)
    assert 1 <= v <= P.NODE_VARIANTS and ms > 0
    status, olb, oub, _, _ = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS)
    op, x, y, z = ctx.bytecode()
    base = np.ascontiguousarray(np.stack([blb, bub], 1))
    ostatus, ostore, _ = oracle.fixpoint_nodes(op, x, y, z, base, off, var, lb, ub)
    np.testing.assert_array_equal(status, ostatus)
    ok = ostatus == oracle.OK
    np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])


def test_nodes_events_follow_a_changed_base(P, oracle):
    """The working stores are reused while the base store is unchanged and
    reloaded when it changes (embed + fixpoint, restore, a smaller batch):
    every launch matches the oracle run on the base of that moment."""
    import workloads as W
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, seed=5, nnodes=256)
    op, x, y, z = ctx.bytecode()
    snap = ctx.snapshot()

    def check(o, v, l, u):
        cl, cu = ctx.read_store()
        base = np.ascontiguousarray(np.stack([cl, cu], 1))
        status, olb, oub, _, _ = ctx.fixpoint_nodes(o, v, l, u, sched=P.SCHED_EVENTS)
        ostatus, ostore, _ = oracle.fixpoint_nodes(op, x, y, z, base, o, v, l, u)
        np.testing.assert_array_equal(status, ostatus)
        ok = ostatus == oracle.OK
        np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])
        np.testing.assert_array_equal(oub[ok], ostore[ok, :, 1])

    check(off, var, lb, ub)
    check(off, var, lb, ub)  # same base: working stores reused
    # a new base: one unfixed variable bisected, then propagated
    free = np.where(blb < bub)[0]
    v0 = int(free[0])
    ctx.embed(v0, int(blb[v0]), int(blb[v0] + (bub[v0] - blb[v0]) // 2))
    rc, _ = ctx.fixpoint()
    assert rc == P.OK
    nl, nu = ctx.read_store()
    _, off2, var2, lb2, ub2 = W.nodes(5000, 20_000, 256, 6, 48, base_store=(nl, nu))
    check(off2, var2, lb2, ub2)
    # back to the first base, then a smaller batch on the same base
    ctx.restore(snap)
    check(off, var, lb, ub)
    check(off[:41], var, lb, ub)


def test_nodes_events_need_a_fixpoint_base(P, oracle):
    """When the base store is not a fixpoint the event schedule is not exact;
    the call then runs AC-1 rounds and still matches the oracle."""
    import workloads as W
    base = W.plain(5000, 20_000, 10**6, 7)
    ctx = P.Context(0)
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    blb, bub = ctx.read_store()
    _, off, var, lb, ub = W.nodes(5000, 20_000, 64, 7, 16, base_store=(blb, bub))
    status, olb, oub, _, _ = ctx.fixpoint_nodes(off, var, lb, ub, sched=P.SCHED_EVENTS)
    op, x, y, z = ctx.bytecode()
    bs = np.ascontiguousarray(np.stack([blb, bub], 1))
    ostatus, ostore, _ = oracle.fixpoint_nodes(op, x, y, z, bs, off, var, lb, ub)
    np.testing.assert_array_equal(status, ostatus)
    ok = ostatus == oracle.OK
    np.testing.assert_array_equal(olb[ok], ostore[ok, :, 0])


@pytest.mark.parametrize("sched", SCHEDS)
def test_instances_cluster_path(sched, P, oracle):
    """More large instances than clusters (work stealing across clusters of 8
    CTAs sharing the store through distributed shared memory) plus small ones
    in the same call: every store bit-exact."""
    import workloads as W
    insts = [W.plain(30_000 + 997 * j, 120_000 + 3000 * j, 1000, 40 + j, mix=W.MIX_UNEVEN) for j in range(24)]
    insts += [W.plain(400 + 10 * j, 1600 + 40 * j, 1000, 90 + j, mix=W.MIX_UNEVEN) for j in range(8)]
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    ctx = P.Context(0)
    status, rounds, ms, st = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb, ub, sched=_sched(P, sched))
    for j, inst in enumerate(insts):
        s = inst.store()
        oracle.install(inst.op, inst.x, inst.y, inst.z, s)
        orc, _ = oracle.fixpoint(inst.op, inst.x, inst.y, inst.z, s)
        assert status[j] == orc == oracle.OK, j
        np.testing.assert_array_equal(lb[var_off[j]:var_off[j + 1]], s[:, 0])
        np.testing.assert_array_equal(ub[var_off[j]:var_off[j + 1]], s[:, 1])
    capped, r2, _, _ = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb.copy(), ub.copy(), max_rounds=1,
                                              sched=_sched(P, sched))
    assert np.all(r2 <= 1)


def test_instances_reject_bad_bytecode(P):
    """Validation (on the host's threads) names the first bad instance and
    leaves the stores untouched."""
    import workloads as W
    insts = [W.plain(500, 2000, 1000, 70 + j) for j in range(40)]
    prop_off, var_off, op, x, y, z, lb, ub = W.pack(insts)
    lb0 = lb.copy()
    ctx = P.Context(0)
    for j_bad, field, value, msg in [(17, "x", 10**6, "instance 17: var index out of range"),
                                      (3, "op", 11, "instance 3: bad opcode"),
                                      (31, "z", -1, "instance 31: var index out of range")]:
        arrs = dict(op=op.copy(), x=x.copy(), y=y.copy(), z=z.copy())
        arrs[field][prop_off[j_bad] + 5] = value
        arrs["x"][prop_off[39] + 1] = 10**6  # a later bad instance is not the one reported
        with pytest.raises(P.PirError, match=msg):
            ctx.fixpoint_instances(prop_off, var_off, arrs["op"], arrs["x"], arrs["y"], arrs["z"], lb, ub)
        np.testing.assert_array_equal(lb, lb0)


def test_nodes_staged_graph_matches_watch(P):
    """pir_nodes_stage + pir_fixpoint_nodes_staged (each batch one CUDA graph,
    updated in place, rebuilt when the staging grows) give what
    pir_fixpoint_nodes_watch gives, batch after batch; a bad variable in the
    staging is rejected before anything runs."""
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, nnodes=200, seed=7)
    watch = np.arange(0, 5000, 7, dtype=np.int32)
    for j0, j1 in ((0, 60), (60, 120), (120, 200), (0, 30)):
        o = (off[j0:j1 + 1] - off[j0]).astype(np.int32)
        sl = slice(off[j0], off[j1])
        ws, wl, wu, wr, _ = ctx.fixpoint_nodes_watch(o, var[sl], lb[sl], ub[sl], watch)
        nn, nt, nw = j1 - j0, int(o[-1]), len(watch)
        buf = ctx.nodes_stage(nn, nt, nw)
        buf[:nw] = watch
        buf[nw:nw + nn + 1] = o
        buf[nw + nn + 1:nw + nn + 1 + nt] = var[sl]
        buf[nw + nn + 1 + nt:nw + nn + 1 + 2 * nt] = lb[sl]
        buf[nw + nn + 1 + 2 * nt:] = ub[sl]
        ss, sl_, su, sr, st = ctx.fixpoint_nodes_staged(nn, nt, nw)
        np.testing.assert_array_equal(ss, ws)
        np.testing.assert_array_equal(sr, wr)
        np.testing.assert_array_equal(sl_, wl)
        np.testing.assert_array_equal(su, wu)
        assert st["certify_narrowed"] == 0
    buf = ctx.nodes_stage(2, 1, 0)
    buf[:] = [0, 1, 1, 5000, 0, 0]  # off 0, 1, 1; var 5000 is out of range
    with pytest.raises(P.PirError):
        ctx.fixpoint_nodes_staged(2, 1, 0)


def test_nodes_staged_after_instances(P):
    """Staged node batches and uneven instances on one context: the instance
    install growing its own pinned staging leaves the node staging and the
    batch graph alone, so the batch after it still matches
    pir_fixpoint_nodes_watch (and the context tears down cleanly)."""
    import workloads as W
    ctx, (blb, bub), off, var, lb, ub = _nodes_setup(P, nnodes=80, seed=3)
    watch = np.arange(0, 5000, 11, dtype=np.int32)
    nn, nt, nw = 80, int(off[-1]), len(watch)
    ws, wl, wu, wr, _ = ctx.fixpoint_nodes_watch(off, var, lb, ub, watch)

    def staged():
        buf = ctx.nodes_stage(nn, nt, nw)
        buf[:nw] = watch
        buf[nw:nw + nn + 1] = off
        buf[nw + nn + 1:nw + nn + 1 + nt] = var
        buf[nw + nn + 1 + nt:nw + nn + 1 + 2 * nt] = lb
        buf[nw + nn + 1 + 2 * nt:] = ub
        ss, sl_, su, sr, st = ctx.fixpoint_nodes_staged(nn, nt, nw)
        np.testing.assert_array_equal(ss, ws)
        np.testing.assert_array_equal(sr, wr)
        np.testing.assert_array_equal(sl_, wl)
        np.testing.assert_array_equal(su, wu)

    staged()
    for n in (4, 12):  # the second set grows the instance staging again
        prop_off, var_off, op, x, y, z, ilb, iub = W.pack(_uneven_set(5, n=n))
        status, _, _, _ = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, ilb, iub)
        assert np.all(status == P.OK)
        staged()
    ctx.close()
