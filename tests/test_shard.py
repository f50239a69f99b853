"""Sharding of search nodes and instances across ranks: the partition, the
re-packing, and two gloo ranks on CPU whose gathered results equal the
unsharded run (the oracle stands in for the GPU kernel of each rank)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "lala-pc_gb300"))
sys.path.insert(0, ROOT)

import shard  # noqa: E402


def test_lpt_partition_is_a_balanced_partition():
    rng = np.random.default_rng(0)
    for nparts in (1, 2, 3, 8):
        costs = rng.integers(1, 1000, 257)
        parts = shard.lpt_partition(costs, nparts)
        assert len(parts) == nparts
        allidx = np.sort(np.concatenate(parts))
        np.testing.assert_array_equal(allidx, np.arange(len(costs)))
        loads = [int(costs[p].sum()) for p in parts]
        assert max(loads) <= costs.sum() / nparts + costs.max()
        # deterministic
        again = shard.lpt_partition(costs, nparts)
        for a, b in zip(parts, again):
            np.testing.assert_array_equal(a, b)


def test_lpt_more_parts_than_units():
    parts = shard.lpt_partition([5, 3], 4)
    assert sorted(len(p) for p in parts) == [0, 0, 1, 1]


def test_select_nodes_and_scatter_round_trip():
    rng = np.random.default_rng(1)
    k = rng.integers(0, 5, 20)
    off = np.zeros(21, np.int32)
    np.cumsum(k, out=off[1:])
    var = rng.integers(0, 50, off[-1]).astype(np.int32)
    lb = rng.integers(-9, 0, off[-1]).astype(np.int32)
    ub = rng.integers(0, 9, off[-1]).astype(np.int32)

    def summary(o, v, l, u, j):
        a, b = o[j], o[j + 1]
        return [b - a, int(v[a:b].sum()), int(l[a:b].sum()), int(u[a:b].sum())]

    parts = shard.lpt_partition(shard.node_costs(off), 3)
    rows = []
    for idx in parts:
        o2, v2, l2, u2 = shard.select_nodes(off, var, lb, ub, idx)
        assert len(o2) == len(idx) + 1
        rows.append(np.array([summary(o2, v2, l2, u2, j) for j in range(len(idx))], np.int64).reshape(-1, 4))
    back = shard.scatter_rows(20, parts, rows)
    for i in range(20):
        np.testing.assert_array_equal(back[i], summary(off, var, lb, ub, i))


def test_select_instances_round_trip():
    import workloads as W
    insts = W.uneven(7, 1000, 3000, 4)
    po, vo, op, x, y, z, lb, ub = W.pack(insts)
    idx = np.array([5, 0, 3])
    p2, v2, o2, x2, y2, z2, l2, u2 = shard.select_instances(po, vo, op, x, y, z, lb, ub, idx)
    for j, i in enumerate(idx):
        np.testing.assert_array_equal(o2[p2[j]:p2[j + 1]], op[po[i]:po[i + 1]])
        np.testing.assert_array_equal(z2[p2[j]:p2[j + 1]], z[po[i]:po[i + 1]])
        np.testing.assert_array_equal(l2[v2[j]:v2[j + 1]], lb[vo[i]:vo[i + 1]])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_nodes(rank, ws, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import workloads as W
    from oracle import oracle as O
    base = W.plain(2000, 8000, 10**6, 3)
    s = base.store()
    rc, _ = O.install_and_fixpoint(base.op, base.x, base.y, base.z, s)
    assert rc == O.OK
    op, x, y, z = base.op, base.x, base.y, base.z
    _, off, var, lb, ub = W.nodes(2000, 8000, 48, 5, 16, base_store=(s[:, 0].copy(), s[:, 1].copy()))
    parts = shard.lpt_partition(shard.node_costs(off), ws)
    mine = parts[rank]
    o2, v2, l2, u2 = shard.select_nodes(off, var, lb, ub, mine)
    status, stores, _ = O.fixpoint_nodes(op, x, y, z, s, o2, v2, l2, u2, threads=1)
    got = shard.gather_to_root(dist, (status, stores))
    if rank == 0:
        st = shard.scatter_rows(len(off) - 1, parts, [g[0] for g in got])
        sto = shard.scatter_rows(len(off) - 1, parts, [g[1] for g in got])
        ref_status, ref_stores, _ = O.fixpoint_nodes(op, x, y, z, s, off, var, lb, ub, threads=1)
        np.testing.assert_array_equal(st, ref_status)
        ok = ref_status == O.OK
        np.testing.assert_array_equal(sto[ok], ref_stores[ok])
        open(os.path.join(outdir, "nodes_ok"), "w").write("%d %d" % (len(st), int(ok.sum())))
    dist.destroy_process_group()


def _rank_instances(rank, ws, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import workloads as W
    from oracle import oracle as O
    insts = W.uneven(12, 1000, 6000, 2)
    po, vo, op, x, y, z, lb, ub = W.pack(insts)
    parts = shard.lpt_partition(shard.instance_costs(po), ws)
    mine = parts[rank]
    p2, v2, o2, x2, y2, z2, l2, u2 = shard.select_instances(po, vo, op, x, y, z, lb, ub, mine)
    s2 = np.ascontiguousarray(np.stack([l2, u2], 1))
    status, _ = O.fixpoint_instances(p2, v2, o2, x2, y2, z2, s2, threads=1)
    stores = [s2[v2[j]:v2[j + 1]] for j in range(len(mine))]
    got = shard.gather_to_root(dist, (status, stores))
    if rank == 0:
        st = shard.scatter_rows(len(insts), parts, [g[0] for g in got])
        s_ref = np.ascontiguousarray(np.stack([lb, ub], 1))
        ref_status, _ = O.fixpoint_instances(po, vo, op, x, y, z, s_ref, threads=1)
        np.testing.assert_array_equal(st, ref_status)
        for p, g in zip(parts, got):
            for j, i in enumerate(p):
                if ref_status[i] == O.OK:
                    np.testing.assert_array_equal(g[1][j], s_ref[vo[i]:vo[i + 1]])
        open(os.path.join(outdir, "instances_ok"), "w").write("%d" % len(st))
    dist.destroy_process_group()


def _spawn(fn, tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(fn, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)


def test_two_ranks_nodes_gloo(tmp_path, oracle):
    pytest.importorskip("torch")
    _spawn(_rank_nodes, tmp_path)
    n, ok = map(int, open(tmp_path / "nodes_ok").read().split())
    assert n == 48 and ok > 0


def test_two_ranks_instances_gloo(tmp_path, oracle):
    pytest.importorskip("torch")
    _spawn(_rank_instances, tmp_path)
    assert int(open(tmp_path / "instances_ok").read()) == 12
