"""Sharding of the batched workloads across ranks (one process per GPU).

Search nodes over one base model, and independent instances, are independent
units: each rank runs its own share in its own launch, with no collective on
the data path, and the results come back to rank 0 after the timed region.
The single instance does not shard (every round would need an all-reduce of
the store), so it runs as replicas.

The share of each rank is chosen by a cost estimate and a greedy
longest-processing-time-first assignment (each unit, heaviest first, goes to
the least loaded rank), whose largest load is at most the mean load plus the
largest unit cost.  The assignment is deterministic, so every rank computes the
same partition without exchanging anything.

Cost estimates:
  * a search node: 1 + the number of tightened bounds (propagation starts from
    the tightened variables; the base is at its fixpoint);
  * an instance: its propagator count (a round sweeps every propagator).
"""
import heapq

import numpy as np


def node_costs(off):
    """Cost estimate of each node of a tightening table (off: nnodes + 1 offsets)."""
    off = np.asarray(off, np.int64)
    return 1 + np.diff(off)


def instance_costs(prop_off):
    """Cost estimate of each packed instance (prop_off: ninst + 1 offsets)."""
    return np.maximum(np.diff(np.asarray(prop_off, np.int64)), 1)


def lpt_partition(costs, nparts):
    """Indices of the units of each part (ascending within a part).

    Units in order of decreasing cost (ties: lower index first) go to the part
    with the least load (ties: lower part first)."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    costs = np.asarray(costs, np.int64)
    order = np.lexsort((np.arange(len(costs)), -costs))
    heap = [(0, p) for p in range(nparts)]
    parts = [[] for _ in range(nparts)]
    for u in order:
        load, p = heapq.heappop(heap)
        parts[p].append(int(u))
        heapq.heappush(heap, (load + int(costs[u]), p))
    return [np.array(sorted(p), np.int64) for p in parts]


def select_nodes(off, var, lb, ub, idx):
    """The tightening table of the nodes `idx`, in that order."""
    off = np.asarray(off, np.int64)
    idx = np.asarray(idx, np.int64)
    cnt = off[idx + 1] - off[idx]
    new_off = np.zeros(len(idx) + 1, np.int32)
    np.cumsum(cnt, out=new_off[1:])
    take = np.concatenate([np.arange(off[i], off[i + 1]) for i in idx]) if len(idx) else np.zeros(0, np.int64)
    take = take.astype(np.int64)
    return (new_off, np.asarray(var, np.int32)[take], np.asarray(lb, np.int32)[take],
            np.asarray(ub, np.int32)[take])


def select_instances(prop_off, var_off, op, x, y, z, lb, ub, idx):
    """The packed instances `idx`, in that order, re-packed back to back (variable
    indices are relative to each instance, so they carry over unchanged)."""
    prop_off = np.asarray(prop_off, np.int64)
    var_off = np.asarray(var_off, np.int64)
    idx = np.asarray(idx, np.int64)
    pc = prop_off[idx + 1] - prop_off[idx]
    vc = var_off[idx + 1] - var_off[idx]
    po = np.zeros(len(idx) + 1, np.int64)
    vo = np.zeros(len(idx) + 1, np.int64)
    np.cumsum(pc, out=po[1:])
    np.cumsum(vc, out=vo[1:])

    def gather(a, offs, ids):
        if not len(ids):
            return np.zeros(0, np.int32)
        return np.ascontiguousarray(np.concatenate([a[offs[i]:offs[i + 1]] for i in ids]), np.int32)

    return (po, vo, gather(op, prop_off, idx), gather(x, prop_off, idx), gather(y, prop_off, idx),
            gather(z, prop_off, idx), gather(lb, var_off, idx), gather(ub, var_off, idx))


def scatter_rows(n, parts, values):
    """Puts the per-part result rows back in unit order: values[p][j] is the
    result of unit parts[p][j]."""
    first = next((v for v in values if len(v)), None)
    if first is None:
        return np.zeros((n,), np.int64)
    first = np.asarray(first)
    out = np.empty((n,) + first.shape[1:], first.dtype)
    for idx, v in zip(parts, values):
        if len(idx):
            out[np.asarray(idx)] = np.asarray(v)
    return out


def instance_var_slices(var_off, idx):
    """(start, stop) of each selected instance's variables in the packed store."""
    var_off = np.asarray(var_off, np.int64)
    return [(int(var_off[i]), int(var_off[i + 1])) for i in idx]


def gather_to_root(dist, obj, root=0):
    """Every rank's `obj` on the root rank (a list in rank order), None elsewhere;
    [obj] without a process group.  Called after the timed region."""
    if dist is None:
        return [obj]
    ws = dist.get_world_size()
    out = [None] * ws if dist.get_rank() == root else None
    dist.gather_object(obj, out, dst=root)
    return out
