"""Benchmark of the pirgpu propagation engine (one JSON line on stdout).

Default workload (one step = one full fixpoint from the initial store):
1,000,000 int32 variables with lb ~ U[-1e6, 0], ub = lb + U[0, 2e6];
4,000,000 PIR propagators (45% x=y+z, 15% x=y*z, 5% min, 5% max, 10% x=y-z,
20% reified x=(y<=z)) with a planted solution, plus a 20,000-link chain
x_{i+1} = x_i + c_i (c_i ~ U[1, 5]) that keeps changing one bound per round
for ~20,000 rounds.  Metric: propagator executions per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload single_large|single_small|out_of_l2|nodes|uneven|learned|search|pc]

--impl reference times the reference algorithm's CPU path (the C++
restatement of lala-pc's PIR::deduce driven by the Gauss-Seidel loop) on
bounded samples of the same workload on the host cores.
Under torchrun (N > 1) the single instance does not shard: each rank runs an
independent replica on its own GPU; value = executions of all ranks / max time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "lala-pc_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

ALG_BYTES_PER_EXEC = 40   # 16 B bytecode + 3 x 8 B intervals read
ALG_BYTES_PER_JOIN = 4    # one int32 bound written per narrowing join
L2_FLUSH_BYTES = 256 << 20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------ CUDA runtime --
class Cudart:
    """Minimal libcudart access (pinned host buffers, L2 flush, device sync)."""

    def __init__(self):
        for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
            try:
                self.L = ctypes.CDLL(name)
                break
            except OSError:
                continue
        else:
            raise RuntimeError("libcudart not found")
        self.flush_ptr = None

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed with CUDA error %d" % (what, rc))

    def set_device(self, d):
        self.check(self.L.cudaSetDevice(d), "cudaSetDevice")

    def sync(self):
        self.check(self.L.cudaDeviceSynchronize(), "cudaDeviceSynchronize")

    def pinned(self, n, dtype=np.int32):
        p = ctypes.c_void_p()
        nbytes = int(n) * np.dtype(dtype).itemsize
        self.check(self.L.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 16)), 0),
                   "cudaHostAlloc")
        buf = (ctypes.c_byte * max(nbytes, 16)).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype, count=int(n))

    def flush_l2(self):
        """Overwrite a 256 MiB buffer (twice the L2) so the next step starts cold."""
        if self.flush_ptr is None:
            p = ctypes.c_void_p()
            self.check(self.L.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(L2_FLUSH_BYTES)), "cudaMalloc")
            self.flush_ptr = p
        self.check(self.L.cudaMemset(self.flush_ptr, 1, ctypes.c_size_t(L2_FLUSH_BYTES)), "cudaMemset")
        self.sync()


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms.  start() returns
    once the first sample is in (nvidia-smi takes a while to start); a timed
    region shorter than the interval gets the sample taken right after it."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.n0 = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        t0 = time.time()
        while len(self.lines) <= self.n0 and time.time() - t0 < 1.0 and self.proc.poll() is None:
            time.sleep(0.005)
        in_region = max(0, len(self.lines) - self.n0)
        self.lines = self.lines[max(0, self.n0 - 1):]  # the last sample before the region and the ones after
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names[1:], f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "interval_ms": 50,
                "samples_after_start": in_region}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_fields(name):
    """The 'key: number' lines of the ncu summary profiles/<name>.md (the
    figures a bench line quotes from ncu), as a dict of floats."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    out = {}
    if not os.path.exists(p):
        return out
    for line in open(p):
        t = line.strip()
        if ":" not in t or t.startswith(("#", "|", "`")) or " " in t.split(":", 1)[0]:
            continue
        k, v = t.split(":", 1)
        try:
            out[k] = float(v.strip().split()[0])
        except (ValueError, IndexError):
            continue
    return out


def ncu_traffic(name):
    """DRAM bytes per launch recorded by the ncu summary profiles/<name>.md
    (line 'traffic_bytes_per_launch: N'), or None."""
    return profile_fields(name).get("traffic_bytes_per_launch")


# --------------------------------------------------------------- workloads --
def make_workload(name):
    import workloads as W
    if name == "single_large":
        inst = W.single_large(0)
        desc = ("1,000,000 vars / 4,000,000 propagators (planted solution, bounds scale 1e6) "
                "+ 20,000-link chain")
    elif name == "single_small":
        inst = W.single_small(0)
        desc = "1,000 vars / 3,000 propagators (planted solution, bounds scale 1e3)"
    elif name == "out_of_l2":
        inst = W.plain(4_000_000, 16_000_000, 10**6, 0)
        desc = ("4,000,000 vars / 16,000,000 propagators (planted solution, bounds scale 1e6, base mix); "
                "bytecode 256 MB + store 32 MB")
    else:
        raise ValueError(name)
    return inst, desc


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def dist_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------- CPU baseline --
def cpu_sample(inst, target_s=12.0, min_sweeps=1):
    """Gauss-Seidel sweeps of the oracle from the initial store (reference
    order), as many as fit in ~target_s; returns (execs/s, sweeps, seconds)."""
    from oracle import oracle as O
    s = inst.store()
    st, perm = O.install(inst.op, inst.x, inst.y, inst.z, s)
    op, x, y, z = (np.ascontiguousarray(a[perm]) for a in (inst.op, inst.x, inst.y, inst.z))
    t0 = time.perf_counter()
    O.sweeps(op, x, y, z, s, 1)
    one = time.perf_counter() - t0
    n = max(min_sweeps, int(target_s / max(one, 1e-9)) - 1)
    t0 = time.perf_counter()
    O.sweeps(op, x, y, z, s, n)
    dt = time.perf_counter() - t0
    return (n * inst.nprops) / dt, n + 1, dt + one, (n + 1) * inst.nprops / (dt + one)


def cpu_time_to_fixpoint(sec_per_sweep):
    """The reference loop's time to the fixpoint of the 1M / 4M + chain
    instance on one host core: its two parts share no variable, so the
    Gauss-Seidel loop over the whole instance needs the larger of the parts'
    sweep counts (each part run to its own fixpoint here, on the oracle),
    each sweep costing the measured seconds of a sweep of the whole instance."""
    import workloads as W
    from oracle import oracle as O
    rnd = W.single_large(0, chain=0)
    s = rnd.store()
    t0 = time.perf_counter()
    rc, info = O.install_and_fixpoint(rnd.op, rnd.x, rnd.y, rnd.z, s)
    t_rnd = time.perf_counter() - t0
    empty = W.Instance(np.zeros(0, np.int32), np.zeros(0, np.int32), *(np.zeros(0, np.int32),) * 4)
    chain = W.add_chain(empty, 20_000, 1_000_000, 0)
    c = chain.store()
    t0 = time.perf_counter()
    rc2, cinfo = O.install_and_fixpoint(chain.op, chain.x, chain.y, chain.z, c)
    t_chain = time.perf_counter() - t0
    sweeps = max(info["sweeps"], cinfo["sweeps"])
    return {"seconds": sweeps * sec_per_sweep, "sweeps": sweeps, "random_part_sweeps": info["sweeps"],
            "chain_sweeps": cinfo["sweeps"], "seconds_per_sweep": sec_per_sweep, "cores": 1,
            "method": "sweeps to the fixpoint (the larger of the random part's and the chain's, each run "
                      "to its fixpoint on the oracle: %.1f s + %.1f s) x the measured seconds of one sweep "
                      "of the whole instance" % (t_rnd, t_chain)}


def out_of_l2_record(cr, hbm):
    """AC-1 and event fixpoints of a 4,000,000-var / 16,000,000-propagator
    instance (256 MB of bytecode + 32 MB of store: more than twice the 129 MB
    L2), where the per-round bytecode stream comes from HBM."""
    import pirgpu
    import workloads as W
    t0 = time.perf_counter()
    inst = W.plain(4_000_000, 16_000_000, 10**6, 0)
    gen_s = time.perf_counter() - t0
    ctx = pirgpu.Context(0)
    ctx.load_store(inst.lb, inst.ub)
    t0 = time.perf_counter()
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    tell_s = time.perf_counter() - t0
    snap = ctx.snapshot()
    tuned = ctx.autotune(16)
    runs = []
    for k in range(4):  # one warm-up, three timed, the L2 flushed before each
        ctx.restore(snap)
        cr.flush_l2()
        rc, st = ctx.fixpoint()
        if rc != pirgpu.OK:
            raise RuntimeError("out-of-L2 fixpoint status %s" % pirgpu.STATUS[rc])
        if k:
            runs.append(st)
    ac1_lb, ac1_ub = ctx.read_store()
    best = min(runs, key=lambda r: r["device_ms"])
    ctx.restore(snap)
    cr.flush_l2()
    rc, ev = ctx.fixpoint(sched=pirgpu.SCHED_EVENTS)
    ev_lb, ev_ub = ctx.read_store()
    same = bool(rc == pirgpu.OK and np.array_equal(ac1_lb, ev_lb) and np.array_equal(ac1_ub, ev_ub))
    alg = best["executions"] * ALG_BYTES_PER_EXEC + best["narrowed"] * ALG_BYTES_PER_JOIN
    achieved = alg / (best["device_ms"] / 1e3) / 1e9
    prof = profile_fields("persistent_fixpoint_out_of_l2")
    rec = {
        "workload": "4,000,000 vars / 16,000,000 propagators (planted solution, bounds scale 1e6, base mix); "
                    "bytecode 256 MB + store 32 MB",
        "value": best["executions"] / (best["device_ms"] / 1e3), "unit": "executions/s",
        "time_to_fixpoint_ms": best["device_ms"], "rounds": best["rounds"], "executions": best["executions"],
        "kernel_variant": list(tuned),
        "roofline": {"bound": "l2", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "dram_bytes_per_round": prof.get("dram_bytes_per_round"),
                     "dram_gbs_ncu": prof.get("dram_gbs"),
                     "note": "the 256 MB bytecode streams from HBM every round (dram_bytes_per_round); the "
                             "interval gathers hit the L2-resident 32 MB store, and the round is bound by the "
                             "L1/L2 gather path and issue (profiles/persistent_fixpoint_out_of_l2.md)",
                     "bytes_model": "40 B per execution + 4 B per narrowing join"},
        "events_schedule": {"time_to_fixpoint_ms": ev["device_ms"], "executions": ev["executions"],
                            "rounds": ev["rounds"], "certify_narrowed": ev["certify_narrowed"],
                            "store_equal_to_ac1": same},
        "l2": "flushed before each fixpoint (256 MiB cudaMemset)", "generate_s": gen_s, "tell_s": tell_s,
    }
    ctx.close()
    return rec


def _nodes_bit_exact(ctx, base, off, var, lb, ub, m):
    """Nodes 0 .. m-1 of a batch: GPU stores (pir_fixpoint_nodes, event
    schedule) against the oracle run node by node on the host's threads."""
    import pirgpu
    from oracle import oracle as O
    o = off[:m + 1]
    status, olb, oub, _, _ = ctx.fixpoint_nodes(o, var, lb, ub, sched=pirgpu.SCHED_EVENTS)
    op, x, y, z = ctx.bytecode()
    bs = np.ascontiguousarray(np.stack(base, 1))
    ost, ostore, _ = O.fixpoint_nodes(op, x, y, z, bs, o, var, lb, ub, threads=os.cpu_count() or 1)
    eq = 0
    for j in range(m):
        if status[j] == ost[j] and (ost[j] != O.OK or (np.array_equal(olb[j], ostore[j, :, 0]) and
                                                       np.array_equal(oub[j], ostore[j, :, 1]))):
            eq += 1
    return {"nodes_checked": m, "nodes_equal": eq, "failed_nodes": int((ost == O.FAILED).sum())}


def _nodes_sequential(ctx, snap, off, var, lb, ub, sample, sched):
    """The plain single-instance GPU loop, node after node: restore the base,
    embed the node's tightenings, pir_fixpoint (AC-1 rounds or the event
    schedule with its certifying sweep)."""
    import pirgpu
    dev, ex, t0 = 0.0, 0, time.perf_counter()
    for j in range(sample):
        ctx.restore(snap)
        ctx.embed_many(var[off[j]:off[j + 1]], lb[off[j]:off[j + 1]], ub[off[j]:off[j + 1]])
        rc, st = ctx.fixpoint(sched=sched)
        dev += st["device_ms"] / 1e3
        ex += st["executions"]
    wall = time.perf_counter() - t0
    ctx.restore(snap)
    return {"nodes_per_s_device": sample / dev, "nodes_per_s_wall": sample / wall, "sample_nodes": sample,
            "executions_per_node": ex / sample}


def nodes_record(cr, args):
    """The batched-search-node workload (4,096 nodes over a 100,000-var /
    400,000-propagator base at its fixpoint) measured beside the default
    line: batched device nodes/s, the plain single-instance GPU loop node
    after node under both schedules, end to end through the C ABI, and an
    inline bit-exact check of a sample of nodes against the oracle."""
    import pirgpu
    ctx, base, (blb, bub), off, var, lb, ub = _nodes_workload()
    nn = len(off) - 1
    tuned = ctx.autotune_nodes(off, var, lb, ub)
    for _ in range(3):
        ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=pirgpu.SCHED_EVENTS)
        cr.flush_l2()
    runs = []
    for _ in range(5):
        status, _, _, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=pirgpu.SCHED_EVENTS)
        runs.append(st)
        cr.flush_l2()
    dev_ms = float(np.median([r["device_ms"] for r in runs]))
    value = nn / (dev_ms / 1e3)
    st = runs[0]
    # the same batch without the per-node certifying sweeps (opts.certify < 0):
    # the node kernel's own rounds; the statuses must be the certified ones
    unc = []
    for _ in range(5):
        s_unc, _, _, _, st_unc = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=pirgpu.SCHED_EVENTS,
                                                    certify=-1)
        unc.append(st_unc)
        cr.flush_l2()
    unc_ms = float(np.median([r["device_ms"] for r in unc]))
    _, _, _, _, st_ac1 = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=pirgpu.SCHED_AC1)
    snap = ctx.snapshot()
    ctx.autotune(8)
    ctx.restore(snap)
    seq_ac1 = _nodes_sequential(ctx, snap, off, var, lb, ub, args.seq_nodes, pirgpu.SCHED_AC1)
    seq_ev = _nodes_sequential(ctx, snap, off, var, lb, ub, args.seq_nodes, pirgpu.SCHED_EVENTS)
    p_off, p_var, p_lb, p_ub = (cr.pinned(len(a)) for a in (off, var, lb, ub))
    p_off[:], p_var[:], p_lb[:], p_ub[:] = off, var, lb, ub
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        ctx.fixpoint_nodes(p_off, p_var, p_lb, p_ub, want_stores=False, sched=pirgpu.SCHED_EVENTS)
        ts.append(time.perf_counter() - t0)
    e2e_t = float(np.median(ts))
    # end to end through the staged batches (pir_nodes_stage: the batch written
    # into the context's pinned staging, one CUDA graph per batch), the call a
    # solver's own search loop makes; per node its status out
    # the batch sits in the staging as the plain path's inputs sit in pinned
    # buffers; every call copies it in and the statuses out (its CUDA graph)
    nt = int(off[-1])
    buf = ctx.nodes_stage(nn, nt, 0)
    buf[:nn + 1] = off
    buf[nn + 1:nn + 1 + nt] = var
    buf[nn + 1 + nt:nn + 1 + 2 * nt] = lb
    buf[nn + 1 + 2 * nt:] = ub
    ctx.fixpoint_nodes_staged(nn, nt, 0)  # builds the graph
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        ctx.fixpoint_nodes_staged(nn, nt, 0)
        ts.append(time.perf_counter() - t0)
    staged_t = float(np.median(ts))
    exact = _nodes_bit_exact(ctx, (blb, bub), off, var, lb, ub, min(nn, args.cpu_nodes))
    rec = {
        "workload": "nodes: 100,000 vars / 400,000 propagators (bounds scale 1e6) at its fixpoint, 4,096 nodes, "
                    "k ~ U[1,64] bisections of unfixed vars",
        "value": value, "unit": "nodes/s", "ms_per_batch": dev_ms, "schedule": "events (certified)",
        "node_kernel_variant": list(tuned), "executions_per_batch": st["executions"],
        "certify": {"executions": st["certify_executions"], "narrowed": st["certify_narrowed"]},
        "uncertified": {"ms_per_batch": unc_ms, "nodes_per_s": nn / (unc_ms / 1e3),
                        "executions_per_batch": unc[0]["executions"],
                        "statuses_equal_to_certified": bool(np.array_equal(s_unc, status))},
        "max_rounds": int(rounds.max()), "nodes_failed": int((status == pirgpu.FAILED).sum()),
        "batched_ac1": {"ms_per_batch": st_ac1["device_ms"], "nodes_per_s": nn / (st_ac1["device_ms"] / 1e3),
                        "executions_per_batch": st_ac1["executions"]},
        "sequential_ac1": seq_ac1, "sequential_events": seq_ev,
        "batched_over_sequential_ac1": value / seq_ac1["nodes_per_s_device"],
        "batched_over_sequential_events": value / seq_ev["nodes_per_s_device"],
        "e2e": {"value": nn / e2e_t, "unit": "nodes/s", "h2d_bytes_per_step": int(len(var) * 12 + len(off) * 4),
                "d2h_bytes_per_step": int(nn * 8),
                "over_sequential_events_wall": (nn / e2e_t) / seq_ev["nodes_per_s_wall"],
                "staged_graph": {"value": nn / staged_t, "unit": "nodes/s",
                                 "note": "pir_fixpoint_nodes_staged on a batch already written into the "
                                         "context's pinned staging (pir_nodes_stage), as the plain path's inputs "
                                         "are already in pinned buffers: one CUDA graph per batch (counters "
                                         "cleared, batch copied in, node kernel, statuses copied out)"}},
        "bit_exact": exact,
        "l2": "flushed between batches (256 MiB cudaMemset); median of 5 batches, CUDA events",
    }
    ctx.close()
    return rec


# ------------------------------------------------------------------- ours ---
def run_ours(args):
    import pirgpu
    ws, rank, local = dist_env()
    dist = dist_init(ws)
    cr = Cudart()
    cr.set_device(local)
    inst, desc = make_workload(args.workload)
    ctx = pirgpu.Context(local)
    ctx.load_store(inst.lb, inst.ub)
    t0 = time.perf_counter()
    ctx.tell(inst.op, inst.x, inst.y, inst.z)  # install: the (op, y, x, z) sort, on the device from 65,536 on
    tell_s = time.perf_counter() - t0
    snap = ctx.snapshot()
    nprops = ctx.num_deductions()
    init_lb, init_ub = ctx.read_store()  # store after install (reified targets met with [0,1])
    kw = dict(mode=args.mode, max_rounds=args.max_rounds, variant=args.variant)
    tuned = None
    if args.mode in (0, 1) and args.variant == 0:
        tuned = ctx.autotune(64)
        ctx.restore(snap)
    ok = (pirgpu.OK, pirgpu.TIMEOUT) if args.max_rounds else (pirgpu.OK,)

    def step():
        ctx.restore(snap)
        rc, st = ctx.fixpoint(**kw)
        if rc not in ok:
            raise RuntimeError("fixpoint status %s" % pirgpu.STATUS[rc])
        return st

    for _ in range(args.warmup):
        step()
        cr.flush_l2()
    if dist:
        dist.barrier()
    cr.sync()
    clk = ClockSampler(local)
    clk.start()
    stats = []
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        stats.append(step())
        cr.flush_l2()
    cr.sync()
    wall = time.perf_counter() - wall0
    clocks = clk.stop()
    dev_ms = sum(s["device_ms"] for s in stats)
    execs = sum(s["executions"] for s in stats)
    joins = sum(s["narrowed"] for s in stats)
    rounds = [s["rounds"] for s in stats]
    t_max = dist_max(dist, dev_ms / 1e3)
    execs_all = dist_sum(dist, execs)
    value = execs_all / t_max
    ac1_store = ctx.read_store() if args.max_rounds == 0 else None

    # end to end through the C ABI: pinned host store in, fixpoint, store out
    lb_h = cr.pinned(inst.nvars)
    ub_h = cr.pinned(inst.nvars)
    lb_o = cr.pinned(inst.nvars)
    ub_o = cr.pinned(inst.nvars)
    lb_h[:] = init_lb
    ub_h[:] = init_ub
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 3))
    e2e_execs = 0
    if dist:
        dist.barrier()
    cr.sync()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.load_store(lb_h, ub_h)
        rc, st = ctx.fixpoint(**kw)
        ctx._check(ctx._L.pir_read_store(ctx.h, lb_o.ctypes.data_as(pirgpu._I32P),
                                         ub_o.ctypes.data_as(pirgpu._I32P)))
        e2e_execs += st["executions"]
    cr.sync()
    e2e_t = dist_max(dist, time.perf_counter() - t0)
    e2e_value = dist_sum(dist, e2e_execs) / e2e_t if e2e_steps else None

    # the same fixpoint under the event schedule (only the propagators of the
    # variables narrowed in the previous round run), for its time to fixpoint
    ev = None
    if args.mode in (0, 1) and args.max_rounds == 0 and not args.no_events:
        ev_runs = []
        first_wall = None
        for _ in range(3):
            ctx.restore(snap)
            cr.flush_l2()
            t0 = time.perf_counter()
            rc, st = ctx.fixpoint(sched=pirgpu.SCHED_EVENTS)
            if first_wall is None:  # includes building the adjacency and the path segments
                first_wall = time.perf_counter() - t0
            if rc != pirgpu.OK:
                raise RuntimeError("event fixpoint status %s" % pirgpu.STATUS[rc])
            ev_runs.append(st)
        ev_store = ctx.read_store()
        st = sorted(ev_runs, key=lambda s: s["device_ms"])[1]  # median of 3
        ev = {"time_to_fixpoint_ms": st["device_ms"], "first_call_wall_ms": first_wall * 1e3,
              "executions": st["executions"], "rounds": st["rounds"],
              "certify_executions": st["certify_executions"], "certify_narrowed": st["certify_narrowed"],
              "ac1_over_events_time": (dev_ms / args.steps) / st["device_ms"],
              "ac1_over_events_executions": (execs / args.steps) / max(st["executions"], 1),
              "store_equal_to_ac1": bool(np.array_equal(ev_store[0], ac1_store[0]) and
                                         np.array_equal(ev_store[1], ac1_store[1])),
              "fixpoint": "certified by a final sweep of every propagator; bit-exact vs the oracle in tests"}
    if rank != 0:
        return
    hbm, hbm_src = peaks()
    achieved = (execs * ALG_BYTES_PER_EXEC + joins * ALG_BYTES_PER_JOIN) / (dev_ms / 1e3) / 1e9
    prof = profile_fields("persistent_fixpoint_" + args.workload)
    traffic = prof.get("traffic_bytes_per_launch")
    cpu = None
    cpu_fix = None
    extras = ws == 1 and not args.no_cpu
    if extras:
        v, sw, secs, _ = cpu_sample(inst, args.cpu_seconds)
        cpu = {"value": v, "unit": "executions/s", "cores": 1, "kind": "port",
               "sample": "%d Gauss-Seidel sweeps (%d executions) of the same instance from its "
                         "initial store, %.1f s, 1 host thread" % (sw, sw * nprops, secs)}
        if args.workload == "single_large":
            cpu_fix = cpu_time_to_fixpoint(secs / sw)
            cpu_fix["over_gpu_ac1"] = cpu_fix["seconds"] / (dev_ms / args.steps / 1e3)
            if ev:
                cpu_fix["over_gpu_events"] = cpu_fix["seconds"] / (ev["time_to_fixpoint_ms"] / 1e3)
    l2_resident = args.workload == "single_large"
    roofline = {"bound": "l2" if l2_resident else "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic,
                "peak_source": hbm_src + " (MEASURED_PEAKS.json hbm_gbs)",
                "bytes_model": "40 B per execution + 4 B per narrowing join"}
    if l2_resident:
        roofline["note"] = ("the 64 MB bytecode and 8.3 MB store stay in the 129 MB L2 across rounds: DRAM traffic "
                            "is the 'traffic' figure; frac is against the HBM copy peak, the only measured "
                            "memory peak; the ncu L2 figures are in 'l2'")
        roofline["l2"] = {k: prof.get(k) for k in ("l2_hit_rate_pct", "lts_throughput_pct", "l1tex_throughput_pct",
                                                   "issue_active_pct", "dram_bytes_per_round")}
    more = {}
    if ws == 1 and args.workload == "single_large" and not args.no_extras:
        more["out_of_l2"] = out_of_l2_record(cr, hbm)
        more["nodes"] = nodes_record(cr, args)
        more["uneven"] = uneven_record(cr, args)
        more["learned"] = learned_record(args)
    out = {
        "metric": "propagator executions/sec", "value": value, "unit": "executions/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic: seeded generator, planted-solution instance",
        "config": {"workload": args.workload + ": " + desc, "nvars": inst.nvars,
                   "propagators": int(nprops), "parallelism": "replicas" if ws > 1 else "single",
                   "mode": ["auto", "persistent", "hostloop", "smem"][args.mode],
                   "l2": "flushed between steps (256 MiB cudaMemset); step timed with CUDA events",
                   "rounds_per_step": rounds[0], "fixpoint": "bit-exact vs CPU oracle in tests",
                   "kernel_variant": list(tuned) if tuned else args.variant},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "executions/s",
                "h2d_bytes_per_step": int(inst.nvars * 8), "d2h_bytes_per_step": int(inst.nvars * 8),
                "steps": e2e_steps},
        "gpu_launches": args.steps * (1 if args.mode in (0, 1, 3) else rounds[0] * 2),
        "clocks": clocks,
        "time_to_fixpoint_ms": dev_ms / args.steps,
        "tell_ms": tell_s * 1e3,
        "events_schedule": ev,
        "cpu_time_to_fixpoint": cpu_fix,
        "wall_s": wall,
    }
    out.update(more)
    print(json.dumps(out), flush=True)


def _nodes_workload():
    import workloads as W
    import pirgpu
    base = W.plain(100_000, 400_000, 10**6, 0)
    ctx = pirgpu.Context(dist_env()[2])
    ctx.load_store(base.lb, base.ub)
    ctx.tell(base.op, base.x, base.y, base.z)
    rc, _ = ctx.fixpoint()
    if rc != pirgpu.OK:
        raise RuntimeError("base instance failed")
    blb, bub = ctx.read_store()
    _, off, var, lb, ub = W.nodes(100_000, 400_000, 4096, 0, 64, base_store=(blb, bub))
    return ctx, base, (blb, bub), off, var, lb, ub


def run_nodes(args):
    """Batched search nodes: 4,096 nodes over a 100,000-var / 400,000-propagator
    base at its fixpoint, each bisecting k ~ U[1, 64] variables."""
    import pirgpu
    import shard
    ws, rank, local = dist_env()
    dist = dist_init(ws)
    cr = Cudart()
    cr.set_device(local)
    ctx, base, (blb, bub), off, var, lb, ub = _nodes_workload()
    nn_all = len(off) - 1
    if ws > 1:
        # this rank's nodes (cost-balanced partition, no collective on the data path)
        parts = shard.lpt_partition(shard.node_costs(off), ws)
        off, var, lb, ub = shard.select_nodes(off, var, lb, ub, parts[rank])
    nn = len(off) - 1
    sched = pirgpu.SCHED_EVENTS if args.node_sched == "events" else pirgpu.SCHED_AC1
    tuned = ctx.autotune_nodes(off, var, lb, ub) if sched == pirgpu.SCHED_EVENTS else None
    for _ in range(args.warmup):
        ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=sched)
        cr.flush_l2()
    if dist:
        dist.barrier()
    cr.sync()
    clk = ClockSampler(local)
    clk.start()
    runs = []
    for _ in range(args.steps):
        status, _, _, rounds, st = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=sched)
        runs.append(st)
        cr.flush_l2()
    clocks = clk.stop()
    dev_s = sum(r["device_ms"] for r in runs) / 1e3
    t_max = dist_max(dist, dev_s)
    value = nn_all * args.steps / t_max
    n_ok = int(dist_sum(dist, int((status == 0).sum())))
    n_failed = int(dist_sum(dist, int((status == 1).sum())))
    max_rounds = int(dist_max(dist, int(rounds.max()) if nn else 0))
    if rank != 0:
        return
    extras = ws == 1  # comparison runs and the CPU baseline: rank 0 at N=1 only
    # the batched AC-1 kernel, for reference
    st_ac1 = {"device_ms": None, "executions": None}
    if extras and not args.no_cpu:
        _, _, _, _, st_ac1 = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=pirgpu.SCHED_AC1)
    execs = sum(r["executions"] for r in runs)
    joins = sum(r["narrowed"] for r in runs)
    snap = ctx.snapshot()
    # the first batch after the base store changed (working stores reloaded,
    # entailment at the base recomputed); restore() marks the store changed
    first_ms = None
    if extras:
        ctx.restore(snap)
        cr.flush_l2()
        _, _, _, _, st_first = ctx.fixpoint_nodes(off, var, lb, ub, want_stores=False, sched=sched)
        first_ms = st_first["device_ms"]
    # the plain single-instance GPU loop, node after node (sample), under
    # AC-1 rounds and under the event schedule
    sample = min(nn, args.seq_nodes) if extras else 0
    seq_ac1 = seq_ev = None
    if sample:
        ctx.autotune(8)
        ctx.restore(snap)
        seq_ac1 = _nodes_sequential(ctx, snap, off, var, lb, ub, sample, pirgpu.SCHED_AC1)
        seq_ev = _nodes_sequential(ctx, snap, off, var, lb, ub, sample, pirgpu.SCHED_EVENTS)
    # end to end through the C ABI: host tightenings in, per-node status and
    # rounds out (what a search driver reads; the sequential loop reads the
    # same), and separately with every node's store downloaded as well
    # (inputs from pinned host buffers, filled before the timed calls)
    e2e_t = e2e_stores_t = None
    if extras and not args.no_e2e:
        p_off, p_var, p_lb, p_ub = (cr.pinned(len(a)) for a in (off, var, lb, ub))
        p_off[:], p_var[:], p_lb[:], p_ub[:] = off, var, lb, ub
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            ctx.fixpoint_nodes(p_off, p_var, p_lb, p_ub, want_stores=False, sched=sched)
            ts.append(time.perf_counter() - t0)
        e2e_t = float(np.median(ts))
        t0 = time.perf_counter()
        ctx.fixpoint_nodes(p_off, p_var, p_lb, p_ub, want_stores=True, sched=sched)
        e2e_stores_t = time.perf_counter() - t0
    hbm, hbm_src = peaks()
    achieved = (execs * ALG_BYTES_PER_EXEC + joins * ALG_BYTES_PER_JOIN) / dev_s / 1e9
    cpu = None
    exact = None
    if extras and not args.no_cpu:
        from oracle import oracle as O
        exact = _nodes_bit_exact(ctx, (blb, bub), off, var, lb, ub, min(nn, args.cpu_nodes))
        op, x, y, z = ctx.bytecode()
        bs = np.ascontiguousarray(np.stack([blb, bub], 1))
        m = min(nn, args.cpu_nodes)
        th = os.cpu_count() or 1
        t0 = time.perf_counter()
        ost, _, _ = O.fixpoint_nodes(op, x, y, z, bs, off[:m + 1], var, lb, ub, threads=th)
        ct = time.perf_counter() - t0
        cpu = {"value": m / ct, "unit": "nodes/s", "cores": th, "kind": "port",
               "sample": "%d nodes, Gauss-Seidel per node, %d host threads, %.1f s" % (m, th, ct)}
    out = {
        "metric": "batched nodes/sec", "value": value, "unit": "nodes/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic: planted-solution base instance at its fixpoint, bisected nodes",
        "config": {"workload": "nodes: 100,000 vars / 400,000 propagators (bounds scale 1e6) at its fixpoint, 4,096 nodes, k ~ U[1,64] bisections of unfixed vars",
                   "parallelism": "nodes sharded over %d ranks (cost-balanced, no collective)" % ws
                   if ws > 1 else "single",
                   "nodes_ok": n_ok, "nodes_failed": n_failed,
                   "max_rounds": max_rounds, "mean_rounds_rank0": float(rounds.mean()) if nn else 0.0,
                   "schedule": args.node_sched, "executions_per_step": execs // args.steps,
                   "node_kernel_variant": list(tuned) if tuned else None,
                   "batched_ac1_ms": st_ac1["device_ms"], "batched_ac1_executions": st_ac1["executions"],
                   "first_batch_on_new_base_ms": first_ms},
        "sequential_ac1": seq_ac1, "sequential_events": seq_ev,
        "batched_over_sequential_ac1": value / seq_ac1["nodes_per_s_device"] if seq_ac1 else None,
        "batched_over_sequential_events": value / seq_ev["nodes_per_s_device"] if seq_ev else None,
        "certify": {"executions": runs[0]["certify_executions"], "narrowed": runs[0]["certify_narrowed"]},
        "bit_exact": exact,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": ncu_traffic("nodes_events_4096_nodes"),
                     "peak_source": hbm_src},
        "cpu_baseline": cpu,
        "e2e": {"value": nn_all / e2e_t if e2e_t else None, "unit": "nodes/s",
                "h2d_bytes_per_step": int(len(var) * 12 + len(off) * 4),
                "d2h_bytes_per_step": int(nn * 8),
                "with_stores": {"value": nn_all / e2e_stores_t if e2e_stores_t else None,
                                "d2h_bytes_per_step": int(nn * len(blb) * 8)}},
        "gpu_launches": args.steps, "clocks": clocks,
    }
    print(json.dumps(out), flush=True)


def learned_measure(args):
    """Learned scheduler on search nodes of the 100,000-var / 400,000-propagator
    base: trained on change traces of the plain fixpoint of 1,024 nodes (up to
    1M samples), then run node by node (restore the base, embed the node's
    bisections, fixpoint) on 256 held-out nodes under AC-1, the event schedule,
    the learned frontier rounds (at the given wake fraction, a quarter, and
    everything woken) and the learned grid kernel; every result checked against
    AC-1's store.  Returns a dict."""
    import pirgpu
    ctx, base, (blb, bub), off, var, lb, ub = _nodes_workload()
    ntrain, ntest = 1024, 256
    t0 = time.perf_counter()
    ns, npos = ctx.sched_collect(off[:ntrain + 1], var, lb, ub, max_samples=1_000_000, keep_negative=0.01)
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = ctx.sched_train(epochs=args.epochs, batch=8192, lr=3e-3, pos_weight=4.0)
    t_train = time.perf_counter() - t0
    snap = ctx.snapshot()

    def run(sched, frac=0.0, **kw):
        ex, cex, dev, rounds, outs = 0, 0, 0.0, 0, []
        for j in range(ntrain, ntrain + ntest):
            ctx.restore(snap)
            ctx.embed_many(var[off[j]:off[j + 1]], lb[off[j]:off[j + 1]], ub[off[j]:off[j + 1]])
            rc, st = ctx.fixpoint(mode=1, sched=sched, wake_fraction=frac, **kw)
            ex += st["executions"]
            cex += st["certify_executions"]
            dev += st["device_ms"]
            rounds += st["rounds"]
            outs.append((rc, ctx.read_store()))
        return {"executions": ex, "certify_executions": cex, "device_ms": dev, "rounds": rounds}, outs

    def same_as(o0, o1):
        return sum(1 for (a, (l0, u0)), (b, (l1, u1)) in zip(o0, o1)
                   if a == b and (a != pirgpu.OK or (np.array_equal(l0, l1) and np.array_equal(u0, u1))))

    run(pirgpu.SCHED_AC1)  # warm-up
    ac1, o0 = run(pirgpu.SCHED_AC1)
    ev, oe = run(pirgpu.SCHED_EVENTS)
    lrn, o1 = run(pirgpu.SCHED_LEARNED, args.wake_fraction)
    quarter, oq = run(pirgpu.SCHED_LEARNED, 0.25)
    allw, oa = run(pirgpu.SCHED_LEARNED, 1.0)
    grid, og = run(pirgpu.SCHED_LEARNED, args.wake_fraction, local_frontier=-1)
    for r, o in ((ev, oe), (lrn, o1), (quarter, oq), (allw, oa), (grid, og)):
        r["bit_exact_nodes"] = same_as(o0, o)
    ctx.restore(snap)
    ctx.close()
    return {"ntrain": ntrain, "ntest": ntest, "samples": ns, "positives": npos, "collect_s": t_collect,
            "train_s": t_train, "loss": [float(v) for v in loss], "ac1": ac1, "events": ev, "learned": lrn,
            "quarter": quarter, "all_woken": allw, "grid": grid}


def learned_record(args):
    """The learned scheduler beside the single instance in the default line."""
    m = learned_measure(args)
    e0, e1 = m["ac1"]["executions"], m["learned"]["executions"]
    return {"workload": "learned: 100,000 vars / 400,000 propagators, trained on %d nodes, %d held-out nodes, "
                        "each restored, embedded and propagated" % (m["ntrain"], m["ntest"]),
            "value": e0 / max(e1, 1), "unit": "x fewer executions than AC-1",
            "wake_fraction": args.wake_fraction, "samples": m["samples"], "train_s": m["train_s"],
            "ac1": m["ac1"], "events": m["events"], "learned": m["learned"],
            "learned_all_woken": m["all_woken"], "learned_grid": m["grid"],
            "bit_exact_nodes": m["learned"]["bit_exact_nodes"], "nodes": m["ntest"],
            "wall_ratio_ac1_over_learned": m["ac1"]["device_ms"] / max(m["learned"]["device_ms"], 1e-9)}


def run_learned(args):
    """The learned scheduler's own line (see learned_measure)."""
    ws, rank, local = dist_env()
    cr = Cudart()
    cr.set_device(local)
    m = learned_measure(args)
    ac1, lrn, allw = m["ac1"], m["learned"], m["all_woken"]
    e0, e1, d0, d1 = ac1["executions"], lrn["executions"], ac1["device_ms"], lrn["device_ms"]
    out = {
        "metric": "propagator executions to fixpoint (learned vs AC-1)", "value": e0 / max(e1, 1),
        "unit": "x fewer executions", "n_gpus": 1, "steps": m["ntest"], "warmup": m["ntest"],
        "ms_per_step": d1 / m["ntest"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32 propagation, bf16 weights / fp32 accumulate scorer",
        "data": "synthetic: planted-solution base at its fixpoint, bisected nodes",
        "config": {"workload": "learned: 100,000 vars / 400,000 propagators, trained on %d nodes, tested on %d "
                               "held-out nodes" % (m["ntrain"], m["ntest"]),
                   "samples": m["samples"], "positives": m["positives"], "collect_s": m["collect_s"],
                   "train_s": m["train_s"], "epochs": args.epochs, "loss": m["loss"],
                   "wake_fraction": args.wake_fraction},
        "ac1": ac1,
        "events": m["events"],
        "learned": lrn,
        "learned_wake_quarter": dict(m["quarter"], note="the frontier rounds waking at least a quarter of the frontier"),
        "learned_all_woken": dict(allw, note="the same frontier rounds with every entry woken: what the network "
                                             "adds over the frontier alone"),
        "learned_grid": dict(m["grid"], note="the grid kernel: every propagator scored every round"),
        "wall_ratio_ac1_over_learned": d0 / max(d1, 1e-9),
        "wall_ratio_events_over_learned": m["events"]["device_ms"] / max(d1, 1e-9),
        "executions_all_woken_over_learned": allw["executions"] / max(e1, 1),
        "bit_exact_nodes": lrn["bit_exact_nodes"], "nodes": m["ntest"],
        "gpu_launches": m["ntest"],  # one learned fixpoint launch per held-out node (the timed device time)
    }
    print(json.dumps(out), flush=True)


UNEVEN_DESC = ("uneven: 512 instances, propagators log-uniform [1e3, 2e5], vars = props/4, "
               "5% tdiv + 5% tmod")


def _uneven_pinned(cr, packed):
    """The packed instances in pinned host buffers (the stores are reset from
    lb0 / ub0 before every call)."""
    prop_off, var_off, op, x, y, z, lb0, ub0 = packed
    pinned = []
    for a in (op, x, y, z, lb0, ub0):
        b = cr.pinned(len(a))
        b[:] = a
        pinned.append(b)
    return (prop_off, var_off) + tuple(pinned) + (lb0, ub0)


def _uneven_time(cr, ctx, pk, sched, steps, warmup):
    """pir_fixpoint_instances from pinned host buffers (install, copies in and
    out inside each call), `steps` timed calls after `warmup`: device seconds
    (CUDA events around the kernels), wall seconds of the calls, per-instance
    device ms, the last call's statuses, stats and stores."""
    prop_off, var_off, op, x, y, z, lb, ub, lb0, ub0 = pk
    for _ in range(warmup):
        lb[:], ub[:] = lb0, ub0
        ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb, ub, sched=sched)
    cr.sync()
    runs, walls, per = [], [], []
    for _ in range(steps):
        lb[:], ub[:] = lb0, ub0
        t0 = time.perf_counter()
        status, rounds, ms, st = ctx.fixpoint_instances(prop_off, var_off, op, x, y, z, lb, ub, sched=sched)
        walls.append(time.perf_counter() - t0)
        runs.append(st)
        per.append(ms)
    return {"dev_s": sum(r["device_ms"] for r in runs) / 1e3, "wall_s": sum(walls), "per": np.concatenate(per),
            "status": status, "rounds": rounds, "executions": sum(r["executions"] for r in runs),
            "lb": lb.copy(), "ub": ub.copy()}


def _uneven_cpu(packed):
    """The oracle on every instance (install + Gauss-Seidel each) over the
    host's threads: (seconds, statuses, stores)."""
    from oracle import oracle as O
    prop_off, var_off, op, x, y, z, lb0, ub0 = packed
    s = np.ascontiguousarray(np.stack([lb0, ub0], 1))
    th = os.cpu_count() or 1
    t0 = time.perf_counter()
    ost, _ = O.fixpoint_instances(prop_off, var_off, op, x, y, z, s, threads=th)
    return time.perf_counter() - t0, th, ost, s


def _uneven_equal(r, packed, ost, s):
    """Instances whose status equals the oracle's and, when OK, whose store is
    the oracle's bit for bit."""
    var_off = packed[1]
    n = 0
    for j in range(len(ost)):
        if r["status"][j] != ost[j]:
            continue
        v0, v1 = var_off[j], var_off[j + 1]
        if ost[j] != 0 or (np.array_equal(r["lb"][v0:v1], s[v0:v1, 0]) and
                           np.array_equal(r["ub"][v0:v1], s[v0:v1, 1])):
            n += 1
    return n


def uneven_record(cr, args):
    """The uneven-instance workload beside the single instance in the default
    line: instances/s under the event-filtered rounds and under AC-1 (device
    time and end to end through the C ABI), p50 / p99 per-instance time, every
    instance checked against the oracle, which is also the CPU baseline."""
    import pirgpu
    import workloads as W
    t0 = time.perf_counter()
    insts = W.uneven(512, 1000, 200_000, 0)
    packed = W.pack(insts)
    gen_s = time.perf_counter() - t0
    n = len(insts)
    ctx = pirgpu.Context(0)
    pk = _uneven_pinned(cr, packed)
    steps = max(3, min(args.steps, 5))
    res = {name: _uneven_time(cr, ctx, pk, sched, steps, 2)
           for name, sched in (("events", pirgpu.SCHED_EVENTS), ("ac1", pirgpu.SCHED_AC1))}
    ctx.close()
    cpu_s, th, ost, s = _uneven_cpu(packed)
    hbm, _ = peaks()
    out = {"workload": UNEVEN_DESC, "propagators": int(packed[0][-1]), "generate_s": gen_s}
    for name, r in res.items():
        out[name] = {"value": n * steps / r["dev_s"], "unit": "instances/s", "ms_per_step": r["dev_s"] * 1e3 / steps,
                     "instance_ms_p50": float(np.percentile(r["per"], 50)),
                     "instance_ms_p99": float(np.percentile(r["per"], 99)),
                     "executions_per_step": r["executions"] // steps,
                     "max_rounds": int(r["rounds"].max()),
                     "roofline_frac": r["executions"] * ALG_BYTES_PER_EXEC / r["dev_s"] / 1e9 / hbm,
                     "e2e": {"value": n * steps / r["wall_s"], "unit": "instances/s",
                             "h2d_bytes_per_step": int(packed[0][-1] * 16 + packed[1][-1] * 8),
                             "d2h_bytes_per_step": int(packed[1][-1] * 8)},
                     "bit_exact": {"instances_checked": n, "instances_equal": _uneven_equal(r, packed, ost, s)}}
    out["events_over_ac1"] = res["ac1"]["dev_s"] / res["events"]["dev_s"]
    out["cpu_baseline"] = {"value": n / cpu_s, "unit": "instances/s", "cores": th, "kind": "port",
                           "sample": "all %d instances (install + Gauss-Seidel each), %d host threads, %.1f s"
                                     % (n, th, cpu_s)}
    out["schedule"] = "events: a round runs the propagators of the variables the previous round narrowed"
    out["l2"] = "not flushed: each step copies 387 MB of instances in, more than the 129 MB L2"
    return out


def run_uneven(args):
    """512 independent instances, propagators log-uniform in [1e3, 2e5]."""
    import pirgpu
    import shard
    import workloads as W
    ws, rank, local = dist_env()
    dist = dist_init(ws)
    cr = Cudart()
    cr.set_device(local)
    insts_all = W.uneven(512, 1000, 200_000, 0)
    n_all = len(insts_all)
    packed = W.pack(insts_all)
    total_props = int(packed[0][-1])
    if ws > 1:
        # this rank's instances (cost-balanced partition, no collective on the data path)
        parts = shard.lpt_partition(shard.instance_costs(packed[0]), ws)
        packed = shard.select_instances(*packed, parts[rank])
    sched = {"events": pirgpu.SCHED_EVENTS, "ac1": pirgpu.SCHED_AC1}[args.inst_sched]
    ctx = pirgpu.Context(local)
    pk = _uneven_pinned(cr, packed)
    if dist:
        dist.barrier()
    clk = ClockSampler(local)
    clk.start()
    r = _uneven_time(cr, ctx, pk, sched, args.steps, args.warmup)
    clocks = clk.stop()
    t_max = dist_max(dist, r["dev_s"])
    wall_max = dist_max(dist, r["wall_s"])
    n_failed = int(dist_sum(dist, int((r["status"] == 1).sum())))
    per_all = shard.gather_to_root(dist, r["per"])
    if rank != 0:
        return
    per_all = np.concatenate(per_all)
    hbm, hbm_src = peaks()
    achieved = r["executions"] * ALG_BYTES_PER_EXEC / r["dev_s"] / 1e9
    cpu = None
    if ws == 1 and not args.no_cpu:
        ct, th, ost, s = _uneven_cpu(packed)
        cpu = {"value": n_all / ct, "unit": "instances/s", "cores": th, "kind": "port",
               "sample": "all %d instances (install + Gauss-Seidel each), %d host threads, %.1f s" % (n_all, th, ct),
               "instances_equal": _uneven_equal(r, packed, ost, s)}
    prof = "instances_cluster_uneven_512" if args.inst_sched == "ac1" else "instances_events_uneven_512"
    out = {
        "metric": "batched instances/sec", "value": n_all * args.steps / t_max, "unit": "instances/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic: planted-solution instances",
        "config": {"workload": UNEVEN_DESC, "propagators": total_props, "schedule": args.inst_sched,
                   "parallelism": "instances sharded over %d ranks (cost-balanced, no collective)" % ws
                   if ws > 1 else "single",
                   "instance_ms_p50": float(np.percentile(per_all, 50)),
                   "instance_ms_p99": float(np.percentile(per_all, 99)),
                   "executions_per_step": r["executions"] // args.steps,
                   "failed": n_failed},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": ncu_traffic(prof), "peak_source": hbm_src},
        "cpu_baseline": cpu,
        "e2e": {"value": n_all * args.steps / wall_max, "unit": "instances/s",
                "h2d_bytes_per_step": int(packed[0][-1] * 16 + packed[1][-1] * 8),
                "d2h_bytes_per_step": int(packed[1][-1] * 8)},
        # per step: store pack, the cluster kernel, the one-CTA-per-instance kernel, store unpack
        "gpu_launches": 4 * args.steps, "clocks": clocks,
    }
    print(json.dumps(out), flush=True)


def run_search(args):
    """The search driver on n-queens (all solutions, bisection of the first
    unfixed queen): nodes propagated per second; the CPU oracle's depth-first
    search of the same tree beside it."""
    import pirgpu
    import workloads as W
    ws, rank, local = dist_env()
    cr = Cudart()
    cr.set_device(local)
    n = args.queens
    inst = W.queens(n)
    dec = np.arange(n, dtype=np.int32)
    ctx = pirgpu.Context(local)
    ctx.load_store(inst.lb, inst.ub)
    ctx.tell(inst.op, inst.x, inst.y, inst.z)
    for _ in range(args.warmup):
        ctx.search(dec)
    clk = ClockSampler(local)
    clk.start()
    runs, walls = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        status, _, st = ctx.search(dec)
        walls.append(time.perf_counter() - t0)
        runs.append(st)
    clocks = clk.stop()
    st = runs[0]
    dev_s = sum(r["device_ms"] for r in runs) / 1e3
    nodes = sum(r["nodes"] for r in runs)
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        s = inst.store()
        _, perm = O.install(inst.op, inst.x, inst.y, inst.z, s)
        cap = args.cpu_search_nodes
        t0 = time.perf_counter()
        rc, _, info = O.search(inst.op[perm], inst.x[perm], inst.y[perm], inst.z[perm], s, dec, max_nodes=cap)
        ct = time.perf_counter() - t0
        cpu = {"value": info["nodes"] / ct, "unit": "nodes/s", "cores": 1, "kind": "port",
               "sample": "%s: %d nodes of the same depth-first tree (%d solutions), Gauss-Seidel per node, "
                         "1 host thread, %.1f s" % ("the whole tree" if rc == O.OK else "the first nodes",
                                                    info["nodes"], info["solutions"], ct)}
    out = {
        "metric": "search nodes/sec", "value": nodes / dev_s, "unit": "nodes/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(walls) * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic: the %d-queens model" % n,
        "config": {"workload": "search: %d-queens, all solutions, bisection of the first unfixed queen, "
                               "4,096 open nodes per launch" % n,
                   "nodes": st["nodes"], "failures": st["failures"], "solutions": st["solutions"],
                   "launches": st["launches"], "max_depth": st["max_depth"],
                   "device_ms_per_search": dev_s * 1e3 / args.steps},
        "roofline": None,
        "cpu_baseline": cpu,
        "e2e": {"value": nodes / sum(walls), "unit": "nodes/s", "h2d_bytes_per_step": st["h2d_bytes"],
                "d2h_bytes_per_step": st["d2h_bytes"], "note": "whole pir_search calls: host bookkeeping, "
                                                               "tightenings in and watched bounds out per launch"},
        "gpu_launches": st["launches"] * args.steps, "clocks": clocks,
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- PC trees --
def _pc_workload(args):
    import workloads as W
    tape, roots, lb, ub, _ = W.pc_mix(args.pc_vars, args.pc_props, seed=0)
    kinds = tape[:, 0]
    leaves = int(np.isin(kinds, [0, 16, 17]).sum())  # VAR, PVAR, NVAR nodes
    desc = ("PC trees: %d vars / %d formula propagators (40%% 4-term linear <=, 30%% reified "
            "differences, 20%% disjunctive temporal, 10%% max equalities; planted solution, bounds "
            "scale 1e3), %d tape nodes" % (args.pc_vars, args.pc_props, len(tape)))
    return tape, roots, lb, ub, leaves, desc


def run_pc(args):
    """Fixpoint of the PC tree propagators (pc_fixpoint): executions/s."""
    import pirgpu
    ws, rank, local = dist_env()
    dist = dist_init(ws)
    cr = Cudart()
    cr.set_device(local)
    tape, roots, lb, ub, leaves, desc = _pc_workload(args)
    nvars, nprops, nnodes = len(lb), len(roots), len(tape)
    ctx = pirgpu.Context(local)
    ctx.load_store(lb, ub)
    ctx.pc_tell(tape, roots)
    snap = ctx.snapshot()

    def step():
        ctx.restore(snap)
        rc, st = ctx.pc_fixpoint(max_rounds=args.max_rounds)
        if rc not in ((pirgpu.OK, pirgpu.TIMEOUT) if args.max_rounds else (pirgpu.OK,)):
            raise RuntimeError("pc fixpoint status %s" % pirgpu.STATUS[rc])
        return st

    for _ in range(args.warmup):
        step()
        cr.flush_l2()
    if dist:
        dist.barrier()
    cr.sync()
    clk = ClockSampler(local)
    clk.start()
    stats = []
    for _ in range(args.steps):
        stats.append(step())
        cr.flush_l2()
    cr.sync()
    clocks = clk.stop()
    dev_ms = sum(s["device_ms"] for s in stats)
    execs = sum(s["executions"] for s in stats)
    joins = sum(s["narrowed"] for s in stats)
    rounds = stats[0]["rounds"]
    t_max = dist_max(dist, dev_ms / 1e3)
    value = dist_sum(dist, execs) / t_max

    # the same fixpoint under the event schedule (a round runs only the
    # formulas whose variables the previous round narrowed)
    ev_runs = []
    for _ in range(2):
        ctx.restore(snap)
        rc, st = ctx.pc_fixpoint(sched=pirgpu.SCHED_EVENTS)
        if rc != pirgpu.OK:
            raise RuntimeError("pc event fixpoint status %s" % pirgpu.STATUS[rc])
        ev_runs.append(st)
        cr.flush_l2()
    evb = min(ev_runs, key=lambda x: x["device_ms"])
    ev = {"time_to_fixpoint_ms": evb["device_ms"], "executions": evb["executions"], "rounds": evb["rounds"],
          "full_over_events_time": (dev_ms / args.steps) / evb["device_ms"],
          "full_over_events_executions": (execs / args.steps) / max(evb["executions"], 1),
          "fixpoint": "identical to the full rounds (same rounds and stores, tested)"}

    lb_h, ub_h, lb_o, ub_o = (cr.pinned(nvars) for _ in range(4))
    lb_h[:] = lb
    ub_h[:] = ub
    e2e_steps = 0 if args.no_e2e else max(1, min(args.steps, 3))
    e2e_execs = 0
    cr.sync()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.load_store(lb_h, ub_h)
        rc, st = ctx.pc_fixpoint()
        ctx._check(ctx._L.pir_read_store(ctx.h, lb_o.ctypes.data_as(pirgpu._I32P),
                                         ub_o.ctypes.data_as(pirgpu._I32P)))
        e2e_execs += st["executions"]
    cr.sync()
    e2e_t = dist_max(dist, time.perf_counter() - t0)
    e2e_value = dist_sum(dist, e2e_execs) / e2e_t if e2e_steps else None
    if rank != 0:
        return
    # bytes a round must move: every tree node once (16 B), every variable leaf
    # once (8 B), the round's store copy (B -> A, 16 B per variable); per
    # fixpoint the initial copy (16 B per variable); 4 B per narrowing join
    per_round = nnodes * 16 + leaves * 8 + nvars * 16
    alg_bytes = args.steps * (rounds * per_round + nvars * 16) + joins * 4
    hbm, hbm_src = peaks()
    achieved = alg_bytes / (dev_ms / 1e3) / 1e9
    cpu = None
    if ws == 1 and not args.no_cpu:
        from oracle import oracle as O
        s = np.ascontiguousarray(np.stack([lb, ub], 1))
        order = O.pc_order(tape, roots)
        t0 = time.perf_counter()
        rc, info = O.pc_fixpoint(tape, order, s)
        dt = time.perf_counter() - t0
        cpu = {"value": info["execs"] / dt, "unit": "executions/s", "cores": 1, "kind": "port",
               "sample": "the whole Gauss-Seidel fixpoint of the same instance (%d sweeps, %d executions), "
                         "%.1f s, 1 host thread" % (info["sweeps"], info["execs"], dt)}
    out = {
        "metric": "propagator executions/sec", "value": value, "unit": "executions/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic: seeded generator, planted-solution instance",
        "config": {"workload": "pc: " + desc, "nvars": nvars, "propagators": nprops, "tape_nodes": nnodes,
                   "parallelism": "replicas" if ws > 1 else "single",
                   "schedule": "Jacobi rounds, one cooperative launch",
                   "l2": "flushed between steps (256 MiB cudaMemset); step timed with CUDA events",
                   "rounds_per_step": rounds, "fixpoint": "bit-exact vs the CPU oracle in tests"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": ncu_traffic("pc_fixpoint_pc"),
                     "peak_source": hbm_src + " (MEASURED_PEAKS.json hbm_gbs)",
                     "bytes_model": "per round 16 B per tape node + 8 B per variable leaf + 16 B per variable "
                                    "(store copy); 16 B per variable per fixpoint; 4 B per narrowing join"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "executions/s", "h2d_bytes_per_step": int(nvars * 8),
                "d2h_bytes_per_step": int(nvars * 8), "steps": e2e_steps},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "time_to_fixpoint_ms": dev_ms / args.steps,
        "tree_nodes_per_s": args.steps * rounds * nnodes / (dev_ms / 1e3),
        "events_schedule": ev,
    }
    print(json.dumps(out), flush=True)


def run_reference_pc(args):
    """The reference's PC loop on the host: the Gauss-Seidel fixpoint of the
    oracle (a restatement of pc.hpp / formula.hpp / terms.hpp), 1 thread."""
    from oracle import oracle as O
    tape, roots, lb, ub, _, desc = _pc_workload(args)
    order = O.pc_order(tape, roots)
    s0 = np.ascontiguousarray(np.stack([lb, ub], 1))
    for _ in range(args.warmup):
        O.pc_fixpoint(tape, order, s0.copy(), max_sweeps=1)
    times, execs = [], 0
    for _ in range(args.steps):
        s = s0.copy()
        t0 = time.perf_counter()
        rc, info = O.pc_fixpoint(tape, order, s, max_sweeps=args.ref_sweeps)
        times.append(time.perf_counter() - t0)
        execs += info["execs"]
    tot = sum(times)
    v = execs / tot
    out = {
        "metric": "propagator executions/sec", "value": v, "unit": "executions/s",
        "n_gpus": dist_env()[0], "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic: seeded generator, planted-solution instance",
        "config": {"workload": "pc: " + desc, "nvars": len(lb), "propagators": len(roots)},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "executions/s", "cores": 1, "kind": "port",
                         "sample": "each step = the first %d Gauss-Seidel sweeps of the fixpoint from the "
                                   "initial store (the reference loop is sequential: 1 host thread)"
                                   % args.ref_sweeps},
        "e2e": {"value": v, "unit": "executions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "pc":
        return run_reference_pc(args)
    inst, desc = make_workload(args.workload)
    from oracle import oracle as O
    s0 = inst.store()
    st, perm = O.install(inst.op, inst.x, inst.y, inst.z, s0)
    op, x, y, z = (np.ascontiguousarray(a[perm]) for a in (inst.op, inst.x, inst.y, inst.z))
    sweeps_per_step = args.ref_sweeps
    for _ in range(args.warmup):
        s = s0.copy()
        O.sweeps(op, x, y, z, s, 1)
    times, execs = [], 0
    s = s0.copy()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.sweeps(op, x, y, z, s, sweeps_per_step)
        times.append(time.perf_counter() - t0)
        execs += sweeps_per_step * inst.nprops
    tot = sum(times)
    v = execs / tot
    out = {
        "metric": "propagator executions/sec", "value": v, "unit": "executions/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tot * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic: seeded generator, planted-solution instance",
        "config": {"workload": args.workload + ": " + desc, "nvars": inst.nvars,
                   "propagators": int(inst.nprops)},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "executions/s", "cores": 1, "kind": "port",
                         "sample": "each step = %d Gauss-Seidel sweeps over the sorted bytecode "
                                   "(the reference loop is sequential: 1 host thread)" % sweeps_per_step},
        "e2e": {"value": v, "unit": "executions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="single_large")
    ap.add_argument("--mode", type=int, default=1, help="0 auto, 1 persistent, 2 host loop, 3 smem")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-sweeps", type=int, default=3)
    ap.add_argument("--max-rounds", type=int, default=0, help="round cap (profiling runs)")
    ap.add_argument("--variant", type=int, default=0, help="persistent kernel variant, 0: autotuned")
    ap.add_argument("--no-events", action="store_true", help="skip the event-schedule run of the single instance")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the out-of-L2 and batched-node records")
    ap.add_argument("--seq-nodes", type=int, default=128, help="nodes timed in the sequential loop")
    ap.add_argument("--cpu-nodes", type=int, default=256)
    ap.add_argument("--cpu-instances", type=int, default=128)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--node-sched", default="events", choices=["events", "ac1"])
    ap.add_argument("--inst-sched", default="events", choices=["events", "ac1"],
                    help="uneven workload: event-filtered or AC-1 rounds")
    ap.add_argument("--wake-fraction", type=float, default=1 / 32)
    ap.add_argument("--queens", type=int, default=12, help="search workload: board size")
    ap.add_argument("--cpu-search-nodes", type=int, default=2_000_000, help="search workload: CPU node cap")
    ap.add_argument("--pc-vars", type=int, default=1_000_000, help="pc workload: variables")
    ap.add_argument("--pc-props", type=int, default=1_000_000, help="pc workload: formula propagators")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        log("note: fewer than 3 warm-up steps")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "nodes":
        run_nodes(args)
    elif args.workload == "uneven":
        run_uneven(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "search":
        run_search(args)
    elif args.workload == "pc":
        run_pc(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
