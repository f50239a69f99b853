"""The ncu summaries under profiles/ carry the 'key: number' lines bench.py
quotes in its JSON line (DRAM traffic per launch, the L2-resident round's L2
figures, the out-of-L2 instance's DRAM bytes per round): a summary reworded
without them would leave those fields null."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_profiles_carry_the_quoted_figures():
    B = _bench()
    for name in ("persistent_fixpoint_single_large", "events_fixpoint_single_large", "nodes_events_4096_nodes",
                 "instances_events_uneven_512", "instances_cluster_uneven_512", "pc_fixpoint_pc"):
        t = B.ncu_traffic(name)
        assert t is not None and t > 0, name
    sl = B.profile_fields("persistent_fixpoint_single_large")
    for k in ("l2_hit_rate_pct", "lts_throughput_pct", "l1tex_throughput_pct", "issue_active_pct",
              "dram_bytes_per_round"):
        assert sl.get(k, 0) > 0, k
    ol = B.profile_fields("persistent_fixpoint_out_of_l2")
    assert ol.get("dram_bytes_per_round", 0) > 0 and ol.get("dram_gbs", 0) > 0


def test_profiles_name_no_removed_capture_style():
    """Launch lists collect the device time only; DRAM or L2 counters come
    from one-kernel captures (-k ... -c 1)."""
    for f in os.listdir(os.path.join(ROOT, "profiles")):
        text = open(os.path.join(ROOT, "profiles", f)).read()
        commands = text.replace("\\\n", " ").splitlines()  # continued lines joined
        for cmd in commands:
            if cmd.startswith("ncu --metrics") and " -k " not in cmd:
                assert cmd.split()[2] == "gpu__time_duration.sum", (f, cmd)
            if cmd.startswith("ncu "):
                assert "--clock-control none" in cmd, (f, cmd)
