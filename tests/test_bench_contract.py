"""bench.py's reference arm (the CPU restatement of the reference routines
on the host cores) prints the one JSON line of the bench contract; it needs
no GPU, so its shape is checked here on the smallest workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "c1", "--steps", "3",
                        "--warmup", "3", "--relax-steps", "0"], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == d["unit"] == "particle-steps/s"
    assert d["steps"] == 3 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["config"]["workload"] == "c1"
    # the GPU arm's stored tuning: the same skins in both arms' config
    from simulationcode_gb300.autotune import load_tuned
    assert d["config"]["skins"] == load_tuned("c1")["skins"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_force_bytes_model_follows_the_list_read():
    """the roofline's algorithmic bytes: per particle its record, count and
    force (plus the velocity stream for Newtonian/Langevin) and 4 B per list
    entry the launch reads (the filtered list's count when one is given)"""
    import bench
    from types import SimpleNamespace as NS
    specs = [NS(N=100, dims=3, dynamics=2), NS(N=50, dims=2, dynamics=0)]
    stats = [NS(list_entries=3000), NS(list_entries=800)]
    per3 = 8 * 3 + 8 + 4 + 8 * 3
    per2 = 8 * 2 + 8 + 4 + 8 * 2 + 16 * 2
    assert bench.force_bytes_per_launch(specs, stats) == 100 * per3 + 50 * per2 + 4 * (3000 + 800)
    assert bench.force_bytes_per_launch(specs, stats, [1500.0, 400.0]) == 100 * per3 + 50 * per2 + 4 * (1500 + 400)


def test_issue_bound_from_the_profile():
    """the force kernel's issue-rate floor: warp instructions per launch over
    4 schedulers x SMs x clock, as a fraction of the measured launch time"""
    import bench
    prof = {"warp_instructions_per_launch": 4 * 152 * 2070e6 * 1e-4, "sm_count": 152}
    ib = bench.issue_bound(prof, 0.2, 2070.0)
    assert abs(ib["floor_ms"] - 0.1) < 1e-12 and abs(ib["frac"] - 0.5) < 1e-12
    assert bench.issue_bound({}, 0.2, 2070.0) is None
    assert bench.issue_bound({"dram_bytes_per_launch": 1}, 0.2, 2070.0) is None
    # the committed profile of the batch workload carries the figures
    with open(os.path.join(ROOT, "profiles", "force_traffic_c4.json")) as f:
        assert bench.issue_bound(json.load(f), 0.238, 2070.0)["frac"] > 0.3


def test_reference_arm_under_torchrun_prints_one_line():
    """--impl reference launched as the driver launches a multi-GPU run (two
    ranks, gloo on the CPU): rank 0 alone runs and prints the line, the
    other rank exits 0 without work"""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--gpus", "2", "--workload", "c1", "--steps", "3", "--warmup", "3", "--relax-steps", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
