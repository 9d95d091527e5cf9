#!/usr/bin/env python3
"""Benchmark of the SimulationCode.jl MD hot path on GB300 (libsimmd).

Prints ONE JSON line.  A "step" is one MD time step of every particle of the
workload (all replicas).  ``value`` = particle-steps/s with the state
resident in HBM (device-timed with CUDA events on the library's stream);
``e2e`` = the same metric through the C ABI with host buffers: the
ArrayStruct arrays from page-locked host memory to the device
(simmd_set_state_all: a caller holding the state between segments),
simmd_step, download of the state, all inside the timed region; a restart
segment (simmd_upload_all, new lists first) is reported beside it.

    python bench.py [--workload c4] [--steps K] [--warmup W] [--gpus N]
    python bench.py --impl reference ...   # the reference algorithm on the host cores

Multi-GPU: independent replicas, no collective on the data path.  The
replica batch is one job of 512 replicas per GPU partitioned over the ranks
by LPT on particles x steps (weak scaling: per-GPU work fixed); a
single-system workload runs one copy per rank.  Max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def rank_specs(workload, rank, precision=None, world=1):
    """the replicas of one rank.  No system spans GPUs.  The replica batch
    (c4) is a job of 512 replicas per GPU, 512 x world in all (the first 512
    are the one-GPU workload), partitioned over the ranks by LPT on
    particles x steps: each rank runs its share, no collective on the data
    path (weak scaling).  A single-system workload (c1-c3) runs one copy per
    rank with the rank's own seed (rank 0: the canonical seed)."""
    from simulationcode_gb300 import workloads as W
    import inspect
    kw = {} if precision is None else {"precision": precision}
    if workload == "c4":
        nrep = 512 * world
        part = W.lpt_partition([int(n) for n in W.c4_sizes(nrep)], world)[rank]
        return W.c4(nrep=nrep, indices=part, **kw)
    fn = W.WORKLOADS[workload]
    if rank:
        kw["seed"] = inspect.signature(fn).parameters["seed"].default + 7919 * rank
    return fn(**kw)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, x):
        return self._reduce(x, "MAX")

    def sum(self, x):
        return self._reduce(x, "SUM")

    def _reduce(self, x, op):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=getattr(self.dist.ReduceOp, op))
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        """start sampling and wait for the first sample (the sampler's own
        start-up stays outside the timed region)"""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            t = time.time()
            while not self.lines and time.time() - t < 10:
                time.sleep(0.05)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def mark(self, begin):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.t0 is not None and self.t1 is not None:
            inside = [x for x in lines if self.t0 - 0.15 <= x[0] <= self.t1 + 0.15]
            if inside:
                lines = inside
        for _, ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def issue_bound(profile, force_ms, sm_mhz):
    """The force kernel against the SMs' instruction-issue rate: its warp
    instructions per launch and the GPU's SM count (ncu, ``profile``) at one
    instruction per scheduler per cycle (4 per SM) at ``sm_mhz`` take
    ``floor_ms``; ``frac`` is that floor over the measured launch time.
    None without a profile."""
    try:
        w = float(profile["warp_instructions_per_launch"])
        sms = int(profile["sm_count"])
        floor_ms = w / (4.0 * sms * float(sm_mhz) * 1e6) * 1e3
        return {"warp_instructions_per_launch": w, "sm_count": sms, "sm_mhz": float(sm_mhz),
                "floor_ms": floor_ms, "frac": floor_ms / force_ms}
    except (KeyError, TypeError, ValueError, ZeroDivisionError):
        return None


def force_bytes_per_launch(specs, stats, entries=None):
    """Algorithmic HBM bytes of one force-kernel launch, independent of the
    kernel's own representation: per particle its position (8 B per
    component) and diameter (8 B), its list count (4 B) and 4 B per list
    entry read, the force write (8 B per component) and, when the second
    half-kick is fused (Newtonian/Langevin), the velocity read and write
    (16 B per component).  Neighbour positions are gathered from L2
    (cell-sorted layout) and not counted.  ``entries``: list entries a
    launch reads per replica (with filtered lists: the filtered list's,
    the full list's on the launches that re-filter), else the full list's."""
    total = 0
    for k, (s, st) in enumerate(zip(specs, stats)):
        per = 8 * s.dims + 8 + 4 + 8 * s.dims
        if s.dynamics != 2:
            per += 16 * s.dims
        e = st.list_entries if entries is None else entries[k]
        total += s.N * per + 4 * int(e)
    return total


def state_bytes(specs):
    """bytes of the particle state every step reads and writes (positions,
    velocities, forces, displacements in FP64), for the L2 statement"""
    return sum(s.N * 8 * s.dims * 4 for s in specs)


def workload_config(workload, specs, n_particles, n_replicas, tuned):
    """the ``config`` object both arms print: the workload, its size and the
    tuning's skins (the rebuild cadence), identical in the GPU arm and the
    reference arm"""
    from simulationcode_gb300 import workloads as W
    from simulationcode_gb300.autotune import group_key, skin_for
    skins = {}
    for s in specs:
        skins[group_key(s)] = skin_for(tuned, s)
    sb = state_bytes(specs)
    # the configuration's own skin is 0.3; the skins the run uses are `skins`
    desc = W.DESCRIPTIONS[workload].replace(", skin 0.3", ", skin 0.3 as configured (the run's: skins)")
    return {"workload": workload, "description": desc, "particles": int(n_particles),
            "replicas": int(n_replicas), "skins": dict(sorted(skins.items())),
            "l2": ("state larger than L2 (%.0f MB of particle state per step), no flush" % (sb / 1e6))
                  if sb > 129e6 else "state fits in L2 (%.0f MB of particle state)" % (sb / 1e6)}


def build_batch(specs, device, tpp):
    from simulationcode_gb300.batch import ReplicaBatch
    b = ReplicaBatch(device, tpp=tpp, graphs=True, graph_steps=16)
    n = sum(s.N for s in specs)
    b.reserve(n + 128 * len(specs), 4 * n // 8 + 64 * len(specs), len(specs) + 1, max(s.max_neighbors for s in specs))
    ids = [b.add(s) for s in specs]
    return b, ids


# kernel launches of the set-up relaxation (for ncu --launch-skip counts)
relax_launches = [0]
relax_counts = [0, 0]


def plain_fp64_one_at_a_time(specs, device, steps=32):
    """The plain FP64 path run one replica at a time: a context per replica,
    device-timed steps summed over replicas."""
    import copy
    from simulationcode_gb300 import _lib
    from simulationcode_gb300.batch import ReplicaBatch
    tot_ps, tot_ms = 0, 0.0
    for s in specs:
        t = copy.copy(s)
        t.precision = _lib.FP64
        b = ReplicaBatch(device, tpp=1, graphs=True, graph_steps=16)
        b.add(t)
        b.rebuild()
        b.step(3)
        b.timer_start()
        b.step(steps)
        tot_ms += b.timer_stop()
        tot_ps += t.N * steps
        b.close()
    return {"value": tot_ps / (tot_ms / 1000.0), "unit": "particle-steps/s", "steps_per_replica": steps,
            "replicas": len(specs)}


def run_serving(device, serve_seconds, capacity_seconds, concurrency=64, seed=5, log=None):
    """Serving (continuous batching): (1) capacity = particle-steps/s of the
    split-precision request mix with ``concurrency`` requests kept in flight
    (closed loop, ``capacity_seconds`` of wall clock); (2) a Poisson stream at
    0.8 x that capacity (in requests/s, from the stream's mean N*steps) for
    ``serve_seconds`` of arrivals, served to completion: p50/p99 completion
    latency and served particle-steps/s; (3) the plain FP64 path, one replica
    at a time, on a sample of the same requests."""
    from simulationcode_gb300 import workloads as W
    from simulationcode_gb300.serving import Request, Server, poisson_arrivals
    t_setup = time.perf_counter()
    say = log or (lambda m: None)
    pool = W.c5_requests(3 * concurrency, seed=seed + 1)
    say("serving: %d capacity requests generated (%.1f s)" % (len(pool), time.perf_counter() - t_setup))
    W.relax_on_device([s for s, _ in pool], device)
    say("serving: relaxed (%.1f s)" % (time.perf_counter() - t_setup))
    srv = Server(device=device, tick_steps=256, download=False)
    it = iter(pool)
    for _ in range(concurrency):
        srv.submit(Request(*next(it)))
    t0 = time.perf_counter()
    exhausted = False
    while time.perf_counter() - t0 < capacity_seconds and (srv.active or srv.waiting):
        srv.admit()
        srv.tick()
        while not exhausted and len(srv.active) + len(srv.waiting) < concurrency:
            try:
                srv.submit(Request(*next(it)))
            except StopIteration:
                exhausted = True
    cap_s = time.perf_counter() - t0
    capacity = srv.particle_steps / cap_s
    cap_failed = sum(1 for c in srv.completions if not c.ok)
    srv.batch.close()
    say("serving: capacity %.3g particle-steps/s over %.1f s, %d ticks, %d completed, %d failed" % (
        capacity, cap_s, srv.ticks, len(srv.completions) - cap_failed, cap_failed))
    if not capacity > 0 or cap_failed:
        msgs = sorted({c.message for c in srv.completions if not c.ok})[:3]
        return {"error": "capacity run failed: %d failed requests %s" % (cap_failed, msgs),
                "capacity_particle_steps_per_s": capacity}
    mean_work = float(np.mean([d[0] * d[4] for d in W.c5_draws(4096, seed=seed + 2)]))
    rate = 0.8 * capacity / mean_work
    n_req = max(16, int(round(rate * serve_seconds)))
    say("serving: rate %.2f requests/s, %d requests" % (rate, n_req))
    reqs = W.c5_requests(n_req, seed=seed + 2)
    W.relax_on_device([s for s, _ in reqs], device)
    rng = np.random.default_rng(seed + 3)
    arrivals = poisson_arrivals(n_req, rate, rng)
    setup_s = time.perf_counter() - t_setup - cap_s
    say("serving: open loop starts (set-up %.1f s)" % setup_s)
    srv = Server(device=device, tick_steps=256, download=True)
    last = [time.perf_counter()]

    def progress(s):
        if time.perf_counter() - last[0] > 5.0:
            last[0] = time.perf_counter()
            say("serving: t=%.1f s active %d waiting %d done %d" % (s.now(), len(s.active), len(s.waiting),
                                                                  len(s.completions)))

    done = srv.run([Request(sp, st, float(a), tag=k) for k, ((sp, st), a) in enumerate(zip(reqs, arrivals))],
                   sleep=lambda dt: time.sleep(min(dt, 1.0)), on_tick=progress)
    summ = srv.summary(done)
    srv.batch.close()
    sample = [sp for sp, _ in reqs[:16]]
    plain = plain_fp64_one_at_a_time(sample, device, steps=256)
    out = {"capacity_particle_steps_per_s": capacity, "capacity_concurrency": concurrency,
           "capacity_seconds": cap_s, "rate_requests_per_s": rate, "load": 0.8,
           "mean_particle_steps_per_request": mean_work,
           "p50_latency_s": summ["p50_s"], "p99_latency_s": summ["p99_s"], "mean_latency_s": summ["mean_s"],
           "served_particle_steps_per_s": summ["particle_steps_per_s"], "requests": summ["requests"],
           "completed": summ["completed"], "failed": summ["failed"], "makespan_s": summ["makespan_s"],
           "peak_active": summ["peak_active"], "peak_admitted_bytes": summ["peak_admitted_bytes"],
           "budget_bytes": summ["budget_bytes"], "ticks": summ["ticks"], "tick_steps": 256,
           "plain_fp64_one_at_a_time": plain,
           "capacity_vs_plain_fp64": capacity / plain["value"],
           "setup_s": setup_s,
           "precision": "f32-split", "arrival_window_s": serve_seconds}
    if log:
        log("serving: capacity %.3g ps/s, rate %.2f req/s, %d requests, p50 %.3f s, p99 %.3f s" % (
            capacity, rate, n_req, summ["p50_s"], summ["p99_s"]))
    return out


def split_precision_error(specs, device, positions=None, nsample=16):
    """FP32-split vs FP64 on the same configurations (pair forces, Newtonian
    copies so no noise enters): force relative RMS and |dE|/N.  positions:
    the workload's states after its timed steps (equilibrated), else the
    set-up configurations."""
    import copy
    from simulationcode_gb300 import _lib
    from simulationcode_gb300.batch import ReplicaBatch
    sample = []
    for k, s0 in enumerate(specs[:nsample]):
        s1 = copy.copy(s0)
        if positions is not None:
            s1.r = positions[k]
        sample.append(s1)
    num = den = 0.0
    de = 0.0
    n = 0
    res = {}
    for prec in (_lib.FP64, _lib.FP32_SPLIT):
        b = ReplicaBatch(device)
        ids = []
        for s in sample:
            t = copy.copy(s)
            t.precision = prec
            t.dynamics = _lib.NEWTONIAN
            t.v = np.zeros_like(s.r)
            ids.append(b.add(t))
        b.rebuild()
        _lib.check(b.lib.simmd_forces(b.ctx, None, None))
        en = b.energies()
        res[prec] = [(b.state(i)[2], en[i].epot) for i in ids]
        b.close()
    for (f64, e64), (f32, e32), s in zip(res[_lib.FP64], res[_lib.FP32_SPLIT], sample):
        num += float(((f32 - f64) ** 2).sum())
        den += float((f64 ** 2).sum())
        de += abs(e32 - e64)
        n += s.N
    return {"force_rel_rms": math.sqrt(num / den), "energy_abs_per_particle": de / n,
            "replicas_sampled": len(sample)}


def cpu_baseline_port(specs, seconds=12.0):
    """The oracle (serial C restatement of the reference) on a bounded sample
    of the same workload: whole replicas, a few steps each."""
    from oracle import build as ob, pyoracle as O
    ob.build_oracle()
    done_ps, t_used = 0, 0.0
    used = []
    for s in specs:
        p = O.make_params(s.dims, s.potential, s.dynamics, s.N, s.box_size, s.force_cutoff2, s.skin,
                          eps=s.lj_eps, sigma=s.lj_sigma, lj_rc=math.sqrt(s.force_cutoff2), zeta=s.b_zeta,
                          berthier_rc=math.sqrt(s.force_cutoff2), kBT=s.kBT, gamma=s.gamma, dt=s.dt, m=s.m)
        sysm = O.OracleSystem(p, s.r, s.D, v=s.v, force_cutoff=s.verlet_force_cutoff, maxK=s.max_neighbors * 2)
        sysm.update_neighbor_lists()
        t0 = time.perf_counter()
        sysm.run(1, seed=s.seed)
        t1 = time.perf_counter()
        per = max(t1 - t0, 1e-6)
        nsteps = int(max(1, min(200, (seconds - t_used) / per)))
        t0 = time.perf_counter()
        sysm.run(nsteps, seed=s.seed, step0=1)
        dt = time.perf_counter() - t0
        done_ps += s.N * nsteps
        t_used += dt + per
        used.append((s.N, s.dims, nsteps))
        if t_used > seconds:
            break
    value = done_ps / max(t_used, 1e-9)
    sample = "%d replica(s) of the workload, %d particle-steps (%s)" % (
        len(used), done_ps, ", ".join("N=%d %dD x%d steps" % u for u in used[:4]) + ("..." if len(used) > 4 else ""))
    return {"value": value, "unit": "particle-steps/s", "cores": 1, "kind": "port", "sample": sample}


def run_reference(args, dist):
    """--impl reference: the reference algorithm (the oracle port, a serial
    restatement of the Julia routines; Julia itself is not available) on the
    host cores, threads over replicas."""
    from concurrent.futures import ThreadPoolExecutor
    from simulationcode_gb300 import autotune as AT, workloads as W
    from oracle import build as ob, pyoracle as O
    ob.build_oracle()
    specs = W.WORKLOADS[args.workload](precision=0)
    # the GPU arm's tuning: the same skin (rebuild cadence) per replica group
    tuned = AT.load_tuned(args.workload) if args.autotune == "stored" else None
    for s in specs:
        s.skin = AT.skin_for(tuned, s)
    # bounded sample: a prefix of the replicas sized so that set-up, warm-up
    # and timed steps take about two minutes at a conservative 1e6
    # particle-steps/s per thread
    threads = max(1, os.cpu_count() or 1)
    budget = 120.0 * 1e6 * threads / float(args.relax_steps + args.warmup + args.steps)
    keep, tot = [], 0
    for s in specs:
        if keep and tot + s.N > budget:
            break
        keep.append(s)
        tot += s.N
    sample = ("the full workload" if len(keep) == len(specs) else
              "the first %d of %d replicas (%d particles)" % (len(keep), len(specs), tot))
    specs = keep
    # the same seeded initial state, relaxed as the GPU arm's set-up does
    # (capped steepest descent, here the oracle's C routine), threads over
    # replicas; the oracle releases the GIL inside its C calls
    systems = []
    for s in specs:
        p = O.make_params(s.dims, s.potential, s.dynamics, s.N, s.box_size, s.force_cutoff2, s.skin,
                          eps=s.lj_eps, sigma=s.lj_sigma, lj_rc=math.sqrt(s.force_cutoff2), zeta=s.b_zeta,
                          berthier_rc=math.sqrt(s.force_cutoff2), kBT=s.kBT, gamma=s.gamma, dt=s.dt, m=s.m)
        sysm = O.OracleSystem(p, s.r, s.D, v=s.v, force_cutoff=s.verlet_force_cutoff, maxK=s.max_neighbors * 2)
        systems.append((s, sysm))
    cores = max(1, min(os.cpu_count() or 1, len(systems)))
    pool = ThreadPoolExecutor(cores)

    def setup(t):
        s, sysm = t
        if s.potential == O.POT_BERTHIER and args.relax_steps > 0:
            sysm.relax_capped(args.relax_steps, 1e-3, 0.05)
        sysm.update_neighbor_lists()

    list(pool.map(setup, systems))
    # replicas are independent: each thread runs a replica's steps in one
    # oracle call (Philox noise keyed by the step, as on the GPU)
    list(pool.map(lambda t: t[1].run(args.warmup, seed=t[0].seed, step0=0), systems))
    t0 = time.perf_counter()
    list(pool.map(lambda t: t[1].run(args.steps, seed=t[0].seed, step0=args.warmup), systems))
    dt = time.perf_counter() - t0
    n = sum(s.N for s, _ in systems)
    value = n * args.steps / dt
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(args.workload, [s for s, _ in systems], n, len(systems), tuned or {}),
            "run": {"parallelism": "threads over replicas", "threads": cores},
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": "%s, %d timed steps" % (sample, args.steps)},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    pool.shutdown()
    return line


def run_gpu(args, dist):
    from simulationcode_gb300 import _lib, build as lb, workloads as W
    lb.build()
    lib = _lib.load()
    device = dist.local
    prec = {"fp64": _lib.FP64, "fp32": _lib.FP32_SPLIT}[args.precision] if args.precision else None
    specs = rank_specs(args.workload, dist.rank, prec, dist.ws)
    # set-up: relax random starts on the GPU (not timed)
    if any(s.potential == _lib.POT_BERTHIER for s in specs) and args.relax_steps > 0:
        fmax, counts = W.relax_on_device(specs, device, steps=args.relax_steps)
        print("relaxed: max |F| %.3g" % fmax, file=sys.stderr, flush=True)
        relax_launches[0] += counts[0]
        relax_counts[0] += counts[1]
        relax_counts[1] += counts[2]
    from simulationcode_gb300 import autotune as AT
    tuned = AT.load_tuned(args.workload) if args.autotune == "stored" else None
    if tuned is not None:
        args.tpp = int(tuned.get("tpp", args.tpp))
    batch, ids = build_batch(specs, device, args.tpp)
    if args.skin is not None:
        batch.set_skin(args.skin)
        tuned = None
    batch.rebuild()
    tune = None
    if tuned is not None:
        AT.apply_tuned(batch, tuned, graphs=args.graphs)
    elif args.autotune == "live":
        skins = [float(x) for x in args.tune_skins.split(",")] if args.tune_skins else None
        tune = AT.autotune(batch, tpps=(1, 2, 4, 8), skins=skins,
                           log=lambda m: print(m, file=sys.stderr, flush=True), group_by=AT.group_key)
        args.tpp = tune.tpp
        tuned = AT.as_tuned(tune, batch)
        print("TUNED %s %s" % (args.workload, json.dumps(tuned)), file=sys.stderr, flush=True)
    if not args.graphs:
        batch.set_tuning(int((tuned or {}).get("tpp", args.tpp)), False, 16)
    batch.step(args.warmup)
    st_before = [batch.stats(i) for i in ids]
    # kernel launches of this process before the timed region (for ncu -s)
    kc = batch.kernel_counts()
    print("LAUNCHES_BEFORE_TIMED=%d FORCE_LAUNCHES_BEFORE_TIMED=%d BUILD_LAUNCHES_BEFORE_TIMED=%d" % (
        relax_launches[0] + batch.launches(), relax_counts[0] + kc[0], relax_counts[1] + kc[1]),
        file=sys.stderr, flush=True)
    clocks = ClockSampler(device)
    clocks.start()
    dist.barrier()
    l0 = batch.launches()
    clocks.mark(True)
    batch.timer_start()
    batch.step(args.steps)
    ms = batch.timer_stop()
    clocks.mark(False)
    launches = batch.launches() - l0
    clk = clocks.stop()
    ms = dist.max(ms)
    n = sum(s.N for s in specs)
    n_all = dist.sum(n)           # particles of every rank (replicas only)
    value = n_all * args.steps / (ms / 1000.0)
    st_after = [batch.stats(i) for i in ids]
    rebuilds = sum(b.rebuilds - a.rebuilds for a, b in zip(st_before, st_after))

    # force-kernel duration: CUDA events around every force launch of an
    # instrumented pass of the same step loop (direct launches)
    if args.no_profile_pass:
        prof = {"force_ms": float("nan"), "force_n": 1, "kick_ms": 0.0, "rebuild_ms": 0.0, "update_ms": 0.0,
                "steps": 1}
    else:
        pr0 = [batch.prune_stats(i)[0] for i in ids] if batch.inner_skin > 0 else None
        batch.profile(True)
        batch.step(max(16, min(args.steps, 64)))
        prof = batch.profile_get()
        batch.profile(False)
    force_ms = prof["force_ms"] / max(prof["force_n"], 1)
    stats = [batch.stats(i) for i in ids]
    entries = None
    if batch.inner_skin > 0 and not args.no_profile_pass:
        # filtered lists: the filtered entries on most launches, the full list
        # on the launches that re-filter (their share per replica)
        entries = []
        for k, (rid, st) in enumerate(zip(ids, stats)):
            n_pr, e_in = batch.prune_stats(rid)
            f = min(1.0, (n_pr - pr0[k]) / max(prof["steps"], 1))
            entries.append(e_in * (1.0 - f) + st.list_entries * f)
    fbytes = force_bytes_per_launch(specs, stats, entries)
    peak, peak_kind = peaks()
    achieved = fbytes / (force_ms / 1000.0) / 1e9
    traffic = None
    fprof = {}
    tfile = os.path.join(ROOT, "profiles", "force_traffic_%s.json" % args.workload)
    if os.path.exists(tfile):
        try:
            with open(tfile) as f:
                fprof = json.load(f)
            traffic = fprof.get("dram_bytes_per_launch")
        except Exception:
            traffic = None

    # e2e through the C ABI: host (page-locked) arrays -> device, K steps,
    # device -> host, every replica at once (one copy per array, one
    # synchronisation each way).  The timed segment is that of a caller that
    # holds the state on the host between calls (the reference's driver
    # between callbacks): simmd_set_state_all (the lists and skin bookkeeping
    # stay valid) + simmd_step(K) + simmd_download_all.  A restart segment
    # (simmd_upload_all: new lists for every replica before the first step)
    # is timed after it and reported beside it.
    total, offs = batch.transfer_layout()
    any_v = any(s.dynamics != 2 for s in specs)
    r_all = np.zeros(total)
    v_all = np.zeros(total) if any_v else None
    D_all = np.zeros(sum(s.N for s in specs))
    F_all = np.zeros(total)
    doff = 0
    for rid, s in sorted(zip(ids, specs), key=lambda t: t[0]):
        D_all[doff:doff + s.N] = s.D
        doff += s.N
    host = [a for a in (r_all, v_all, D_all, F_all) if a is not None]
    for a in host:
        _lib.check(lib.simmd_host_register(C.c_void_p(a.ctypes.data), a.nbytes))
    h2d = r_all.nbytes + (v_all.nbytes if any_v else 0)
    d2h = r_all.nbytes + F_all.nbytes + (v_all.nbytes if any_v else 0)
    e2e_steps = 0 if args.no_e2e else args.steps
    restart = None
    # one untimed round: the host takes the current state, and the staging
    # buffers of the batched transfers are allocated once per context, as in
    # a user's repeated segments
    batch.download_all(r_all, v_all, F_all)
    batch.set_state_all(r_all, v_all)
    dist.barrier()
    t0 = time.perf_counter()
    batch.set_state_all(r_all, v_all)
    if e2e_steps:
        _lib.check(lib.simmd_step(batch.ctx, e2e_steps, None))
    batch.download_all(r_all, v_all, F_all)
    e2e_s = dist.max(time.perf_counter() - t0)
    if e2e_steps:
        dist.barrier()
        t0 = time.perf_counter()
        batch.upload_all(r_all, D_all, v=v_all)
        _lib.check(lib.simmd_step(batch.ctx, e2e_steps, None))
        batch.download_all(r_all, v_all, F_all)
        rs = dist.max(time.perf_counter() - t0)
        restart = {"value": n_all * e2e_steps / rs, "unit": "particle-steps/s",
                   "h2d_bytes_per_step": (h2d + D_all.nbytes) / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps,
                   "what": "simmd_upload_all (r, %sD) + simmd_step(K) + simmd_download_all: new lists for every "
                           "replica before the first step" % ("v, " if any_v else "")}
    for a in host:
        lib.simmd_host_unregister(C.c_void_p(a.ctypes.data))
    e2e_steps = max(e2e_steps, 1)
    e2e = {"value": n_all * e2e_steps / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps,
           "what": "simmd_set_state_all (r%s of every replica from page-locked host arrays; lists kept) + "
                   "simmd_step(K) + simmd_download_all (r, %sF), wall clock" % (", v" if any_v else "",
                                                                                 "v, " if any_v else ""),
           "restart": restart}

    # bytes streamed per step: force launch + positions, velocities, forces,
    # displacements of the integrator pass
    step_bytes = fbytes + sum(s.N * 8 * s.dims * 6 for s in specs)
    dtype = "f64" if all(s.precision == 0 for s in specs) else "f32-split (f32 pair math, f64 integration)"
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": dist.ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": workload_config(args.workload, specs, n_all, int(dist.sum(len(specs))), tuned or {}),
            "run": {"particles_per_rank": n, "replicas_per_rank": len(specs), "threads_per_particle": args.tpp,
                    "bytes_streamed_per_step": step_bytes,
                    "parallelism": ("LPT replica partition over %d ranks" % dist.ws) if dist.ws > 1
                                   else "single GPU",
                    "rebuilds_in_timed_region": rebuilds,
                    "step_loop": "CUDA graph of 16 steps" if args.graphs else "direct launches",
                    "tuning": {"source": {"stored": "simulationcode_gb300/tuned.json (autotuner result)",
                                          "live": "autotuner, this run"}.get(args.autotune, "none"),
                               "tuned": tuned,
                               "trials": None if tune is None else tune.trials}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "k_force", "force_ms_per_launch": force_ms,
                         "alg_bytes_per_launch": fbytes,
                         "issue": issue_bound(fprof, force_ms, clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0)},
            "step_breakdown_ms": {k: prof[k] / max(prof["steps"], 1) for k in ("force_ms", "kick_ms", "rebuild_ms",
                                                                               "update_ms")},
            "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if any(sp.precision == 0 for sp in specs):
        # the plain FP64 path is bound by GB300's FP64 pipe, not HBM: FP64
        # operations of the reference pair arithmetic per list entry (3D soft
        # spheres 45, 2D 39, LJ 3D 32, LJ 2D 24; a correctly rounded
        # reciprocal or divide counted as 4) over the force-pass time
        ops = 0
        for sp, st in zip(specs, stats):
            if sp.precision != 0:
                continue
            per = (45 if sp.dims == 3 else 39) if sp.potential == 1 else (32 if sp.dims == 3 else 24)
            ops += per * int(st.list_entries)
        line["fp64_pipe"] = {"ops_per_launch": ops, "achieved_tops": ops / (force_ms / 1000.0) / 1e12,
                             "nominal_peak_tops": 0.625,
                             "note": "nominal = 1.25 TFLOP/s FP64 counting an FMA as 2; DMUL/DADD issue at the FMA rate"}
    evolved = [batch.state(i)[0] for i in ids[:16]]
    batch.close()
    if dist.rank == 0 and any(s.precision != 0 for s in specs) and not args.no_compare:
        plain = plain_fp64_one_at_a_time(specs, device)
        line["plain_fp64_one_at_a_time"] = plain
        line["speedup_vs_plain_fp64"] = value / plain["value"]
        err = split_precision_error(specs, device, positions=evolved)
        err["states"] = "the workload's states after its timed steps"
        line["split_precision_error"] = err
    if dist.rank == 0 and args.serve_seconds > 0:
        line["serving"] = run_serving(device, args.serve_seconds, args.serve_capacity_seconds,
                                      log=lambda m: print(m, file=sys.stderr, flush=True))
    if dist.rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_port(specs, seconds=args.cpu_seconds)
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c4", choices=["c1", "c2", "c3", "c4"])
    ap.add_argument("--precision", default=None, choices=[None, "fp64", "fp32"])
    ap.add_argument("--tpp", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-FP64 and error comparisons")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-profile-pass", action="store_true")
    ap.add_argument("--relax-steps", type=int, default=300)
    ap.add_argument("--skin", type=float, default=None, help="override the workload's skin (without autotuning)")
    ap.add_argument("--no-graphs", dest="graphs", action="store_false",
                    help="direct launches instead of the captured step loop (for per-kernel profiling: ncu does not "
                         "profile kernel nodes of graphs with conditional nodes)")
    ap.add_argument("--autotune", default="stored", choices=["stored", "live", "off"],
                    help="tuning (threads per particle, per-group skin = rebuild cadence): the autotuner's stored "
                         "result (simulationcode_gb300/tuned.json, the default, shared with the reference arm), "
                         "a live autotuner run, or none")
    ap.add_argument("--tune-skins", default="0.3,0.4,0.5,0.6,0.7",
                    help="skins the autotuner may choose from (the rebuild cadence); empty: keep the configured skin")
    ap.add_argument("--serve-seconds", type=float, default=30.0,
                    help="arrival window of the serving run (0: no serving run)")
    ap.add_argument("--serve-capacity-seconds", type=float, default=6.0,
                    help="closed-loop window that measures the serving capacity")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    if args.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        line = run_reference(args, dist)
    else:
        line = run_gpu(args, dist)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
