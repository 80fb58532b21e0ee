#!/usr/bin/env python3
"""Benchmark of the GB300 photon walk.  Headline: photons/s of the plain
kernel on the 2^30-photon workload (params.h optics: MU_A 2/cm, MU_S 20/cm,
101 shells of 50 um, Philox seed 1, photon ids 0 .. 2^30-1).

One step = one walk of the whole photon batch (one kernel launch).  Prints
one JSON line (rank 0).  Usage:

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Top-level keys (the plain walk):
* value: photons/s over all ranks, device time of the walk (CUDA events on
  the launching stream), L2 flushed between timed steps;
* e2e: the same metric through the C ABI's host-array call
  tmc_photon_batch(heat, heat2, n, params), wall time of the whole call
  (launch, walk, FP64 finalisation, device-to-host copy of the result);
* roofline: the bound named for this path, SFU-class operations (4 per
  photon step: log, 2 sqrt, divide) against the measured MUFU rate, and the
  pipe that actually binds (instruction issue);
* cpu_baseline: the reference's walk on this host's cores (libc rand): one
  lone process, one process per core, and subsamples of the high-albedo and
  batched-sweep workloads, each process running >= 10 s.
Beside it, on one GPU (the default run; --plain-only leaves them out):
* high_albedo: the plain walk at high albedo (MU_A 0.1, MU_S 100, 1001
  shells of 10 um), 2^28 photons per launch;
* sweep: 4096 independent problems in one persistent launch (autotuned,
  CUDA-graph replay) at 1/64 of the photon counts, against one launch per
  problem on a subsample of the problems;
* serve: the request stream (continuous batching, RSE stopping) on the
  server's persistent launch fed from a work queue: capacity, the load
  offered at 2000 requests/s, and p50/p99 latency at 70 % of the capacity;
  serve_waves: the same on the server's default setting (waves of
  launches, which leave SM room for other work between launches).

Multi-GPU (torchrun): each rank walks its own 2^30 photons (ids offset by
rank), no collective on the data path; weak scaling.  After the timed region
the ranks' exact tallies are summed (replicas.reduce_tallies over gloo).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "photons/s on 1 GB300 (plain vs batched/served) at stated error; p50/p99 latency"
UNIT = "photons/s"
SFU_OPS_PER_STEP = 4          # log, sqrt (radius), divide + sqrt (direction)
CPU_SECONDS_PER_PROC = 10.5   # each CPU-baseline process runs at least 10 s
REF_SECONDS_PER_STEP = 3.0    # each reference-arm step: every core walks ~3 s

# Figures from one ncu capture of walk_plain<512, FastMath> at params.h optics
# (one 2^25-photon launch).  They describe the kernel built from the sources
# whose SHA-256 is recorded here; bench.py hashes the current sources and
# marks the figures "stale" when they differ (the kernel changed since the
# capture), in which case they must not be read as this build's.
NCU_WALK = {
    "capture": "profiles/walk_plain_fast_2p25photons_ncu_full.txt",
    "sources": ["tiny_mc_gb300/csrc/tmc_device.cuh", "tiny_mc_gb300/csrc/tmc_walk.cuh",
                "tiny_mc_gb300/csrc/tmc_plain.cu"],
    "sources_sha256": "ea19d338f68d330bf85235a1a34dc1fde124bf73e8b6288c8c512f1da601432c",
    # thread-instructions (predicated on) per photon step
    "thread_instr_per_step": 226.5,
    # busy fraction of each pipe
    "pipes_busy": {"issue_slots": 0.827, "alu": 0.550, "fma": 0.340, "xu_sfu": 0.134,
                   "shared_wavefronts": 0.541, "dram": 0.0},
    # DRAM bytes read + written by one launch (constant and code fetch plus the
    # warps' 101-shell histogram flushes; not proportional to the photon count)
    "dram_bytes_per_launch": 178944,
}


def walk_sources_sha256() -> str:
    h = hashlib.sha256()
    for rel in NCU_WALK["sources"]:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--photons", type=int, default=1 << 30)
    ap.add_argument("--math", choices=["exact", "fast"], default="fast")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--plain-only", action="store_true",
                    help="leave out the high_albedo, sweep and serve legs of the default run")
    ap.add_argument("--optics", choices=["params_h", "high_albedo"], default="params_h",
                    help="plain workload optics: params_h = params.h (101 shells, 50 um, MU_A 2, MU_S 20); "
                         "high_albedo = high albedo (1001 shells, 10 um, MU_A 0.1, MU_S 100)")
    ap.add_argument("--high-albedo-photons", type=int, default=1 << 28)
    ap.add_argument("--high-albedo-steps", type=int, default=2)
    ap.add_argument("--sweep-mu-a-min", type=float, default=0.01,
                    help="sweep workload: lower end of the mu_a range (0.01: the full sweep distribution)")
    ap.add_argument("--workload", choices=["plain", "sweep", "serve"], default="plain",
                    help="plain: 2^30 photons at params.h optics with the other legs beside it (default); "
                         "sweep / serve: that leg alone, as its own line")
    ap.add_argument("--serve-slots", type=int, default=1024)
    ap.add_argument("--serve-steps-per-batch", type=float, default=0.0,
                    help="server RSE batch size in photon steps (0: library default)")
    ap.add_argument("--serve-steps-per-item", type=float, default=-1.0,
                    help="server work item size in photon steps (0: one item per batch; -1: library default)")
    ap.add_argument("--serve-inflight-items", type=int, default=-1,
                    help="server cap on launched, unfinished work items (0: none; -1: library default)")
    ap.add_argument("--serve-waves", type=int, default=-1,
                    help="server launches in flight (1..64; -1: library default)")
    ap.add_argument("--serve-stream", type=int, choices=[-1, 0, 1], default=-1,
                    help="server kernel: 0 per-item barriers, 1 barrier-free, -1 library default")
    ap.add_argument("--serve-persistent", type=int, choices=[-1, 0, 1], default=-1,
                    help="server: 1 one persistent launch fed from a work queue, 0 waves of launches, "
                         "-1 library default")
    ap.add_argument("--serve-calib", type=int, default=256)
    ap.add_argument("--serve-window", type=float, default=10.0)
    ap.add_argument("--serve-duration", type=float, default=25.0)
    ap.add_argument("--serve-drain", type=float, default=60.0)
    ap.add_argument("--sweep-scale", type=float, default=1.0 / 64,
                    help="photon-count multiplier of the sweep (1 = full size, ~3.3e13 steps)")
    ap.add_argument("--sweep-steps", type=int, default=2)
    ap.add_argument("--batch-config", default="",
                    help="sweep: fixed 'block,items_per_block,stream' instead of the autotuner")
    ap.add_argument("--plain-stride", type=int, default=16,
                    help="sweep: the one-launch-per-problem form walks every k-th problem (0: none)")
    return ap.parse_args()


OPTICS = {"params_h": dict(shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0),
          "high_albedo": dict(shells=1001, microns_per_shell=10.0, mu_a=0.1, mu_s=100.0)}


def workload_config(args, world):
    o = OPTICS[args.optics]
    name = ("plain walk, 2^30 photons per GPU, params.h optics" if args.optics == "params_h" and
            args.photons == 1 << 30 else f"plain walk, {args.photons} photons per GPU ({args.optics} optics)")
    return {
        "workload": name,
        "photons_per_step_per_gpu": args.photons,
        "shells": o["shells"], "microns_per_shell": o["microns_per_shell"], "mu_a_per_cm": o["mu_a"],
        "mu_s_per_cm": o["mu_s"],
        "rng": "Philox-4x32-10 keyed by photon id, seed 1",
        "math": args.math,
        "tallies": "u64 shared / u128 global fixed point (2^-40)",
        "l2": "flushed between timed steps (256 MiB write); inputs are only parameters",
        "parallelism": f"replicas x{world} (photon-id ranges)",
    }


# --------------------------------------------------------------- CPU side
def _cpu_worker(job):
    """One process: the reference walk (libc rand) for a list of
    (shells, microns_per_shell, mu_a, mu_s, photons) problems on one core.
    Returns (photons, photon steps, seconds, kind)."""
    problems, seed = job
    sys.path.insert(0, ROOT)
    from oracle import oracle
    photons = steps = 0
    t0 = time.perf_counter()
    kind = "port"
    for shells, mps, mu_a, mu_s, n in problems:
        p = oracle.oparams(int(shells), float(mps), float(mu_a), float(mu_s), seed)
        _, s = oracle.native_rate(p, int(n), seed)
        photons += int(n)
        steps += int(s)
    return photons, steps, time.perf_counter() - t0, kind


class CpuPool:
    def __init__(self, procs):
        import multiprocessing as mp
        self.procs = procs
        self.pool = mp.get_context("spawn").Pool(procs)

    def run(self, jobs):
        """Runs one job per process at once; returns the per-job results and
        the wall time of the whole set."""
        t0 = time.perf_counter()
        res = self.pool.map(_cpu_worker, jobs, chunksize=1)
        return res, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _optics_tuple(name, photons):
    o = OPTICS[name]
    return (o["shells"], o["microns_per_shell"], o["mu_a"], o["mu_s"], photons)


def _calibrate(pool, name, seconds, probe_photons):
    """Photons one core walks in about `seconds` at `name` optics."""
    res, _ = pool.run([([_optics_tuple(name, probe_photons)], 1)])
    rate = res[0][0] / max(res[0][2], 1e-6)
    return max(1, int(rate * seconds)), res[0][1] / res[0][0]


def _leg(res, wall, procs):
    photons = sum(r[0] for r in res)
    steps = sum(r[1] for r in res)
    return {"photons_per_s": photons / wall, "photon_steps_per_s": steps / wall,
            "processes": procs, "seconds": wall,
            "per_process_seconds": [round(r[2], 2) for r in res]}


def cpu_baseline_measure(sweep_problems=None):
    """The reference's walk on this host: (i) one process alone, (ii) one
    process per core, params.h optics; (iii) high albedo and (iv) a subsample
    of the batched sweep, one process per core; every process >= 10 s."""
    from oracle import oracle
    oracle.build(ref=False)
    cores = cpu_cores()
    pool = CpuPool(cores)
    pool.run([([_optics_tuple("params_h", 256)], i + 1) for i in range(cores)])   # start the workers
    n1, spp = _calibrate(pool, "params_h", CPU_SECONDS_PER_PROC, 20000)
    res, wall = pool.run([([_optics_tuple("params_h", n1)], 1)])
    single = _leg(res, wall, 1)
    res, wall = pool.run([([_optics_tuple("params_h", n1)], i + 1) for i in range(cores)])
    per_core = _leg(res, wall, cores)
    nh, _ = _calibrate(pool, "high_albedo", CPU_SECONDS_PER_PROC, 200)
    res, wall = pool.run([([_optics_tuple("high_albedo", nh)], i + 1) for i in range(cores)])
    high = _leg(res, wall, cores)
    sweep = None
    if sweep_problems is not None:
        sweep = cpu_sweep_subsample(pool, cores, sweep_problems)
    pool.close()
    kind = "port"
    out = {
        "value": per_core["photons_per_s"], "unit": UNIT, "cores": cores, "kind": kind,
        "sample": f"params.h optics, libc rand (the reference's walk, replayed by the oracle), "
                  f"{cores} processes x {n1} photons (seeds 1..{cores}), one process per core",
        "single_thread": {**single, "photons_per_process": n1},
        "per_core": {**per_core, "photons_per_process": n1},
        "high_albedo": {**high, "photons_per_process": nh,
                        "workload": "MU_A 0.1, MU_S 100, 1001 shells of 10 um"},
        "single_thread_value": single["photons_per_s"],
    }
    if sweep is not None:
        out["sweep"] = sweep
    return out


def cpu_sweep_subsample(pool, cores, sw):
    """Every core walks a disjoint subsample of the sweep's problems, each
    problem for a photon count sized to its expected steps, ~10 s per core;
    the sweep's CPU photons/s follows from the measured photon-step rate and
    the sweep's total photons and expected steps."""
    import numpy as np

    import tiny_mc_gb300 as tmc
    est = np.array([tmc.expected_steps(float(q["mu_a"]), float(q["mu_s"])) for q in sw])
    # step rate of one core, for sizing
    res, _ = pool.run([([_optics_tuple("params_h", 20000)], 1)])
    step_rate = res[0][1] / res[0][2]
    order = np.random.default_rng(1).permutation(len(sw))
    per_core = [order[c::cores] for c in range(cores)]
    jobs = []
    for c, idx in enumerate(per_core):
        target = step_rate * CPU_SECONDS_PER_PROC / max(1, len(idx))
        probs = []
        for i in idx:
            q = sw[i]
            n = max(1, int(round(target / est[i])))
            probs.append((int(q["shells"]), float(q["microns_per_shell"]), float(q["mu_a"]),
                          float(q["mu_s"]), n))
        jobs.append((probs, c + 1))
    res, wall = pool.run(jobs)
    leg = _leg(res, wall, cores)
    total_photons = float(sw["n_photons"].astype(np.float64).sum())
    total_steps = float((sw["n_photons"].astype(np.float64) * est).sum())
    leg["sweep_photons_per_s"] = total_photons / (total_steps / leg["photon_steps_per_s"])
    leg["workload"] = (f"all {len(sw)} problems of the sweep, each walked for ~{CPU_SECONDS_PER_PROC:.0f} s / "
                       f"{len(per_core[0])} of its expected steps on one of {cores} cores; sweep photons/s = "
                       f"the sweep's photons / (its expected photon steps / the measured step rate)")
    return leg


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    from oracle import oracle
    oracle.build(ref=False)
    cores = cpu_cores()
    pool = CpuPool(cores)
    pool.run([([_optics_tuple("params_h", 256)], i + 1) for i in range(cores)])
    n_step, _ = _calibrate(pool, "params_h", REF_SECONDS_PER_STEP, 20000)
    jobs = [([_optics_tuple("params_h", n_step)], i + 1) for i in range(cores)]
    for _ in range(args.warmup):
        pool.run(jobs)
    times = []
    for _ in range(args.steps):
        _, wall = pool.run(jobs)
        times.append(wall)
    pool.close()
    total = cores * n_step * args.steps
    value = total / sum(times)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(args, world), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step: {cores} processes x {n_step} photons (~{REF_SECONDS_PER_STEP:.0f} s) "
                                   f"of the reference walk (libc rand replay, params.h optics)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id: str | None):
        self.device_id = device_id
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"]
        if self.device_id:
            cmd += ["-i", self.device_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "power_w_max": max(power) if power else None,
            "samples": len(sm),
            "reasons": sorted(reasons),
        }


def _device_id(torch, dev):
    uuid = getattr(torch.cuda.get_device_properties(dev), "uuid", None)
    return f"GPU-{uuid}" if uuid is not None else None


def _sfu_roofline(steps_per_launch, launch_s, sfu_peak):
    achieved = SFU_OPS_PER_STEP * steps_per_launch / launch_s
    return {"bound": "sfu", "achieved": achieved / 1e9, "peak": sfu_peak / 1e9, "unit": "Gop/s",
            "frac": achieved / sfu_peak,
            "algorithmic_unit": "4 SFU-class ops (log, sqrt, divide, sqrt) per photon step",
            "photon_steps_per_launch": steps_per_launch,
            "peak_source": "measured live: MUFU lg2/sqrt/rcp probe (tmc_probe_sfu_rate)"}


# ------------------------------------------------------------------- ours
def run_ours(args):
    import numpy as np
    import torch

    import tiny_mc_gb300 as tmc

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    extra_legs = rank == 0 and world == 1 and not args.plain_only and args.optics == "params_h"

    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sweep_problems = None
        if extra_legs:
            from tiny_mc_gb300.sweep import make_sweep
            sweep_problems = make_sweep(4096, seed=0, photon_scale=args.sweep_scale, min_photons=16,
                                        mu_a_range=(args.sweep_mu_a_min, 10.0))
        cpu_base = cpu_baseline_measure(sweep_problems)

    dev = torch.device("cuda", torch.cuda.current_device())
    props = torch.cuda.get_device_properties(dev)
    device_id = _device_id(torch, dev)

    optics = OPTICS[args.optics]
    S = optics["shells"]
    p = tmc.params(seed=1, photon_id_base=rank * args.photons, math=args.math, **optics)
    tmc.set_plain_launch(args.block, args.blocks_per_sm, 0)
    tally = torch.zeros((S, 4), dtype=torch.int64, device=dev)
    steps_ctr = torch.zeros(1, dtype=torch.int64, device=dev)
    ws = torch.zeros(max(1, tmc.workspace_bytes() // 8), dtype=torch.int64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def one_step(params=p):
        tmc.photon_batch_device(tally.data_ptr(), args.photons, params, steps_ctr.data_ptr(), ws.data_ptr(), sp)

    sfu_peak = tmc.probe_sfu_rate()
    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    steps_ctr.zero_()
    tally.zero_()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = ClockSampler(device_id)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        one_step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    if dist is not None:
        dist.barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(ms)
    photon_steps = int(steps_ctr.item())
    replicas = None
    if dist is not None:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        ps = torch.tensor([photon_steps], device=dev, dtype=torch.int64)
        dist.all_reduce(ps)
        photon_steps_all = int(ps.item())
        # the only exchange of the path: the ranks' exact tallies, summed
        from tiny_mc_gb300.replicas import reduce_tallies
        gloo = dist.new_group(backend="gloo")
        local_tally = tally.cpu().numpy().view(np.uint64).reshape(-1).view(tmc.TALLY_DTYPE).copy()
        total = reduce_tallies(local_tally, group=gloo)
        sw, _ = tmc.tally_sums(total)
        replicas = {"reduced_over_ranks": world, "photons": args.photons * args.steps * world,
                    "sum_w_fixed_point_2^-40": str(sum(sw)),
                    "reduction": "exact 128-bit sum of every rank's tally (all_gather over gloo)"}
    else:
        photon_steps_all = photon_steps
    photons_all = args.photons * args.steps * world
    value = photons_all / (total_ms * 1e-3)

    # roofline of the dominant kernel (the walk is the only kernel per step)
    per_launch_s = (sum(ms) / len(ms)) * 1e-3
    steps_per_launch = photon_steps / args.steps
    roofline = _sfu_roofline(steps_per_launch, per_launch_s, sfu_peak)
    current = walk_sources_sha256() == NCU_WALK["sources_sha256"]
    roofline["traffic"] = NCU_WALK["dram_bytes_per_launch"] if (args.optics == "params_h" and current) else None
    roofline["traffic_note"] = ("DRAM bytes per launch from " + NCU_WALK["capture"] +
                                ("" if current else " (stale: the kernel sources changed since; not reported)"))
    # the pipe that binds: instruction issue (4 warp-instructions per clock per
    # SM); its ceiling at the sampled clock, from the capture's instruction count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    if mhz and args.optics == "params_h" and args.math == "fast":
        ipstep = NCU_WALK["thread_instr_per_step"]
        issue_steps = props.multi_processor_count * mhz * 1e6 * 4 * 32 / ipstep
        roofline["binding_pipe"] = {
            "pipe": "instruction issue", "thread_instr_per_step": ipstep,
            "ceiling_photon_steps_per_s": issue_steps,
            "frac": (steps_per_launch / per_launch_s) / issue_steps,
            "sm_mhz": mhz, "pipes_busy_ncu": NCU_WALK["pipes_busy"],
            "source": NCU_WALK["capture"], "sources_sha256": NCU_WALK["sources_sha256"],
            "stale": not current,
        }

    # the exact (bit-reproducible) arithmetic on the same workload, as many
    # launches as the headline
    exact = None
    if args.math == "fast":
        pe = tmc.params(seed=1, photon_id_base=rank * args.photons, math="exact", **optics)
        one_step(pe)
        torch.cuda.synchronize()
        ex_ms = []
        for _ in range(args.steps):
            ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.zero_()
            ea.record(stream)
            one_step(pe)
            eb.record(stream)
            torch.cuda.synchronize()
            ex_ms.append(ea.elapsed_time(eb))
        exact = {"value": args.photons * world * len(ex_ms) / (sum(ex_ms) * 1e-3), "unit": UNIT,
                 "launches": len(ex_ms), "ms_per_launch": sum(ex_ms) / len(ex_ms),
                 "vs_fast": sum(ms) / len(ms) / (sum(ex_ms) / len(ex_ms))}

    # e2e through the host-array C ABI call
    e2e = None
    if not args.no_e2e:
        heat = np.zeros(S, np.float32)
        heat2 = np.zeros(S, np.float32)
        tmc.photon_batch(heat, heat2, args.photons, p)     # warm
        if dist is not None:
            dist.barrier()
        wall = []
        for _ in range(max(1, min(args.steps, 3))):
            t0 = time.perf_counter()
            tmc.photon_batch(heat, heat2, args.photons, p)
            wall.append(time.perf_counter() - t0)
        tw = sum(wall)
        if dist is not None:
            t = torch.tensor([tw], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tw = float(t.item())
        e2e = {"value": args.photons * len(wall) * world / tw, "unit": UNIT,
               "h2d_bytes_per_step": 40, "d2h_bytes_per_step": 16 * S,
               "call": "tmc_photon_batch(heat, heat2, n, params) with host float arrays"}

    legs = {}
    if extra_legs:
        legs["high_albedo"] = high_albedo_leg(args, tmc, torch, sfu_peak, device_id)
        legs["sweep"] = sweep_leg(args, tmc, torch, device_id, plain_steps_per_s=steps_per_launch / per_launch_s)
        if args.serve_persistent < 0:
            # one persistent launch fed from a work queue (the server's
            # setting for a dedicated GPU), then the default waves of launches
            args.serve_persistent = 1
            legs["serve"] = serve_leg(args, device_id)
            args.serve_persistent = 0
            legs["serve_waves"] = serve_leg(args, device_id)
            args.serve_persistent = -1
        else:
            legs["serve"] = serve_leg(args, device_id)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, world),
            "photon_steps_per_s": photon_steps_all / (total_ms * 1e-3),
            "steps_per_photon": photon_steps_all / photons_all,
            "value_exact_math": exact["value"] if exact else None, "exact_math": exact,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu_base,
            "gpu_launches": args.steps, "clocks": clk, "wall_s_timed_region": t_wall,
            **legs,
        }
        if replicas is not None:
            line["replicas"] = replicas
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def high_albedo_leg(args, tmc, torch, sfu_peak, device_id):
    """The plain walk at high albedo (~7168 steps per photon): 2^28 photons
    per launch, one warm-up launch of 2^24 photons, then timed launches."""
    o = OPTICS["high_albedo"]
    n = args.high_albedo_photons
    dev = torch.device("cuda", torch.cuda.current_device())
    tally = torch.zeros((o["shells"], 4), dtype=torch.int64, device=dev)
    steps_ctr = torch.zeros(1, dtype=torch.int64, device=dev)
    ws = torch.zeros(max(1, tmc.workspace_bytes() // 8), dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    p = tmc.params(seed=1, math=args.math, **o)
    tmc.photon_batch_device(tally.data_ptr(), 1 << 24, p, 0, ws.data_ptr(), sp)
    torch.cuda.synchronize()
    clocks = ClockSampler(device_id)
    clocks.start()
    ms = []
    for _ in range(args.high_albedo_steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        tmc.photon_batch_device(tally.data_ptr(), n, p, steps_ctr.data_ptr(), ws.data_ptr(), sp)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    clk = clocks.stop()
    steps = int(steps_ctr.item())
    launch_s = sum(ms) / len(ms) * 1e-3
    return {
        "workload": "plain walk, 2^28 photons, high albedo (MU_A 0.1/cm, MU_S 100/cm, 1001 shells of 10 um)",
        "value": n * len(ms) / (sum(ms) * 1e-3), "unit": UNIT, "launches": len(ms),
        "ms_per_launch": sum(ms) / len(ms), "photon_steps_per_s": steps / (sum(ms) * 1e-3),
        "steps_per_photon": steps / (n * len(ms)), "math": args.math,
        "roofline": _sfu_roofline(steps / len(ms), launch_s, sfu_peak),
        "clocks": clk,
    }


def sweep_leg(args, tmc, torch, device_id, plain_steps_per_s=None):
    """The batched sweep: 4096 independent problems (seeded draw of the
    sweep's parameter distribution) in one persistent launch per run, tuned by
    the library's two-stage autotuner and replayed through a CUDA graph;
    against the plain form (one launch per problem, back to back on one
    stream) on every k-th problem."""
    from tiny_mc_gb300.sweep import make_sweep

    sw = make_sweep(4096, seed=0, photon_scale=args.sweep_scale, min_photons=16,
                    mu_a_range=(args.sweep_mu_a_min, 10.0))
    photons = int(sw["n_photons"].sum())
    b = tmc.Batch(sw, seed=1, math=args.math)
    t0 = time.perf_counter()
    if args.batch_config:
        blk, ipb, strm = (int(v) for v in args.batch_config.split(","))
        b.set_config(blk, ipb, False, bool(strm))
        tune_ms = None
    else:
        tune_ms = b.autotune(scale=min(1.0, 1.0 / 16), max_steps_per_photon=2e4)
    tune_s = time.perf_counter() - t0
    refine_ms, refine_s = None, None
    if not args.batch_config and args.sweep_scale <= 1.0 / 16:
        t0 = time.perf_counter()
        refine_ms = b.refine(4)
        refine_s = time.perf_counter() - t0
    b.set_config(**{**b.config(), "use_graph": True})
    _, est_steps = b.info()
    stream = torch.cuda.current_stream()
    b.run(stream.cuda_stream)        # warm-up; captures the graph
    torch.cuda.synchronize()
    clocks = ClockSampler(device_id)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.sweep_steps)]
    for k in range(args.sweep_steps):
        ev[k][0].record(stream)
        b.run(stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [a.elapsed_time(c) for a, c in ev]
    _, steps_pp = b.read()
    photon_steps = int(steps_pp.sum())     # one run's steps (each run zeroes the counters)
    batched = photons * len(ms) / (sum(ms) * 1e-3)
    batched_sps = photon_steps * len(ms) / (sum(ms) * 1e-3)
    n_items, _ = b.info()
    cfg = b.config()
    b.close()

    plain = None
    if args.plain_stride > 0:
        sub = sw[::args.plain_stride]
        d = torch.zeros((int(sub["shells"].max()), 4), dtype=torch.int64, device="cuda")
        st = torch.zeros(1, dtype=torch.int64, device="cuda")
        ws = torch.zeros(max(1, tmc.workspace_bytes() // 8), dtype=torch.int64, device="cuda")
        plist = [tmc.params(shells=int(q["shells"]), microns_per_shell=float(q["microns_per_shell"]),
                            mu_a=float(q["mu_a"]), mu_s=float(q["mu_s"]), seed=1,
                            photon_id_base=int(q["photon_id_base"]), math=args.math) for q in sub]
        sp = stream.cuda_stream
        a_, c_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record(stream)
        for q, p in zip(sub, plist):
            tmc.photon_batch_device(d.data_ptr(), int(q["n_photons"]), p, st.data_ptr(), ws.data_ptr(), sp)
        c_.record(stream)
        torch.cuda.synchronize()
        pms = a_.elapsed_time(c_)
        sub_photons = int(sub["n_photons"].sum())
        plain = {"value": sub_photons / (pms * 1e-3), "unit": UNIT,
                 "photon_steps_per_s": int(st.item()) / (pms * 1e-3),
                 "problems": len(sub), "photons": sub_photons, "ms": pms,
                 "form": f"one tmc_photon_batch_device launch per problem, every {args.plain_stride}th "
                         f"problem of the sweep, back to back on one stream"}
    return {
        "workload": "batched sweep: 4096 problems in one persistent launch, CUDA-graph replay",
        "value": batched, "unit": UNIT, "photon_steps_per_s": batched_sps,
        "runs": len(ms), "ms_per_run": sum(ms) / len(ms),
        "photon_scale": args.sweep_scale, "photons_per_run": photons, "photon_steps_per_run": photon_steps,
        "est_photon_steps_per_run": est_steps, "math": args.math, "sweep_seed": 0, "rng_seed": 1,
        "batch_config": cfg, "work_items": n_items,
        "autotune_s": tune_s, "autotune_best_ms": tune_ms, "refine_s": refine_s, "refine_best_ms": refine_ms,
        "plain_form": plain,
        "photons_per_s_over_plain_form": batched / plain["value"] if plain else None,
        "photon_steps_per_s_over_plain_walk": batched_sps / plain_steps_per_s if plain_steps_per_s else None,
        "gpu_launches_per_run": 1, "clocks": clk,
    }


def serve_leg(args, device_id):
    """The served stream: Poisson arrivals of requests with the sweep's
    parameter distribution, a target RSE at shell 10 in [0.5 %, 5 %] and a
    2^24-photon cap.  Three measurements:
      1. calibration: the first requests of the trace submitted at once give
         the mean photon steps per request;
      2. the configured rate (2000/s) for a fixed window: the server is
         saturated, so photon steps walked per second there is its capacity,
         and 2000/s x mean steps per request / capacity is the offered load;
      3. the same trace with arrivals slowed to 70 % of capacity: p50/p99
         latency of a stream the GPU can sustain."""
    import numpy as np

    from tiny_mc_gb300.serve import Server, make_trace

    n_total = 100000
    req, arr = make_trace(n_total, rate=2000.0, seed=0)
    kw = {} if args.serve_stream < 0 else {"stream": args.serve_stream}
    if args.serve_steps_per_batch > 0:
        kw["steps_per_batch"] = args.serve_steps_per_batch
    if args.serve_steps_per_item >= 0:
        kw["steps_per_item"] = args.serve_steps_per_item
    if args.serve_waves >= 0:
        kw["waves"] = args.serve_waves
    if args.serve_inflight_items >= 0:
        kw["inflight_items"] = args.serve_inflight_items
    if args.serve_persistent >= 0:
        kw["persistent"] = args.serve_persistent
    math = 1 if args.math == "fast" else 0
    clocks = ClockSampler(device_id)
    clocks.start()
    s = Server(slots=args.serve_slots, math=math, **kw)
    C = args.serve_calib
    t0 = time.perf_counter()
    res_c, done_c = s.run_trace(req[:C], np.zeros(C), time_limit_s=600.0)
    t_c = time.perf_counter() - t0
    calib_steps = float(res_c["photon_steps"].sum())
    mean_steps = calib_steps / max(1, done_c)
    W = args.serve_window
    sel = slice(C, C + int(2000.0 * W * 1.5))
    a2 = arr[sel] - arr[sel][0]
    w0 = s.work()
    t0 = time.perf_counter()
    res_o, done_o = s.run_trace(req[sel], a2, time_limit_s=W)
    t_o = time.perf_counter() - t0
    saturated = (s.work() - w0) / t_o          # the GPU never runs out of work here
    offered = 2000.0 * mean_steps / saturated
    arrived = int(np.sum(a2 <= t_o))
    got = res_o["photons"] > 0
    lat_o = res_o["latency_s"][got]
    s.close()
    s = Server(slots=args.serve_slots, math=math, **kw)
    kernel = (("barrier-free" if s.cfg.stream else "per-item barriers") +
              (", one persistent launch fed from a work queue" if s.cfg.persistent else ", waves of launches"))
    rate = 0.7 * saturated / mean_steps
    n3 = max(50, min(int(rate * args.serve_duration), n_total - C))
    sel3 = slice(C, C + n3)
    a3 = (arr[sel3] - arr[sel3][0]) * (2000.0 / rate)
    t0 = time.perf_counter()
    res_s, done_s = s.run_trace(req[sel3], a3, time_limit_s=a3[-1] + args.serve_drain)
    t_s = time.perf_counter() - t0
    clk = clocks.stop()
    got3 = res_s["photons"] > 0
    lat = res_s["latency_s"][got3]
    photons3 = float(res_s["photons"].sum())
    steps3 = float(res_s["photon_steps"].sum())
    cfg = {"slots": args.serve_slots, "kernel": kernel, "steps_per_batch": s.cfg.steps_per_batch,
           "steps_per_item": s.cfg.steps_per_item, "waves": s.cfg.waves or 16,
           "inflight_items": s.cfg.inflight_items}
    s.close()
    pct = lambda v, q: float(np.percentile(v, q)) if len(v) else None  # noqa: E731
    return {
        "workload": "served stream: Poisson arrivals, target RSE at shell 10 in [0.5%, 5%], "
                    "cap 2^24 photons, sweep parameter distribution",
        "value": photons3 / t_s, "unit": UNIT, "math": args.math, "trace_seed": 0, "config": cfg,
        "latency_p50_s": pct(lat, 50), "latency_p99_s": pct(lat, 99),
        "photon_steps_per_s": steps3 / t_s, "seconds": t_s,
        "requests": n3, "completed": int(done_s), "arrival_rate_per_s": rate,
        "reached_target_frac": float(np.mean(res_s["reached_target"][got3])) if got3.any() else None,
        "capacity": {"calibration_requests": C, "calibration_s": t_c,
                     "mean_photon_steps_per_request": mean_steps,
                     "saturated_photon_steps_per_s": saturated,
                     "offered_load_at_2000_per_s": offered},
        "at_2000_per_s_window": {"window_s": W, "arrived": arrived, "completed": int(done_o),
                                 "photons_per_s": float(res_o["photons"].sum()) / t_o,
                                 "photon_steps_per_s_completed": float(res_o["photon_steps"].sum()) / t_o,
                                 "latency_p50_s_completed": pct(lat_o, 50),
                                 "latency_p99_s_completed": pct(lat_o, 99),
                                 "overloaded": bool(offered > 1.0)},
        "clocks": clk,
    }


def _alone(args, leg):
    """--workload sweep / serve: that leg as its own line."""
    import torch

    import tiny_mc_gb300 as tmc
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    out = sweep_leg(args, tmc, torch, _device_id(torch, dev)) if leg == "sweep" else \
        serve_leg(args, _device_id(torch, dev))
    line = {"metric": METRIC, "value": out["value"], "unit": UNIT, "n_gpus": 1,
            "steps": out.get("runs", 1), "warmup": 1 if leg == "sweep" else 0,
            "ms_per_step": out.get("ms_per_run", out.get("seconds", 0) * 1e3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": out["workload"]}, leg: out}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in ("sweep", "serve"):
        return _alone(args, args.workload)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
