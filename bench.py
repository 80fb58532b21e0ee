#!/usr/bin/env python3
"""Benchmark of the GB300 photon walk: photons/s of the plain kernel on the
2^30-photon workload (params.h optics: MU_A 2/cm, MU_S 20/cm, 101 shells of
50 um, Philox seed 1, photon ids 0 .. 2^30-1).

One step = one walk of the whole photon batch (one kernel launch).  Prints
one JSON line (rank 0).  Usage:

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* value: photons/s over all ranks, device time of the walk (CUDA events on
  the launching stream), L2 flushed between timed steps;
* e2e: the same metric through the C ABI's host-array call
  tmc_photon_batch(heat, heat2, n, params), wall time of the whole call
  (launch, walk, FP64 finalisation, device-to-host copy of the result);
* roofline: the bound named for this path, SFU-class operations
  (4 per photon step: log, 2 sqrt, divide) against the measured MUFU rate;
* cpu_baseline: the reference's walk on this host's cores (libc rand).

Multi-GPU (torchrun): each rank walks its own 2^30 photons (ids offset by
rank), no collective on the data path; weak scaling.
"""
from __future__ import annotations

import argparse
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
CPU_PHOTONS_PER_PROC = 1 << 16
# Issue-slot accounting of walk_plain<512, FastMath> at params.h optics, from
# ncu --set full of one 2^25-photon launch (profiles/walk_plain_fast_
# 2p25photons_ncu_full.txt): thread-instructions per photon step and the busy
# fraction of each pipe (thread-instructions with the predicate on).  An SM
# issues at most 4 warp-instructions per clock.
WALK_THREAD_INSTR_PER_STEP = 232.2
WALK_PIPES_NCU = {"issue_slots": 0.815, "alu": 0.544, "fma_heavy": 0.489, "xu_sfu": 0.216,
                  "shared_wavefronts": 0.515, "dram": 0.0}
# DRAM bytes (read + write) of one walk launch, from an ncu capture of the walk
# at params.h optics (2^25 photons): only the 101-shell tally flush touches
# DRAM, so the figure does not grow with the photon count.
WALK_DRAM_BYTES_PER_LAUNCH = 20736


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
    ap.add_argument("--optics", choices=["params_h", "high_albedo"], default="params_h",
                    help="plain workload optics: params_h = params.h (101 shells, 50 um, MU_A 2, MU_S 20); "
                         "high_albedo = high albedo (1001 shells, 10 um, MU_A 0.1, MU_S 100)")
    ap.add_argument("--sweep-mu-a-min", type=float, default=0.01,
                    help="sweep workload: lower end of the mu_a range (0.01: the full sweep distribution)")
    ap.add_argument("--workload", choices=["plain", "sweep", "serve"], default="plain",
                    help="plain: 2^30 photons at params.h optics (default); sweep: the 4096-problem batched sweep; "
                         "serve: the request stream")
    ap.add_argument("--serve-slots", type=int, default=1024)
    ap.add_argument("--serve-steps-per-batch", type=float, default=0.0,
                    help="server RSE batch size in photon steps (0: library default)")
    ap.add_argument("--serve-steps-per-item", type=float, default=-1.0,
                    help="server work item size in photon steps (0: one item per batch; -1: library default)")
    ap.add_argument("--serve-inflight-items", type=int, default=-1,
                    help="server cap on launched, unfinished work items (0: none; -1: library default)")
    ap.add_argument("--serve-waves", type=int, default=-1,
                    help="server launches in flight (1..16; -1: library default)")
    ap.add_argument("--serve-stream", type=int, choices=[-1, 0, 1], default=-1,
                    help="server kernel: 0 per-item barriers, 1 barrier-free, -1 library default")
    ap.add_argument("--serve-calib", type=int, default=256)
    ap.add_argument("--serve-window", type=float, default=10.0)
    ap.add_argument("--serve-duration", type=float, default=60.0)
    ap.add_argument("--serve-drain", type=float, default=120.0)
    ap.add_argument("--sweep-scale", type=float, default=1.0 / 64,
                    help="photon-count multiplier of the sweep (1 = full size, ~3.3e13 steps)")
    ap.add_argument("--batch-config", default="",
                    help="sweep: fixed 'block,items_per_block,stream' instead of the autotuner")
    ap.add_argument("--plain-steps", type=int, default=1,
                    help="sweep workload: timed passes of the one-launch-per-problem form")
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
def _cpu_worker(args):
    """One process: photons/s of the reference walk (libc rand) on one core."""
    photons, seed = args
    sys.path.insert(0, ROOT)
    from oracle import oracle
    if oracle.ref_available("params_h", "nat"):
        try:
            L = oracle.ref_lib("params_h", "nat")
            return L.ref_native_rate(photons, seed), "reference"
        except OSError:
            pass
    rate, _ = oracle.native_rate(oracle.cfg("params_h"), photons, seed)
    return rate, "port"


class CpuPool:
    def __init__(self, procs):
        import multiprocessing as mp
        self.procs = procs
        self.pool = mp.get_context("spawn").Pool(procs)

    def step(self, photons_per_proc):
        t0 = time.perf_counter()
        res = self.pool.map(_cpu_worker, [(photons_per_proc, i + 1) for i in range(self.procs)])
        dt = time.perf_counter() - t0
        kind = res[0][1]
        return self.procs * photons_per_proc / dt, kind, [r[0] for r in res]

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline_measure():
    from oracle import oracle
    oracle.build(ref=False)
    cores = cpu_cores()
    pool = CpuPool(cores)
    pool.step(1 << 12)                                    # warm the workers
    rate, kind, per = pool.step(CPU_PHOTONS_PER_PROC * 2)
    pool.close()
    single = statistics.median(per)
    return {
        "value": rate, "unit": UNIT, "cores": cores, "kind": kind,
        "single_thread_value": single,
        "sample": f"{cores} processes x {CPU_PHOTONS_PER_PROC * 2} photons, params.h optics, "
                  f"libc rand seeds 1..{cores} (one process per core); single-thread = median process",
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    from oracle import oracle
    oracle.build(ref=False)
    cores = cpu_cores()
    pool = CpuPool(cores)
    for _ in range(args.warmup):
        pool.step(CPU_PHOTONS_PER_PROC)
    rates, times, kind = [], [], "port"
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r, kind, _ = pool.step(CPU_PHOTONS_PER_PROC)
        times.append(time.perf_counter() - t0)
        rates.append(r)
    pool.close()
    total = cores * CPU_PHOTONS_PER_PROC * args.steps
    value = total / sum(times)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(args, world), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"each step: {cores} processes x {CPU_PHOTONS_PER_PROC} photons of "
                                   f"the reference walk (libc rand, params.h optics)"},
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

    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_base = cpu_baseline_measure()

    dev = torch.device("cuda", torch.cuda.current_device())
    props = torch.cuda.get_device_properties(dev)
    uuid = getattr(props, "uuid", None)
    device_id = f"GPU-{uuid}" if uuid is not None else None

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

    def one_step():
        tmc.photon_batch_device(tally.data_ptr(), args.photons, p, steps_ctr.data_ptr(), ws.data_ptr(), sp)

    sfu_peak = tmc.probe_sfu_rate()
    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    steps_ctr.zero_()

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
    if dist is not None:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        ps = torch.tensor([photon_steps], device=dev, dtype=torch.int64)
        dist.all_reduce(ps)
        photon_steps_all = int(ps.item())
    else:
        photon_steps_all = photon_steps
    photons_all = args.photons * args.steps * world
    value = photons_all / (total_ms * 1e-3)

    # roofline of the dominant kernel (the walk is the only kernel per step)
    per_launch_s = (sum(ms) / len(ms)) * 1e-3
    per_launch_ops = SFU_OPS_PER_STEP * photon_steps / args.steps
    achieved = per_launch_ops / per_launch_s
    roofline = {
        "bound": "sfu", "achieved": achieved / 1e9, "peak": sfu_peak / 1e9, "unit": "Gop/s",
        "frac": achieved / sfu_peak,
        "traffic": WALK_DRAM_BYTES_PER_LAUNCH if args.optics == "params_h" else None,
        "traffic_note": "DRAM bytes per launch (ncu, 101 shells); tally flush only, independent of photons",
        "algorithmic_unit": "4 SFU-class ops (log, sqrt, divide, sqrt) per photon step",
        "photon_steps_per_launch": photon_steps / args.steps,
        "peak_source": "measured live: MUFU lg2/sqrt/rcp probe (tmc_probe_sfu_rate)",
    }
    # the pipe that binds: instruction issue (4 warp-instructions per clock per
    # SM); its ceiling at the sampled clock, and the ncu pipe utilisations
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    if mhz and args.optics == "params_h" and args.math == "fast":
        issue_steps = props.multi_processor_count * mhz * 1e6 * 4 * 32 / WALK_THREAD_INSTR_PER_STEP
        roofline["binding_pipe"] = {
            "pipe": "instruction issue", "thread_instr_per_step": WALK_THREAD_INSTR_PER_STEP,
            "ceiling_photon_steps_per_s": issue_steps,
            "frac": (photon_steps / args.steps / per_launch_s) / issue_steps,
            "sm_mhz": mhz, "pipes_busy_ncu": WALK_PIPES_NCU,
            "source": "ncu --set full, profiles/walk_plain_fast_2p25photons_ncu_full.txt",
        }

    # the exact (bit-reproducible) arithmetic on the same workload, for reference
    value_exact = None
    if args.math == "fast" and not args.no_e2e:
        pe = tmc.params(seed=1, photon_id_base=rank * args.photons, math="exact", **optics)
        tmc.photon_batch_device(tally.data_ptr(), args.photons, pe, 0, ws.data_ptr(), sp)
        torch.cuda.synchronize()
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.zero_()
        ea.record(stream)
        tmc.photon_batch_device(tally.data_ptr(), args.photons, pe, 0, ws.data_ptr(), sp)
        eb.record(stream)
        torch.cuda.synchronize()
        value_exact = args.photons * world / (ea.elapsed_time(eb) * 1e-3)

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

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, world),
            "photon_steps_per_s": photon_steps_all / (total_ms * 1e-3),
            "steps_per_photon": photon_steps_all / photons_all,
            "value_exact_math": value_exact,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu_base,
            "gpu_launches": args.steps, "clocks": clk, "wall_s_timed_region": t_wall,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_sweep(args):
    """The batched sweep: 4096 independent problems (seeded draw of the sweep's
    parameter distribution) in one persistent launch per step, against the
    plain form (one launch per problem, back to back on one stream)."""
    import torch

    import tiny_mc_gb300 as tmc
    from tiny_mc_gb300.sweep import make_sweep

    torch.cuda.set_device(0)
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
        # second stage on the batch itself (4 full runs; skipped at large
        # scales, where each run takes minutes)
        t0 = time.perf_counter()
        refine_ms = b.refine(4)
        refine_s = time.perf_counter() - t0
    b.set_config(**{**b.config(), "use_graph": True})
    _, est_steps = b.info()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        b.run(stream.cuda_stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(None)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        ev[k][0].record(stream)
        b.run(stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [a.elapsed_time(c) for a, c in ev]
    _, steps_pp = b.read()
    photon_steps = int(steps_pp.sum())     # one run's steps (each run zeroes the counters)
    batched = photons * args.steps / (sum(ms) * 1e-3)

    # the plain form: one tmc_photon_batch_device launch per problem
    d = torch.zeros((int(sw["shells"].max()), 4), dtype=torch.int64, device="cuda")
    ws = torch.zeros(max(1, tmc.workspace_bytes() // 8), dtype=torch.int64, device="cuda")
    plist = [tmc.params(shells=int(q["shells"]), microns_per_shell=float(q["microns_per_shell"]),
                        mu_a=float(q["mu_a"]), mu_s=float(q["mu_s"]), seed=1,
                        photon_id_base=int(q["photon_id_base"]), math=args.math) for q in sw]
    sp = stream.cuda_stream
    plain_ms = []
    for _ in range(args.plain_steps):
        a_, c_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record(stream)
        for q, p in zip(sw, plist):
            tmc.photon_batch_device(d.data_ptr(), int(q["n_photons"]), p, 0, ws.data_ptr(), sp)
        c_.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(a_.elapsed_time(c_))
    plain = photons * len(plain_ms) / (sum(plain_ms) * 1e-3) if plain_ms else None
    n_items, _ = b.info()
    line = {
        "metric": METRIC, "value": batched, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(ms) / len(ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched sweep: 4096 problems in one persistent launch",
                   "photon_scale": args.sweep_scale, "photons_per_step": photons,
                   "photon_steps_per_step": photon_steps,
                   "est_photon_steps_per_step": est_steps, "math": args.math,
                   "sweep_seed": 0, "rng_seed": 1, "batch_config": b.config(), "work_items": n_items,
                   "autotune_s": tune_s, "autotune_best_ms": tune_ms,
                   "refine_s": refine_s, "refine_best_ms": refine_ms},
        "photon_steps_per_s": photon_steps * args.steps / (sum(ms) * 1e-3),
        "plain_form": ({"value": plain, "unit": UNIT, "ms_per_pass": sum(plain_ms) / len(plain_ms),
                        "launches_per_pass": len(sw)} if plain_ms else None),
        "batched_over_plain": batched / plain if plain else None,
        "gpu_launches": args.steps, "clocks": clk,
    }
    b.close()
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args):
    """The served stream: Poisson arrivals of requests with the sweep's parameter
    distribution, a target RSE at shell 10 in [0.5 %, 5 %] and a 2^24-photon
    cap.  Three measurements on one server:
      1. calibration: the first requests of the trace submitted at once give
         the mean photon steps per request and the server's throughput, hence
      2. the configured rate for a fixed window (no drain): the server is
         saturated, so photon steps walked per second there is its capacity,
         and 2000/s x mean steps per request / capacity is the offered load;
         plus the latency of what completed while the queue grows;
      3. the same trace with arrivals slowed to 70 % of capacity: p50/p99
         latency of a stream the GPU can sustain."""
    import numpy as np
    import torch

    from tiny_mc_gb300.serve import Server, make_trace

    torch.cuda.set_device(0)
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
    s = Server(slots=args.serve_slots, math=1 if args.math == "fast" else 0, **kw)
    # 1. calibration
    C = args.serve_calib
    t0 = time.perf_counter()
    res_c, done_c = s.run_trace(req[:C], np.zeros(C), time_limit_s=600.0)
    t_c = time.perf_counter() - t0
    calib_steps = float(res_c["photon_steps"].sum())
    mean_steps = calib_steps / max(1, done_c)
    capacity = calib_steps / t_c
    # 2. configured rate, fixed window
    W = args.serve_window
    sel = slice(C, C + int(2000.0 * W * 1.2))
    a2 = arr[sel] - arr[sel][0]
    clocks = ClockSampler(None)
    clocks.start()
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
    # 3. slowed to 70 % of capacity
    s = Server(slots=args.serve_slots, math=1 if args.math == "fast" else 0, **kw)
    kernel = "barrier-free" if s.cfg.stream else "per-item barriers"
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
    s.close()
    pct = lambda v, q: float(np.percentile(v, q)) if len(v) else None  # noqa: E731
    line = {
        "metric": METRIC, "value": photons3 / t_s, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": t_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "served stream: Poisson arrivals, target RSE at shell 10 "
                               "in [0.5%, 5%], cap 2^24 photons, sweep parameter distribution",
                   "trace_seed": 0, "math": args.math, "slots": args.serve_slots,
                   "kernel": kernel, "steps_per_batch": s.cfg.steps_per_batch,
                   "steps_per_item": s.cfg.steps_per_item, "waves": s.cfg.waves or 16,
                   "inflight_items": s.cfg.inflight_items},
        "latency_p50_s": pct(lat, 50), "latency_p99_s": pct(lat, 99),
        "photon_steps_per_s": steps3 / t_s,
        "requests": n3, "completed": int(done_s), "arrival_rate_per_s": rate,
        "reached_target_frac": float(np.mean(res_s["reached_target"][got3])) if got3.any() else None,
        "calibration": {"requests": C, "mean_photon_steps_per_request": mean_steps,
                        "calibration_photon_steps_per_s": capacity,
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
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "sweep":
        return run_sweep(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
