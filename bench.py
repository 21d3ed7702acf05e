#!/usr/bin/env python3
"""Benchmark: Metropolis MC trial moves/s of the bulk-salt Ewald system.

Workload (one step): R independent replica chains of the 20,000-ion bulk
salt system (0.1 M, LJ + Coulomb, real-space erfc cutoff 12 A, alpha 0.3/A,
ncutoff 8 -> 1152 k-vectors, 45^3 cells, atomic translation moves), each
advanced by M trial moves in one persistent chain-kernel launch.

  value   device-timed moves/s with all state resident in HBM, proposals
          from the on-device counter RNG (fau_run_batch).
  e2e     the same moves through the drop-in C ABI (fau_run_proposals_batch):
          proposals drawn on the host in the reference's mt19937 order, in
          pinned host memory that the kernel reads in place (72 B per move cross
          host->device while the chains run), accept flags + dU copied back, all
          inside the timed region.
  --impl reference
          the CPU oracle (the reference algorithm restated: all-pairs
          Nonbonded, O(K) Ewald per state, two-state sync) on all host
          threads, one chain per thread, bounded sample per step.

Multi-GPU: replicas only (one process per GPU, each with its own R replicas,
no collective on the data path); timing is max over ranks.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# algorithmic work per unit (flops; add/mul/compare = 1, FMA = 2)
FLOPS_PER_K_UPDATE = 37.0    # per k-vector per moved atom: midpoint phase (12), sin(D/2) (9), dQ (3),
                             # pending fold (2), dU_rec term (7), accumulation (4)
FLOPS_PER_PAIR = 38.0        # per pair interaction (LJ + Ewald real space)
BYTES_PER_PAIR_CANDIDATE = 16.0


def _env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"fau_clocks_{os.getpid()}.csv"

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist_init(n_gpus):
    rank, local, world = _env_rank()
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return dist, rank, local, world
    return None, 0, 0, 1


def _max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_streams(R: int, rank: int) -> np.ndarray:
    """Device RNG streams of one rank's replicas: disjoint across ranks (replicas only)."""
    return np.arange(R, dtype=np.uint32) + np.uint32(1_000_000 * rank)


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _sum_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def _profile_traffic():
    """DRAM bytes per move of the pipelined chain kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "fast_chain_kernel_bulk_ewald.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["dram_bytes_per_move"]), d.get("source", str(p.name))
        except (ValueError, KeyError):
            pass
    return None, None


def cpu_baseline(spec, seconds_per_thread: float = 1.0, threads: int | None = None) -> dict:
    """The oracle (reference algorithm restated in C++) on the host cores:
    one chain per thread, a bounded number of moves per chain."""
    sys.path.insert(0, str(ROOT / "tests"))
    import ctypes as C

    import oracle_lib as O
    from faunus_gb300.system import move_descs

    threads = threads or os.cpu_count() or 1
    d, keep = spec.to_desc()
    arr, keep2 = move_descs(spec, spec.extra["moves"])
    L = O.lib()
    mps, wall = C.c_double(), C.c_double()
    # calibrate on one chain, then size the sample to ~seconds_per_thread per thread
    rc = L.orc_bench_chains(C.byref(d), arr, 1, 1, 1, 20, C.byref(mps), C.byref(wall))
    if rc != 0:
        raise RuntimeError(f"oracle bench failed: {rc}")
    per_move = wall.value / 20
    m = max(20, int(seconds_per_thread / max(per_move, 1e-9)))
    rc = L.orc_bench_chains(C.byref(d), arr, 1, threads, threads, m, C.byref(mps), C.byref(wall))
    if rc != 0:
        raise RuntimeError(f"oracle bench failed: {rc}")
    return {"value": mps.value, "unit": "moves/s", "cores": threads, "kind": "port",
            "sample": f"{threads} chains x {m} moves of the 20,000-ion bulk Ewald system, one chain per thread "
                      f"({wall.value:.1f} s wall)", "wall_s": wall.value, "moves_per_chain": m}


def run_reference(args) -> None:
    # rank 0 alone runs the CPU reference; the other ranks exit without work
    rank, _, _ = _env_rank()
    if rank != 0:
        return
    from faunus_gb300 import configs
    spec = configs.bulk_ewald(n_salt=10000, seed=1)
    threads = os.cpu_count() or 1
    sample = args.cpu_sample_seconds
    for _ in range(args.warmup):
        cpu_baseline(spec, seconds_per_thread=0.4 * sample, threads=threads)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(spec, seconds_per_thread=sample, threads=threads))
    wall = time.perf_counter() - t0
    total_moves = sum(v["value"] * v["wall_s"] for v in vals)
    tot_wall = sum(v["wall_s"] for v in vals)
    value = total_moves / tot_wall
    line = {
        "impl": "reference", "metric": "MC trial moves/sec", "value": value, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_wall / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "config": {"workload": "bulk-salt Ewald, 20,000 ions, one chain per host thread", "n_particles": 20000,
                   "kvectors": 1152, "parallelism": f"{threads} host threads"},
        "cpu_baseline": {"value": value, "unit": "moves/s", "cores": threads, "kind": "port",
                         "sample": vals[-1]["sample"]},
        "e2e": {"value": value, "unit": "moves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)


# algorithmic bytes of the path: per k-vector and move 12 B k-vector + 4 B A_k + 16 B Q(k) read,
# per accepted move 16 B Q(k) written a k-vector, per candidate particle 20 B (x, y, z, q, type)
BYTES_PER_K_READ, BYTES_PER_K_WRITE, BYTES_PER_CANDIDATE = 32, 16, 20


def _hbm_roofline(alg_bytes_per_s, dram_bytes_per_move, moves_per_launch, alg_bytes_per_move):
    """The HBM roofline: the path's algorithmic bytes per second against the measured copy
    bandwidth of MEASURED_PEAKS.json; `traffic` the DRAM bytes of one launch from the ncu
    capture of the same kernel (cold cache) -- far below the algorithmic bytes, because each
    chain keeps its k-vector table, A_k and Q(k) in shared memory and its particles in L2."""
    peaks = Path(__file__).resolve().parent / "MEASURED_PEAKS.json"
    try:
        peak = float(json.loads(peaks.read_text())["hbm_gbs"])
        src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError):
        peak, src = 6800.0, "fallback 6.8 TB/s"
    achieved = alg_bytes_per_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": dram_bytes_per_move * moves_per_launch if dram_bytes_per_move else None,
            "algorithmic_bytes_per_move": alg_bytes_per_move, "dram_bytes_per_move": dram_bytes_per_move,
            "peak_source": src,
            "work": f"{BYTES_PER_K_READ} B read per k-vector and move + {BYTES_PER_K_WRITE} B written per "
                    f"k-vector and accepted move + {BYTES_PER_CANDIDATE} B per candidate particle",
            "note": "algorithmic bytes are served from shared memory and L2; traffic = ncu DRAM bytes of "
                    "one launch (8 KB a move, cold cache)"}


def run_ours(args) -> None:
    dist, rank, local, world = _dist_init(args.gpus)
    import faunus_gb300 as F
    from faunus_gb300 import _capi as A
    from faunus_gb300 import configs

    ctx = F.Context(local)
    water = args.workload == "water"
    if water and not args.value_only:
        raise SystemExit("--workload water is a profiling case: use it with --value-only")
    base = configs.spce_water(n_mol=1000) if water else configs.bulk_ewald(n_salt=10000, seed=1)
    dp, dprot = (0.5, 0.5) if water else (2.0, 0.0)
    sms = _sm_count(local)
    R = args.replicas or 4 * sms  # four chains per SM: the pipelined kernel's occupancy limit
    M = args.moves
    first = ctx.create(base)
    systems = [first] + [first.clone() for _ in range(R - 1)]
    streams = replica_streams(R, rank)
    resident = ctx.hbm_used()

    # ---- kernel configuration: the autotuner's choice unless --threads is given
    tuned = None
    threads = args.threads
    if water:
        threads = max(threads, 0)  # molecular moves: the pipelined molecular kernel
    if threads < 0:
        from faunus_gb300 import autotune
        tuned = autotune.tune(ctx, first, replicas=max(8, R // 4), moves=1000, force=True,
                              cache=Path(os.environ.get("TMPDIR", "/tmp")) / f"fau_tune_{os.getpid()}.json")
        threads = tuned["threads"]

    # ---- value: device RNG, resident state
    def step(k):
        return ctx.run_batch(systems, M, seed=args.seed, counter_base=k * M, streams=streams, dp=dp,
                             dprot=dprot, threads=threads)

    for w in range(args.warmup):
        step(w)
    clocks = Clocks(local)
    clocks.start()
    _barrier(dist)
    t0 = time.perf_counter()
    stats = [step(args.warmup + k) for k in range(args.steps)]
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_ms = sum(s["device_ms"] for s in stats)
    dev_s = _max_over_ranks(dist, dev_ms * 1e-3)
    moves = sum(s["moves"] for s in stats)
    pairs = sum(s["pair_evals"] for s in stats)
    kup = sum(s["k_updates"] for s in stats)
    acc = sum(s["accepted"] for s in stats)
    tot_moves = _sum_over_ranks(dist, moves)
    value = tot_moves / dev_s

    if args.value_only:
        if rank == 0:
            print(json.dumps({"metric": "MC trial moves/sec", "value": value, "unit": "moves/s",
                              "ms_per_step": 1e3 * dev_s / args.steps, "replicas": R, "moves": M,
                              "workload": args.workload}), flush=True)
        ctx.close()
        _barrier(dist)
        return

    # ---- e2e: reference-stream proposals through the C ABI, host buffers
    gens = [F.MoveGenerator(base, base.extra["moves"], 7 + i, 11 + i, default_seeds=False) for i in range(R)]
    offsets = np.arange(R + 1, dtype=np.int64) * M
    props_buf, acc_buf, du_buf = _pinned(R * M)

    def fill():
        def one(i):
            props_buf[i * M:(i + 1) * M] = gens[i].generate(M)
        with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
            list(ex.map(one, range(R)))

    e2e_systems = systems
    for _ in range(max(1, args.warmup // 2)):
        fill()
        ctx.run_proposals_batch(e2e_systems, props_buf, offsets, acc_buf, du_buf)
    e2e_s = 0.0
    e2e_moves = 0
    for _ in range(args.steps):
        fill()  # the step's inputs (drawn by the caller's Move code), outside the timed region
        _barrier(dist)
        t1 = time.perf_counter()
        st = ctx.run_proposals_batch(e2e_systems, props_buf, offsets, acc_buf, du_buf)
        e2e_s += time.perf_counter() - t1
        e2e_moves += st["moves"]
    e2e_s = _max_over_ranks(dist, e2e_s)
    e2e_value = _sum_over_ranks(dist, e2e_moves) / e2e_s

    # ---- roofline of the chain kernel: HBM (algorithmic bytes) and the FP32 pipe
    peak = ctx.fp32_peak_tflops()
    flops = FLOPS_PER_K_UPDATE * kup + FLOPS_PER_PAIR * pairs
    achieved = flops / (dev_ms * 1e-3) / 1e12
    bytes_per_move, src = _profile_traffic()
    traffic = bytes_per_move * (moves / args.steps) if bytes_per_move else None
    kv = systems[0].K
    alg_bytes = BYTES_PER_K_READ * kup + BYTES_PER_K_WRITE * kv * acc + BYTES_PER_CANDIDATE * pairs / 2
    hbm = _hbm_roofline(alg_bytes / (dev_ms * 1e-3), bytes_per_move, moves / args.steps, alg_bytes / max(moves, 1))

    line = {
        "metric": "MC trial moves/sec", "value": value, "unit": "moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic",
        "config": {"workload": "bulk-salt Ewald (20,000 LJ+Coulomb ions, 0.1 M, erfc Rc 12 A, alpha 0.3, "
                               "ncutoff 8, 45^3 cells, transrot dp 2 A) x R replica chains",
                   "replicas_per_gpu": R, "moves_per_replica_per_step": M, "n_particles": base.n,
                   "kvectors": systems[0].K, "cells": "x".join(map(str, systems[0].cell_grid())),
                   "threads_per_chain": threads or 160,
                   "kernel": "pipelined chain kernel" if threads in (0, 96, 160, 288) else "chain kernel",
                   "autotune": ({"table": tuned["table"], "replicas": tuned["replicas"], "moves": tuned["moves"]}
                                if tuned else "off (--threads given)"),
                   "l2": f"inputs larger than L2: {resident / 2**30:.1f} GiB resident per GPU",
                   "parallelism": f"replicas (dp{world})", "rng": "Philox4x32-10 on device (value); "
                   "reference mt19937 stream on host (e2e)"},
        "pair_interactions_per_s": _sum_over_ranks(dist, pairs) / dev_s,
        "k_updates_per_s": _sum_over_ranks(dist, kup) / dev_s,
        "acceptance": acc / max(moves, 1),
        "e2e": {"value": e2e_value, "unit": "moves/s", "h2d_bytes_per_step": int(R * M * 72 + 8 * (R + 1)),
                "d2h_bytes_per_step": int(R * M * 9)},
        "roofline": hbm,
        "roofline_fp32": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                          "frac": achieved / peak if peak else None, "traffic": traffic,
                          "peak_source": "measured FP32 FMA probe (fau_measure_fp32_peak) in this run",
                          "work": f"{FLOPS_PER_K_UPDATE:g} flop per k-vector x moved atom + {FLOPS_PER_PAIR:g} per pair",
                          "traffic_source": src},
        "clocks": clk,
        "gpu_launches": 3 * args.steps,
        "wall_s": wall,
    }
    if rank == 0 and not args.no_extras:
        line["plain_fp64_single_system"] = plain_form(ctx, base)
        line["plain_fp64_single_system"]["batched_over_plain"] = value / line["plain_fp64_single_system"]["value"]
        line["served"] = served(ctx, F, configs, full=args.served_full)
        line["other_configs"] = other_configs(ctx, configs, R)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(base)
        line["cpu_baseline"].pop("wall_s", None)
    if rank == 0:
        print(json.dumps(line), flush=True)
    for s in systems:
        s.close()
    ctx.close()
    _barrier(dist)


def plain_form(ctx, base, moves: int = 400) -> dict:
    """The in-GPU comparison point: the plain single-system form (FP64 accumulation,
    one trial move per call: device pair/Ewald kernels, host Metropolis)."""
    from faunus_gb300 import _capi as A
    import faunus_gb300 as F
    spec = base.copy()
    spec.precision = A.FAU_PREC_FP64
    g = ctx.create(spec)
    props = F.MoveGenerator(spec, spec.extra["moves"], 5, 6, default_seeds=False).generate(moves + 20)
    g.run_proposals(props[:20])  # warm-up
    t0 = time.perf_counter()
    _, _, st = g.run_proposals(props[20:])
    wall = time.perf_counter() - t0
    g.close()
    return {"value": moves / wall, "unit": "moves/s", "moves": moves,
            "form": "FP64 pair and Ewald kernels per trial move, host Metropolis, same 20,000-ion system"}


def other_configs(ctx, configs, replicas: int) -> dict:
    """Device-timed throughput of the other configurations (seconds each): the primitive
    model (200 hard-sphere ions) and rigid SPC/E water (1,000 molecules, molecular moves)
    as replica batches, and the 256-walker parallel-tempering ladder (N 100..5,000)."""
    out = {}

    def batch_rate(spec, R, M, **kw):
        base = ctx.create(spec)
        systems = [base] + [base.clone() for _ in range(R - 1)]
        mv = spec.extra["moves"][0]
        kw.setdefault("dp", mv.get("dp", 2.0))
        kw.setdefault("dprot", mv.get("dprot", 0.0))
        ctx.run_batch(systems, max(1, M // 5), seed=1, **kw)
        st = ctx.run_batch(systems, M, seed=1, counter_base=M, **kw)
        for s_ in systems:
            s_.close()
        return st["moves"] / (st["device_ms"] * 1e-3), st["pair_evals"] / (st["device_ms"] * 1e-3)

    mps, pps = batch_rate(configs.primitive_model(n=200), replicas, 20000)
    out["primitive_model_200"] = {"replicas": replicas, "moves_per_s": mps, "pair_interactions_per_s": pps}
    mps, pps = batch_rate(configs.spce_water(n_mol=1000), replicas, 5000)
    out["spce_water_1000"] = {"replicas": replicas, "moves_per_s": mps, "pair_interactions_per_s": pps,
                              "kernel": "pipelined molecular kernel (1 preparing + 7 compute warps)"}
    specs, temps = configs.pt_replicas(n_rep=256)
    systems = [ctx.create(s_) for s_ in specs]
    st = ctx.run_batch(systems, swap_interval=2000, n_swap_blocks=5, temperatures=temps, seed=3, dp=2.0)
    for s_ in systems:
        s_.close()
    out["parallel_tempering_256"] = {"moves_per_s": st["moves"] / (st["device_ms"] * 1e-3),
                                     "swaps_attempted": st["swaps_attempted"], "swaps_accepted": st["swaps_accepted"],
                                     "swap_interval_moves": 2000,
                                     "note": "one graph: 5 blocks of 2,000 moves per walker + device swap kernel; "
                                             "each block lasts as long as its largest walker (N up to 5,000)"}
    return out


def served(ctx, F, configs, full: bool = False) -> dict:
    """Served MC jobs: Poisson stream of the three single-system shapes, admitted by HBM
    footprint, continuous batching over 608 slots.  full: the configured stream (N
    log-uniform 64..20,000, 1e4..1e6 moves); default: the same shapes bounded to
    N <= 5,000 and <= 2e5 moves per job, so the run takes seconds, not minutes (the
    full stream's tail is single chains of the largest water jobs)."""
    from faunus_gb300.serve import GpuBackend, Server, jobs_from_stream
    if full:
        n_jobs, rate, n_max, m_max = 1000, 320.0, 20000, 1e6
    else:
        n_jobs, rate, n_max, m_max = 2000, 1000.0, 5000, 2e5
    stream = configs.served_jobs(n_jobs=n_jobs, rate_hz=rate, n_max=n_max, moves_max=m_max, seed=4)
    jobs = jobs_from_stream(stream)
    budget = 128 << 30
    srv = Server(GpuBackend(ctx), hbm_budget=budget, max_slots=608, seed=7, time_slice_s=0.025)
    rep = srv.run(jobs, fast_forward=False)
    rep.update({"jobs": n_jobs, "hbm_budget_bytes": budget, "slots": 608,
                "rounds_are": "25 ms time slices: each chain runs until it has had 25 ms of device time",
                "stream": f"served_jobs(seed 4): Poisson {rate:g} jobs/s, primitive model / bulk Ewald / SPC/E "
                          f"water, N log-uniform 64..{n_max}, moves log-uniform 1e4..{m_max:g}"
                          + ("" if full else " (bounded; --served-full for 20,000 / 1e6)")})
    return rep


def _sm_count(dev: int) -> int:
    try:
        import torch
        return torch.cuda.get_device_properties(dev).multi_processor_count
    except Exception:
        return 152


def _pinned(n):
    """Pinned host buffers for the e2e proposals and results."""
    from faunus_gb300 import _capi as A
    try:
        import torch
        p = torch.empty(n * A.PROPOSAL_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True).numpy()
        a = torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy()
        d = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        return p.view(A.PROPOSAL_DTYPE), a, d
    except Exception:
        return np.zeros(n, dtype=A.PROPOSAL_DTYPE), np.zeros(n, np.uint8), np.zeros(n)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--replicas", type=int, default=0, help="replica chains per GPU (0: 4 x SMs)")
    ap.add_argument("--moves", type=int, default=10000, help="moves per replica per step")
    ap.add_argument("--threads", type=int, default=-1,
                    help="kernel configuration: -1 = autotuned; 0/160, 96, 288 = pipelined kernel with 4, 2, 8 "
                         "compute warps; 128/256 = chain kernel")
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the plain-form and served-stream measurements")
    ap.add_argument("--served-full", action="store_true", help="served stream at the full configured job sizes")
    ap.add_argument("--cpu-sample-seconds", type=float, default=0.5,
                    help="reference arm: seconds of CPU chain work per thread and step")
    ap.add_argument("--value-only", action="store_true", help="device-timed value only (profiling case)")
    ap.add_argument("--workload", default="bulk", choices=["bulk", "water"],
                    help="water: 1,000 rigid SPC/E molecules, molecular moves (profiling case, with --value-only)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
