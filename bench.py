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

Beside them the line carries each launch's error against FP64 (audit probes),
the roofline forms, the plain single-system FP64 form, the served stream
(p50/p99 latency, aggregate moves/s, the jobs' audited errors) and the other
configurations: the primitive model in FP32C and as FP64 replica chains, the
bulk system as FP64 replica chains, rigid SPC/E water, and the 256-walker
parallel-tempering ladder beside its uniform-replica equivalent.

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


def cpu_baseline(spec, seconds_per_thread: float = 1.0, threads: int | None = None, check=None) -> dict:
    """The oracle (reference algorithm restated in C++) on the host cores:
    one chain per thread, a bounded number of moves per chain.  check: optional
    (proposals, device dU) of a fresh copy of `spec` run on the device in this run; the
    oracle replays the proposals and the device dU is compared with its FP64 dU."""
    sys.path.insert(0, str(ROOT / "tests"))
    import ctypes as C

    import oracle_lib as O
    from faunus_gb300.system import move_descs

    parity = None
    if check is not None:
        props, du_dev, acc_dev = check
        det = O.OracleSystem(spec).run_detail(props)
        same = np.nonzero(det["accepted"].astype(np.uint8) != acc_dev)[0]
        upto = int(same[0]) + 1 if len(same) else len(props)
        fin = np.isfinite(det["du"][:upto])
        parity = {"moves": len(props), "compared": int(fin.sum()), "identical_accepts_until": upto,
                  **O.du_errors(du_dev[:upto][fin], det["du"][:upto][fin], det["err_scale"][:upto][fin]),
                  "definition": "rel_scaled = |dU_dev - dU_fp64| / max(|dU|, S) (S: sum of |summands|; "
                                "tolerance 1e-6); rel_du = |dU_dev - dU_fp64| / |dU| for |dU| > 1e-3 kT",
                  "source": "device dU of the reference-stream proposals through fau_run_proposals_batch vs "
                            "the FP64 oracle replaying them"}

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
    out = {"value": mps.value, "unit": "moves/s", "cores": threads, "kind": "port",
           "sample": f"{threads} chains x {m} moves of the 20,000-ion bulk Ewald system, one chain per thread "
                     f"({wall.value:.1f} s wall)", "wall_s": wall.value, "moves_per_chain": m}
    if parity is not None:
        out["du_parity"] = parity
    return out


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


def _roofline(R, stats, dev_ms, kv, fp32_peak, sms, sm_mhz):
    """The contract's HBM form for the pipelined chain kernel (algorithmic bytes per launch over its
    device time against the measured copy bandwidth; `traffic` the DRAM bytes of one launch from the
    committed ncu capture of the same kernel) and every other fraction faunus_gb300.roofline
    defines, with the one that binds."""
    from faunus_gb300 import roofline as RL
    moves = sum(s["moves"] for s in stats)
    pairs = sum(s["pair_evals"] for s in stats)
    acc = sum(s["accepted"] for s in stats)
    launches = len(stats)
    mps = moves / (dev_ms * 1e-3)
    alg_b = RL.single_atom_bytes(pairs, moves, acc, kv) / moves
    flops = RL.single_atom_flops(pairs, moves, kv, ewald_pair=True) / moves
    prof = RL.kernel_profile("fast_chain_kernel_bulk_ewald")
    fr = RL.fractions(mps, alg_b, flops, fp32_peak, sms, sm_mhz, prof)
    per_launch_moves = moves / launches
    hbm = fr["hbm"]
    line = {"bound": "hbm", "achieved": hbm["achieved_gbs"], "peak": hbm["peak_gbs"], "unit": "GB/s",
            "frac": hbm["frac"],
            "traffic": prof["dram_bytes_per_move"] * per_launch_moves if prof and prof.get("dram_bytes_per_move")
            else None,
            "peak_source": hbm["peak_source"], "algorithmic_bytes_per_move": alg_b,
            "work": f"{RL.BYTES_PER_K_READ} B read per k-vector and move + {RL.BYTES_PER_K_WRITE} B written per "
                    f"k-vector and accepted move + {RL.BYTES_PER_CANDIDATE_FP32} B per candidate particle "
                    "(faunus_gb300/roofline.py)",
            "note": "the algorithmic bytes are served from shared memory (k-vectors, A_k, Q(k)) and L2 "
                    "(particles); `traffic` is the measured DRAM bytes of one launch"}
    others = {k: v for k, v in fr.items() if k != "hbm"}
    others["flops_per_move"] = flops
    others["work"] = (f"{RL.FLOPS_PER_K_SINGLE_ATOM_MOVE:g} flop per k-vector and move + "
                      f"{RL.FLOPS_PER_PAIR_LJ_EWALD:g} per pair interaction (faunus_gb300/roofline.py)")
    if prof:
        others["profile_source"] = prof.get("source")
    return line, others


def run_ours(args) -> None:
    dist, rank, local, world = _dist_init(args.gpus)
    import faunus_gb300 as F
    from faunus_gb300 import _capi as A
    from faunus_gb300 import configs

    ctx = F.Context(local)
    water = args.workload == "water"
    fp64 = args.workload in ("pm_fp64", "bulk_fp64")
    if args.workload != "bulk" and not args.value_only:
        raise SystemExit(f"--workload {args.workload} is a profiling case: use it with --value-only")
    if water:
        base = configs.spce_water(n_mol=1000)
    elif args.workload == "pm_fp64":
        base = configs.primitive_model(n=200, precision=A.FAU_PREC_FP64)
    else:
        base = configs.bulk_ewald(n_salt=10000, seed=1, precision=A.FAU_PREC_FP64 if fp64 else A.FAU_PREC_FP32C)
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
    if water or fp64:
        threads = max(threads, 0)  # molecular moves: the pipelined molecular kernel; FP64: FP64 chains
    if threads < 0:
        from faunus_gb300 import autotune
        # measured at the replica count this run uses: the CTA size that fits the most chains
        # per SM wins there, not the one fastest with one chain per SM
        tuned = autotune.tune(ctx, first, replicas=R, moves=1000, force=True,
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

    # ---- e2e: reference-stream proposals through the C ABI, host buffers.  Each step's proposals
    # are drawn on the host (mt19937 in the reference's order, as the caller's Move code would) into
    # one of two pinned buffers while the device runs the previous step from the other; the kernel
    # reads its buffer in place; accept flags and dU come back.  Generation, copies and kernels are
    # all inside the timed region.
    gens = [F.MoveGenerator(base, base.extra["moves"], 7 + i, 11 + i, default_seeds=False) for i in range(R)]
    offsets = np.arange(R + 1, dtype=np.int64) * M
    bufs = [_pinned(R * M) for _ in range(2)]
    gen_threads = max(1, min(16, (os.cpu_count() or 2) - 1))
    pool = cf.ThreadPoolExecutor(max_workers=gen_threads)

    def fill(buf):
        t = time.perf_counter()
        props = buf[0]
        chunk = (R + gen_threads - 1) // gen_threads

        def part(c):
            for i in range(c * chunk, min(R, (c + 1) * chunk)):
                props[i * M:(i + 1) * M] = gens[i].generate(M)
        list(pool.map(part, range(gen_threads)))
        return time.perf_counter() - t

    e2e_systems = systems
    for w in range(max(1, args.warmup // 2)):
        fill(bufs[0])
        ctx.run_proposals_batch(e2e_systems, bufs[0][0], offsets, bufs[0][1], bufs[0][2])
    gen_s = []
    kern_s = []
    e2e_moves = 0
    _barrier(dist)
    t1 = time.perf_counter()
    gen_s.append(fill(bufs[0]))
    for k in range(args.steps):
        cur = bufs[k % 2]
        nxt = pool.submit(fill, bufs[(k + 1) % 2]) if k + 1 < args.steps else None
        tk = time.perf_counter()
        st = ctx.run_proposals_batch(e2e_systems, cur[0], offsets, cur[1], cur[2])
        kern_s.append(time.perf_counter() - tk)
        e2e_moves += st["moves"]
        if nxt is not None:
            gen_s.append(nxt.result())
    e2e_wall = time.perf_counter() - t1
    e2e_s = _max_over_ranks(dist, e2e_wall)
    e2e_value = _sum_over_ranks(dist, e2e_moves) / e2e_s
    pool.shutdown()

    # ---- parity of this run's device dU: a fresh copy of the system, the reference stream's first
    # moves through the same entry point (checked against the oracle in the CPU-baseline leg)
    chk = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        fresh = ctx.create(base)
        pg = F.MoveGenerator(base, base.extra["moves"], 7, 11, default_seeds=False).generate(args.parity_moves)
        acc_c = np.zeros(len(pg), np.uint8)
        du_c = np.zeros(len(pg))
        ctx.run_proposals_batch([fresh], pg, np.array([0, len(pg)], np.int64), acc_c, du_c)
        fresh.close()
        chk = (pg, du_c, acc_c)

    # ---- roofline of the pipelined chain kernel
    peak = ctx.fp32_peak_tflops()
    roof, roof_other = _roofline(R, stats, dev_ms, systems[0].K, peak, sms, clk.get("sm_mhz"))

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
                "d2h_bytes_per_step": int(R * M * 9),
                "covers": "host proposal generation (reference mt19937 stream, "
                          f"{gen_threads} host threads, double-buffered) + host->device reads of the pinned "
                          "proposals + kernels + accept flags and dU back",
                "generation_s_per_step": statistics.mean(gen_s), "call_s_per_step": statistics.mean(kern_s),
                "generation_moves_per_s": R * M / statistics.mean(gen_s),
                "wall_s": e2e_wall},
        "du_err_vs_fp64_audit": {
            "rel_scaled_max": max(s["du_err_scaled_max"] for s in stats),
            "rel_du_max": max(s["du_err_rel_max"] for s in stats),
            "probes": sum(s["du_err_samples"] for s in stats),
            "how": "every launch: each chain's probe move (its next proposal, not decided) re-evaluated in FP64 on "
                   "the same state; rel_scaled = |dU32 - dU64| / max(|dU64|, S), rel_du = / |dU64| (|dU64| > 1e-3)"},
        "roofline": roof,
        "roofline_other": roof_other,
        "clocks": clk,
        # per timed step (one fau_run_batch call): the chain kernel and its FP64 audit in the graph,
        # and the two counter gathers around it
        "gpu_launches": 4 * args.steps,
        "wall_s": wall,
    }
    if rank == 0 and not args.no_extras:
        line["plain_fp64_single_system"] = plain_form(ctx, base)
        line["plain_fp64_single_system"]["batched_over_plain"] = value / line["plain_fp64_single_system"]["value"]
        line["served"] = served(ctx, F, configs, full=not args.served_bounded)
        line["other_configs"] = other_configs(ctx, configs, R, sweeps=args.pt_sweeps, pt_blocks=args.pt_blocks,
                                              pt_budget_s=args.pt_budget_s)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(base, check=chk)
        line["cpu_baseline"].pop("wall_s", None)
        if "du_parity" in line["cpu_baseline"]:
            line["du_rel_err_max"] = {k: line["cpu_baseline"]["du_parity"][k]
                                      for k in ("rel_scaled_max", "rel_du_max", "rel_du_median")}
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


def other_configs(ctx, configs, replicas: int, sweeps: int = 1000, pt_blocks: int = 2, pt_budget_s: float = 60.0) -> dict:
    """Device-timed throughput of the other configurations (seconds each): the primitive
    model (200 hard-sphere ions; FP32C and, as specified, FP64) and rigid SPC/E water (1,000
    molecules, molecular moves) as replica batches, and the 256-walker parallel-tempering ladder
    (N 100..5,000)."""
    from faunus_gb300 import _capi as A
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
        audit.clear()
        if st["du_err_samples"]:
            audit.update({"rel_scaled_max": st["du_err_scaled_max"], "rel_du_max": st["du_err_rel_max"],
                          "probes": st["du_err_samples"]})
        return st["moves"] / (st["device_ms"] * 1e-3), st["pair_evals"] / (st["device_ms"] * 1e-3)

    audit = {}  # the timed launch's audit probes (error of the FP32 changes against FP64)

    mps, pps = batch_rate(configs.primitive_model(n=200), replicas, 20000)
    out["primitive_model_200"] = {"replicas": replicas, "moves_per_s": mps, "pair_interactions_per_s": pps,
                                  "du_err_vs_fp64_audit": dict(audit)}
    # the primitive model as specified, in FP64: FP64 replica chains (fau_fp64.cu)
    mps, pps = batch_rate(configs.primitive_model(n=200, precision=A.FAU_PREC_FP64), replicas, 20000)
    out["primitive_model_200_fp64"] = {"replicas": replicas, "moves_per_s": mps, "pair_interactions_per_s": pps,
                                       "kernel": "FP64 replica chains (plain FP64 pair sums and decision, "
                                                 "all pairs, one CTA per system)"}
    # the benchmark system itself as FP64 replica chains: what the FP32C form gains over FP64
    mps, pps = batch_rate(configs.bulk_ewald(n_salt=10000, seed=1, precision=A.FAU_PREC_FP64), replicas, 1000)
    out["bulk_ewald_20000_fp64"] = {"replicas": replicas, "moves_per_s": mps, "pair_interactions_per_s": pps,
                                    "kernel": "FP64 replica chains (FP64 pairs over each state's cell stencil, "
                                              "FP64 sin/cos of k.r for the K = 1152 k-vectors)"}
    mps, pps = batch_rate(configs.spce_water(n_mol=1000), replicas, 5000)
    out["spce_water_1000"] = {"replicas": replicas, "moves_per_s": mps, "pair_interactions_per_s": pps,
                              "kernel": "pipelined molecular kernel (1 preparing + 7 compute warps)",
                              "du_err_vs_fp64_audit": dict(audit)}
    out["parallel_tempering_256"] = parallel_tempering(ctx, configs, sweeps, pt_blocks, pt_budget_s)
    return out


def parallel_tempering(ctx, configs, sweeps: int, blocks: int, budget_s: float) -> dict:
    """Config 3: 256 primitive-model walkers, N ~ U{100..5000}, T 250-400 K geometric, a swap
    round every `sweeps` sweeps of each walker (sweeps x N_i moves per walker between rounds), all
    blocks and swap rounds in one CUDA graph.  A one-sweep calibration block measures each walker's
    cycles per move first; the configured sweeps run when the predicted time of the blocks fits
    `budget_s` (the longest walker sets a block's length), otherwise the most sweeps that fit."""
    specs, temps = configs.pt_replicas(n_rep=256)
    systems = [ctx.create(s_) for s_ in specs]
    n = np.array([s_.n for s_ in specs], np.int64)
    cyc = np.zeros(len(specs), np.uint64)
    cal = ctx.run_batch(systems, moves_per_system=n, swap_interval=1, n_swap_blocks=1, temperatures=temps, seed=3,
                        dp=2.0, cycles_out=cyc)
    sec_per_sweep = float(cal["device_ms"]) * 1e-3
    run_sweeps = sweeps
    if sec_per_sweep * sweeps * blocks > budget_s:
        run_sweeps = max(1, int(budget_s / (sec_per_sweep * blocks)))
    lens = n * run_sweeps
    st = ctx.run_batch(systems, moves_per_system=lens, swap_interval=1, n_swap_blocks=blocks, temperatures=temps,
                       seed=3, dp=2.0, counter_base=1)
    for s_ in systems:
        s_.close()
    # the uniform-replica comparison at equal total particles: 256 walkers of the ladder's mean
    # size at its middle temperature, 10 sweeps each
    nm = int(round(n.mean() / 2) * 2)
    uni = configs.primitive_model(n=nm, L=50.0 * (nm / 200.0) ** (1.0 / 3.0), lB=7.1 * 298.0 / 316.0,
                                  temperature=316.0, seed=5)
    ub = ctx.create(uni)
    usys = [ub] + [ub.clone() for _ in range(len(specs) - 1)]
    ctx.run_batch(usys, nm, seed=1, dp=2.0)
    su = ctx.run_batch(usys, 10 * nm, seed=1, counter_base=nm, dp=2.0)
    for s_ in usys:
        s_.close()
    uni_mps = su["moves"] / (su["device_ms"] * 1e-3)
    longest = int(np.argmax(cyc))
    return {"moves_per_s": st["moves"] / (st["device_ms"] * 1e-3), "moves": st["moves"],
            "device_s": st["device_ms"] * 1e-3, "swap_rounds": blocks,
            "sweeps_between_swaps": run_sweeps, "configured_sweeps_between_swaps": sweeps,
            "swaps_attempted": st["swaps_attempted"], "swaps_accepted": st["swaps_accepted"],
            "swap_acceptance": st["swaps_accepted"] / max(1, st["swaps_attempted"]),
            "walkers": len(specs), "particles_total": int(n.sum()),
            "uniform_equivalent": {"walkers": len(specs), "n": nm, "moves_per_s": uni_mps,
                                   "pt_over_uniform": st["moves"] / (st["device_ms"] * 1e-3) / uni_mps,
                                   "what": "the same number of walkers of the ladder's mean size (equal total "
                                           "particles), no swaps, 10 sweeps each"},
            "calibration_s_per_sweep": sec_per_sweep,
            "longest_walker": {"n": int(n[longest]), "cycles_per_move": float(cyc[longest]) / float(n[longest])},
            "note": ("walker i moves sweeps x N_i times between swap rounds (ParallelTempering every 1,000 sweeps); "
                     "a block lasts as long as its longest chain; walkers start in descending order of work")}


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
                          + (" (the configured stream)" if full else " (bounded)")})
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
    ap.add_argument("--served-bounded", action="store_true",
                    help="served stream bounded to N <= 5,000 and 2e5 moves a job (default: the configured stream, "
                         "N log-uniform 64..20,000, 1e4..1e6 moves)")
    ap.add_argument("--parity-moves", type=int, default=2000,
                    help="moves of the device dU checked against the oracle in the CPU-baseline leg")
    ap.add_argument("--cpu-sample-seconds", type=float, default=0.5,
                    help="reference arm: seconds of CPU chain work per thread and step")
    ap.add_argument("--pt-sweeps", type=int, default=1000, help="parallel tempering: sweeps between swap rounds")
    ap.add_argument("--pt-blocks", type=int, default=2, help="parallel tempering: swap rounds measured")
    ap.add_argument("--pt-budget-s", type=float, default=60.0,
                    help="parallel tempering: device seconds allowed; fewer sweeps run if the calibration predicts more")
    ap.add_argument("--value-only", action="store_true", help="device-timed value only (profiling case)")
    ap.add_argument("--workload", default="bulk", choices=["bulk", "water", "pm_fp64", "bulk_fp64"],
                    help="profiling cases, with --value-only: water (1,000 rigid SPC/E molecules, molecular "
                         "moves), pm_fp64 / bulk_fp64 (the 200-ion primitive model / the bulk system as FP64 "
                         "replica chains)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
