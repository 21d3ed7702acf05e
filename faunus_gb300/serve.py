"""Continuous-batching server for Metropolis MC jobs on one GPU.

A job is one Faunus system (``SystemSpec``) and a number of single-atom or
molecular translate/rotate moves.  The server

  * admits queued jobs while a slot is free and the job's device footprint
    (positions, records, cell list, Q(k), pair tables: ``fau_sys_footprint``)
    fits in the HBM budget beside the jobs already resident; a job that can
    never fit is rejected at once;
  * keeps every admitted job's state resident on the device between launches;
  * advances all resident jobs together in one ``fau_run_batch`` launch per
    round (per-system dp and dprot; single-atom jobs in the pipelined kernel,
    molecular ones beside them in the pipelined molecular kernel) -- jobs join and leave
    between rounds, so work that arrives while others run overlaps with them;
  * gives every job the same device time a round: with ``time_slice_s`` each
    chain runs until it has had that much time of its own (the kernels stop at
    the first move boundary past it and report the moves done), so no chain
    waits for another's share; without it, a job's first round is a
    ``block_moves`` calibration, after which its measured SM cycles per move
    set how many moves fit in ``round_cycles``;
  * retires a job when its moves are done and reports, per job, the queueing
    and run time and the error of its FP32 energy changes against FP64 (the
    kernels' audit probes: a job's last round ends with one; a probe with an
    infinite energy change, a hard-sphere overlap, has no finite error and is
    not counted), and for the
    stream, p50/p99 latency (arrival -> result), the aggregate moves/s and the
    largest of those errors.

Each job's moves come from the device counter RNG keyed by (server seed, job
id, move counter), so a job's trajectory -- and its result -- is the same
alone and in any mix of other jobs.

The scheduler talks to a small backend interface (``GpuBackend`` drives the
C ABI); tests of the scheduling logic substitute a host-only backend.
"""
from __future__ import annotations

import time
import dataclasses
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import _capi as A
from ._capi import FauError
from .system import Context, SystemSpec, footprint


@dataclass
class Job:
    spec: SystemSpec
    moves: int
    id: int
    dp: float = 2.0
    dprot: float = 0.0
    arrival_s: float = 0.0  # seconds after the stream starts


@dataclass
class JobResult:
    id: int
    status: str                  # "done" or "rejected: ..."
    moves: int = 0
    accepted: int = 0
    energy: float = float("nan")  # running total energy at the end (kT)
    positions: Optional[np.ndarray] = None
    # the audit probes' error against FP64 ({"rel_scaled_max", "rel_du_max", "samples"}), if any
    du_err: Optional[dict] = None
    arrival_s: float = 0.0
    admitted_s: float = float("nan")
    finished_s: float = float("nan")

    @property
    def latency_s(self) -> float:
        return self.finished_s - self.arrival_s


@dataclass
class _Active:
    job: Job
    handle: object
    bytes: int
    done: int = 0
    admitted_s: float = 0.0
    cycles_per_move: float = 0.0  # measured; 0 until the first round


class GpuBackend:
    """The device through the C ABI: one resident system per job.  `threads` is a fixed
    kernel width (160: the pipelined kernel with 4 compute warps, molecular jobs in 256-thread
    CTAs of the pipelined molecular kernel), so that a job's chain is the same whatever other
    jobs share its launches."""

    def __init__(self, ctx: Context, threads: int = 160):
        self.ctx = ctx
        self.threads = threads

    def footprint(self, spec: SystemSpec) -> int:
        return footprint(spec)

    def create(self, spec: SystemSpec):
        # one code path for every chain of a mixed batch: whole-cell staging (a batch of many
        # shapes with several staging paths side by side measured slower: p50 3.8 s against 2.8 s)
        return self.ctx.create(dataclasses.replace(spec, cell_staging=1))

    def run(self, handles, moves: Sequence[int], *, seed: int, streams: Sequence[int], counters: Sequence[int],
            dp: Sequence[float], dprot: Sequence[float]) -> np.ndarray:
        """Advance each system by its move count in one launch (CUDA graph); returns the SM
        cycles each system's chain took."""
        cycles = np.zeros(len(handles), dtype=np.uint64)
        self.ctx.run_batch(handles, moves_per_system=np.asarray(moves, dtype=np.int64), seed=seed,
                           streams=np.asarray(streams, dtype=np.uint32),
                           counters=np.asarray(counters, dtype=np.uint64), dp_per_system=dp,
                           dprot_per_system=dprot, threads=self.threads, cycles_out=cycles)
        return cycles

    def run_timed(self, handles, moves: Sequence[int], time_budget_s: float, *, seed: int,
                  streams: Sequence[int], counters: Sequence[int], dp: Sequence[float],
                  dprot: Sequence[float]) -> np.ndarray:
        """Advance each system by up to its move count, each chain ending at the first move
        boundary after time_budget_s of its own (one launch); returns the moves each performed."""
        done = np.zeros(len(handles), dtype=np.int64)
        try:
            self.ctx.run_batch(handles, moves_per_system=np.asarray(moves, dtype=np.int64), seed=seed,
                               streams=np.asarray(streams, dtype=np.uint32),
                               counters=np.asarray(counters, dtype=np.uint64), dp_per_system=dp,
                               dprot_per_system=dprot, threads=self.threads, time_budget_s=time_budget_s,
                               moves_out=done)
        except FauError as e:
            # a chain filled a cell list: the library doubled it; every chain's progress is in
            # `done`, and the next round continues from there
            if e.status != A.FAU_ERR_CAPACITY:
                raise
        return done

    def result(self, handle, with_positions: bool) -> dict:
        c = handle.counters()
        return {"energy": handle.running_energy(), "accepted": c["accepted"], "moves": c["moves"],
                "positions": handle.positions() if with_positions else None, "du_err": handle.audit()}

    def close(self, handle) -> None:
        handle.close()


class Server:
    def __init__(self, backend, hbm_budget: int, max_slots: int = 608, block_moves: int = 2000, seed: int = 1,
                 keep_positions: bool = False, clock: Callable[[], float] = time.perf_counter,
                 round_cycles: float = 2e8, min_block: int = 100, time_slice_s: Optional[float] = None):
        """time_slice_s: rounds are time slices -- every resident job runs until its chain has
        had that much device time or its moves are done (backend.run_timed), so no chain waits
        for the slowest share of a round; None: shares of round_cycles from measured cycles
        per move (backend.run)."""
        if hbm_budget <= 0:
            raise ValueError("hbm_budget must be positive")
        self.backend = backend
        self.budget = int(hbm_budget)
        self.max_slots = int(max_slots)
        self.block = int(block_moves)
        self.round_cycles = float(round_cycles)
        self.min_block = int(min_block)
        self.time_slice = None if time_slice_s is None else float(time_slice_s)
        if self.time_slice is not None and not self.time_slice > 0:
            raise ValueError("time_slice_s must be positive")
        self.seed = int(seed)
        self.keep_positions = keep_positions
        self.clock = clock
        self.queue: List[Job] = []
        self.active: Dict[int, _Active] = {}
        self.results: Dict[int, JobResult] = {}
        self.moves_done = 0
        self.rounds = 0
        self.resident = 0  # footprint of the admitted jobs (the budget covers only these)
        self.need: Dict[int, int] = {}
        self.t0 = None

    # ---------------------------------------------------------------- time
    def now(self) -> float:
        if self.t0 is None:
            self.t0 = self.clock()
        return self.clock() - self.t0

    # ---------------------------------------------------------------- jobs
    def submit(self, job: Job) -> None:
        if job.id in self.active or job.id in self.results or any(q.id == job.id for q in self.queue):
            raise ValueError(f"job id {job.id} already used")
        if job.moves < 0:
            raise ValueError("negative move count")
        self.need[job.id] = int(self.backend.footprint(job.spec))  # once per job, not per admission attempt
        self.queue.append(job)

    def _admit(self) -> None:
        now = self.now()
        keep = []
        for job in self.queue:
            if job.arrival_s > now:
                keep.append(job)
                continue
            need = self.need[job.id]
            if need > self.budget:
                self.results[job.id] = JobResult(job.id, f"rejected: footprint {need} B exceeds the HBM budget "
                                                         f"{self.budget} B", arrival_s=job.arrival_s,
                                                 finished_s=now)
                continue
            if len(self.active) >= self.max_slots or self.resident + need > self.budget:
                keep.append(job)  # waits for a slot / memory to free up
                continue
            self.active[job.id] = _Active(job, self.backend.create(job.spec), need, admitted_s=now)
            self.resident += need
        self.queue = keep

    def _retire(self) -> None:
        now = self.now()
        for jid in [j for j, a in self.active.items() if a.done >= a.job.moves]:
            a = self.active.pop(jid)
            r = self.backend.result(a.handle, self.keep_positions)
            self.backend.close(a.handle)
            self.resident -= a.bytes
            self.results[jid] = JobResult(jid, "done", moves=r["moves"], accepted=r["accepted"], energy=r["energy"],
                                          positions=r["positions"], du_err=r.get("du_err"), arrival_s=a.job.arrival_s,
                                          admitted_s=a.admitted_s, finished_s=now)

    def step(self) -> int:
        """Admit, run one round of moves over every resident job, retire; returns moves run."""
        self._admit()
        self._retire()  # zero-move jobs
        if not self.active:
            return 0
        members = list(self.active.values())
        kw = dict(seed=self.seed, streams=[a.job.id for a in members], counters=[a.done for a in members],
                  dp=[a.job.dp for a in members], dprot=[a.job.dprot for a in members])
        total = 0
        if self.time_slice is not None:
            ran = self.backend.run_timed([a.handle for a in members], [a.job.moves - a.done for a in members],
                                         self.time_slice, **kw)
            for a, m in zip(members, ran):
                a.done += int(m)
                total += int(m)
        else:
            moves = [min(self._share(a), a.job.moves - a.done) for a in members]
            cycles = self.backend.run([a.handle for a in members], moves, **kw)
            for i, (a, m) in enumerate(zip(members, moves)):
                a.done += m
                total += m
                if cycles is not None and m > 0 and cycles[i] > 0:
                    c = float(cycles[i]) / m
                    a.cycles_per_move = c if a.cycles_per_move == 0.0 else 0.5 * (a.cycles_per_move + c)
        self.moves_done += total
        self.rounds += 1
        self._retire()
        return total

    def _share(self, a: _Active) -> int:
        """Moves of job `a` that fit in this round's cycle budget."""
        if a.cycles_per_move <= 0.0:
            return self.block
        return max(self.min_block, int(self.round_cycles / a.cycles_per_move))

    def idle(self) -> bool:
        return not self.active and not self.queue

    def run(self, jobs: Sequence[Job] = (), fast_forward: bool = True) -> dict:
        """Serve a stream until every job has a result.  With fast_forward, idle gaps
        before the next arrival are skipped (the clock jumps) instead of slept."""
        for j in jobs:
            self.submit(j)
        self.now()
        while not self.idle():
            ran = self.step()
            if ran == 0 and not self.active and self.queue:
                wait = min(j.arrival_s for j in self.queue) - self.now()
                if wait > 0:
                    if fast_forward:
                        self.t0 -= wait
                    else:
                        time.sleep(wait)
        return self.report()

    def report(self) -> dict:
        done = [r for r in self.results.values() if r.status == "done"]
        lat = np.array([r.latency_s for r in done]) if done else np.zeros(0)
        audited = [r.du_err for r in done if r.du_err and r.du_err.get("samples", 0) > 0]
        wall = self.now()
        return {
            "jobs_done": len(done),
            "jobs_rejected": sum(1 for r in self.results.values() if r.status != "done"),
            "moves": int(self.moves_done),
            "rounds": self.rounds,
            "wall_s": wall,
            "moves_per_s": self.moves_done / wall if wall > 0 else 0.0,
            "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "jobs_audited": len(audited),
            "du_err_rel_scaled_max": max((d["rel_scaled_max"] for d in audited), default=None),
        }


def jobs_from_stream(stream: Sequence[dict]) -> List[Job]:
    """Jobs from configs.served_jobs() records, with the shape's displacement parameters."""
    out = []
    for rec in stream:
        spec = rec["spec"]
        mv = spec.extra["moves"][0]
        out.append(Job(spec=spec, moves=int(rec["moves"]), id=int(rec["id"]), dp=float(mv.get("dp", 2.0)),
                       dprot=float(mv.get("dprot", 0.0)), arrival_s=float(rec["arrival_s"])))
    return out
