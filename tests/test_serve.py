"""Scheduling logic of the continuous-batching server (host only).

A fake backend stands in for the device: each "system" advances a
deterministic counter, and a fake clock advances a fixed time per launched
move, so admission, slot limits, memory limits, rejection, continuous
joining and latency accounting are checked exactly.
"""
import numpy as np
import pytest

from faunus_gb300.serve import Job, Server


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeSystem:
    def __init__(self, spec):
        self.spec = spec
        self.moves = 0
        self.state = 0
        self.closed = False


class FakeBackend:
    """Footprint = spec["bytes"]; a run advances each system's state by a hash of
    (seed, stream, counter) per move, independent of the other systems."""

    def __init__(self, clock, seconds_per_move=1e-6):
        self.clock = clock
        self.spm = seconds_per_move
        self.live = []
        self.launches = []
        self.moves_per_launch = []

    def footprint(self, spec):
        return spec["bytes"]

    def create(self, spec):
        s = FakeSystem(spec)
        self.live.append(s)
        return s

    def run(self, handles, moves, *, seed, streams, counters, dp, dprot):
        self.launches.append(sorted(streams))
        self.moves_per_launch.append(dict(zip(streams, moves)))
        for h, m, st, c in zip(handles, moves, streams, counters):
            for k in range(c, c + m):
                h.state = (h.state * 6364136223846793005 + (seed ^ (st << 20) ^ k)) & (2**64 - 1)
            h.moves += m
        cyc = [m * h.spec.get("cpm", 1000) for h, m in zip(handles, moves)]
        self.clock.t += self.spm * max(c / 1000 for c in cyc)  # the launch lasts as long as its slowest chain
        return np.array(cyc, dtype=np.uint64)

    def run_timed(self, handles, moves, time_budget_s, *, seed, streams, counters, dp, dprot):
        """each chain runs moves of cpm cycles at 1 GHz until its time is spent (at least one)"""
        done = []
        for h, m, st, c in zip(handles, moves, streams, counters):
            per = h.spec.get("cpm", 1000) * 1e-9
            k = min(m, max(1, int(time_budget_s / per + 1e-9))) if m > 0 else 0
            for j in range(c, c + k):
                h.state = (h.state * 6364136223846793005 + (seed ^ (st << 20) ^ j)) & (2**64 - 1)
            h.moves += k
            done.append(k)
        self.launches.append(sorted(streams))
        self.moves_per_launch.append(dict(zip(streams, done)))
        self.clock.t += max(k * h.spec.get("cpm", 1000) * 1e-9 for k, h in zip(done, handles))
        return np.array(done, dtype=np.int64)

    def result(self, h, with_positions):
        return {"energy": float(h.state % 1000003), "accepted": h.moves // 2, "moves": h.moves,
                "positions": None}

    def close(self, h):
        h.closed = True
        self.live.remove(h)


def _server(budget=100, slots=4, block=1000, **kw):
    clock = FakeClock()
    be = FakeBackend(clock)
    return Server(be, hbm_budget=budget, max_slots=slots, block_moves=block, clock=clock, **kw), be, clock


def test_every_job_finishes_with_its_moves():
    srv, be, _ = _server()
    jobs = [Job(spec={"bytes": 10}, moves=m, id=i) for i, m in enumerate([500, 2500, 1000, 0, 7000])]
    rep = srv.run(jobs)
    assert rep["jobs_done"] == 5 and rep["jobs_rejected"] == 0
    assert [srv.results[i].moves for i in range(5)] == [500, 2500, 1000, 0, 7000]
    assert rep["moves"] == 11000 and not be.live


def test_oversize_job_is_rejected_and_others_run():
    srv, be, _ = _server(budget=100)
    rep = srv.run([Job(spec={"bytes": 101}, moves=10, id=0), Job(spec={"bytes": 50}, moves=10, id=1)])
    assert srv.results[0].status.startswith("rejected")
    assert srv.results[1].status == "done"
    assert rep["jobs_rejected"] == 1


def test_admission_waits_for_memory_and_slots():
    srv, be, _ = _server(budget=100, slots=2, block=1000)
    jobs = [Job(spec={"bytes": 60}, moves=3000, id=0), Job(spec={"bytes": 60}, moves=1000, id=1),
            Job(spec={"bytes": 30}, moves=1000, id=2), Job(spec={"bytes": 10}, moves=1000, id=3)]
    srv.run(jobs)
    # job 1 cannot share memory with job 0; jobs 2 and 3 fill the second slot one after the other
    for launch in be.launches:
        assert len(launch) <= 2
        assert sum(jobs[i].spec["bytes"] for i in launch) <= 100
    assert be.launches[0] == [0, 2]
    assert all(r.status == "done" for r in srv.results.values())


def test_continuous_batching_jobs_join_between_rounds():
    srv, be, clock = _server(budget=1000, slots=8, block=1000, round_cycles=1e6)
    # one second per launched move would be too slow: 1 ms per 1000-move round
    be.spm = 1e-6
    jobs = [Job(spec={"bytes": 1}, moves=10000, id=0, arrival_s=0.0),
            Job(spec={"bytes": 1}, moves=2000, id=1, arrival_s=0.0025)]
    srv.run(jobs)
    # job 1 arrived while job 0 was running and was launched together with it
    joint = [l for l in be.launches if l == [0, 1]]
    assert len(joint) == 2
    r0, r1 = srv.results[0], srv.results[1]
    assert r1.admitted_s >= 0.0025 and r1.finished_s < r0.finished_s
    assert r1.latency_s == pytest.approx(r1.finished_s - 0.0025)


def test_result_is_the_same_alone_and_in_the_mix():
    a, _, _ = _server(block=700)
    a.run([Job(spec={"bytes": 1}, moves=5000, id=42)])
    b, _, _ = _server(block=700, slots=8)
    b.run([Job(spec={"bytes": 1}, moves=m, id=i) for i, m in [(1, 900), (2, 12000), (42, 5000), (3, 10)]])
    assert a.results[42].energy == b.results[42].energy


def test_report_percentiles_and_idle_gaps_are_skipped():
    srv, be, clock = _server(budget=100, slots=4, block=1000)
    jobs = [Job(spec={"bytes": 1}, moves=1000 * (i + 1), id=i, arrival_s=10.0 * i) for i in range(10)]
    rep = srv.run(jobs, fast_forward=True)
    lat = np.array([srv.results[i].latency_s for i in range(10)])
    assert rep["p50_latency_s"] == pytest.approx(np.percentile(lat, 50))
    assert rep["p99_latency_s"] == pytest.approx(np.percentile(lat, 99))
    assert (lat > 0).all() and lat.max() < 1.0  # the 10 s gaps were fast-forwarded, not slept


def test_duplicate_ids_and_bad_budget_are_rejected():
    srv, _, _ = _server()
    srv.submit(Job(spec={"bytes": 1}, moves=1, id=7))
    with pytest.raises(ValueError):
        srv.submit(Job(spec={"bytes": 1}, moves=1, id=7))
    with pytest.raises(ValueError):
        Server(FakeBackend(FakeClock()), hbm_budget=0)


def test_time_slices_same_result_and_no_chain_waits():
    """In time-slice rounds each chain runs for the slice (a slow job does fewer moves per
    round, never holding fast ones back); results equal those of the cycle-share rounds."""
    jobs = lambda: [Job(spec={"bytes": 1, "cpm": 1000}, moves=40000, id=0),
                    Job(spec={"bytes": 1, "cpm": 4000}, moves=10000, id=1),
                    Job(spec={"bytes": 1, "cpm": 2000}, moves=7, id=2)]
    a, _, _ = _server(budget=100, slots=4, block=500, round_cycles=4e6)
    a.run(jobs())
    b, be, _ = _server(budget=100, slots=4, time_slice_s=4e-3)
    b.run(jobs())
    assert be.moves_per_launch[0] == {0: 4000, 1: 1000, 2: 7}
    for i in range(3):
        assert a.results[i].energy == b.results[i].energy and b.results[i].moves == a.results[i].moves
    with pytest.raises(ValueError):
        _server(time_slice_s=0.0)


def test_round_shares_follow_measured_cycles_per_move():
    """A slow job (4x the cycles per move) gets a quarter of a fast job's moves per round
    after its calibration round, so neither waits on the other."""
    srv, be, _ = _server(budget=100, slots=4, block=500, round_cycles=4e6, min_block=10)
    srv.run([Job(spec={"bytes": 1, "cpm": 1000}, moves=40000, id=0),
             Job(spec={"bytes": 1, "cpm": 4000}, moves=10000, id=1)])
    first, second = be.moves_per_launch[0], be.moves_per_launch[1]
    assert first == {0: 500, 1: 500}          # calibration
    assert second == {0: 4000, 1: 1000}       # 4e6 cycles each
    assert srv.results[0].moves == 40000 and srv.results[1].moves == 10000


def test_gpu_backend_keeps_progress_when_a_cell_list_fills():
    """fau_run_batch reports FAU_ERR_CAPACITY after doubling the full cell list; the moves each
    chain made are in moves_out, so the time-sliced backend returns them and the next round
    continues; other errors still raise."""
    from faunus_gb300._capi import FAU_ERR_ARG, FAU_ERR_CAPACITY, FauError
    from faunus_gb300.serve import GpuBackend

    class Ctx:
        def __init__(self, status):
            self.status = status

        def run_batch(self, handles, moves_per_system=None, moves_out=None, **kw):
            moves_out[:] = np.minimum(moves_per_system, 7)
            raise FauError(self.status, "fau_run_batch", "full cell")

    be = GpuBackend(Ctx(FAU_ERR_CAPACITY))
    done = be.run_timed([object(), object()], [100, 3], 0.01, seed=1, streams=[1, 2], counters=[0, 0],
                        dp=[1.0, 1.0], dprot=[0.0, 0.0])
    assert list(done) == [7, 3]
    with pytest.raises(FauError):
        GpuBackend(Ctx(FAU_ERR_ARG)).run_timed([object()], [5], 0.01, seed=1, streams=[1], counters=[0],
                                                dp=[1.0], dprot=[0.0])


def test_report_carries_each_jobs_error_against_fp64():
    """The backend's audit of a job (its probes' error against FP64) is kept in the job's result,
    and the stream report gives how many jobs carry one and the largest error; a job whose
    backend reports no probe (or none at all) counts as unaudited."""
    srv, be, _ = _server(budget=100, slots=4)
    audits = {0: {"rel_scaled_max": 2e-7, "rel_du_max": 1e-5, "samples": 3},
              1: {"rel_scaled_max": 5e-7, "rel_du_max": 4e-5, "samples": 1},
              2: {"rel_scaled_max": 0.0, "rel_du_max": 0.0, "samples": 0}}
    plain = be.result

    def result(h, with_positions):
        r = plain(h, with_positions)
        if h.spec["id"] in audits:
            r["du_err"] = audits[h.spec["id"]]
        return r

    be.result = result
    jobs = [Job(spec={"bytes": 10, "id": i}, moves=1000, id=i) for i in range(4)]
    rep = srv.run(jobs)
    assert rep["jobs_done"] == 4
    assert rep["jobs_audited"] == 2 and rep["du_err_rel_scaled_max"] == 5e-7
    assert srv.results[0].du_err["samples"] == 3 and srv.results[3].du_err is None
