"""The continuous-batching server on the device: a job's result is the same
alone and in a mix of jobs that join and leave around it -- the same moves
(device RNG keyed by job id and move counter), bit-identical positions,
acceptance counts and running energy, although the server sizes each job's share
of a round from measured cycles (or from device time, in time-slice rounds) so
launch boundaries differ between the runs (pending Q(k) changes and partial
energy sums stay on the device across launches); p50/p99 latency and throughput
are reported; an over-size job is rejected without disturbing the others."""
import numpy as np
import pytest

from faunus_gb300 import configs
from faunus_gb300.serve import GpuBackend, Job, Server, jobs_from_stream
from faunus_gb300.system import footprint

pytestmark = pytest.mark.gpu


def _job(kind, jid, moves, arrival=0.0):
    if kind == "pm":
        spec, dp, dprot = configs.primitive_model(n=200, seed=jid), 2.0, 0.0
    elif kind == "bulk":
        spec, dp, dprot = configs.bulk_ewald(n_salt=500, seed=jid), 2.0, 0.0
    else:
        spec, dp, dprot = configs.spce_water(n_mol=256, L=18.6, seed=jid), 0.5, 0.5
    return Job(spec=spec, moves=moves, id=jid, dp=dp, dprot=dprot, arrival_s=arrival)


@pytest.mark.parametrize("kind,slice_s", [("pm", None), ("bulk", None), ("water", None), ("pm", 2e-4),
                                          ("bulk", 1e-4), ("water", 5e-4)])
def test_served_job_same_alone_and_in_mix(ctx, kind, slice_s):
    budget = 2 << 30
    alone = Server(GpuBackend(ctx), hbm_budget=budget, block_moves=1500, seed=9, keep_positions=True)
    alone.run([_job(kind, 17, 6000)])
    mix = Server(GpuBackend(ctx), hbm_budget=budget, block_moves=1500, seed=9, keep_positions=True,
                 time_slice_s=slice_s)
    others = [_job("pm", 3, 2500), _job("bulk", 4, 9000), _job("water", 5, 4000, arrival=0.0),
              _job("bulk", 6, 3000, arrival=0.002)]
    mix.run(others[:2] + [_job(kind, 17, 6000)] + others[2:])
    a, b = alone.results[17], mix.results[17]
    assert a.status == b.status == "done" and a.moves == b.moves == 6000
    if slice_s:
        assert mix.rounds > 2  # the job took several time slices
    assert np.array_equal(a.positions, b.positions)
    assert a.accepted == b.accepted
    assert a.energy == b.energy


def test_served_stream_reports_latency_and_rejects_oversize(ctx):
    stream = configs.served_jobs(n_jobs=12, rate_hz=200.0, n_min=64, n_max=2000, moves_min=2e3, moves_max=2e4,
                                 seed=4)
    jobs = jobs_from_stream(stream)
    big = configs.bulk_ewald(n_salt=10000, seed=1)
    budget = max(footprint(j.spec) for j in jobs) * 6
    assert footprint(big) > budget
    jobs.append(Job(spec=big, moves=100, id=999, arrival_s=0.0))
    srv = Server(GpuBackend(ctx), hbm_budget=budget, block_moves=2000, seed=3)
    rep = srv.run(jobs)
    assert rep["jobs_done"] == 12 and rep["jobs_rejected"] == 1
    assert srv.results[999].status.startswith("rejected")
    assert rep["p50_latency_s"] is not None and rep["p99_latency_s"] >= rep["p50_latency_s"] > 0
    assert rep["moves"] == sum(j.moves for j in jobs if j.id != 999)
    assert srv.resident == 0
