"""The continuous-batching server on the device: a job's result is the same
alone and in a mix of jobs that join and leave around it -- the same moves
(device RNG keyed by job id and move counter), bit-identical positions,
acceptance counts and running energy, although the server sizes each job's share
of a round from measured cycles (or from device time, in time-slice rounds) so
launch boundaries differ between the runs (pending Q(k) changes and partial
energy sums stay on the device across launches); p50/p99 latency and throughput
are reported, with every job's error against FP64 from the kernels' audit probes; an over-size job
is rejected without disturbing the others."""
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
    # every result carries the error of its FP32 energy changes against FP64 (audit probes)
    assert rep["jobs_audited"] == 12 and 0.0 < rep["du_err_rel_scaled_max"] <= 1e-6
    assert all(r.du_err["samples"] >= 1 for r in srv.results.values() if r.status == "done")



def test_batched_chain_continues_after_a_full_cell_list(ctx):
    """fau_run_batch stops a chain that fills a cell after that move, doubles the cell list and
    reports FAU_ERR_CAPACITY with every chain's progress in moves_out; continued from there the
    chain ends exactly as one whose cells never fill (no interactions: every move accepted)."""
    from faunus_gb300 import FauError, SystemSpec
    from faunus_gb300 import _capi as A
    L, c = 40.0, 40.0 / 3
    centres = np.array([[(i + 0.5) * c - L / 2, (j + 0.5) * c - L / 2, (k + 0.5) * c - L / 2]
                        for i in range(3) for j in range(3) for k in range(3)])
    pos = np.concatenate([centres, centres[1:8] + 0.1])  # one per cell, 2 in cells 1..7: capacity 8
    n = len(pos)

    def make(cap):
        return ctx.create(SystemSpec(box=np.full(3, L), pos=pos.copy(), charge=np.zeros(n),
                                     type=np.zeros(n, np.int32), group_begin=np.array([0, n], np.int32),
                                     group_flags=np.array([1], np.int32), n_types=1, pair_terms=0,
                                     pair_cutoff=12.0, cell_capacity=cap))

    a, b = make(1), make(64)
    # fill cell (0,0,0) to its capacity of 8 with host proposals (no overflow yet)
    props = np.zeros(7, dtype=A.PROPOSAL_DTYPE)
    props["kind"] = A.FAU_MOVE_ATOMIC
    props["index"] = np.arange(27, 34)
    props["dr"] = centres[0] + 0.2 * np.arange(1, 8)[:, None] / 8 - pos[27:34]
    props["u"] = 0.0
    for s in (a, b):
        s.run_proposals(props)
        assert (s.cells() == 0).sum() == 8
    total, done, fills = 4000, 0, 0
    while done < total:
        out = np.zeros(1, np.int64)
        try:
            ctx.run_batch([a], moves_per_system=[total - done], seed=2, counters=[done], dp=9.0, threads=160,
                          moves_out=out)
        except FauError as e:
            assert e.status == A.FAU_ERR_CAPACITY
            fills += 1
        done += int(out[0])
    ctx.run_batch([b], total, seed=2, dp=9.0, threads=160)
    assert fills >= 1
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.cells(), b.cells())
