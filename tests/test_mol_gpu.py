"""GPU parity of the pipelined molecular-move kernel (fau_run_batch with the default
kernel choice runs every molecular-move system in it, in 512-thread CTAs when every molecular
chain of the launch fits on the GPU at once, else in 256-thread CTAs (threads=160 fixes those);
threads=256 forces the chain kernel; systems wide enough for more than 3 x 3 x 3 mass-centre cells of the largest
group cutoff take their GroupCutoff candidates from those cells, the chain kernel from every
group).  Under the same device proposals both kernels must give the same chain --
the same accept count and bit-identical FP64 positions and mass centres -- barring a
near tie (u between the two FP32C energy changes' exponentials); the running energy
must agree with an FP64 recomputation; a batch mixing atomic systems (pipelined
single-atom kernel) with molecular ones runs both kernels in one graph."""
import dataclasses

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

pytestmark = pytest.mark.gpu

CASES = {
    "water_small": lambda: configs.spce_water(n_mol=256, L=18.6, seed=3),
    "water_1000": lambda: configs.spce_water(n_mol=1000, seed=4),
    "water_surface": lambda: configs.spce_water(n_mol=256, L=18.6, seed=5, epss=1.0),
    "water_two_kinds": lambda: configs.spce_water(n_mol=512, L=24.8, seed=6, molecules=("M", "Q"),
                                                  cutoff_g2g={"default": 7.0, "M Q": 10.0}),
    "water_4000": lambda: configs.spce_water(n_mol=4000, L=49.3, seed=12),            # mass-centre cells 4^3
    "water_6666": lambda: configs.spce_water(n_mol=6666, L=58.5, seed=14),            # mass-centre cells 5^3
    "water_4000_two_kinds": lambda: configs.spce_water(n_mol=4000, L=49.3, seed=15, molecules=("M", "Q"),
                                                       cutoff_g2g={"default": 7.0, "M Q": 10.0}),
    "water_2000_no_cutoff": lambda: configs.spce_water(n_mol=2000, L=39.1, seed=13, cutoff_g2g=0.0),  # chunks
    "water_reaction_field": lambda: dataclasses.replace(
        configs.spce_water(n_mol=256, L=18.6, seed=7), ewald=None,
        **F.coulomb_scheme("reactionfield", epsr=1.0, cutoff=9.0, epsrf=80.0, temperature=300.0)),
}


def _consistent(s):
    e_run = s.running_energy()
    s.q_rebuild()
    e_tot = s.energy_total()["total"]
    assert abs(e_run - e_tot) <= 1e-6 * max(1.0, abs(e_tot)), (e_run, e_tot)


@pytest.mark.parametrize("threads", [0, 160])
@pytest.mark.parametrize("case", sorted(CASES))
def test_molecular_kernel_equals_chain_kernel(ctx, case, threads):
    """threads 0: a launch of one molecular chain runs it in a 512-thread CTA (1 preparing + 15
    compute warps); 160: the 256-thread CTA (1 + 7)."""
    spec = CASES[case]()
    a, b = ctx.create(spec), ctx.create(spec)
    moves = 3000
    sa = ctx.run_batch([a], moves, seed=17, streams=[3], dp=0.5, dprot=0.5, threads=threads)
    sb = ctx.run_batch([b], moves, seed=17, streams=[3], dp=0.5, dprot=0.5, threads=256)
    assert sa["moves"] == sb["moves"] == moves
    assert sa["accepted"] == sb["accepted"] and sa["accepted"] > 300
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.mass_centers(), b.mass_centers())
    assert abs(a.running_energy() - b.running_energy()) <= 1e-6 * abs(b.running_energy())
    if a.K:
        assert np.abs(a.q() - b.q()).max() < 1e-4
    _consistent(a)


def test_molecular_kernel_replicas_and_mixed_batch(ctx):
    w = configs.spce_water(n_mol=256, L=18.6, seed=8)
    pm = configs.primitive_model(n=200, seed=9)
    ws = [ctx.create(w) for _ in range(4)]
    ps = [ctx.create(pm) for _ in range(3)]
    ref_w = [ctx.create(w) for _ in range(4)]
    batch = ws[:2] + ps + ws[2:]
    st = ctx.run_batch(batch, 2000, seed=5, dp_per_system=[0.5, 0.5, 2.0, 2.0, 2.0, 0.5, 0.5],
                       dprot_per_system=[0.5] * 7)
    assert st["moves"] == 7 * 2000
    # each water replica alone in the chain kernel, same stream id as in the batch
    for k, (sw, rw) in enumerate(zip(ws, ref_w)):
        sid = [0, 1, 5, 6][k]
        ctx.run_batch([rw], 2000, seed=5, streams=[sid], dp=0.5, dprot=0.5, threads=256)
        assert np.array_equal(sw.positions(), rw.positions())
        _consistent(sw)
    for s in ps:
        _consistent(s)


def test_molecular_kernel_parallel_tempering_and_counters(ctx):
    w = configs.spce_water(n_mol=256, L=18.6, seed=10)
    reps = [ctx.create(w) for _ in range(4)]
    st = ctx.run_batch(reps, seed=3, dp=0.5, dprot=0.5, swap_interval=500, n_swap_blocks=4,
                       temperatures=[280.0, 300.0, 320.0, 340.0])
    assert st["moves"] == 4 * 2000 and st["swaps_attempted"] > 0
    c = [r.counters() for r in reps]
    assert sum(x["moves"] for x in c) == 8000 and sum(x["accepted"] for x in c) == st["accepted"]
    for r in reps:
        _consistent(r)


@pytest.mark.parametrize("dp,dprot", [(0.5, 0.0), (0.0, 0.5), (0.0, 0.0)])
def test_molecular_kernel_translation_rotation_only_and_empty_moves(ctx, dp, dprot):
    spec = configs.spce_water(n_mol=256, L=18.6, seed=11)
    a, b = ctx.create(spec), ctx.create(spec)
    pos0 = a.positions()
    sa = ctx.run_batch([a], 1500, seed=3, dp=dp, dprot=dprot, threads=0)
    sb = ctx.run_batch([b], 1500, seed=3, dp=dp, dprot=dprot, threads=256)
    assert sa["moves"] == sb["moves"] and sa["accepted"] == sb["accepted"]
    assert np.array_equal(a.positions(), b.positions())
    if dp == 0.0 and dprot == 0.0:  # empty changes: nothing moves, nothing is counted as a move
        assert sa["moves"] == 0 and np.array_equal(a.positions(), pos0)
    else:
        assert sa["accepted"] > 100
    _consistent(a)


def test_molecular_kernel_host_proposals(ctx):
    """fau_run_proposals_batch runs systems of molecules whose proposals are all molecular (the
    reference's moltransrot stream) in the pipelined molecular kernel: its chain matches the
    FP64 oracle and is the chain kernel's (fau_run_proposals) bit for bit."""
    import oracle_lib  # noqa: F401  (the oracle comparison helper below loads it)
    from test_pipelined_gpu import _oracle_compare
    specs = [configs.spce_water(n_mol=256, L=18.6, seed=31), configs.spce_water(n_mol=4000, L=49.3, seed=32)]
    M = 1500
    props = [F.MoveGenerator(s, s.extra["moves"], 71 + i, 73 + i, default_seeds=False).generate(M)
             for i, s in enumerate(specs)]
    systems = [ctx.create(s) for s in specs]
    allp = np.concatenate(props)
    off = np.arange(len(specs) + 1, dtype=np.int64) * M
    acc = np.zeros(len(allp), np.uint8)
    du = np.zeros(len(allp))
    st = ctx.run_proposals_batch(systems, allp, off, acc, du)
    assert st["moves"] > 0
    for i, (s, spec) in enumerate(zip(systems, specs)):
        sl = slice(i * M, (i + 1) * M)
        assert _oracle_compare(s.positions(), acc[sl], du[sl], spec, props[i]) > 100
        c = ctx.create(spec)
        acc_c, du_c, _ = c.run_proposals(props[i])
        assert np.array_equal(acc_c.astype(np.uint8), acc[sl])
        assert np.array_equal(c.positions(), s.positions())
        assert np.allclose(du_c, du[sl], rtol=1e-9, atol=1e-9)


def test_molecular_kernel_reports_its_error_against_fp64(ctx):
    """Each launch's molecular chains end with a probe move (the next proposal, evaluated on the
    final state and not decided) that probe_audit_kernel re-evaluates in FP64: the batch and each
    system report its error, within the parity tolerance, and the probe leaves the chains as they
    were (the same chain as one launch without probes)."""
    specs = [configs.spce_water(n_mol=256, L=18.6, seed=40 + i) for i in range(3)]
    specs.append(configs.spce_water(n_mol=256, L=18.6, seed=44, epss=1.0))
    specs.append(configs.spce_water(n_mol=512, L=24.8, seed=45, molecules=("M", "Q"),
                                    cutoff_g2g={"default": 7.0, "M Q": 10.0}))
    systems = [ctx.create(s) for s in specs]
    quiet = [ctx.create(s) for s in specs]
    streams = np.arange(len(specs), dtype=np.uint32)
    for b in range(3):
        st = ctx.run_batch(systems, 400, seed=3, dp=0.5, dprot=0.5, streams=streams, counters=[400 * b] * len(specs),
                           threads=160)
        assert st["du_err_samples"] == len(specs)
        assert 0.0 < st["du_err_scaled_max"] <= 1e-6
    ctx.run_batch(quiet, 1200, seed=3, dp=0.5, dprot=0.5, streams=streams, threads=160, audit=False)
    for s, q in zip(systems, quiet):
        a = s.audit()
        assert a["samples"] == 3 and 0.0 < a["rel_scaled_max"] <= 1e-6
        assert q.audit()["samples"] == 0
        assert np.array_equal(s.positions(), q.positions())
        assert s.running_energy() == q.running_energy()
        _consistent(s)
    # host proposals (the reference stream) through the molecular kernel report theirs too
    spec = specs[0]
    g = ctx.create(spec)
    props = F.MoveGenerator(spec, spec.extra["moves"], 5, 6, default_seeds=False).generate(300)
    st = ctx.run_proposals_batch([g], props, np.array([0, 300], np.int64))
    assert st["du_err_samples"] == 1 and st["du_err_scaled_max"] <= 1e-6
