"""FP64 replica chains: systems made with FAU_PREC_FP64 run in fau_run_batch and
fau_run_proposals_batch as persistent chains in plain FP64 arithmetic (fau_fp64.cu), for
single-atom and rigid-molecule moves.

The primitive model of the 200-ion electrolyte is specified in FP64 with 1e5 moves: its
reference-stream chain is compared with the FP64 oracle move by move.  Both sides are FP64 and
differ only in the order of the pair sums, so dU is held to 1e-12 of max(|dU|, S) and the accept
sequence must be identical (a near tie at that level would be listed); positions are
bit-identical.  The Ewald and surface terms add FP64 phases: both sides form
q (e^{i k.r_new} - e^{i k.r_old}) from sin/cos of k.r, whose rounding (a few ulp of |k.r|, up to
~25 rad here) leaves an absolute error near 1e-12 kT in dU however small the move; those systems
are held to 1e-10 max(|dU|, S) + 1e-11 kT, and the chain to the plain FP64 form, which evaluates
the same arithmetic one move per call, within 1e-13 kT.
"""
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12


def _props(spec, n, seeds=(11, 13)):
    return F.MoveGenerator(spec, spec.extra["moves"], seeds[0], seeds[1], default_seeds=False).generate(n)


def _fp64_vs_oracle(ctx, spec, n_moves, tol, atol=0.0):
    """The caller's proposals through the FP64 chain kernel (fau_run_proposals_batch) against the
    oracle's performMove loop."""
    g = ctx.create(spec)
    props = _props(spec, n_moves)
    acc = np.zeros(n_moves, np.uint8)
    du = np.zeros(n_moves)
    st = ctx.run_proposals_batch([g], props, np.array([0, n_moves], np.int64), acc, du)
    o = O.OracleSystem(spec)
    det = o.run_detail(props)
    acc_o, du_o, scale = det["accepted"].astype(np.uint8), det["du"], det["err_scale"]
    assert np.array_equal(acc, acc_o), f"first differing decision at move {np.argmax(acc != acc_o)}"
    fin = np.isfinite(du_o)
    assert np.array_equal(np.isfinite(du), fin)
    assert np.array_equal(np.sign(du[~fin]), np.sign(du_o[~fin]))
    den = np.maximum(np.abs(du_o[fin]), scale[fin])
    rel = np.maximum(np.abs(du[fin] - du_o[fin]) - atol, 0.0) / np.where(den > 0, den, 1.0)
    assert rel.max(initial=0.0) <= tol, f"max rel err {rel.max():.3e} at move {np.argmax(rel)}"
    assert np.array_equal(g.positions(), o.positions())
    print(f"FP64 CHAIN {spec.name} moves={n_moves} accepted={int(acc.sum())} max_rel={rel.max(initial=0.0):.3e}")
    return g, o, st, acc, props, du


def test_fp64_chain_primitive_model_as_specified(ctx):
    """The 200-ion primitive model (Coulomb 24 A cutoff + WCA + hard spheres, L = 50 A) in FP64,
    1e5 reference-stream moves."""
    spec = configs.primitive_model(n=200, precision=A.FAU_PREC_FP64)
    g, o, st, acc, _, _ = _fp64_vs_oracle(ctx, spec, 100000, TOL_FP64)
    assert st["moves"] == 100000
    assert acc.sum() > 5000
    # the running FP64 energy agrees with a fresh total and with the oracle's
    e_run, e_tot = g.running_energy(), g.energy_total()["total"]
    assert abs(e_run - e_tot) <= 1e-9 * max(1.0, abs(e_tot))
    assert abs(e_tot - o.energy_total()["total"]) <= 1e-9 * max(1.0, abs(e_tot))


@pytest.mark.parametrize("epss", [0.0, 1.0])
def test_fp64_chain_ewald(ctx, epss):
    """Bulk salt with Ewald (reciprocal Q(k) updates, and the surface term at epss = 1) and a cell
    list kept by the commit."""
    spec = configs.bulk_ewald(n_salt=500, epss=epss, precision=A.FAU_PREC_FP64)
    g, o, st, acc, props, du = _fp64_vs_oracle(ctx, spec, 2000, 1e-10, atol=1e-11)
    assert acc.sum() > 500
    # the plain FP64 form (one move per call, host decision) on the same proposals
    p = ctx.create(spec)
    acc_p, du_p, _ = p.run_proposals(props)
    assert np.array_equal(acc_p, acc)
    fin = np.isfinite(du)
    assert np.abs(du[fin] - du_p[fin]).max() <= 1e-13
    assert np.array_equal(p.positions(), g.positions())
    p.close()
    cells, dims, _, _ = O.cell_bin(spec.box, spec.pair_cutoff, o.positions())
    assert np.array_equal(g.cells(), cells)
    assert np.abs(g.q() - o.q()).max() < 1e-9
    e_run, e_tot = g.running_energy(), g.energy_total()["total"]
    assert abs(e_run - e_tot) <= 1e-9 * max(1.0, abs(e_tot))


def test_fp64_batch_equals_each_chain_alone(ctx):
    """Device proposals: each FP64 chain of a batch of clones ends where it ends alone, bit for
    bit, and its running energy equals its total."""
    spec = configs.primitive_model(n=200, precision=A.FAU_PREC_FP64)
    base = ctx.create(spec)
    reps = [base] + [base.clone() for _ in range(5)]
    streams = np.arange(6, dtype=np.uint32) + 40
    st = ctx.run_batch(reps, 3000, seed=9, dp=2.0, streams=streams)
    assert st["moves"] == 6 * 3000
    assert st["accepted"] > 1000
    for k, r in enumerate(reps):
        alone = ctx.create(spec)
        ctx.run_batch([alone], 3000, seed=9, dp=2.0, streams=streams[k:k + 1])
        assert np.array_equal(alone.positions(), r.positions())
        assert alone.running_energy() == r.running_energy()
        e_tot = r.energy_total()["total"]
        assert abs(r.running_energy() - e_tot) <= 1e-9 * max(1.0, abs(e_tot))
        alone.close()
    for r in reps:
        r.close()


def test_fp64_parallel_tempering(ctx):
    """FP64 walkers of uneven size under parallel tempering: every walker's running energy
    equals its total after the swap rounds."""
    specs, temps = configs.pt_replicas(n_rep=8, n_min=100, n_max=400, precision=A.FAU_PREC_FP64)
    walkers = [ctx.create(s) for s in specs]
    n = np.array([s.n for s in specs], np.int64)
    st = ctx.run_batch(walkers, moves_per_system=20 * n, swap_interval=1, n_swap_blocks=3, temperatures=temps,
                       seed=3, dp=2.0)
    assert st["moves"] == 3 * int((20 * n).sum())
    assert st["swaps_attempted"] > 0
    for w in walkers:
        e_tot = w.energy_total()["total"]
        assert abs(w.running_energy() - e_tot) <= 1e-9 * max(1.0, abs(e_tot))
        w.close()


def test_fp64_and_fp32c_systems_do_not_share_a_batch(ctx):
    a = ctx.create(configs.primitive_model(n=200, precision=A.FAU_PREC_FP64))
    b = ctx.create(configs.primitive_model(n=200))
    with pytest.raises(F.FauError, match="FP64"):
        ctx.run_batch([a, b], 100, seed=1, dp=2.0)
    props = _props(a.spec, 10)
    with pytest.raises(F.FauError, match="FP64"):
        ctx.run_proposals_batch([a, b], np.concatenate([props, props]), np.array([0, 10, 20], np.int64))
    a.close()
    b.close()


@pytest.mark.parametrize("make", [
    lambda: configs.spce_water(n_mol=256, L=18.6, seed=3, precision=A.FAU_PREC_FP64),
    lambda: configs.spce_water(n_mol=256, L=18.6, seed=5, epss=1.0, precision=A.FAU_PREC_FP64),
    lambda: configs.spce_water(n_mol=512, L=24.8, seed=6, molecules=("M", "Q"), cutoff_g2g={"default": 7.0, "M Q": 10.0},
                               precision=A.FAU_PREC_FP64),
])
def test_fp64_chain_rigid_molecules(ctx, make):
    """Rigid SPC/E water (TranslateRotate moves of the reference stream, GroupCutoff per molecule
    pair, Ewald and its surface term) through the FP64 chain kernel: the oracle's chain, and the
    plain FP64 form's dU within 1e-13 of max(1, |dU|) kT (the two sum the group's pairs in
    different orders); positions and mass centres bit-identical."""
    spec = make()
    g, o, st, acc, props, du = _fp64_vs_oracle(ctx, spec, 1000, 1e-10, atol=1e-11)
    assert (props["kind"] == A.FAU_MOVE_MOLECULAR).all() and acc.sum() > 200
    assert np.array_equal(g.mass_centers(), o.mass_centers())
    p = ctx.create(spec)
    acc_p, du_p, _ = p.run_proposals(props)
    assert np.array_equal(acc_p, acc)
    fin = np.isfinite(du)
    assert (np.abs(du[fin] - du_p[fin]) <= 1e-13 * np.maximum(1.0, np.abs(du_p[fin]))).all()
    assert np.array_equal(p.positions(), g.positions())
    e_run, e_tot = g.running_energy(), g.energy_total()["total"]
    assert abs(e_run - e_tot) <= 1e-9 * max(1.0, abs(e_tot))
    p.close()


def test_fp64_molecular_batch_equals_each_chain_alone(ctx):
    """Device proposals (moltransrot): each FP64 water chain of a batch ends where it ends alone."""
    spec = configs.spce_water(n_mol=256, L=18.6, seed=4, precision=A.FAU_PREC_FP64)
    reps = [ctx.create(spec) for _ in range(3)]
    streams = np.array([7, 8, 9], np.uint32)
    st = ctx.run_batch(reps, 800, seed=2, dp=0.5, dprot=0.5, streams=streams)
    assert st["moves"] == 3 * 800 and st["accepted"] > 300
    for k, r in enumerate(reps):
        alone = ctx.create(spec)
        ctx.run_batch([alone], 800, seed=2, dp=0.5, dprot=0.5, streams=streams[k:k + 1])
        assert np.array_equal(alone.positions(), r.positions())
        assert np.array_equal(alone.mass_centers(), r.mass_centers())
        assert alone.running_energy() == r.running_energy()
        e_tot = r.energy_total()["total"]
        assert abs(r.running_energy() - e_tot) <= 1e-9 * max(1.0, abs(e_tot))
        alone.close()
    for r in reps:
        r.close()


def _two_spheres(pos, sigma2=16.0, terms=A.FAU_PAIR_HS | A.FAU_PAIR_COULOMB):
    return F.SystemSpec(box=np.full(3, 20.0), pos=np.array(pos, dtype=float), charge=np.array([1.0, -1.0]),
                        type=np.zeros(2, np.int32), group_begin=np.array([0, 2], np.int32),
                        group_flags=np.array([A.FAU_GROUP_ATOMIC], np.int32), n_types=1,
                        hs_sigma2=np.full((1, 1), 16.0), sigma2=np.full((1, 1), sigma2),
                        eps4=np.full((1, 1), 1.0), pair_terms=terms, coulomb_type=A.FAU_COUL_PLAIN,
                        bjerrum_length=7.0, precision=A.FAU_PREC_FP64)


def _moves(rows):
    p = np.zeros(len(rows), dtype=A.PROPOSAL_DTYPE)
    for m, (i, dr, u) in enumerate(rows):
        p["kind"][m] = A.FAU_MOVE_ATOMIC
        p["index"][m] = i
        p["dr"][m] = dr
        p["u"][m] = u
    return p


def test_fp64_chain_infinities_follow_get_energy_change(ctx):
    """Hard-sphere overlaps in an FP64 chain: into overlap +inf (rejected, unless u = 0, as
    u <= exp(-dU) has it), out of overlap -inf (accepted); the oracle decides the same."""
    spec = _two_spheres([[0, 0, 0], [5, 0, 0]])
    props = _moves([(1, (-2.0, 0, 0), 0.5), (1, (-2.0, 0, 0), 0.0), (1, (2.0, 0, 0), 0.999)])
    g = ctx.create(spec)
    acc = np.zeros(3, np.uint8)
    du = np.zeros(3)
    ctx.run_proposals_batch([g], props, np.array([0, 3], np.int64), acc, du)
    det = O.OracleSystem(spec).run_detail(props)
    assert list(acc) == [0, 1, 1] == list(det["accepted"].astype(np.uint8))
    assert du[0] == math.inf and du[1] == math.inf and du[2] == -math.inf
    assert np.array_equal(np.sign(du), np.sign(det["du"]))


def test_fp64_chain_nan_pair_energy_is_rejected(ctx):
    """A missing coefficient makes both states NaN: getEnergyChange maps a NaN trial energy to
    +inf (src/montecarlo.cpp:198-200), rejected, and the chain goes on."""
    spec = _two_spheres([[0, 0, 0], [5, 0, 0]], sigma2=float("nan"), terms=A.FAU_PAIR_WCA)
    props = _moves([(1, (0.5, 0, 0), 0.5), (0, (0.0, 0.5, 0), 0.5)])
    g = ctx.create(spec)
    acc = np.ones(2, np.uint8)
    du = np.zeros(2)
    st = ctx.run_proposals_batch([g], props, np.array([0, 2], np.int64), acc, du)
    assert st["moves"] == 2
    assert list(acc) == [0, 0] and du[0] == math.inf and du[1] == math.inf
