"""GPU parity: the sm_103a path (through the C ABI) against the FP64 oracle.

Tolerance (FP32 pair and Ewald terms with compensated sums, FP64 totals):
    |dU_gpu - dU_oracle| <= 1e-6 * max(|dU|, S)
where S is the sum of |summand| magnitudes the change is summed from over both
states: every pair potential term of every pair counted separately (Coulomb,
and the r^-12 and r^-6 parts of LJ and WCA, which cancel near r = sigma), plus (2 pi lB / V) sum_k A_k (|2 Re(Q_k* d_k)| + |d_k|^2) for the
reciprocal change -- the floating-point error scale of the sum.  Accept sequences must be identical under the same proposal stream
except at near ties, where u falls between exp(-dU_gpu) and exp(-dU_oracle);
positions after an identical accept sequence are bit-identical (FP64 move
arithmetic is IEEE-exact on both sides).  The plain FP64 form is held to
1e-12.
"""
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O

pytestmark = pytest.mark.gpu

TOL_FP32C = 1e-6
TOL_FP64 = 1e-12


def _props(spec, n, seeds=(11, 13)):
    return F.MoveGenerator(spec, spec.extra["moves"], seeds[0], seeds[1], default_seeds=False).generate(n)


def _compare_chain(gpu_sys, spec, props, tol, expect_bit_exact=True, label="", median_tol=None):
    acc_g, du_g, st = gpu_sys.run_proposals(props)
    o = O.OracleSystem(spec)
    det = o.run_detail(props)
    acc_o, du_o, scale = det["accepted"].astype(np.uint8), det["du"], det["err_scale"]
    mism = np.nonzero(acc_g != acc_o)[0]
    first = int(mism[0]) if len(mism) else len(props)
    sl = slice(0, first + 1 if first < len(props) else first)
    fin = np.isfinite(du_o[sl])
    assert np.array_equal(np.isfinite(du_g[sl]), fin)
    assert np.array_equal(np.sign(du_g[sl][~fin]), np.sign(du_o[sl][~fin]))
    err = np.abs(du_g[sl][fin] - du_o[sl][fin])
    den = np.maximum(np.abs(du_o[sl][fin]), scale[sl][fin])
    den = np.where(den > 0, den, 1.0)
    rel = err / den
    assert rel.max(initial=0.0) <= tol, f"max rel err {rel.max():.3e} at move {np.argmax(rel)}"
    errs = O.du_errors(du_g[sl][fin], du_o[sl][fin], scale[sl][fin])
    print(f"PARITY {label or spec.name} moves={len(props)} near_ties={len(mism)} " +
          " ".join(f"{k}={v:.3e}" if isinstance(v, float) else f"{k}={v}" for k, v in errs.items()))
    # the benchmark forms (bulk Ewald, primitive model): the median error relative to |dU| itself
    # is held too; elsewhere (truncated-Coulomb polynomials, rigid molecules' nine site pairs a
    # neighbour) the summands cancel more and S bounds the error
    if median_tol is not None:
        assert errs["rel_du_median"] <= median_tol, f"median err / |dU| {errs['rel_du_median']:.3e}"
    report = {"moves": len(props), "accepted": int(acc_g[:first].sum()), "max_rel_err": float(rel.max(initial=0)),
              "near_ties": len(mism) > 0, "first_mismatch": first, "stats": st, "errors": errs}
    if len(mism):
        # a near tie: the decisions straddle u; the chains differ from here on
        m = first
        u = props["u"][m]
        lo, hi = sorted([math.exp(-min(du_g[m], 700)), math.exp(-min(du_o[m], 700))])
        assert lo <= u <= hi or abs(u - lo) < 1e-12 or abs(u - hi) < 1e-12
        assert first > len(props) // 10, "accept sequence diverged early"
    elif expect_bit_exact:
        assert np.array_equal(gpu_sys.positions(), o.positions())
        if spec.n_groups > 1:
            assert np.array_equal(gpu_sys.mass_centers(), o.mass_centers())
    return report, o


# ---------------------------------------------------------------- total energies
@pytest.mark.parametrize("make", [
    lambda: configs.primitive_model(n=200),
    lambda: configs.bulk_ewald(n_salt=1000),
    lambda: configs.bulk_ewald(n_salt=1000, epss=1.0),
    lambda: configs.spce_water(n_mol=256, L=18.6),
    lambda: configs.spce_water(n_mol=1000),
    lambda: configs.spce_water(n_mol=512, L=24.8, molecules=("M", "Q"), cutoff_g2g={"default": 7.0, "M Q": 10.0}),
])
def test_energy_total_matches_oracle(ctx, make):
    spec = make()
    g = ctx.create(spec)
    eg = g.energy_total()
    eo = O.OracleSystem(spec).energy_total()
    for key in ("self", "nonbonded", "ewald_rec", "ewald_surf", "total"):
        a, b = eg[key], eo[key]
        assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (key, a, b)
    assert g.K == (1152 if spec.ewald and spec.ewald["ncutoff"] == 8 else g.K)
    # Q(k) of the device (FP64 from fixed-point phases) against the oracle's FP64 Q
    if spec.ewald:
        qg, qo = g.q(), O.OracleSystem(spec).q()
        assert np.abs(qg - qo).max() < 1e-5


@pytest.mark.parametrize("make,K", [(lambda: configs.bulk_ewald(n_salt=1000), 1152),
                                    (lambda: configs.bulk_ewald(n_salt=10000), 1152),
                                    (lambda: configs.spce_water(n_mol=1000), 911)])
def test_kvector_table_matches_oracle(ctx, make, K):
    """PolicyIonIon::updateBox (src/energy.cpp:133-186): the device table holds the oracle's
    k-vectors in the oracle's order, element by element, and the same A_k."""
    spec = make()
    g = ctx.create(spec)
    kv, ak = O.OracleSystem(spec).kvectors()
    assert g.K == len(kv) == K
    kv_g, ak_g = g.kvectors()
    assert np.array_equal(kv_g, kv)
    np.testing.assert_allclose(ak_g, ak, rtol=1e-15, atol=0)


# ---------------------------------------------------------------- chains, FP32C
def test_chain_primitive_model(ctx):
    """Config 0 as specified: 1e5 reference-stream moves of the 200-ion primitive model."""
    spec = configs.primitive_model(n=200)
    rep, _ = _compare_chain(ctx.create(spec), spec, _props(spec, 100000), TOL_FP32C, median_tol=O.TOL_REL_DU_MEDIAN)
    assert rep["accepted"] > 5000


def test_chain_bulk_ewald_small(ctx):
    spec = configs.bulk_ewald(n_salt=1000)
    g = ctx.create(spec)
    assert g.cell_grid() == (21, 21, 21)
    rep, o = _compare_chain(g, spec, _props(spec, 5000), TOL_FP32C, median_tol=O.TOL_REL_DU_MEDIAN)
    assert rep["accepted"] > 1000
    if not rep["near_ties"]:
        # device cell list equals the reference grid binning of the final positions
        cells, dims, _, _ = O.cell_bin(spec.box, spec.pair_cutoff, o.positions())
        assert np.array_equal(g.cells(), cells)
        # Q(k): running device copy vs oracle, then an FP64 rebuild
        assert np.abs(g.q() - o.q()).max() < 1e-4
        drift = g.q_rebuild()
        assert drift < 1e-4
        assert np.abs(g.q() - o.q()).max() < 1e-5


def test_chain_bulk_ewald_surface_term(ctx):
    spec = configs.bulk_ewald(n_salt=1000, epss=1.0)
    _compare_chain(ctx.create(spec), spec, _props(spec, 3000), TOL_FP32C)


def test_chain_bulk_ewald_full_size(ctx):
    """The benchmark system: 20,000 ions, K = 1152, 45^3 cells."""
    spec = configs.bulk_ewald(n_salt=10000)
    g = ctx.create(spec)
    assert g.cell_grid() == (45, 45, 45) and g.K == 1152
    rep, _ = _compare_chain(g, spec, _props(spec, 1000), TOL_FP32C, median_tol=O.TOL_REL_DU_MEDIAN)
    assert rep["accepted"] > 200


def test_chain_water(ctx):
    spec = configs.spce_water(n_mol=1000)
    rep, _ = _compare_chain(ctx.create(spec), spec, _props(spec, 1500), TOL_FP32C)
    assert rep["stats"]["moves"] == 1500


def test_chain_small_water_box(ctx):
    spec = configs.spce_water(n_mol=256, L=18.6)
    _compare_chain(ctx.create(spec), spec, _props(spec, 2000), TOL_FP32C)


@pytest.mark.parametrize("cut", [{"default": 7.0, "M Q": 10.0}, {"M Q": 8.0}])
def test_chain_water_per_pair_group_cutoff(ctx, cut):
    """GroupCutoff::getCutoff per molecule-kind pair (two kinds, M and Q) in the chain
    kernel, the plain FP64 form and a batch of clones."""
    spec = configs.spce_water(n_mol=512, L=24.8, molecules=("M", "Q"), cutoff_g2g=cut)
    props = _props(spec, 1500)
    _compare_chain(ctx.create(spec), spec, props, TOL_FP32C)
    w = configs.spce_water(n_mol=512, L=24.8, molecules=("M", "Q"), cutoff_g2g=cut, precision=A.FAU_PREC_FP64)
    _compare_chain(ctx.create(w), w, _props(w, 300), 1e-10)
    base = ctx.create(spec)
    reps = [base] + [base.clone() for _ in range(3)]
    ctx.run_batch(reps, 500, seed=2, dp=0.5, dprot=0.5)
    for r in reps:
        e_run = r.running_energy()
        r.q_rebuild()
        assert abs(e_run - r.energy_total()["total"]) <= 1e-6 * abs(e_run)


def test_running_energy_has_no_drift(ctx):
    spec = configs.bulk_ewald(n_salt=1000)
    g = ctx.create(spec)
    g.run_proposals(_props(spec, 5000), want_acc=False, want_du=False)
    e_run = g.running_energy()
    g.q_rebuild()
    e_tot = g.energy_total()["total"]
    assert abs(e_run - e_tot) <= 1e-6 * abs(e_tot)


# ---------------------------------------------------------------- plain FP64 form
def test_plain_fp64_form(ctx):
    spec = configs.primitive_model(n=200, precision=A.FAU_PREC_FP64)
    _compare_chain(ctx.create(spec), spec, _props(spec, 1500), TOL_FP64)


def test_plain_fp64_form_ewald_and_water(ctx):
    spec = configs.bulk_ewald(n_salt=500, precision=A.FAU_PREC_FP64)
    _compare_chain(ctx.create(spec), spec, _props(spec, 300), 1e-10)
    w = configs.spce_water(n_mol=256, L=18.6, precision=A.FAU_PREC_FP64)
    _compare_chain(ctx.create(w), w, _props(w, 300), 1e-10)


# ---------------------------------------------------------------- single-move API
def test_trial_single_moves(ctx):
    spec = configs.bulk_ewald(n_salt=1000)
    g = ctx.create(spec)
    o = O.OracleSystem(spec)
    rng = np.random.default_rng(5)
    for _ in range(50):
        i = int(rng.integers(spec.n))
        dr = rng.normal(size=3)
        u = float(rng.random())
        rg = g.trial_atomic(i, dr, u)
        ro = o.trial_atomic(i, dr, u)
        assert rg["accepted"] == ro["accepted"]
        assert abs(rg["du"] - ro["du"]) <= TOL_FP32C * max(abs(ro["du"]), ro["err_scale"])
        assert abs(rg["du_ewald"] - ro["du_ewald"]) <= TOL_FP32C * max(abs(ro["du"]), ro["err_scale"])
    assert np.array_equal(g.positions(), o.positions())


def test_trial_group_moves(ctx):
    spec = configs.spce_water(n_mol=256, L=18.6)
    g = ctx.create(spec)
    o = O.OracleSystem(spec)
    props = _props(spec, 40)
    for p in props:
        if p["kind"] != A.FAU_MOVE_MOLECULAR:
            continue
        rg = g.trial_group(p["index"], p["dr"], p["quat"], p["u"])
        ro = o.trial_group(p["index"], p["dr"], p["quat"], p["u"])
        assert rg["accepted"] == ro["accepted"]
        assert abs(rg["du"] - ro["du"]) <= TOL_FP32C * max(abs(ro["du"]), ro["err_scale"])
    assert np.array_equal(g.positions(), o.positions())
    assert np.array_equal(g.mass_centers(), o.mass_centers())


# ---------------------------------------------------------------- edge cases
def _two_spheres(pos, precision=A.FAU_PREC_FP32C, sigma2=16.0, terms=A.FAU_PAIR_HS | A.FAU_PAIR_COULOMB):
    return F.SystemSpec(box=np.full(3, 20.0), pos=np.array(pos, dtype=float), charge=np.array([1.0, -1.0]),
                        type=np.zeros(2, np.int32), group_begin=np.array([0, 2], np.int32),
                        group_flags=np.array([A.FAU_GROUP_ATOMIC], np.int32), n_types=1,
                        hs_sigma2=np.full((1, 1), 16.0), sigma2=np.full((1, 1), sigma2),
                        eps4=np.full((1, 1), 1.0), pair_terms=terms, coulomb_type=A.FAU_COUL_PLAIN,
                        bjerrum_length=7.0, precision=precision)


@pytest.mark.parametrize("prec", [A.FAU_PREC_FP32C, A.FAU_PREC_FP64])
def test_hard_sphere_infinities(ctx, prec):
    g = ctx.create(_two_spheres([[0, 0, 0], [5, 0, 0]], prec))
    r = g.trial_atomic(1, (-2.0, 0, 0), 0.5)  # into overlap: +inf, rejected
    assert r["du"] == math.inf and r["new_inf"] == 1 and r["accepted"] == 0
    # u == 0 accepts even +inf, as `u <= exp(-dU)` does in the reference
    r = g.trial_atomic(1, (-2.0, 0, 0), 0.0)
    assert r["du"] == math.inf and r["accepted"] == 1
    g2 = ctx.create(_two_spheres([[0, 0, 0], [3, 0, 0]], prec))
    r = g2.trial_atomic(1, (2.0, 0, 0), 0.999)  # out of overlap: -inf, accepted
    assert r["du"] == -math.inf and r["accepted"] == 1 and r["old_inf"] == 1


def test_nan_pair_energy_is_rejected(ctx):
    """A missing coefficient makes both states NaN; getEnergyChange maps a NaN
    trial energy to +inf (src/montecarlo.cpp:198-200): rejected, no error."""
    spec = _two_spheres([[0, 0, 0], [5, 0, 0]], sigma2=float("nan"), terms=A.FAU_PAIR_WCA)
    g = ctx.create(spec)
    r = g.trial_atomic(1, (0.5, 0, 0), 0.5)
    o = O.OracleSystem(spec)
    ro = o.trial_atomic(1, (0.5, 0, 0), 0.5)
    assert r["du"] == ro["du"] == math.inf
    assert r["accepted"] == ro["accepted"] == 0
    assert math.isnan(g.energy_total()["total"])


def test_empty_changes_and_invalid_arguments(ctx):
    spec = configs.primitive_model(n=20, L=20.0)
    g = ctx.create(spec)
    props = np.zeros(5, dtype=A.PROPOSAL_DTYPE)
    props["kind"] = A.FAU_MOVE_NONE
    props["u"] = 0.5
    acc, du, st = g.run_proposals(props)
    assert st["moves"] == 0 and not acc.any()
    with pytest.raises(F.FauError) as e:
        g.trial_atomic(999, (0, 0, 0), 0.5)
    assert e.value.status == A.FAU_ERR_ARG
    with pytest.raises(F.FauError) as e:
        g.trial_group(0, (0, 0, 0), (0, 0, 0, 0), 0.5)
    assert e.value.status == A.FAU_ERR_ARG
    bad = props.copy()
    bad["kind"] = 7
    with pytest.raises(F.FauError):
        g.run_proposals(bad)


def test_cell_capacity_overflow_recovers(ctx):
    """Pile particles into one cell: the device list overflows, the host regrows
    it and resumes; positions and binning still match the oracle."""
    n = 64
    rng = np.random.default_rng(9)
    L = 40.0
    pos = (rng.random((n, 3)) - 0.5) * L * 0.999
    spec = F.SystemSpec(box=np.full(3, L), pos=pos, charge=np.zeros(n), type=np.zeros(n, np.int32),
                        group_begin=np.array([0, n], np.int32), group_flags=np.array([1], np.int32), n_types=1,
                        pair_terms=0, pair_cutoff=12.0, cell_capacity=1)
    g = ctx.create(spec)
    assert g.cell_grid() == (3, 3, 3)
    props = np.zeros(n, dtype=A.PROPOSAL_DTYPE)
    props["kind"] = A.FAU_MOVE_ATOMIC
    props["index"] = np.arange(n)
    target = -0.5 * L + 1.0 + rng.random((n, 3)) * 10.0  # all into cell (0,0,0)
    props["dr"] = target - pos
    props["u"] = 0.0
    acc, du, st = g.run_proposals(props)
    assert acc.all()
    o = O.OracleSystem(spec)
    o.run_proposals(props)
    assert np.array_equal(g.positions(), o.positions())
    cells, _, _, _ = O.cell_bin(spec.box, 12.0, o.positions())
    assert np.array_equal(g.cells(), cells) and (cells == 0).sum() >= n - 1


# ---------------------------------------------------------------- batched replicas
def test_batch_mixed_systems_energy_consistency(ctx):
    specs = [configs.primitive_model(n=200, seed=1), configs.bulk_ewald(n_salt=1000, seed=2),
             configs.spce_water(n_mol=256, L=18.6, seed=3)]
    systems = [ctx.create(s) for s in specs]
    st = ctx.run_batch(systems, 3000, seed=7, dp=1.0, dprot=0.3, threads=256)
    assert st["moves"] == 9000 and st["accepted"] > 0
    for s in systems:
        e_run = s.running_energy()
        s.q_rebuild()
        e_tot = s.energy_total()["total"]
        assert abs(e_run - e_tot) <= 1e-6 * max(1.0, abs(e_tot)), (e_run, e_tot)


def test_batch_result_same_alone_and_in_mix(ctx):
    """Continuous-batching invariant: a system's trajectory depends only on its
    (seed, stream, counter), not on which other systems share the launch."""
    a1 = ctx.create(configs.bulk_ewald(n_salt=500, seed=4))
    ctx.run_batch([a1], 2000, seed=3, streams=[42], counters=[0], threads=256)
    others = [ctx.create(configs.primitive_model(n=200, seed=s)) for s in range(3)]
    a2 = ctx.create(configs.bulk_ewald(n_salt=500, seed=4))
    ctx.run_batch(others[:1] + [a2] + others[1:], 2000, seed=3, streams=[1, 42, 2, 3], counters=[0, 0, 0, 0],
                  threads=256)
    assert np.array_equal(a1.positions(), a2.positions())
    assert a1.running_energy() == a2.running_energy()
    # resuming with a counter offset equals one longer run
    b1 = ctx.create(configs.primitive_model(n=200, seed=8))
    ctx.run_batch([b1], 1000, seed=5, streams=[9], counters=[0], threads=256)
    ctx.run_batch([b1], 1000, seed=5, streams=[9], counters=[1000], threads=256)
    b2 = ctx.create(configs.primitive_model(n=200, seed=8))
    ctx.run_batch([b2], 2000, seed=5, streams=[9], counters=[0], threads=256)
    assert np.array_equal(b1.positions(), b2.positions())


def test_parallel_tempering_swaps(ctx):
    specs, temps = configs.pt_replicas(n_rep=8, n_min=100, n_max=300)
    systems = [ctx.create(s) for s in specs]
    st = ctx.run_batch(systems, swap_interval=400, n_swap_blocks=6, temperatures=temps, seed=11, dp=2.0,
                       threads=128)
    assert st["swaps_attempted"] >= 6 * 3 and st["moves"] == 8 * 400 * 6
    for s in systems:
        e_run = s.running_energy()
        e_tot = s.energy_total()["total"]
        assert abs(e_run - e_tot) <= 1e-6 * max(1.0, abs(e_tot))


# ---------------------------------------------------------------- two-phase (EnergyTerm-level) form
def test_energy_change_then_commit_matches_oracle(ctx):
    """The caller decides: evaluate, draw Metropolis on the host, commit or drop."""
    for spec in (configs.bulk_ewald(n_salt=500), configs.spce_water(n_mol=256, L=18.6)):
        g = ctx.create(spec)
        o = O.OracleSystem(spec)
        props = _props(spec, 300)
        for p in props:
            if p["kind"] == A.FAU_MOVE_NONE:
                continue
            r = g.energy_change(p)
            ro = (o.trial_atomic(p["index"], p["dr"], p["u"]) if p["kind"] == A.FAU_MOVE_ATOMIC
                  else o.trial_group(p["index"], p["dr"], p["quat"], p["u"]))
            assert abs(r["du"] - ro["du"]) <= TOL_FP32C * max(abs(ro["du"]), ro["err_scale"])
            accept = (not math.isnan(r["du"])) and (r["du"] == -math.inf or p["u"] <= math.exp(-min(r["du"], 700)))
            assert bool(accept) == bool(ro["accepted"])
            g.commit(accept)
        assert np.array_equal(g.positions(), o.positions())
        e_run = g.running_energy()
        g.q_rebuild()
        assert abs(e_run - g.energy_total()["total"]) <= 1e-6 * abs(e_run)
        with pytest.raises(F.FauError) as e:
            g.commit(True)
        assert e.value.status == A.FAU_ERR_STATE


def test_clone_is_an_independent_copy(ctx):
    spec = configs.bulk_ewald(n_salt=500)
    a = ctx.create(spec)
    b = a.clone()
    assert np.array_equal(a.positions(), b.positions())
    assert a.running_energy() == b.running_energy()
    ctx.run_batch([a], 500, seed=1, streams=[3], threads=256)
    assert not np.array_equal(a.positions(), b.positions())
    ctx.run_batch([b], 500, seed=1, streams=[3], threads=256)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.q(), b.q()) and np.array_equal(a.cells(), b.cells())


def test_chain_kernel_reports_its_error_against_fp64(ctx):
    """Proposal streams (fau_run_proposals) and chain-kernel batches (threads 256) end each launch
    with an audit probe re-evaluated in FP64: fau_run_stats.max_rel_err and the batch's du_err_*
    carry the error of the FP32 energy changes, within the parity tolerance; the chain is the
    oracle's all the same."""
    spec = configs.bulk_ewald(n_salt=1000, epss=1.0)
    g = ctx.create(spec)
    rep, _ = _compare_chain(g, spec, _props(spec, 1500), TOL_FP32C)
    assert 0.0 < rep["stats"]["max_rel_err"] <= TOL_FP32C
    assert g.audit()["samples"] == 1
    w = configs.spce_water(n_mol=256, L=18.6, seed=3)
    systems = [ctx.create(w), ctx.create(configs.primitive_model(n=200, seed=4))]
    st = ctx.run_batch(systems, 600, seed=5, dp_per_system=[0.5, 2.0], dprot_per_system=[0.5, 0.0], threads=256)
    assert st["du_err_samples"] == 2 and 0.0 < st["du_err_scaled_max"] <= TOL_FP32C
