"""GPU parity of splined pair potentials (FAU_PAIR_SPLINE, nonbonded_splined) against
the FP64 oracle evaluating the same tables: total energies, single-atom chains in the
chain kernel, the pipelined kernel (reference-stream host proposals) and the plain
FP64 form, hard-sphere repulsion below the first knot, and rigid-water molecular
moves in the molecular kernel (bit-identical to the chain kernel).  Tolerance as in
test_parity_gpu: 1e-6 of max(|dU|, S), S the sum of |summand| magnitudes (for a
splined pair sum_k |c_k| |r^2 - z_i|^k); the FP64 form 1e-12."""
import dataclasses

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O
from test_parity_gpu import TOL_FP32C, TOL_FP64, _compare_chain, _props
from test_pipelined_gpu import _energy_consistent, _oracle_compare

pytestmark = pytest.mark.gpu


def _type_q_sigma(spec):
    q = [float(spec.charge[spec.type == t][0]) for t in range(spec.n_types)]
    return q, np.sqrt(np.diag(spec.sigma2))


def _salt(scheme="fanourgakis", seed=4, molar=1.0, n_salt=1000, **kw):
    spec = configs.bulk_ewald(n_salt=n_salt, molar=molar, seed=seed)
    if scheme != "ewald":
        spec = dataclasses.replace(spec, ewald=None, **F.coulomb_scheme(scheme, epsr=80.0, cutoff=12.0))
    spec = dataclasses.replace(spec, pair_cutoff=0.0)
    q, sig = _type_q_sigma(spec)
    return F.splined(spec, q, sig, **kw)


def _water(seed=3):
    # a reaction field: S(1) = 0, so the functor is continuous at Rc and splines within utol
    # (the Ewald real-space jump at Rc = 9, alpha = 0.2 is above utol: no piece could meet it)
    w = configs.spce_water(n_mol=256, L=18.6, seed=seed)
    w = dataclasses.replace(w, ewald=None, **F.coulomb_scheme("reactionfield", epsr=1.0, cutoff=9.0, epsrf=80.0,
                                                              temperature=300.0))
    return F.splined(w, [-0.8476, 0.4238], [3.166, 2.0], rmax=10.0)


CASES = {
    "salt_fanourgakis": lambda: _salt("fanourgakis"),
    "salt_ewald": lambda: _salt("ewald"),
    "salt_fine_tolerance": lambda: _salt("fanourgakis", seed=5, utol=1e-6, ftol=-1.0),
    "salt_hardsphere": lambda: _salt("fanourgakis", seed=6, hardsphere=True),
}


@pytest.mark.parametrize("case", sorted(CASES) + ["water"])
def test_total_energy_matches_oracle(ctx, case):
    spec = _water() if case == "water" else CASES[case]()
    assert spec.pair_terms & A.FAU_PAIR_SPLINE
    g = ctx.create(spec)
    eg = g.energy_total()
    eo = O.OracleSystem(spec).energy_total()
    for key in ("self", "nonbonded", "total"):
        assert abs(eg[key] - eo[key]) <= 1e-9 * max(1.0, abs(eo[key])), (key, eg[key], eo[key])


@pytest.mark.parametrize("case", sorted(CASES))
def test_chain_kernel_matches_oracle(ctx, case):
    spec = CASES[case]()
    rep, _ = _compare_chain(ctx.create(spec), spec, _props(spec, 3000), TOL_FP32C)
    assert rep["accepted"] > 100


def test_plain_fp64_form_matches_oracle(ctx):
    spec = dataclasses.replace(CASES["salt_fanourgakis"](), precision=A.FAU_PREC_FP64)
    _compare_chain(ctx.create(spec), spec, _props(spec, 500), TOL_FP64)


def test_pipelined_kernel_matches_oracle(ctx):
    names = sorted(CASES)
    specs = [CASES[n]() for n in names]
    systems = [ctx.create(s) for s in specs]
    M = 3000
    props = [F.MoveGenerator(s, s.extra["moves"], 61 + i, 67 + i, default_seeds=False).generate(M)
             for i, s in enumerate(specs)]
    allp = np.concatenate(props)
    off = np.arange(len(specs) + 1, dtype=np.int64) * M
    acc = np.zeros(len(allp), np.uint8)
    du = np.zeros(len(allp))
    st = ctx.run_proposals_batch(systems, allp, off, acc, du)
    assert st["moves"] == len(allp)
    for i, (s, spec) in enumerate(zip(systems, specs)):
        sl = slice(i * M, (i + 1) * M)
        assert _oracle_compare(s.positions(), acc[sl], du[sl], spec, props[i]) > 100
        _energy_consistent(s)


def test_hardsphere_below_first_knot(ctx):
    """A trial that puts two like ions inside their table's first knot is +inf (rejected)
    on both sides; without the flag the exact functor decides and the move is finite."""
    for hs in (True, False):
        spec = _salt("fanourgakis", seed=7, hardsphere=hs)
        assert (spec.spline["hs"][0] == 1) == hs
        z0 = spec.spline["r2"][0]
        i, j = 0, 1  # two cations (type 0)
        d = spec.pos[j] - spec.pos[i]
        target = spec.pos[j] - d / np.linalg.norm(d) * (0.9 * np.sqrt(z0))
        dr = target - spec.pos[i]
        g = ctx.create(spec)
        rg = g.trial_atomic(i, dr, 0.5)
        ro = O.OracleSystem(spec).trial_atomic(i, dr, 0.5)
        assert rg["new_inf"] == ro["new_inf"] == (1 if hs else 0)
        if not hs:
            assert abs(rg["du"] - ro["du"]) <= TOL_FP32C * max(abs(ro["du"]), ro["err_scale"])


def test_molecular_kernel_water(ctx):
    spec = _water(seed=9)
    a, b = ctx.create(spec), ctx.create(spec)
    moves = 3000
    sa = ctx.run_batch([a], moves, seed=19, streams=[2], dp=0.5, dprot=0.5, threads=0)
    sb = ctx.run_batch([b], moves, seed=19, streams=[2], dp=0.5, dprot=0.5, threads=256)
    assert sa["moves"] == sb["moves"] == moves
    assert sa["accepted"] == sb["accepted"] and sa["accepted"] > 300
    assert np.array_equal(a.positions(), b.positions())
    # the two kernels sum in different orders (7 and 8 warps): equal to rounding
    assert abs(a.running_energy() - b.running_energy()) <= 1e-12 * abs(b.running_energy())
    _energy_consistent(a)
    # and the chain kernel against the oracle on host proposals
    _compare_chain(ctx.create(spec), spec, _props(spec, 1500), TOL_FP32C)


@pytest.mark.parametrize("dp", [2.0, 20.0])
def test_reference_cluster_example(ctx, dp):
    """examples/cluster (ten splined waters in a 40 A box: 4 x 4 x 4 mass-centre cells of the
    10 A group cutoff): device total equal to the oracle's; the molecular kernel (candidates
    from the cells; dp 20 moves span more than a cell's neighbours, every group a candidate)
    gives the chain kernel's chain."""
    from test_spline import _cluster_example
    spec, _ = _cluster_example()
    g = ctx.create(spec)
    eg, eo = g.energy_total(), O.OracleSystem(spec).energy_total()
    for key in ("self", "nonbonded", "total"):
        assert abs(eg[key] - eo[key]) <= 1e-9 * max(1.0, abs(eo[key])), key
    a, b = ctx.create(spec), ctx.create(spec)
    sa = ctx.run_batch([a], 4000, seed=5, dp=dp, dprot=1.0, threads=0)
    sb = ctx.run_batch([b], 4000, seed=5, dp=dp, dprot=1.0, threads=256)
    assert sa["accepted"] == sb["accepted"] > 100
    assert np.array_equal(a.positions(), b.positions())
    assert abs(a.running_energy() - b.running_energy()) <= 1e-9 * abs(b.running_energy())
    _energy_consistent(a)
