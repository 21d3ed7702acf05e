"""Splined pair potentials (nonbonded_splined) on the host and in the oracle.

The table generator (fau_andrea_generate, fau_spline_tabulate) is pinned by the
reference's own Andrea known-answer test (src/tabulate.h:316-366) and by
SplinedPotential's contract (src/potentials.cpp:1453-1597): the spline within
utol of the exact functor on [rmin, rmax], |u(rmin)| within 10 % of u_at_rmin,
|u(rmax)| <= u_at_rmax, hard-sphere repulsion dropped for attractive pairs.
The oracle's splined energy is checked against an independent numpy sum that
evaluates the same tables (SplinedPotential::operator(), src/potentials.h:807-823).
"""
import dataclasses
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs
from faunus_gb300.input import load_input

import oracle_lib as O


def test_andrea_kat():
    # TEST_CASE("[Faunus] Andrea"): f = x sin(x) / 2 + 2 on ]0, 10], utol 2e-6, ftol 1e-4
    f = lambda x: 0.5 * x * math.sin(x) + 2
    z, c = F.andrea_spline(f, 0.0, 10.0, 2e-6, 1e-4)
    assert len(z) == 19 and c.size == 108
    assert z[0] == pytest.approx(0.0, abs=1e-12) and z[-1] == pytest.approx(10.0)
    assert z[1] == pytest.approx(0.212991, rel=1e-5) and z[2] == pytest.approx(0.782554, rel=1e-5)
    assert c[0][0] == pytest.approx(2.0) and c[0][1] == pytest.approx(0.0, abs=1e-9)
    assert c[0][2] == pytest.approx(0.5, rel=1e-5) and c[-1][-1] == pytest.approx(-0.0441931, rel=1e-5)
    for x in (1e-9, 5.0, 10.0):
        assert F.andrea_eval(z, c, x) == pytest.approx(f(x), rel=1e-5)


def test_andrea_tolerance_failure_raises():
    # a step that no quintic piece can follow within utol (the reference throws too)
    with pytest.raises(F.FauError):
        F.andrea_spline(lambda z: 1.0 if z < 4.0 else 0.0, 1.0, 9.0, 1e-6)


def _salt(n_salt=200, seed=3, scheme=None):
    spec = configs.bulk_ewald(n_salt=n_salt, seed=seed)
    if scheme:
        spec = dataclasses.replace(spec, ewald=None, **F.coulomb_scheme(scheme, epsr=80.0, cutoff=12.0))
    return spec


def _type_q_sigma(spec):
    q = [float(spec.charge[spec.type == t][0]) for t in range(spec.n_types)]
    return q, np.sqrt(np.diag(spec.sigma2))


def _exact(spec, a, b, r2):
    """the unsplined pair energy of two type-a, type-b particles (oracle, FP64)"""
    q, _ = _type_q_sigma(spec)
    plain = dataclasses.replace(spec, pair_cutoff=0.0)
    return O.pair_u(plain, a, b, q[a], q[b], r2)


@pytest.mark.parametrize("scheme", [None, "fanourgakis"])
def test_pair_tables_meet_the_spline_contract(scheme):
    spec = _salt(scheme=scheme)
    q, sig = _type_q_sigma(spec)
    sp = F.splined(spec, q, sig)
    tb = sp.spline
    T = spec.n_types
    assert len(tb["begin"]) == T * T + 1 and tb["begin"][0] == 0
    for a in range(T):
        for b in range(T):
            ab = a * T + b
            z = tb["r2"][tb["begin"][ab]:tb["begin"][ab + 1]]
            c = tb["coef"][6 * (tb["begin"][ab] - ab):6 * (tb["begin"][ab + 1] - ab - 1)].reshape(-1, 6)
            rmin, rmax = math.sqrt(z[0]), math.sqrt(z[-1])
            assert np.all(np.diff(z) > 0)
            u_min = abs(_exact(spec, a, b, z[0]))
            assert 20.0 / 1.1 <= u_min <= 20.0 * 1.1  # findLowerDistance
            assert abs(_exact(spec, a, b, z[-1])) <= 1e-6  # findUpperDistance
            for r in np.arange(rmin + 0.01, rmax, 0.01):  # createKnots' error scan
                assert abs(F.andrea_eval(z, c, r * r) - _exact(spec, a, b, r * r)) <= 1e-3 + 1e-12
            # symmetric tables
            ba = b * T + a
            assert np.array_equal(z, tb["r2"][tb["begin"][ba]:tb["begin"][ba + 1]])
    # every pair is zero beyond its last knot: pair_cutoff follows the longest table
    assert sp.pair_cutoff == pytest.approx(min(spec.pair_cutoff, math.sqrt(tb["r2"].max()) * (1 + 1e-9)))
    assert sp.pair_terms & A.FAU_PAIR_SPLINE


def test_hardsphere_flag_only_for_repulsive_pairs():
    spec = _salt()
    q, sig = _type_q_sigma(spec)
    sp = F.splined(spec, q, sig, hardsphere=True)
    assert list(sp.spline["hs"]) == [1, 1, 1, 1]  # LJ repulsion at every pair's inner end
    # without LJ between unlike ions, their Coulomb attraction is -20 kT at rmin: no hard sphere
    eps4 = spec.eps4.copy()
    eps4[0, 1] = eps4[1, 0] = 0.0
    sp = F.splined(dataclasses.replace(spec, eps4=eps4), q, sig, hardsphere=True)
    assert list(sp.spline["hs"]) == [1, 0, 0, 1]
    ab = 1
    z0 = sp.spline["r2"][sp.spline["begin"][ab]]
    assert _exact(dataclasses.replace(spec, eps4=eps4), 0, 1, z0) < 0


def test_unsplinable_functors_raise():
    spec = configs.primitive_model(n=50)
    q = [1.0, -1.0]
    with pytest.raises(F.FauError):  # hard-sphere contact below 20 kT: rmin oscillates at sigma
        F.splined(spec, q, [4.0, 4.0])
    plain = dataclasses.replace(spec, pair_terms=A.FAU_PAIR_COULOMB | A.FAU_PAIR_WCA, coulomb_type=A.FAU_COUL_PLAIN)
    with pytest.raises(F.FauError):  # 1/r never falls below 1e-6 kT within 1e6 steps
        F.splined(plain, q, [4.0, 4.0])


def _numpy_splined_energy(sp):
    """SplinedPotential::operator() over all atom pairs (minimum image), numpy FP64"""
    x, L, T = sp.pos, sp.box, sp.n_types
    i, j = np.triu_indices(sp.n, 1)
    d = x[i] - x[j]
    d -= L * np.round(d / L)
    r2 = (d * d).sum(1)
    ab = sp.type[i] * T + sp.type[j]
    tb = sp.spline
    u = np.zeros(len(r2))
    exact = []
    for k in range(T * T):
        sel = np.nonzero(ab == k)[0]
        z = tb["r2"][tb["begin"][k]:tb["begin"][k + 1]]
        c = tb["coef"][6 * (tb["begin"][k] - k):6 * (tb["begin"][k + 1] - k - 1)].reshape(-1, 6)
        inside = (r2[sel] > z[0]) & (r2[sel] < z[-1]) & (r2[sel] < sp.pair_cutoff ** 2)
        for s in sel[inside]:
            u[s] = F.andrea_eval(z, c, r2[s])
        exact.extend(sel[r2[sel] <= z[0]].tolist())
    assert not exact  # no pair below rmin at this density
    return float(u.sum())


def test_oracle_splined_energy_matches_numpy():
    spec = _salt(scheme="fanourgakis")
    q, sig = _type_q_sigma(spec)
    sp = F.splined(spec, q, sig)
    e = O.OracleSystem(sp).energy_total()["nonbonded"]
    assert e == pytest.approx(_numpy_splined_energy(sp), rel=1e-12, abs=1e-12)
    # and close to the exact functor: utol per pair at most
    e0 = O.OracleSystem(spec).energy_total()["nonbonded"]
    assert abs(e - e0) < 1e-3 * spec.n


def test_descriptor_rejects_bad_tables():
    spec = _salt()
    q, sig = _type_q_sigma(spec)
    sp = F.splined(spec, q, sig)
    bad = sp.copy()
    bad.spline["r2"] = bad.spline["r2"].copy()
    bad.spline["r2"][1] = bad.spline["r2"][0]  # not ascending
    with pytest.raises(F.FauError):
        F.footprint(bad)
    bad = sp.copy()
    bad.spline = None  # FAU_PAIR_SPLINE without tables
    with pytest.raises(F.FauError):
        F.footprint(bad)
    assert F.footprint(sp) > F.footprint(spec)


_SPLINED_INPUT = """
temperature: 298.15
geometry: {type: cuboid, length: 60}
mcloop: {macro: 2, micro: 10}
random: {seed: fixed}
atomlist:
  - Na: {q: 1.0, sigma: 3.33, eps: 0.01158968, dp: 1.0}
  - Cl: {q: -1.0, sigma: 4.4, eps: 0.4184, dp: 0.5}
moleculelist:
  - salt: {atoms: [Na, Cl], atomic: true}
insertmolecules:
  - salt: {N: 40}
energy:
  - nonbonded_splined:
      utol: 0.0001
      default:
        - lennardjones: {mixing: LB}
        - coulomb: {type: fanourgakis, epsr: 80, cutoff: 14}
moves:
  - transrot: {molecule: salt}
"""


def test_input_nonbonded_splined():
    st = load_input(_SPLINED_INPUT)
    sp = st.spec
    assert sp.pair_terms & A.FAU_PAIR_SPLINE and sp.pair_terms & A.FAU_PAIR_LJ
    assert sp.spline is not None and len(sp.spline["begin"]) == 5
    # the exact input (nonbonded) gives the same functor; the splined energy is within utol a pair
    exact = load_input(_SPLINED_INPUT.replace("nonbonded_splined", "nonbonded").replace("      utol: 0.0001\n", ""))
    assert not exact.spec.pair_terms & A.FAU_PAIR_SPLINE
    es = O.OracleSystem(sp).energy_total()["nonbonded"]
    ee = O.OracleSystem(exact.spec).energy_total()["nonbonded"]
    assert abs(es - ee) <= 1e-4 * sp.n * (sp.n - 1) / 2
    with pytest.raises(NotImplementedError):
        load_input(_SPLINED_INPUT.replace("nonbonded_splined", "nonbonded_cached"))


def _cluster_example():
    import json
    from pathlib import Path
    from faunus_gb300.input import apply_state
    fx = json.loads((Path(__file__).parent / "golden" / "cluster_example.json").read_text())
    st = load_input(fx["input"])
    apply_state(st, fx["state"])
    return st.spec, fx["expected"]


def test_reference_cluster_example_energy():
    """examples/cluster: ten rigid waters, nonbonded_splined (fanourgakis, epsr 1.2, LB
    Lennard-Jones, cutoff_g2g 10).  The reference reported SystemEnergy -533.93 kT (2 decimals)
    for the state its run started from: the exact functor plus the documented fanourgakis self
    energy give it within the rounding, and the splined tables within utol a pair."""
    sp, exp = _cluster_example()
    assert sp.pair_terms & A.FAU_PAIR_SPLINE
    assert sp.bjerrum_length == pytest.approx(exp["bjerrum_length"], abs=0.005)
    exact = sp.copy()
    exact.spline = None
    exact.pair_terms &= ~A.FAU_PAIR_SPLINE
    ee = O.OracleSystem(exact).energy_total()
    assert abs(ee["total"] - exp["systemenergy_init"]) <= 0.005 + 1e-9
    es = O.OracleSystem(sp).energy_total()
    # pairs of atoms in different waters whose mass centres are within cutoff_g2g
    cm = sp.mass_center
    d = cm[:, None, :] - cm[None, :, :]
    d -= sp.box * np.round(d / sp.box)
    close = ((d * d).sum(-1) < 100.0).sum() - sp.n_groups  # ordered pairs of groups, self excluded
    n_pairs = close // 2 * 9
    assert abs(es["total"] - ee["total"]) <= 1e-3 * n_pairs
    assert es["self"] == ee["self"]


def test_tabulate_argument_errors():
    import ctypes as C
    spec = _salt()
    d, keep = spec.to_desc()
    opts = A.SplineOpts(1e-3, 1e-2, 20.0, 1e-6, 0.0, 0, 0)
    z, c = np.zeros(4), np.zeros(24)
    n, hs = C.c_int(), C.c_int()
    lib = A.lib()
    # a table larger than the output capacity, a type out of range, a non-positive rmin
    assert lib.fau_spline_tabulate(C.byref(d), 0, 0, 1.0, 1.0, 3.0, C.byref(opts), 4, A.as_dptr(z),
                                   A.as_dptr(c), C.byref(n), C.byref(hs)) == A.FAU_ERR_ARG
    assert lib.fau_spline_tabulate(C.byref(d), 5, 0, 1.0, 1.0, 3.0, C.byref(opts), 4, A.as_dptr(z),
                                   A.as_dptr(c), C.byref(n), C.byref(hs)) == A.FAU_ERR_ARG
    assert lib.fau_spline_tabulate(C.byref(d), 0, 0, 1.0, 1.0, 0.0, C.byref(opts), 4, A.as_dptr(z),
                                   A.as_dptr(c), C.byref(n), C.byref(hs)) == A.FAU_ERR_ARG
    assert b"spline" in lib.fau_last_error()


def test_input_splined_options_reach_the_tables():
    hard = load_input(_SPLINED_INPUT.replace("      utol: 0.0001\n", "      utol: 0.0001\n      hardsphere: true\n"))
    assert list(hard.spec.spline["hs"]) == [1, 1, 1, 1]
    coarse = load_input(_SPLINED_INPUT.replace("utol: 0.0001", "utol: 0.01"))
    fine = load_input(_SPLINED_INPUT)
    assert len(coarse.spec.spline["r2"]) < len(fine.spec.spline["r2"])
