"""Truncated Coulomb short-range functions S(q) (NewCoulombGalore, src/potentials.cpp:1628-1700;
docs/_docs/energy.md:169-224) at infinite Debye length.

The host helper writes each named scheme as e erfc(alpha r) + sum_k c_k q^k
(FAU_COUL_TRUNC).  Its polynomials are checked against the documented formulas
evaluated directly, and against the documentation's own table of poisson (C, D)
equivalents (plain within cutoff, undamped Wolf, Levitt / undamped Fennell,
Stenqvist, Fanourgakis).  The oracle's pair energy is lB qa qb S(q) / (r + eps)
below Rc and 0 beyond; its self energy is lB q^2 S'(0) / (2 Rc), the limit of
the documented U_self, which reduces to -lB alpha q^2 / sqrt(pi) for Ewald (the
value the reference's own Ewald KAT pins).  The reference splines S(q) through
CoulombGalore (not vendored), so these forms are restated, not pinned.
"""
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300.system import SystemSpec

import oracle_lib as O

RC, ALPHA, EPSR = 12.0, 0.2, 80.0
Q = np.linspace(0.0, 0.999, 37)
E = math.erfc(ALPHA * RC)
G = 2 * ALPHA * RC / math.sqrt(math.pi) * math.exp(-(ALPHA * RC) ** 2)
erfc = np.vectorize(math.erfc)

DOCS = {  # docs/_docs/energy.md:179-190, written out independently of the helper
    "reactionfield": lambda q, epsrf=40.0: 1 + (epsrf - EPSR) / (2 * epsrf + EPSR) * q ** 3
    - 3 * epsrf / (2 * epsrf + EPSR) * q,
    "qpotential": lambda q: np.prod([1 - q ** n for n in range(1, 5)], axis=0),
    "fanourgakis": lambda q: 1 - 7 / 4 * q + 21 / 4 * q ** 5 - 7 * q ** 6 + 5 / 2 * q ** 7,
    "fennell": lambda q: erfc(ALPHA * RC * q) - q * E + (q - 1) * q * (E + G),
    "zerodipole": lambda q: erfc(ALPHA * RC * q) - q * E + (q * q - 1) / 2 * q * (E + G),
    "zahn": lambda q: erfc(ALPHA * RC * q) - (q - 1) * q * (E + G),
    "wolf": lambda q: erfc(ALPHA * RC * q) - E * q,
    "poisson": lambda q: (1 - q) ** 4 * sum((3 - c) / 3 * math.comb(2 + c, c) * q ** c for c in range(3)),
}
KW = {"reactionfield": dict(epsrf=40.0), "qpotential": dict(order=4)}


def s_of(f, q):
    poly = f["coulomb_poly"]
    s = np.polyval(poly[::-1], q)
    if f["coulomb_erfc"]:
        s = s + f["coulomb_erfc"] * erfc(f["coulomb_alpha"] * RC * q)
    return s


@pytest.mark.parametrize("name", sorted(DOCS))
def test_scheme_polynomial_matches_documented_formula(name):
    f = F.coulomb_scheme(name, epsr=EPSR, cutoff=RC, alpha=ALPHA, **KW.get(name, {}))
    assert f["coulomb_type"] == A.FAU_COUL_TRUNC
    assert np.allclose(s_of(f, Q), DOCS[name](Q), rtol=1e-12, atol=1e-13)
    s1 = s_of(f, np.array([1.0]))[0]  # S(1) = 0 (continuous at the cutoff) except Zahn's erfc(alpha Rc)
    assert abs(s1 - (E if name == "zahn" else 0.0)) < 1e-12
    assert abs(s_of(f, np.array([0.0]))[0] - 1.0) < 1e-12  # S(0) = 1


@pytest.mark.parametrize("C,D,equivalent", [
    (1, -1, lambda q: np.ones_like(q)),                   # plain Coulomb within cutoff
    (1, 0, lambda q: 1 - q),                              # undamped Wolf
    (1, 1, lambda q: (1 - q) ** 2),                       # Levitt / undamped Fennell
    (3, 3, DOCS["poisson"]),                              # Stenqvist
    (4, 3, DOCS["fanourgakis"]),                          # Fanourgakis
])
def test_poisson_equivalence_table(C, D, equivalent):
    f = F.coulomb_scheme("poisson", epsr=EPSR, cutoff=RC, C=C, D=D)
    assert np.allclose(s_of(f, Q), equivalent(Q), rtol=1e-12, atol=1e-13)


def test_undamped_limits_of_erfc_schemes():
    """alpha -> 0: Wolf -> poisson(1, 0), Fennell -> poisson(1, 1)."""
    for name, (C, D) in (("wolf", (1, 0)), ("fennell", (1, 1))):
        a = F.coulomb_scheme(name, epsr=EPSR, cutoff=RC, alpha=0.0)
        b = F.coulomb_scheme("poisson", epsr=EPSR, cutoff=RC, C=C, D=D)
        assert np.allclose(s_of(a, Q), s_of(b, Q), atol=1e-14)


def test_scheme_argument_errors():
    with pytest.raises(ValueError):
        F.coulomb_scheme("plain", epsr=EPSR, cutoff=10.0)
    with pytest.raises(ValueError):
        F.coulomb_scheme("wolf", epsr=EPSR)
    with pytest.raises(ValueError):
        F.coulomb_scheme("qpotential", epsr=EPSR, cutoff=RC)
    with pytest.raises(ValueError):
        F.coulomb_scheme("qpotential", epsr=EPSR, cutoff=RC, order=6)  # degree 21 > 15
    with pytest.raises(ValueError):
        F.coulomb_scheme("yukawa", epsr=EPSR, cutoff=RC)


def _two_ions(f, r):
    return SystemSpec(box=np.full(3, 100.0), pos=np.array([[0.0, 0, 0], [r, 0, 0]]), charge=np.array([1.0, -1.0]),
                      type=np.array([0, 0], np.int32), group_begin=np.array([0, 2], np.int32),
                      group_flags=np.array([1], np.int32), n_types=1, pair_terms=A.FAU_PAIR_COULOMB, **f)


@pytest.mark.parametrize("name", sorted(DOCS))
def test_oracle_pair_and_self_energy(name):
    f = F.coulomb_scheme(name, epsr=EPSR, cutoff=RC, alpha=ALPHA, **KW.get(name, {}))
    lB = f["bjerrum_length"]
    for r in (3.0, 7.5, 11.9):
        e = O.OracleSystem(_two_ions(f, r)).energy_total()
        rr = r + np.finfo(float).eps
        assert e["nonbonded"] == pytest.approx(-lB * DOCS[name](np.array([rr / RC]))[0] / rr, rel=1e-12, abs=1e-15)
        # U_self = -1/2 sum_i lim (u - u~) = lB q^2 S'(0) / (2 Rc), by a central difference of S
        h = 1e-6
        ds0 = (DOCS[name](np.array([h]))[0] - DOCS[name](np.array([-h]))[0]) / (2 * h)
        assert e["self"] == pytest.approx(2 * lB * ds0 / (2 * RC), rel=1e-6)
    assert O.OracleSystem(_two_ions(f, 12.5)).energy_total()["nonbonded"] == 0.0


def test_descriptor_rejects_bad_scheme():
    f = F.coulomb_scheme("wolf", epsr=EPSR, cutoff=RC, alpha=ALPHA)
    spec = _two_ions(f, 3.0)
    spec.coulomb_poly = np.full(17, 1.0)
    with pytest.raises(ValueError):
        spec.to_desc()
    spec = _two_ions(dict(f, coulomb_cutoff=0.0), 3.0)
    with pytest.raises(F.FauError):
        F.footprint(spec)
    spec = _two_ions(dict(f, coulomb_type=7), 3.0)
    with pytest.raises(F.FauError):
        F.footprint(spec)
