"""The CPU oracle against the reference's own known-answer tests.

Golden values come from tests/golden/kat.json (extracted from the reference's
doctest sources by tests/golden/make_kat.py; each carries its file:line).
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from faunus_gb300 import _capi as A
from faunus_gb300.system import SystemSpec, bjerrum_length, kjmol_to_kt

import oracle_lib as O

KAT = {k: v["value"] for k, v in json.loads((Path(__file__).parent / "golden" / "kat.json").read_text()).items()}
# doctest::Approx default: relative epsilon = FLT_EPSILON * 100
APPROX = 1.1920929e-07 * 100


def approx(a, b, rel=APPROX):
    return abs(a - b) <= rel * (max(abs(a), abs(b)) + 1.0) if b == 0 else abs(a - b) <= rel * max(abs(a), abs(b))


# ---------------------------------------------------------------- Ewald (src/energy.cpp:74-99, 249-317)
def test_ewald_kvector_counts():
    L = np.full(3, 10.0)
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    q = np.array([1.0, -1.0])
    pbc = O.ewald_policy(pos, q, L, KAT["ewald_alpha"], 11.0, True, 1.0, 1.0, ipbc=False)
    ipbc = O.ewald_policy(pos, q, L, KAT["ewald_alpha"], 11.0, True, 1.0, 1.0, ipbc=True)
    assert pbc["K"] == KAT["ewald_kvectors_pbc"] == 2975
    assert ipbc["K"] == KAT["ewald_kvectors_ipbc"] == 846


@pytest.mark.parametrize("ipbc", [False, True])
def test_ewald_two_ion_energies(ipbc):
    lB = bjerrum_length(1.0, 298.15)
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    q = np.array([1.0, -1.0])
    e = O.ewald_policy(pos, q, np.full(3, 10.0), KAT["ewald_alpha"], 11.0, True, 1.0, lB, ipbc=ipbc)
    assert approx(e["self"], KAT["ewald_self_per_lB"] * lB)
    assert approx(e["surface"], KAT["ewald_surface_per_lB"] * lB)
    key = "ewald_reciprocal_ipbc_per_lB" if ipbc else "ewald_reciprocal_pbc_per_lB"
    assert approx(e["reciprocal"], KAT[key] * lB)
    # tighter than doctest::Approx: the restatement reproduces the reference to ~1e-9
    assert abs(e["reciprocal"] / lB - KAT[key]) < 1e-9


def _nacl_ewald_spec():
    """SpaceFactory::makeNaCl (src/space.cpp:696-713) with two ions at (0,0,0)
    and (1,0,0) in a 10 A cube, Ewald epsr 1, alpha 0.894..., ncutoff 11, epss 1."""
    lB = bjerrum_length(1.0, 298.15)
    return SystemSpec(
        box=np.full(3, 10.0), pos=np.array([[0.0, 0, 0], [1.0, 0, 0]]), charge=np.array([1.0, -1.0]),
        type=np.array([0, 1], dtype=np.int32), group_begin=np.array([0, 2], dtype=np.int32),
        group_flags=np.array([A.FAU_GROUP_ATOMIC], dtype=np.int32), n_types=2, pair_terms=0,
        bjerrum_length=lB, ewald={"alpha": KAT["ewald_alpha"], "ncutoff": 11.0, "spherical_sum": 1, "epss": 1.0},
        precision=A.FAU_PREC_FP64, temperature=298.15)


def test_ewald_update_restore():
    """Energy::Ewald (src/energy.cpp:665-762): energy 103.73 after moving the first
    ion to (0.1, 0.1, 0.1), dU -16.838 through a partial (index) update."""
    spec = _nacl_ewald_spec()
    o = O.OracleSystem(spec)
    e0 = o.energy_total()
    lB = spec.bjerrum_length
    assert approx(e0["total"], (KAT["ewald_surface_per_lB"] + KAT["ewald_reciprocal_pbc_per_lB"]) * lB)
    r = o.trial_atomic(0, (0.1, 0.1, 0.1), 0.0)
    assert r["accepted"] == 1
    assert approx(r["du"], KAT["ewald_energy_change"])
    e1 = o.energy_total()
    assert approx(e1["total"], KAT["ewald_energy_after_move"])
    # partial (cumulative) Q equals a full rebuild
    full = O.OracleSystem(SystemSpec(**{**spec.__dict__, "pos": np.array([[0.1, 0.1, 0.1], [1.0, 0, 0]])}))
    assert np.allclose(o.q(), full.q(), rtol=0, atol=1e-12)
    # and back: restore gives the reference energy again
    r2 = o.trial_atomic(0, (-0.1, -0.1, -0.1), 0.0)
    assert approx(r2["du"], -KAT["ewald_energy_change"])


# ---------------------------------------------------------------- pair potentials
def _lj_spec(sigma, eps_kjmol, custom=None, mixing="LB"):
    sig = np.array(sigma, dtype=float)
    eps = np.array([kjmol_to_kt(e, 298.15) for e in eps_kjmol])
    if mixing == "LB":
        s = 0.5 * (sig[:, None] + sig[None, :])
    else:
        s = np.sqrt(sig[:, None] * sig[None, :])
    e = np.sqrt(eps[:, None] * eps[None, :])
    if custom:
        for (a, b), (cs, ce) in custom.items():
            s[a, b] = s[b, a] = cs
            e[a, b] = e[b, a] = kjmol_to_kt(ce, 298.15)
    n = len(sig)
    return SystemSpec(box=np.full(3, 100.0), pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.zeros(1, np.int32),
                      group_begin=np.array([0, 1], np.int32), group_flags=np.array([1], np.int32), n_types=n,
                      sigma2=s * s, eps4=4 * e, pair_terms=A.FAU_PAIR_LJ)


def test_lennard_jones_mixing():
    """LennardJones (src/potentials.cpp:711-782): A(2, 0.9) B(8, 0.1) C(5, 1.1), d = 9 A."""
    d = 9.0

    def lj(sig, eps_kjmol):
        e = kjmol_to_kt(eps_kjmol, 298.15)
        return 4 * e * ((sig / d) ** 12 - (sig / d) ** 6)

    lb = _lj_spec([2, 8, 5], [0.9, 0.1, 1.1])
    assert approx(O.pair_u(lb, 0, 0, 0, 0, d * d), lj(2.0, 0.9))
    assert approx(O.pair_u(lb, 0, 1, 0, 0, d * d), lj(5.0, 0.3))
    geo = _lj_spec([2, 8, 5], [0.9, 0.1, 1.1], mixing="geometric")
    assert approx(O.pair_u(geo, 0, 1, 0, 0, d * d), lj(4.0, 0.3))
    cus = _lj_spec([2, 8, 5], [0.9, 0.1, 1.1], custom={(0, 1): (8.0, 0.5)})
    assert approx(O.pair_u(cus, 0, 1, 0, 0, d * d), lj(8.0, 0.5))
    assert approx(O.pair_u(cus, 0, 0, 0, 0, d * d), lj(2.0, 0.9))


def test_lennard_jones_force_kat():
    """force.x = 0.0142838474 for a custom A-B pair (eps 2, sigma 8) 9 A apart:
    F_x on a = dU/dr for a at the origin and b at +9 x."""
    spec = _lj_spec([2, 8, 5], [0.9, 0.1, 1.1], custom={(0, 1): (8.0, 2.0)})
    h = 1e-5
    up = O.pair_u(spec, 0, 1, 0, 0, (9 + h) ** 2)
    um = O.pair_u(spec, 0, 1, 0, 0, (9 - h) ** 2)
    fx = (up - um) / (2 * h)
    assert abs(fx - KAT["lj_force_x"]) < 1e-8


def test_hard_sphere():
    """HardSphere (src/potentials.cpp:979-1016): arithmetic and custom mixing."""
    base = dict(box=np.full(3, 100.0), pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.zeros(1, np.int32),
                group_begin=np.array([0, 1], np.int32), group_flags=np.array([1], np.int32), n_types=2,
                pair_terms=A.FAU_PAIR_HS)
    s = np.array([2.0, 8.0])
    ar = 0.5 * (s[:, None] + s[None, :])
    spec = SystemSpec(hs_sigma2=ar * ar, **base)
    assert O.pair_u(spec, 0, 0, 0, 0, 2.01 ** 2) == 0
    assert O.pair_u(spec, 0, 0, 0, 0, 1.99 ** 2) == math.inf
    assert O.pair_u(spec, 0, 1, 0, 0, 5.01 ** 2) == 0
    assert O.pair_u(spec, 0, 1, 0, 0, 4.99 ** 2) == math.inf
    cus = ar.copy()
    cus[0, 1] = cus[1, 0] = 6.0
    spec = SystemSpec(hs_sigma2=cus * cus, **base)
    assert O.pair_u(spec, 0, 1, 0, 0, 6.01 ** 2) == 0
    assert O.pair_u(spec, 0, 1, 0, 0, 5.99 ** 2) == math.inf


def test_wca_missing_coefficient_is_nan():
    """WCA with a missing sigma gives NaN at any distance (src/potentials.cpp:1811-1817)."""
    base = dict(box=np.full(3, 100.0), pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.zeros(1, np.int32),
                group_begin=np.array([0, 1], np.int32), group_flags=np.array([1], np.int32), n_types=1,
                pair_terms=A.FAU_PAIR_WCA)
    spec = SystemSpec(sigma2=np.full((1, 1), np.nan), eps4=np.full((1, 1), 4 * 0.36), **base)
    assert math.isnan(O.pair_u(spec, 0, 0, 0, 0, 100.0))
    assert math.isnan(O.pair_u(spec, 0, 0, 0, 0, 1.0))
    ok = SystemSpec(sigma2=np.full((1, 1), 4.0), eps4=np.full((1, 1), 1.0), **base)
    assert O.pair_u(ok, 0, 0, 0, 0, 4.0 * 1.26) == 0.0
    assert O.pair_u(ok, 0, 0, 0, 0, 4.0) == pytest.approx(0.25)


def test_coulomb_bjerrum_length_and_force():
    """lB(epsr 80) = 7.0056973292 A (src/potentials.cpp:660); plain Coulomb force
    between +1/-1 ions 7 A apart is 0.1429734149 kT/A (src/potentials.cpp:1612-1626)."""
    lB = bjerrum_length(80.0, 298.15)
    assert abs(lB - KAT["coulomb_lB_epsr80"]) < 1e-9
    base = dict(box=np.full(3, 100.0), pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.zeros(1, np.int32),
                group_begin=np.array([0, 1], np.int32), group_flags=np.array([1], np.int32), n_types=1,
                pair_terms=A.FAU_PAIR_COULOMB, coulomb_type=A.FAU_COUL_PLAIN, bjerrum_length=lB)
    spec = SystemSpec(**base)
    h = 1e-5
    fz = (O.pair_u(spec, 0, 0, 1, -1, (7 + h) ** 2) - O.pair_u(spec, 0, 0, 1, -1, (7 - h) ** 2)) / (2 * h)
    assert abs(fz - KAT["newcoulombgalore_plain_force_z"]) < 1e-8
    # |F| for r = (lB, 0.2, -0.1) (CustomPairPotential test, src/potentials.cpp:645-664)
    r = math.sqrt(lB ** 2 + 0.2 ** 2 + 0.1 ** 2)
    fn = (O.pair_u(spec, 0, 0, 1, 1, (r + h) ** 2) - O.pair_u(spec, 0, 0, 1, 1, (r - h) ** 2)) / (2 * h)
    assert abs(abs(fn) - KAT["coulomb_force_norm"]) < 1e-8


def test_functor_potential_coulomb_wca_sum():
    """FunctorPotential (src/potentials.cpp:1333-1368): default pair set Coulomb
    (epsr 80, plain), A-B Coulomb + WCA (LB mixing), C-C hard sphere only.  The
    descriptor's pair terms are global; a pair without a term has its coefficient
    zeroed (eps4 = 0 for WCA, hs_sigma2 = 0 for HS), which reproduces the per-pair
    sets: u(a,a) = coulomb, u(b,b) = coulomb, u(a,b) = coulomb + wca; C-C is 0 just
    outside contact and +inf just inside."""
    lB = bjerrum_length(80.0, 298.15)
    sig = np.array([2.2, 4.0, 2.0])  # 2 r
    eps = np.array([0.1, 0.05, 0.0])  # kJ/mol
    q = np.array([1.0, -1.0, 0.0])
    s2 = (0.5 * (sig[:, None] + sig[None, :])) ** 2
    e4 = np.zeros((3, 3))
    e4[0, 1] = e4[1, 0] = 4 * kjmol_to_kt(math.sqrt(eps[0] * eps[1]), 298.15)
    hs2 = np.zeros((3, 3))
    hs2[2, 2] = s2[2, 2]
    spec = SystemSpec(box=np.full(3, 100.0), pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.zeros(1, np.int32),
                      group_begin=np.array([0, 1], np.int32), group_flags=np.array([1], np.int32), n_types=3,
                      sigma2=s2, eps4=e4, hs_sigma2=hs2, bjerrum_length=lB, coulomb_type=A.FAU_COUL_PLAIN,
                      pair_terms=A.FAU_PAIR_COULOMB | A.FAU_PAIR_WCA | A.FAU_PAIR_HS)
    r2 = 4.0  # r = (2, 0, 0)

    def coulomb(a, b):
        return lB * q[a] * q[b] / math.sqrt(r2)

    def wca(a, b):
        x = (s2[a, b] / r2) ** 3  # (sigma/r)^6
        return 0.0 if r2 > s2[a, b] * 2 ** (1 / 3) else e4[a, b] * (x * x - x + 0.25)

    assert approx(O.pair_u(spec, 0, 0, q[0], q[0], r2), coulomb(0, 0))
    assert approx(O.pair_u(spec, 1, 1, q[1], q[1], r2), coulomb(1, 1))
    assert wca(0, 1) > 0  # the WCA part is not trivially zero at this distance
    assert approx(O.pair_u(spec, 0, 1, q[0], q[1], r2), coulomb(0, 1) + wca(0, 1))
    assert O.pair_u(spec, 2, 2, 0.0, 0.0, r2 * 1.01 ** 2) == 0
    assert O.pair_u(spec, 2, 2, 0.0, 0.0, r2 * 0.99 ** 2) == math.inf


def test_chameleon_cuboid_consistency():
    """Chameleon vs Cuboid (src/geometry.cpp:1320-1371, subcase "cuboid"): points
    drawn in a box 2^(1/3) larger than the periodic cell (2, 3, 4); boundary() and
    vdist() agree with Cuboid's (anint wrap; +-L where |d| > L/2), and
    sqdist(a, b) = |vdist(a, b)|^2."""
    L = np.array([2.0, 3.0, 4.0])
    big = np.cbrt(2.0) * L
    rng = np.random.default_rng(7)
    a = (rng.random((100, 3)) - 0.5) * big
    b = (rng.random((100, 3)) - 0.5) * big
    aw, vd, sq = O.geometry(L, a, b)
    # Cuboid::boundary / vdist (src/geometry.cpp:91-129), restated with numpy
    anint = lambda x: np.trunc(np.where(x > 0, x + 0.5, x - 0.5))
    cw = np.where(np.abs(a) > L / 2, a - L * anint(a / L), a)
    d = a - b
    cd = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
    for x, y in ((aw, cw), (vd, cd)):
        assert all(approx(u, v) for u, v in zip(x.ravel(), y.ravel()))
    assert all(approx(s, float((v * v).sum())) for s, v in zip(sq, vd))
    assert (np.abs(aw) <= L / 2 + 1e-12).all()


def test_ewald_real_space_self_energy():
    """Real-space Ewald S = erfc(alpha r) and self energy -lB alpha/sqrt(pi) q^2,
    matching PolicyIonIon::selfEnergy (src/energy.cpp:484-518) for kappa = 0."""
    lB, alpha = 7.0, 0.3
    spec = SystemSpec(box=np.full(3, 40.0), pos=np.array([[0.0, 0, 0], [3.0, 0, 0]]), charge=np.array([1.0, -1.0]),
                      type=np.array([0, 0], np.int32), group_begin=np.array([0, 2], np.int32),
                      group_flags=np.array([1], np.int32), n_types=1, pair_terms=A.FAU_PAIR_COULOMB,
                      coulomb_type=A.FAU_COUL_EWALD, bjerrum_length=lB, coulomb_cutoff=12.0, coulomb_alpha=alpha)
    e = O.OracleSystem(spec).energy_total()
    r = 3.0 + np.finfo(float).eps
    assert e["nonbonded"] == pytest.approx(-lB * math.erfc(alpha * r) / r, rel=1e-14)
    assert e["self"] == pytest.approx(2 * -lB * alpha / math.sqrt(math.pi), rel=1e-14)


# ---------------------------------------------------------------- cell grid (src/celllistimpl.cpp:46-174)
def test_cell_grid_kat():
    box = np.array([20.0, 30.0, 40.0])
    pts_grid = np.array([[3.0, 2.5, 3.0], [3.0, 3.0, 3.0], [19.0, 29.0, 39.0], [1.0, 1.0, 1.0],
                         [0.0, 0.0, 0.0], [20.0, 30.0, 40.0], [21.0, 10.0, 10.0], [1.0, 10.0, 10.0]])
    cells, dims, omin, omax = O.cell_bin(box, 1.5, pts_grid - 0.5 * box)
    assert dims == (200 // 15, 300 // 15, 400 // 15)
    nx, ny, nz = dims

    def idx(c):
        return c[0] + nx * (c[1] + ny * c[2])

    assert cells[0] == idx((1, 1, 1))
    assert cells[1] == idx((1, 2, 1))
    assert cells[2] == idx((nx - 1, ny - 1, nz - 1)) == nx * ny * nz - 1
    assert cells[3] == 0
    assert cells[4] == cells[5]  # periodic: indexAt(0,0,0) == indexAt(20,30,40)
    assert cells[6] == cells[7]  # indexAt(21,10,10) == indexAt(1,10,10)


def test_cell_neighbour_offsets():
    """Neighbour offsets never wrap onto themselves (src/celllistimpl.h:409-415)."""
    for L, rc, want in [(50.0, 24.0, ((0, 0, 0), (1, 1, 1))), (549.65, 12.0, ((-1,) * 3, (1,) * 3)),
                        (30.0, 12.0, ((0, 0, 0), (1, 1, 1))), (10.0, 12.0, ((0, 0, 0), (0, 0, 0)))]:
        _, dims, omin, omax = O.cell_bin(np.full(3, L), rc, np.zeros((1, 3)))
        assert (omin, omax) == want, (L, rc, dims)


# ---------------------------------------------------------------- RNG (src/random.cpp:65-101)
def test_rng_determinism_and_state():
    L = O.lib()
    assert L.orc_random_default_first() == L.orc_random_default_first()
    import ctypes as C
    b1 = C.create_string_buffer(1 << 16)
    b2 = C.create_string_buffer(1 << 16)
    L.orc_random_state(0, 1, b1, len(b1))
    L.orc_random_state(5489, 0, b2, len(b2))
    assert b1.value == b2.value  # default seed of std::mt19937 is 5489
    # the 10000th output of a default-constructed mt19937 is 4123659995 (C++ [rand.predef])
    state = list(map(int, b1.value.split()))
    assert len(state) == 625
    mt = _MT(state)
    for _ in range(9999):
        mt.next()
    assert mt.next() == 4123659995


class _MT:
    """Minimal MT19937 stepping from a libstdc++ text state (624 words + index)."""

    def __init__(self, st):
        self.x = st[:624]
        self.i = st[624]

    def next(self):
        if self.i >= 624:
            x = self.x
            for k in range(624):
                y = (x[k] & 0x80000000) | (x[(k + 1) % 624] & 0x7FFFFFFF)
                x[k] = x[(k + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            self.i = 0
        y = self.x[self.i]
        self.i += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF


# ---------------------------------------------------------------- Metropolis / energy change policy
def test_energy_change_policy_hard_sphere_overlap():
    """getEnergyChange (src/montecarlo.cpp:193-209): a move into overlap is +inf
    (reject), out of an overlap is -inf (accept)."""
    spec = SystemSpec(box=np.full(3, 20.0), pos=np.array([[0.0, 0, 0], [5.0, 0, 0]]), charge=np.zeros(2),
                      type=np.zeros(2, np.int32), group_begin=np.array([0, 2], np.int32),
                      group_flags=np.array([1], np.int32), n_types=1, hs_sigma2=np.full((1, 1), 16.0),
                      pair_terms=A.FAU_PAIR_HS)
    o = O.OracleSystem(spec)
    r = o.trial_atomic(1, (-2.0, 0, 0), 0.5)  # to 3 A < 4 A
    assert r["du"] == math.inf and r["accepted"] == 0 and r["new_inf"] == 1
    spec2 = SystemSpec(**{**spec.__dict__, "pos": np.array([[0.0, 0, 0], [3.0, 0, 0]])})
    o2 = O.OracleSystem(spec2)
    r = o2.trial_atomic(1, (2.0, 0, 0), 0.99)
    assert r["du"] == -math.inf and r["accepted"] == 1
