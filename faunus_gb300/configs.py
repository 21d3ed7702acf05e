"""Seeded synthetic systems with the shapes of the benchmark configurations.

There is no public dataset for this path; these generators stand in for the
reference's example inputs with the named sizes, charges, potentials and
densities:

  primitive_model   200 hard-sphere ions (+1/-1, sigma 4 A) in L = 50 A,
                    Coulomb (lB 7.1 A, 24 A cutoff) + WCA + hard spheres
  bulk_ewald        20,000 LJ + Coulomb ions at 0.1 M salt, real-space erfc
                    cutoff 12 A (LJ truncated there too), alpha 0.3/A,
                    ncutoff 8, cell lists
  spce_water        1,000 rigid 3-site waters in L = 31 A, Ewald alpha 0.2,
                    Rc 9 A, ncutoff 7.3, cutoff_g2g 10 A (the reference's
                    examples/water/ewald.yml parameters), moltransrot moves
  pt_replicas       256 primitive-model systems, N ~ U{100..5000}, PT ladder
                    250-400 K
  served_jobs       Poisson stream of jobs with the shapes above
"""
from __future__ import annotations

import math

import numpy as np

from . import _capi as A
from .system import SystemSpec, bjerrum_length, group_cutoff, kjmol_to_kt

AVOGADRO = 6.022137e23


def _nonoverlapping(n: int, L: float, radii_sum_min: np.ndarray, rng: np.random.Generator,
                    sig: np.ndarray) -> np.ndarray:
    """Uniform random positions in [-L/2, L/2)^3 with no pair closer than
    (sig_i + sig_j)/2; overlapping particles are redrawn until none remain."""
    from scipy.spatial import cKDTree

    pos = rng.random((n, 3)) * L
    smax = float(sig.max()) if n else 0.0
    for _ in range(10000):
        tree = cKDTree(pos, boxsize=L)
        pairs = tree.query_pairs(smax, output_type="ndarray")
        if len(pairs):
            d = pos[pairs[:, 0]] - pos[pairs[:, 1]]
            d -= L * np.round(d / L)
            r = np.sqrt((d * d).sum(1))
            bad = r < 0.5 * (sig[pairs[:, 0]] + sig[pairs[:, 1]])
            pairs = pairs[bad]
        if len(pairs) == 0:
            break
        redo = np.unique(pairs[:, 1])
        pos[redo] = rng.random((len(redo), 3)) * L
    else:
        raise RuntimeError("could not place non-overlapping particles")
    out = pos - 0.5 * L
    out = np.minimum(out, np.nextafter(0.5 * L, 0))
    return out


def _lb_tables(sigma: np.ndarray, eps_kt: np.ndarray):
    """Lorentz-Berthelot mixing (src/potentials.cpp:18-48): arithmetic sigma,
    geometric epsilon; returns sigma^2 and 4 eps tables."""
    s = 0.5 * (sigma[:, None] + sigma[None, :])
    e = np.sqrt(eps_kt[:, None] * eps_kt[None, :])
    return s * s, 4.0 * e


def primitive_model(n: int = 200, L: float = 50.0, sigma: float = 4.0, lB: float = 7.1, rc: float = 24.0,
                    eps_kjmol: float = 0.5, temperature: float = 298.0, seed: int = 0,
                    precision: int = A.FAU_PREC_FP32C, wca: bool = True, hs: bool = True) -> SystemSpec:
    rng = np.random.default_rng(seed)
    assert n % 2 == 0
    types = np.array([0] * (n // 2) + [1] * (n // 2), dtype=np.int32)
    charge = np.where(types == 0, 1.0, -1.0)
    sig = np.full(n, sigma)
    pos = _nonoverlapping(n, L, sig, rng, sig)
    T = 2
    sigma2, eps4 = _lb_tables(np.full(T, sigma), np.full(T, kjmol_to_kt(eps_kjmol, temperature)))
    terms = A.FAU_PAIR_COULOMB | (A.FAU_PAIR_WCA if wca else 0) | (A.FAU_PAIR_HS if hs else 0)
    rcut = min(rc, 0.5 * L)
    return SystemSpec(
        box=np.full(3, L), pos=pos, charge=charge, type=types,
        group_begin=np.array([0, n], dtype=np.int32), group_flags=np.array([A.FAU_GROUP_ATOMIC], dtype=np.int32),
        n_types=T, sigma2=sigma2, eps4=eps4, hs_sigma2=np.full((T, T), sigma * sigma),
        pair_terms=terms, coulomb_type=A.FAU_COUL_CUT, bjerrum_length=lB, coulomb_cutoff=rcut,
        pair_cutoff=rcut, precision=precision, temperature=temperature,
        name=f"primitive-model N={n} L={L:g}",
        extra={"moves": [{"kind": A.FAU_MOVE_ATOMIC, "repeat": n, "dp": 2.0, "groups": [0]}]},
    )


def salt_box_length(n_salt: int, molar: float) -> float:
    """Cube side (A) holding n_salt formula units at `molar` mol/L."""
    return (n_salt / (molar * AVOGADRO * 1e-27)) ** (1.0 / 3.0)


def bulk_ewald(n_salt: int = 10000, molar: float = 0.1, sigma=(3.0, 4.0), eps_kjmol: float = 0.5,
               rc: float = 12.0, alpha: float = 0.3, ncutoff: float = 8.0, epsr: float = 80.0,
               temperature: float = 298.15, epss: float = 0.0, seed: int = 1, L: float | None = None,
               precision: int = A.FAU_PREC_FP32C, dp: float = 2.0) -> SystemSpec:
    rng = np.random.default_rng(seed)
    n = 2 * n_salt
    if L is None:
        L = salt_box_length(n_salt, molar)
    types = np.array([0] * n_salt + [1] * n_salt, dtype=np.int32)
    charge = np.where(types == 0, 1.0, -1.0)
    sig_t = np.array(sigma, dtype=np.float64)
    sig = sig_t[types]
    pos = _nonoverlapping(n, L, sig, rng, sig)
    eps = np.full(2, kjmol_to_kt(eps_kjmol, temperature))
    sigma2, eps4 = _lb_tables(sig_t, eps)
    return SystemSpec(
        box=np.full(3, L), pos=pos, charge=charge, type=types,
        group_begin=np.array([0, n], dtype=np.int32), group_flags=np.array([A.FAU_GROUP_ATOMIC], dtype=np.int32),
        n_types=2, sigma2=sigma2, eps4=eps4,
        pair_terms=A.FAU_PAIR_COULOMB | A.FAU_PAIR_LJ, coulomb_type=A.FAU_COUL_EWALD,
        bjerrum_length=bjerrum_length(epsr, temperature), coulomb_cutoff=rc, coulomb_alpha=alpha,
        pair_cutoff=rc, ewald={"alpha": alpha, "ncutoff": ncutoff, "spherical_sum": 1, "epss": epss},
        precision=precision, temperature=temperature, name=f"bulk-ewald N={n} L={L:.2f}",
        extra={"moves": [{"kind": A.FAU_MOVE_ATOMIC, "repeat": n, "dp": dp, "groups": [0]}]},
    )


def _random_quaternions(n: int, rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=(n, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def _rotate(q: np.ndarray, v: np.ndarray) -> np.ndarray:
    w, u = q[:, :1], q[:, 1:]
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def _wrap(x: np.ndarray, L) -> np.ndarray:
    L = np.asarray(L, dtype=np.float64)
    half = 0.5 * L
    out = x.copy()
    m = np.abs(out) > half
    t = out / L
    n = np.where(t > 0, np.floor(t + 0.5), np.ceil(t - 0.5))
    out = np.where(m, out - L * n, out)
    return out


def mass_centers(pos: np.ndarray, group_begin: np.ndarray, masses: np.ndarray, L: np.ndarray) -> np.ndarray:
    """Group::updateMassCenter (reference src/group.cpp:136-157): shift by the
    middle particle, mass-weighted centre with periodic wrap, shift back."""
    G = len(group_begin) - 1
    cm = np.zeros((G, 3))
    for g in range(G):
        b, e = group_begin[g], group_begin[g + 1]
        mid = b + (e - b) // 2
        sh = -pos[mid]
        p = _wrap(pos[b:e] + sh, L)
        w = masses[b:e]
        c = (w[:, None] * p).sum(0) / w.sum() - sh
        cm[g] = _wrap(c[None, :], L)[0]
    return cm


def spce_water(n_mol: int = 1000, L: float = 31.0, temperature: float = 300.0, epsr: float = 1.0,
               alpha: float = 0.2, rc: float = 9.0, ncutoff: float = 7.3, cutoff_g2g: float = 10.0,
               epss: float = 0.0, seed: int = 2, precision: int = A.FAU_PREC_FP32C, dp: float = 0.5,
               dprot: float = 0.5, molecules: tuple = ("SOL",)) -> SystemSpec:
    """Rigid SPC/E water (O -0.8476, H +0.4238; O-H 1 A, H-O-H 109.47 deg);
    mass centres on a cubic lattice with random orientations.

    With several `molecules` names, molecule g is of kind g mod len(molecules)
    (same chemistry, distinct molecule ids), and `cutoff_g2g` may be any
    GroupCutoff input form (a number or a {"default": .., "A B": ..} dict)."""
    rng = np.random.default_rng(seed)
    theta = math.radians(109.47) / 2
    geo = np.array([[0.0, 0.0, 0.0], [math.sin(theta), math.cos(theta), 0.0], [-math.sin(theta), math.cos(theta), 0.0]])
    mw = np.array([15.999, 1.007, 1.007])
    geo = geo - (mw[:, None] * geo).sum(0) / mw.sum()
    m = int(math.ceil(n_mol ** (1 / 3)))
    a = L / m
    grid = np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)], dtype=np.float64)
    sites = rng.permutation(len(grid))[:n_mol]
    centres = (grid[sites] + 0.5) * a - 0.5 * L + rng.uniform(-0.05, 0.05, size=(n_mol, 3)) * a
    q = _random_quaternions(n_mol, rng)
    pos = np.zeros((3 * n_mol, 3))
    for s in range(3):
        pos[s::3] = centres + _rotate(q, np.repeat(geo[s:s + 1], n_mol, axis=0))
    pos = _wrap(pos, np.full(3, L))
    types = np.tile(np.array([0, 1, 1], dtype=np.int32), n_mol)
    charge = np.where(types == 0, -0.8476, 0.4238)
    sig_t = np.array([3.166, 2.0])
    eps_t = np.array([kjmol_to_kt(0.65, temperature), 0.0])
    sigma2, eps4 = _lb_tables(sig_t, eps_t)
    gb = np.arange(0, 3 * n_mol + 1, 3, dtype=np.int32)
    masses = np.tile(mw, n_mol)
    box = np.full(3, L)
    cm = mass_centers(pos, gb, masses, box)
    return SystemSpec(
        box=box, pos=pos, charge=charge, type=types, group_begin=gb,
        group_flags=np.full(n_mol, A.FAU_GROUP_RIGID, dtype=np.int32),
        group_molid=(np.arange(n_mol) % len(molecules)).astype(np.int32),
        mass_center=cm, n_types=2, sigma2=sigma2, eps4=eps4, type_mass=np.array([15.999, 1.007]),
        pair_terms=A.FAU_PAIR_COULOMB | A.FAU_PAIR_LJ, coulomb_type=A.FAU_COUL_EWALD,
        bjerrum_length=bjerrum_length(epsr, temperature), coulomb_cutoff=rc, coulomb_alpha=alpha,
        cutoff_g2g=cutoff_g2g if not isinstance(cutoff_g2g, dict) else 0.0,
        cutoff_g2g_pairs=group_cutoff(cutoff_g2g, molecules) if isinstance(cutoff_g2g, dict) else None,
        ewald={"alpha": alpha, "ncutoff": ncutoff, "spherical_sum": 1, "epss": epss},
        precision=precision, temperature=temperature, name=f"spce-water N={n_mol}",
        extra={"moves": [{"kind": A.FAU_MOVE_MOLECULAR, "repeat": n_mol, "dp": dp, "dprot": dprot,
                          "groups": list(range(n_mol))}]},
    )


def pt_ladder(n: int = 256, t_min: float = 250.0, t_max: float = 400.0) -> np.ndarray:
    """Geometric temperature ladder T_r = t_min (t_max/t_min)^(r/(n-1))."""
    r = np.arange(n)
    return t_min * (t_max / t_min) ** (r / max(n - 1, 1))


def pt_replicas(n_rep: int = 256, n_min: int = 100, n_max: int = 5000, seed: int = 3,
                precision: int = A.FAU_PREC_FP32C):
    """Primitive-model replicas with uneven sizes and a PT temperature ladder.
    lB and epsilon/kT follow each replica's temperature (lB = 7.1 A at 298 K)."""
    rng = np.random.default_rng(seed)
    sizes = 2 * rng.integers(n_min // 2, n_max // 2 + 1, size=n_rep)
    temps = pt_ladder(n_rep)
    specs = []
    for r in range(n_rep):
        N = int(sizes[r])
        L = 50.0 * (N / 200.0) ** (1.0 / 3.0)
        T = float(temps[r])
        specs.append(primitive_model(n=N, L=L, lB=7.1 * 298.0 / T, temperature=T, seed=seed * 1000 + r,
                                     precision=precision))
    return specs, temps


def served_jobs(n_jobs: int = 64, rate_hz: float = 50.0, n_min: int = 64, n_max: int = 20000,
                moves_min: float = 1e4, moves_max: float = 1e6, seed: int = 4):
    """Poisson arrival stream of jobs mixing the three single-system shapes.
    Returns a list of dicts {arrival_s, spec, moves, shape}."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for j in range(n_jobs):
        t += rng.exponential(1.0 / rate_hz)
        shape = int(rng.integers(0, 3))
        N = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
        moves = int(math.exp(rng.uniform(math.log(moves_min), math.log(moves_max))))
        if shape == 0:
            N = max(2, N - N % 2)
            spec = primitive_model(n=N, L=50.0 * (N / 200.0) ** (1 / 3), seed=10_000 + j)
        elif shape == 1:
            ns = max(1, N // 2)
            spec = bulk_ewald(n_salt=ns, seed=20_000 + j)
        else:
            nm = max(256, N // 3)  # >= 256 waters: L >= 18.6 A keeps Rc and cutoff_g2g below L/2
            spec = spce_water(n_mol=nm, L=31.0 * (nm / 1000.0) ** (1 / 3), seed=30_000 + j)
        jobs.append({"arrival_s": t, "spec": spec, "moves": moves, "shape": shape, "id": j})
    return jobs
