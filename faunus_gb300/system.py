"""Python host API over the C ABI: a Faunus ``Space`` + ``Hamiltonian``
description (:class:`SystemSpec`), a GPU context, resident systems and the
reference-stream move generator.

Units follow the reference (src/units.h:10-45, :230-233): energies in kT,
lengths in angstrom, epsilon input in kJ/mol converted with the same
physical constants.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _capi as A

# PhysicalConstants (reference src/units.h:10-45)
ELEMENTARY_CHARGE = 1.602177e-19
VACUUM_PERMITTIVITY = 8.85419e-12
BOLTZMANN = 1.380658e-23
AVOGADRO = 6.022137e23
PI = float(np.pi)


def group_cutoff(value, molecule_names: Sequence[str]) -> np.ndarray:
    """GroupCutoff's mass-centre cutoff per molecule-kind pair from the reference's input
    forms (GroupCutoff from_json, src/energy.cpp:1868-1953; KAT src/energy.cpp:1955-2002):

      12.0                              every pair 12
      {"default": 13.0}                 every pair 13
      {"default": 13.0, "M Q": 14.0}    M-Q (both orders) 14, the rest 13
      {"M Q": 11.0}                     M-Q 11, the rest without cutoff (+inf)
    """
    n = len(molecule_names)
    index = {name: i for i, name in enumerate(molecule_names)}
    if isinstance(value, (int, float)):
        return np.full((n, n), float(value))
    out = np.full((n, n), float(value.get("default", np.inf)))
    for key, c in value.items():
        if key == "default":
            continue
        a, b = key.split()
        i, j = index[a], index[b]
        out[i, j] = out[j, i] = float(c)
    return out


def _poly_mul(a, b):
    out = [0.0] * (len(a) + len(b) - 1)
    for i, x in enumerate(a):
        for j, y in enumerate(b):
            out[i + j] += x * y
    return out


def _gbinom(n: int, k: int) -> float:
    """Generalised binomial coefficient n (n-1) ... (n-k+1) / k! (n may be negative)."""
    v = 1.0
    for i in range(k):
        v = v * (n - i) / (i + 1)
    return v


def coulomb_scheme(type: str, *, epsr: float, cutoff: float = 0.0, alpha: float = 0.0, epsrf: float = 0.0,
                   C: int = 3, D: int = 3, order: Optional[int] = None, temperature: float = 298.15) -> dict:
    """SystemSpec fields of a NewCoulombGalore `coulomb` block (src/potentials.cpp:1628-1700)
    at infinite Debye length: S(q = r/Rc) of docs/_docs/energy.md:169-213 written as
    e erfc(alpha r) + sum_k c_k q^k (FAU_COUL_TRUNC), or the plain / Ewald forms.

      plain          S = 1, no cutoff
      ewald          erfc(alpha Rc q)
      reactionfield  1 + (epsrf - epsr)/(2 epsrf + epsr) q^3 - 3 epsrf/(2 epsrf + epsr) q
      poisson        (1-q)^(D+1) sum_{c<C} (C-c)/C binom(D-1+c, c) q^c     (C=3, D=3)
      qpotential     prod_{n=1..order} (1 - q^n)
      fanourgakis    1 - 7/4 q + 21/4 q^5 - 7 q^6 + 5/2 q^7
      fennell        erfc(alpha Rc q) - q E + (q-1) q (E + G)
      zerodipole     erfc(alpha Rc q) - q E + (q^2-1)/2 q (E + G)
      zahn           erfc(alpha Rc q) - (q-1) q (E + G)
      wolf           erfc(alpha Rc q) - q E
    with E = erfc(alpha Rc), G = 2 alpha Rc / sqrt(pi) exp(-alpha^2 Rc^2).
    """
    import math

    lB = bjerrum_length(epsr, temperature)
    out = {"bjerrum_length": lB, "coulomb_cutoff": float(cutoff),
           "coulomb_alpha": float(alpha), "coulomb_erfc": 0.0, "coulomb_poly": None}
    if type == "plain":
        if cutoff:
            raise ValueError("unexpected cutoff for plain: it is always infinity")
        out.update(coulomb_type=A.FAU_COUL_PLAIN, coulomb_cutoff=0.0)
        return out
    if not cutoff > 0:
        raise ValueError(f"coulomb type '{type}' needs a cutoff")
    if type == "ewald":
        out.update(coulomb_type=A.FAU_COUL_EWALD)
        return out
    E = math.erfc(alpha * cutoff)
    G = 2 * alpha * cutoff / math.sqrt(math.pi) * math.exp(-(alpha * cutoff) ** 2)
    e = 0.0
    if type == "reactionfield":
        den = 2 * epsrf + epsr
        poly = [1.0, -3 * epsrf / den, 0.0, (epsrf - epsr) / den]
    elif type == "poisson":
        if C < 1 or D < -1:
            raise ValueError("poisson needs C >= 1 and D >= -1")
        head = [1.0]
        for _ in range(D + 1):
            head = _poly_mul(head, [1.0, -1.0])
        tail = [(C - c) / C * _gbinom(D - 1 + c, c) for c in range(C)]
        poly = _poly_mul(head, tail)
    elif type == "qpotential":
        if order is None or order < 1:
            raise ValueError("qpotential needs order >= 1")
        poly = [1.0]
        for n in range(1, order + 1):
            f = [0.0] * (n + 1)
            f[0], f[n] = 1.0, -1.0
            poly = _poly_mul(poly, f)
    elif type == "fanourgakis":
        poly = [1.0, -7 / 4, 0.0, 0.0, 0.0, 21 / 4, -7.0, 5 / 2]
    elif type == "fennell":
        e, poly = 1.0, [0.0, -E - (E + G), E + G]
    elif type == "zerodipole":
        e, poly = 1.0, [0.0, -E - 0.5 * (E + G), 0.0, 0.5 * (E + G)]
    elif type == "zahn":
        e, poly = 1.0, [0.0, E + G, -(E + G)]
    elif type == "wolf":
        e, poly = 1.0, [0.0, -E]
    else:
        raise ValueError(f"unknown coulomb type '{type}'")
    while len(poly) > 1 and poly[-1] == 0.0:
        poly.pop()
    if len(poly) > A.FAU_COUL_MAX_POLY:
        raise ValueError(f"S(q) has degree {len(poly) - 1} > {A.FAU_COUL_MAX_POLY - 1}")
    out.update(coulomb_type=A.FAU_COUL_TRUNC, coulomb_erfc=e, coulomb_poly=np.array(poly, dtype=np.float64))
    return out


def pressure_kt(value: float, unit: str, temperature: float = 298.15) -> float:
    """Isobaric pressure in kT / A^3 (Isobaric::pressure_units, src/energy.cpp:903-908;
    src/units.h:162-190: Pa / kT / 1 m^3, atm = 101325 Pa, bar = 1e5 Pa, mM = 1e-3 mol/l)."""
    kT = BOLTZMANN * temperature
    conv = {"P/kT": 1.0, "P/Pa": 1.0 / kT / 1e30, "P/atm": 101325.0 / kT / 1e30, "P/bar": 1e5 / kT / 1e30,
            "P/mM": 1e-3 * AVOGADRO / 1e27}
    if unit not in conv:
        raise ValueError(f"unknown pressure unit '{unit}'")
    return value * conv[unit]


def bjerrum_length(epsr: float, temperature: float = 298.15) -> float:
    """Bjerrum length in angstrom (pc::bjerrumLength, src/units.h:37-41)."""
    kT = temperature * BOLTZMANN
    return ELEMENTARY_CHARGE ** 2 / (4 * PI * VACUUM_PERMITTIVITY * epsr * 1e-10 * kT)


def kjmol_to_kt(x: float, temperature: float = 298.15) -> float:
    """operator""_kJmol (src/units.h:230-233): kJ/mol per particle in kT."""
    return x / (temperature * BOLTZMANN) / AVOGADRO * 1e3


def andrea_spline(f, zmin: float, zmax: float, utol: float, ftol: float = -1.0, cap: int = 1201):
    """Tabulate::Andrea::generate (src/tabulate.h:212-298) of a Python function f(z) on
    ]zmin, zmax] through fau_andrea_generate: (knots ascending, coefficients (pieces, 6))."""
    cb = A.SCALAR_FN(lambda z, _ctx: float(f(z)))
    z = np.zeros(cap)
    c = np.zeros(6 * cap)
    n = C.c_int()
    A.check(A.lib().fau_andrea_generate(cb, None, float(zmin), float(zmax), float(utol), float(ftol), cap,
                                        A.as_dptr(z), A.as_dptr(c), C.byref(n)), "fau_andrea_generate")
    m = n.value
    return z[:m].copy(), c[:6 * (m - 1)].reshape(m - 1, 6).copy()


def andrea_eval(knots: np.ndarray, coef: np.ndarray, z: float) -> float:
    """Andrea::eval (src/tabulate.h:188-207): Horner in z - z_i on the piece z_i < z <= z_{i+1}."""
    i = int(np.searchsorted(knots, z, side="left")) - 1
    i = min(max(i, 0), len(knots) - 2)
    dz = z - knots[i]
    s = 0.0
    for k in range(5, 0, -1):
        s = dz * (s + coef[i][k])
    return s + coef[i][0]


@dataclass
class SystemSpec:
    """Space + Hamiltonian of one system, as numpy arrays (see fau_sys_desc)."""

    box: np.ndarray                       # (3,)
    pos: np.ndarray                       # (N, 3) inside [-L/2, L/2]
    charge: np.ndarray                    # (N,)
    type: np.ndarray                      # (N,) int
    group_begin: np.ndarray               # (G+1,)
    group_flags: np.ndarray               # (G,)
    n_types: int
    sigma2: Optional[np.ndarray] = None   # (T, T)
    eps4: Optional[np.ndarray] = None     # (T, T) in kT
    hs_sigma2: Optional[np.ndarray] = None
    type_mass: Optional[np.ndarray] = None
    group_molid: Optional[np.ndarray] = None
    mass_center: Optional[np.ndarray] = None  # (G, 3)
    pair_terms: int = 0
    coulomb_type: int = A.FAU_COUL_PLAIN
    bjerrum_length: float = 0.0
    coulomb_cutoff: float = 0.0
    coulomb_alpha: float = 0.0
    coulomb_erfc: float = 0.0             # FAU_COUL_TRUNC: weight of erfc(alpha r) in S
    coulomb_poly: Optional[np.ndarray] = None  # FAU_COUL_TRUNC: c_k of S(q) = .. + sum c_k q^k
    pair_cutoff: float = 0.0
    cutoff_g2g: float = 0.0
    cutoff_g2g_pairs: Optional[np.ndarray] = None  # (n_molids, n_molids) per molecule-kind pair; see group_cutoff
    isobaric_pressure: Optional[float] = None  # Isobaric term's pressure (kT/A^3, see pressure_kt); None: no term
    maxenergy: Optional[float] = None     # Hamiltonian maxenergy (kT): terms summed up to the first >= it; None: +inf
    cell_staging: int = 0                 # pipelined kernel: 0 occupied slots of stencil cells, 1 whole cells,
                                          # 2 occupied slots when there are more particles than cells
    spline: Optional[dict] = None         # FAU_PAIR_SPLINE tables: begin (T*T+1), r2, coef, hs (see splined)
    ewald: Optional[dict] = None          # alpha, ncutoff, spherical_sum, epss
    precision: int = A.FAU_PREC_FP32C
    cell_capacity: int = 0
    temperature: float = 298.15
    name: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_groups(self) -> int:
        return int(self.group_flags.shape[0])

    def copy(self) -> "SystemSpec":
        import copy
        return copy.deepcopy(self)

    def to_desc(self):
        """Build a fau_sys_desc; returns (desc, keepalive) -- keep both alive."""
        keep = []

        def f64(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return A.as_dptr(a)

        def i32(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.int32)
            keep.append(a)
            return A.as_iptr(a)

        d = A.SysDesc()
        d.n_particles = self.n
        d.box = (C.c_double * 3)(*[float(x) for x in self.box])
        d.pos = f64(self.pos.reshape(-1))
        d.charge = f64(self.charge)
        d.type = i32(self.type)
        d.n_groups = self.n_groups
        d.group_begin = i32(self.group_begin)
        d.group_molid = i32(self.group_molid)
        d.group_flags = i32(self.group_flags)
        d.group_mass_center = f64(None if self.mass_center is None else self.mass_center.reshape(-1))
        d.n_types = int(self.n_types)
        d.type_mass = f64(self.type_mass)
        d.sigma2 = f64(None if self.sigma2 is None else self.sigma2.reshape(-1))
        d.eps4 = f64(None if self.eps4 is None else self.eps4.reshape(-1))
        d.hs_sigma2 = f64(None if self.hs_sigma2 is None else self.hs_sigma2.reshape(-1))
        d.pair_terms = int(self.pair_terms)
        d.coulomb_type = int(self.coulomb_type)
        d.bjerrum_length = float(self.bjerrum_length)
        d.coulomb_cutoff = float(self.coulomb_cutoff)
        d.coulomb_alpha = float(self.coulomb_alpha)
        d.coulomb_erfc = float(self.coulomb_erfc)
        if self.isobaric_pressure is not None:
            d.isobaric = 1
            d.pressure = float(self.isobaric_pressure)
        d.cell_staging = int(self.cell_staging)
        if self.maxenergy is not None and self.maxenergy != math.inf:
            d.maxenergy_set = 1
            d.maxenergy = float(self.maxenergy)
        if self.coulomb_poly is not None:
            cp = np.asarray(self.coulomb_poly, dtype=np.float64).reshape(-1)
            if len(cp) > A.FAU_COUL_MAX_POLY:
                raise ValueError("coulomb_poly has more than FAU_COUL_MAX_POLY coefficients")
            d.coulomb_poly_n = len(cp)
            for k, c in enumerate(cp):
                d.coulomb_poly[k] = float(c)
        d.pair_cutoff = float(self.pair_cutoff)
        d.cutoff_g2g = float(self.cutoff_g2g)
        if self.ewald:
            d.ewald.enabled = 1
            d.ewald.alpha = float(self.ewald["alpha"])
            d.ewald.ncutoff = float(self.ewald["ncutoff"])
            d.ewald.spherical_sum = int(self.ewald.get("spherical_sum", 1))
            d.ewald.epss = float(self.ewald.get("epss", 0.0))
        d.precision = int(self.precision)
        d.cell_capacity = int(self.cell_capacity)
        if self.cutoff_g2g_pairs is not None:
            m = np.asarray(self.cutoff_g2g_pairs, dtype=np.float64)
            if m.ndim != 2 or m.shape[0] != m.shape[1]:
                raise ValueError("cutoff_g2g_pairs must be a square matrix")
            d.n_molids = int(m.shape[0])
            d.cutoff_g2g_pairs = f64(m.reshape(-1))
        if self.spline is not None:
            d.spline_begin = i32(self.spline["begin"])
            d.spline_r2 = f64(self.spline["r2"])
            d.spline_coef = f64(self.spline["coef"])
            d.spline_hs = i32(self.spline.get("hs"))
        return d, keep


def splined(spec: "SystemSpec", type_charge, type_sigma, *, utol: float = 1e-3, ftol: float = 1e-2,
            u_at_rmin: float = 20.0, u_at_rmax: float = 1e-6, rmax: Optional[float] = None,
            hardsphere: bool = False) -> "SystemSpec":
    """nonbonded_splined: the spec's pair terms tabulated per atom-type pair as
    SplinedPotential::from_json does (src/potentials.cpp:1513-1553; the defaults are its own),
    through fau_spline_tabulate with the atom types' charges and sigmas (AtomData q, sigma).

    Returns a copy with FAU_PAIR_SPLINE and the tables.  Every pair is zero beyond its table's
    last knot, so pair_cutoff is set just beyond the longest table (the device's cell lists
    then follow the tables without changing any energy); a smaller positive pair_cutoff
    already in the spec is kept."""
    T = int(spec.n_types)
    base = spec.copy()
    base.spline = None
    base.pair_terms = int(base.pair_terms) & ~A.FAU_PAIR_SPLINE
    d, keep = base.to_desc()
    opts = A.SplineOpts(float(utol), float(ftol), float(u_at_rmin), float(u_at_rmax),
                        float(rmax) if rmax else 0.0, int(bool(hardsphere)), 0)
    cap = 1201
    tables = {}
    for a in range(T):
        for b in range(a + 1):
            z = np.zeros(cap)
            c = np.zeros(6 * cap)
            n, hs = C.c_int(), C.c_int()
            A.check(A.lib().fau_spline_tabulate(C.byref(d), a, b, float(type_charge[a]), float(type_charge[b]),
                                                0.5 * (float(type_sigma[a]) + float(type_sigma[b])), C.byref(opts),
                                                cap, A.as_dptr(z), A.as_dptr(c), C.byref(n), C.byref(hs)),
                    "fau_spline_tabulate")
            m = n.value
            tables[a, b] = tables[b, a] = (z[:m].copy(), c[:6 * (m - 1)].copy(), hs.value)
    begin, r2, coef, hsl = [0], [], [], []
    for a in range(T):
        for b in range(T):
            z, c, h = tables[a, b]
            begin.append(begin[-1] + len(z))
            r2.append(z)
            coef.append(c)
            hsl.append(h)
    out = base
    out.spline = {"begin": np.array(begin, np.int32), "r2": np.concatenate(r2), "coef": np.concatenate(coef),
                  "hs": np.array(hsl, np.int32)}
    out.pair_terms = int(out.pair_terms) | A.FAU_PAIR_SPLINE
    reach = math.sqrt(max(float(t[0][-1]) for t in tables.values())) * (1.0 + 1e-9)
    out.pair_cutoff = reach if not spec.pair_cutoff > 0 else min(float(spec.pair_cutoff), reach)
    return out


class Context:
    """One GPU, one stream, an optional HBM budget (bytes, 0 = unlimited)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._lib = A.lib()
        h = C.c_void_p()
        A.check(self._lib.fau_ctx_create(device, hbm_budget, C.byref(h)), "fau_ctx_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self._lib.fau_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def hbm_used(self) -> int:
        v = C.c_size_t()
        A.check(self._lib.fau_ctx_hbm_used(self.handle, C.byref(v)), "fau_ctx_hbm_used")
        return int(v.value)

    def create(self, spec: SystemSpec) -> "System":
        return System(self, spec)

    def run_batch(self, systems: Sequence["System"], moves=None, *, moves_per_system=None, seed: int = 1,
                  counter_base: int = 0, dp: float = 1.0, dprot: float = 0.0, swap_interval: int = 0,
                  n_swap_blocks: int = 0, temperatures=None, threads: int = 0, streams=None,
                  counters=None, dp_per_system=None, dprot_per_system=None, cycles_out=None,
                  sampler: Optional["Sampler"] = None, sample_slots=None, sample_interval: int = 0,
                  n_sample_blocks: int = 0, time_budget_s: Optional[float] = None, moves_out=None,
                  swap_log: bool = False, audit: bool = True, volume_interval: int = 0, n_volume_blocks: int = 0,
                  volume_dv: float = 0.0, volume_method: int = 0) -> dict:
        """Advance the systems with device proposals (fau_run_batch).  cycles_out, if given,
        is a uint64 array of len(systems) that receives each system's SM cycles.  With a
        sampler, the systems are sampled on the device after every block of moves (the PT
        swap blocks, or n_sample_blocks blocks of sample_interval moves, or once at the end).
        time_budget_s: each chain ends at the first move boundary after that much time of its
        own (or after its move count); moves_out (int64, one entry a system) receives the
        moves each performed -- continue a chain at counter + moves done.  Under parallel
        tempering moves_per_system gives each walker's block length between swaps, and
        swap_log=True adds the record of every round to the result: "swap_slots"
        (n_swap_blocks, n) systems per temperature slot after each round, "swap_energy"
        (n_swap_blocks, n) each system's running energy when the round was decided.
        NPT: n_volume_blocks blocks of volume_interval moves per system, each followed by one
        VolumeMove per system with logarithmic displacement volume_dv and scaling volume_method
        (fau_volume_method); "volume_attempted" / "volume_accepted" count them."""
        n = len(systems)
        arr = (C.c_void_p * n)(*[s.handle for s in systems])
        p = A.BatchParams()
        p.moves = int(moves or 0)
        keep = []
        if moves_per_system is not None:
            m = np.ascontiguousarray(moves_per_system, dtype=np.int64)
            keep.append(m)
            p.moves_per_system = m.ctypes.data_as(C.POINTER(C.c_int64))
        p.seed = int(seed)
        p.counter_base = int(counter_base)
        p.dp = float(dp)
        p.dprot = float(dprot)
        p.swap_interval_moves = int(swap_interval)
        p.n_swap_blocks = int(n_swap_blocks)
        if temperatures is not None:
            t = np.ascontiguousarray(temperatures, dtype=np.float64)
            keep.append(t)
            p.temperatures = A.as_dptr(t)
        p.threads = int(threads)
        if streams is not None:
            sv = np.ascontiguousarray(streams, dtype=np.uint32)
            keep.append(sv)
            p.streams = sv.ctypes.data_as(C.POINTER(C.c_uint32))
        for name, arr_ in (("dp_per_system", dp_per_system), ("dprot_per_system", dprot_per_system)):
            if arr_ is not None:
                v = np.ascontiguousarray(arr_, dtype=np.float64)
                keep.append(v)
                setattr(p, name, A.as_dptr(v))
        if cycles_out is not None:
            if cycles_out.dtype != np.uint64 or not cycles_out.flags.c_contiguous or len(cycles_out) != n:
                raise ValueError("cycles_out must be a contiguous uint64 array with one entry per system")
            p.cycles_out = cycles_out.ctypes.data_as(C.POINTER(C.c_uint64))
        if counters is not None:
            cv = np.ascontiguousarray(counters, dtype=np.uint64)
            keep.append(cv)
            p.counters = cv.ctypes.data_as(C.POINTER(C.c_uint64))
        if sampler is not None:
            p.sampler = sampler.handle
            p.sample_interval_moves = int(sample_interval)
            p.n_sample_blocks = int(n_sample_blocks)
            if sample_slots is not None:
                sl = np.ascontiguousarray(sample_slots, dtype=np.int32)
                keep.append(sl)
                p.sample_slots = A.as_iptr(sl)
        if time_budget_s is not None:
            if not time_budget_s > 0:
                raise ValueError("time_budget_s must be positive")
            p.time_budget_ns = int(time_budget_s * 1e9)
        if moves_out is not None:
            if moves_out.dtype != np.int64 or not moves_out.flags.c_contiguous or len(moves_out) != n:
                raise ValueError("moves_out must be a contiguous int64 array with one entry per system")
            p.moves_out = moves_out.ctypes.data_as(C.POINTER(C.c_int64))
        p.no_audit = 0 if audit else 1
        p.volume_interval_moves = int(volume_interval)
        p.n_volume_blocks = int(n_volume_blocks)
        p.volume_dv = float(volume_dv)
        p.volume_method = int(volume_method)
        log = None
        if swap_log and n_swap_blocks > 0:
            log = (np.zeros((n_swap_blocks, n), np.int32), np.zeros((n_swap_blocks, n)))
            p.swap_slots_out = A.as_iptr(log[0])
            p.swap_energy_out = A.as_dptr(log[1])
        st = A.BatchStats()
        A.check(self._lib.fau_run_batch(self.handle, arr, n, C.byref(p), C.byref(st)), "fau_run_batch")
        out = st.as_dict()
        if log is not None:
            out["swap_slots"], out["swap_energy"] = log
        return out


    def run_proposals_batch(self, systems: Sequence["System"], props: np.ndarray, offsets: np.ndarray,
                            acc_out: Optional[np.ndarray] = None, du_out: Optional[np.ndarray] = None) -> dict:
        """Host-fed proposals for many systems in one launch; props/acc_out/du_out
        may live in pinned host memory (any C-contiguous buffers work)."""
        n = len(systems)
        arr = (C.c_void_p * n)(*[s.handle for s in systems])
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        st = A.BatchStats()
        A.check(self._lib.fau_run_proposals_batch(
            self.handle, arr, n, props.ctypes.data, off.ctypes.data_as(C.POINTER(C.c_int64)),
            acc_out.ctypes.data if acc_out is not None else None,
            A.as_dptr(du_out) if du_out is not None else None, C.byref(st)), "fau_run_proposals_batch")
        return st.as_dict()

    def fp32_peak_tflops(self) -> float:
        v = C.c_double()
        A.check(self._lib.fau_measure_fp32_peak(self.handle, C.byref(v)), "fau_measure_fp32_peak")
        return float(v.value)


def footprint(spec: SystemSpec) -> int:
    d, keep = spec.to_desc()
    v = C.c_size_t()
    A.check(A.lib().fau_sys_footprint(C.byref(d), C.byref(v)), "fau_sys_footprint")
    return int(v.value)


class System:
    """A Space + Hamiltonian resident on the device."""

    def __init__(self, ctx: Context, spec: SystemSpec):
        self._lib = A.lib()
        self.ctx = ctx
        self.spec = spec
        d, keep = spec.to_desc()
        h = C.c_void_p()
        A.check(self._lib.fau_sys_create(ctx.handle, C.byref(d), C.byref(h)), "fau_sys_create")
        self.handle = h
        k = C.c_int()
        A.check(self._lib.fau_sys_num_kvectors(h, C.byref(k)), "fau_sys_num_kvectors")
        self.K = int(k.value)

    def close(self) -> None:
        if self.handle:
            self._lib.fau_sys_destroy(self.handle)
            self.handle = None

    def clone(self) -> "System":
        """Device-to-device deep copy (same context)."""
        h = C.c_void_p()
        A.check(self._lib.fau_sys_clone(self.handle, C.byref(h)), "fau_sys_clone")
        other = System.__new__(System)
        other._lib, other.ctx, other.spec, other.handle, other.K = self._lib, self.ctx, self.spec, h, self.K
        return other

    def energy_total(self) -> dict:
        t = A.EnergyTerms()
        A.check(self._lib.fau_energy_total(self.handle, C.byref(t)), "fau_energy_total")
        return t.as_dict()

    def trial_atomic(self, particle: int, dr, u: float) -> dict:
        r = A.TrialResult()
        drv = (C.c_double * 3)(*map(float, dr))
        A.check(self._lib.fau_trial_atomic(self.handle, int(particle), drv, float(u), C.byref(r)), "fau_trial_atomic")
        return r.as_dict()

    def trial_group(self, group: int, dr, quat, u: float) -> dict:
        r = A.TrialResult()
        drv = (C.c_double * 3)(*map(float, dr))
        q = (C.c_double * 4)(*map(float, quat))
        A.check(self._lib.fau_trial_group(self.handle, int(group), drv, q, float(u), C.byref(r)), "fau_trial_group")
        return r.as_dict()

    def energy_change(self, proposal) -> dict:
        """Evaluate one trial (kept pending on the device); see commit()."""
        p = A.Proposal()
        p.kind = int(proposal["kind"])
        p.index = int(proposal["index"])
        p.dr = (C.c_double * 3)(*map(float, proposal["dr"]))
        p.quat = (C.c_double * 4)(*map(float, proposal["quat"]))
        p.u = float(proposal["u"])
        r = A.TrialResult()
        A.check(self._lib.fau_energy_change(self.handle, C.byref(p), C.byref(r)), "fau_energy_change")
        return r.as_dict()

    def commit(self, accept: bool) -> None:
        A.check(self._lib.fau_commit_pending(self.handle, 1 if accept else 0), "fau_commit_pending")

    def run_proposals(self, props: np.ndarray, want_acc: bool = True, want_du: bool = True):
        props = np.ascontiguousarray(props, dtype=A.PROPOSAL_DTYPE)
        n = len(props)
        acc = np.zeros(n, dtype=np.uint8) if want_acc else None
        du = np.zeros(n, dtype=np.float64) if want_du else None
        st = A.RunStats()
        A.check(self._lib.fau_run_proposals(self.handle, props.ctypes.data, n,
                                            acc.ctypes.data if acc is not None else None,
                                            A.as_dptr(du) if du is not None else None, C.byref(st)),
                "fau_run_proposals")
        return acc, du, st.as_dict()

    def positions(self) -> np.ndarray:
        out = np.zeros((self.spec.n, 3), dtype=np.float64)
        A.check(self._lib.fau_get_positions(self.handle, A.as_dptr(out)), "fau_get_positions")
        return out

    def mass_centers(self) -> np.ndarray:
        out = np.zeros((self.spec.n_groups, 3), dtype=np.float64)
        A.check(self._lib.fau_get_mass_centers(self.handle, A.as_dptr(out)), "fau_get_mass_centers")
        return out

    def cells(self) -> np.ndarray:
        out = np.zeros(self.spec.n, dtype=np.int32)
        A.check(self._lib.fau_get_cells(self.handle, A.as_iptr(out)), "fau_get_cells")
        return out

    def cell_grid(self) -> tuple:
        out = np.zeros(3, dtype=np.int32)
        A.check(self._lib.fau_get_cell_grid(self.handle, A.as_iptr(out)), "fau_get_cell_grid")
        return tuple(int(x) for x in out)

    def running_energy(self) -> float:
        v = C.c_double()
        A.check(self._lib.fau_get_running_energy(self.handle, C.byref(v)), "fau_get_running_energy")
        return float(v.value)

    def counters(self) -> dict:
        """Moves, accepted moves, pair evaluations and k-vector updates since creation."""
        v = (C.c_int64 * 4)()
        A.check(self._lib.fau_get_counters(self.handle, v), "fau_get_counters")
        return {"moves": int(v[0]), "accepted": int(v[1]), "pair_evals": int(v[2]), "k_updates": int(v[3])}

    def accepted_moves(self) -> int:
        return self.counters()["accepted"]

    def refresh_energy(self) -> float:
        """Make the FP64 total energy the running energy (fau_refresh_energy)."""
        v = C.c_double()
        A.check(self._lib.fau_refresh_energy(self.handle, C.byref(v)), "fau_refresh_energy")
        return float(v.value)

    def box(self) -> np.ndarray:
        out = np.zeros(3)
        A.check(self._lib.fau_get_box(self.handle, A.as_dptr(out)), "fau_get_box")
        return out

    def volume_move(self, new_volume: float, u: float, method: str = "isotropic") -> dict:
        """One VolumeMove to `new_volume` with Metropolis uniform `u` (fau_volume_move); the
        Isobaric term is the spec's (`isobaric_pressure`)."""
        r = A.TrialResult()
        A.check(self._lib.fau_volume_move(self.handle, float(new_volume), VOLUME_METHODS[method], float(u),
                                          C.byref(r)), "fau_volume_move")
        return r.as_dict()

    def set_temperature_scale(self, scale: float) -> None:
        A.check(self._lib.fau_set_temperature_scale(self.handle, float(scale)), "fau_set_temperature_scale")

    def q(self) -> np.ndarray:
        out = np.zeros(2 * max(self.K, 1), dtype=np.float64)
        A.check(self._lib.fau_get_q(self.handle, A.as_dptr(out)), "fau_get_q")
        return out[: 2 * self.K].view(np.complex128)

    def save_state(self) -> bytes:
        """The exact device state (fau_sys_save_state): load it into a system made from the same
        spec with the saved box, and its chains continue bit for bit."""
        n = C.c_size_t()
        A.check(self._lib.fau_sys_state_size(self.handle, C.byref(n)), "fau_sys_state_size")
        buf = (C.c_char * n.value)()
        A.check(self._lib.fau_sys_save_state(self.handle, buf, n.value), "fau_sys_save_state")
        return bytes(buf)

    def load_state(self, blob: bytes) -> None:
        buf = C.create_string_buffer(blob, len(blob))
        A.check(self._lib.fau_sys_load_state(self.handle, buf, len(blob)), "fau_sys_load_state")

    def audit(self) -> dict:
        """The pipelined kernel's audit of this system (fau_get_audit): the largest error of its FP32
        energy changes against FP64 re-evaluations of its probe moves."""
        e = np.zeros(2)
        n = C.c_int64()
        A.check(self._lib.fau_get_audit(self.handle, A.as_dptr(e), C.byref(n)), "fau_get_audit")
        return {"rel_scaled_max": float(e[0]), "rel_du_max": float(e[1]), "samples": int(n.value)}

    def kvectors(self):
        """The resident k-vector table: ((K, 3) wavevectors (2 pi)(n / L), (K,) A_k)."""
        kv = np.zeros((max(self.K, 1), 3))
        ak = np.zeros(max(self.K, 1))
        A.check(self._lib.fau_get_kvectors(self.handle, None, A.as_dptr(kv), A.as_dptr(ak)), "fau_get_kvectors")
        return kv[: self.K], ak[: self.K]

    def q_rebuild(self) -> float:
        v = C.c_double()
        A.check(self._lib.fau_q_rebuild(self.handle, C.byref(v)), "fau_q_rebuild")
        return float(v.value)


VOLUME_METHODS = {"isotropic": A.FAU_VOLUME_ISOTROPIC, "xy": A.FAU_VOLUME_XY, "z": A.FAU_VOLUME_Z,
                  "isochoric": A.FAU_VOLUME_ISOCHORIC}


def move_descs(spec: SystemSpec, moves: Sequence[dict]):
    """fau_move_desc array from dicts {kind, repeat, dp, dprot, dir, groups, type_dp, type_dprot};
    a volume move is {kind: FAU_MOVE_VOLUME, repeat, dV, method}."""
    keep = []
    arr = (A.MoveDesc * len(moves))()
    for i, m in enumerate(moves):
        if int(m["kind"]) == A.FAU_MOVE_VOLUME:
            arr[i].kind = A.FAU_MOVE_VOLUME
            arr[i].repeat = float(m.get("repeat", 1.0))
            arr[i].dp = float(m["dV"])
            arr[i].volume_method = VOLUME_METHODS[m.get("method", "isotropic")]
            continue
        g = np.ascontiguousarray(m["groups"], dtype=np.int32)
        keep.append(g)
        arr[i].kind = int(m["kind"])
        arr[i].repeat = float(m["repeat"])
        arr[i].dp = float(m.get("dp", 0.0))
        arr[i].dprot = float(m.get("dprot", 0.0))
        arr[i].dir = (C.c_double * 3)(*m.get("dir", (1.0, 1.0, 1.0)))
        arr[i].n_groups = len(g)
        arr[i].groups = A.as_iptr(g)
        for key in ("type_dp", "type_dprot"):
            if m.get(key) is not None:
                t = np.ascontiguousarray(m[key], dtype=np.float64)
                keep.append(t)
                setattr(arr[i], key, A.as_dptr(t))
    return arr, keep


class MoveGenerator:
    """Proposals drawn in the reference's RNG order (fau_movegen_*)."""

    def __init__(self, spec: SystemSpec, moves: Sequence[dict], slump_seed: int = 0, random_seed: int = 0,
                 default_seeds: bool = True):
        self._lib = A.lib()
        d, self._keep = spec.to_desc()
        arr, keep2 = move_descs(spec, moves)
        self._keep2 = (arr, keep2)
        h = C.c_void_p()
        A.check(self._lib.fau_movegen_create(C.byref(d), arr, len(moves), slump_seed, random_seed,
                                             1 if default_seeds else 0, C.byref(h)), "fau_movegen_create")
        self.handle = h

    def generate(self, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=A.PROPOSAL_DTYPE)
        A.check(self._lib.fau_movegen_generate(self.handle, out.ctypes.data, n), "fau_movegen_generate")
        return out

    def state(self) -> str:
        buf = C.create_string_buffer(1 << 16)
        A.check(self._lib.fau_movegen_get_state(self.handle, buf, len(buf)), "fau_movegen_get_state")
        return buf.value.decode()

    def set_state(self, s: str) -> None:
        A.check(self._lib.fau_movegen_set_state(self.handle, s.encode()), "fau_movegen_set_state")

    def close(self) -> None:
        if self.handle:
            self._lib.fau_movegen_destroy(self.handle)
            self.handle = None


class Sampler:
    """Device analysis accumulators (fau_sampler): AtomRDF between atom types a and b
    and SystemEnergy, per slot (src/analysis.cpp:339-357, 1556-1600)."""

    def __init__(self, ctx: Context, n_slots: int = 1, rdf: Optional[tuple] = None, energy: bool = True):
        """rdf = (type_a, type_b, dr, n_bins) or None."""
        self._lib = A.lib()
        d = A.SamplerDesc()
        d.n_slots = int(n_slots)
        if rdf is not None:
            d.rdf_type_a, d.rdf_type_b, d.rdf_dr, d.rdf_bins = int(rdf[0]), int(rdf[1]), float(rdf[2]), int(rdf[3])
        d.energy = int(bool(energy))
        self.desc = d
        h = C.c_void_p()
        A.check(self._lib.fau_sampler_create(ctx.handle, C.byref(d), C.byref(h)), "fau_sampler_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self._lib.fau_sampler_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self) -> None:
        A.check(self._lib.fau_sampler_reset(self.handle), "fau_sampler_reset")

    def sample(self, systems: Sequence["System"], slots=None) -> None:
        n = len(systems)
        arr = (C.c_void_p * n)(*[s.handle for s in systems])
        sl = None if slots is None else np.ascontiguousarray(slots, dtype=np.int32)
        A.check(self._lib.fau_sampler_sample(self.handle, arr, n, None if sl is None else A.as_iptr(sl)),
                "fau_sampler_sample")

    def read(self) -> dict:
        ns, nb = self.desc.n_slots, self.desc.rdf_bins
        hist = np.zeros((ns, nb + 1), dtype=np.uint64)
        vol, es, e2 = np.zeros(ns), np.zeros(ns), np.zeros(ns)
        nr, ne = np.zeros(ns, dtype=np.int64), np.zeros(ns, dtype=np.int64)
        A.check(self._lib.fau_sampler_read(self.handle, hist.ctypes.data if nb else None, A.as_dptr(vol),
                                           nr.ctypes.data, A.as_dptr(es), A.as_dptr(e2), ne.ctypes.data),
                "fau_sampler_read")
        return {"rdf_hist": hist[:, :nb], "rdf_beyond": hist[:, nb], "rdf_volume_sum": vol, "rdf_samples": nr,
                "energy_sum": es, "energy_sum2": e2, "energy_samples": ne}

    def g_of_r(self, data: Optional[dict] = None, slots=None):
        """(r, g) per PairFunction::_to_disk (src/analysis.cpp:724-737): r the bin's left
        edge i dr, g = N <V> / (4 pi r^2 dr sum N) over the selected slots (default all),
        bins with r = 0 omitted."""
        data = data or self.read()
        sel = slice(None) if slots is None else np.asarray(slots)
        return rdf_normalise(data["rdf_hist"][sel].sum(0), self.desc.rdf_dr,
                             data["rdf_volume_sum"][sel].sum() / max(1, int(data["rdf_samples"][sel].sum())))


def rdf_normalise(hist: np.ndarray, dr: float, mean_volume: float):
    """PairFunction::_to_disk: g(r_i) = N_i <V> / (4 pi r_i^2 dr sum_j N_j), r_i = i dr
    (Equidistant2DTable::from_bin), skipping r = 0 (zero volume element)."""
    hist = np.asarray(hist, dtype=np.float64)
    r = np.arange(len(hist)) / (1.0 / dr)
    total = hist.sum()
    keep = r > 0
    g = hist[keep] * mean_volume / (4.0 * np.pi * r[keep] ** 2 * dr * total)
    return r[keep], g
