"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure only: the tests compare the product against the oracle; the product
path never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from faunus_gb300 import _capi as A

ROOT = Path(__file__).resolve().parent.parent
# FAU_ORACLE_LIB: another build of the same oracle (e.g. oracle/Makefile's sanitize target)
LIB = Path(os.environ.get("FAU_ORACLE_LIB", ROOT / "oracle" / "_build" / "liboracle.so"))
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        src = ROOT / "oracle" / "oracle.cpp"
        if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
            subprocess.run(["make", "-C", str(ROOT / "oracle")], check=True, capture_output=True)
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        sd = C.POINTER(A.SysDesc)
        sig = {
            "orc_sys_create": ([sd, C.POINTER(P)], C.c_int),
            "orc_sys_destroy": ([P], C.c_int),
            "orc_energy_total": ([P, C.POINTER(A.EnergyTerms)], C.c_int),
            "orc_trial_atomic": ([P, C.c_int, A.dptr, C.c_double, C.POINTER(A.TrialResult)], C.c_int),
            "orc_trial_group": ([P, C.c_int, A.dptr, A.dptr, C.c_double, C.POINTER(A.TrialResult)], C.c_int),
            "orc_run_proposals": ([P, P, C.c_int, P, A.dptr, C.POINTER(A.RunStats)], C.c_int),
            "orc_run_proposals_detail": ([P, P, C.c_int, P], C.c_int),
            "orc_get_positions": ([P, A.dptr], C.c_int),
            "orc_get_mass_centers": ([P, A.dptr], C.c_int),
            "orc_get_q": ([P, A.dptr], C.c_int),
            "orc_num_kvectors": ([P], C.c_int),
            "orc_kvectors": ([P, A.dptr, A.dptr], C.c_int),
            "orc_du_atomic": ([P, C.c_int, A.dptr, C.POINTER(A.TrialResult)], C.c_int),
            "orc_ewald_policy": ([C.c_int, A.dptr, A.dptr, A.dptr, C.c_double, C.c_double, C.c_int, C.c_double,
                                  C.c_double, C.c_int, A.dptr, A.iptr], C.c_int),
            "orc_pair_u": ([sd, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, A.dptr], C.c_int),
            "orc_get_box": ([P, A.dptr], C.c_int),
            "orc_volume_move": ([P, C.c_double, C.c_int, C.c_double, C.POINTER(A.TrialResult)], C.c_int),
            "orc_rdf": ([C.c_int, A.dptr, A.iptr, A.dptr, C.c_int, C.c_int, C.c_double, C.c_int, P], C.c_int),
            "orc_geometry": ([A.dptr, C.c_int, A.dptr, A.dptr, A.dptr, A.dptr, A.dptr], C.c_int),
            "orc_cell_bin": ([A.dptr, C.c_double, C.c_int, A.dptr, A.iptr, A.iptr, A.iptr, A.iptr], C.c_int),
            "orc_movegen_create": ([P, C.POINTER(A.MoveDesc), C.c_int, C.c_uint32, C.c_uint32, C.c_int,
                                    C.POINTER(P)], C.c_int),
            "orc_movegen_destroy": ([P], C.c_int),
            "orc_movegen_generate": ([P, P, C.c_int], C.c_int),
            "orc_mc_run": ([P, P, C.c_int, P, A.dptr, C.POINTER(A.RunStats)], C.c_int),
            "orc_bench_chains": ([sd, C.POINTER(A.MoveDesc), C.c_int, C.c_int, C.c_int, C.c_int, A.dptr, A.dptr],
                                 C.c_int),
            "orc_random_default_first": ([], C.c_double),
            "orc_random_state": ([C.c_uint32, C.c_int, C.c_char_p, C.c_size_t], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


# The two error denominators of a device energy change against the oracle's FP64 value:
#   rel_scaled = |dU_gpu - dU_fp64| / max(|dU|, S), S the sum of |summand| the change is summed
#                from (the tolerance's definition, <= 1e-6);
#   rel_du     = |dU_gpu - dU_fp64| / |dU| over moves with |dU| > 1e-3 kT: its median is held
#                to TOL_REL_DU_MEDIAN on the benchmark forms (bulk Ewald, primitive model) and
#                reported elsewhere; its maximum is reported (where the terms cancel, |dU| << S
#                and the FP32 rounding of the summands, bounded through S, dominates).
DU_FLOOR = 1e-3
TOL_REL_DU_MEDIAN = 1e-6


def du_errors(du_g, du_o, scale) -> dict:
    du_g, du_o, scale = np.asarray(du_g), np.asarray(du_o), np.asarray(scale)
    err = np.abs(du_g - du_o)
    den = np.maximum(np.abs(du_o), scale)
    rel_s = err / np.where(den > 0, den, 1.0)
    big = np.abs(du_o) > DU_FLOOR
    rel_d = err[big] / np.abs(du_o[big])
    return {"rel_scaled_max": float(rel_s.max(initial=0.0)), "rel_scaled_p99": float(np.quantile(rel_s, 0.99))
            if len(rel_s) else 0.0, "rel_du_max": float(rel_d.max(initial=0.0)),
            "rel_du_p99": float(np.quantile(rel_d, 0.99)) if len(rel_d) else 0.0,
            "rel_du_median": float(np.median(rel_d)) if len(rel_d) else 0.0,
            "moves_du_above_floor": int(big.sum())}


def _ok(rc: int, where: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{where}: oracle status {rc}")


class OracleSystem:
    """The CPU FP64 restatement of one Space + Hamiltonian."""

    def __init__(self, spec):
        self.spec = spec
        d, self._keep = spec.to_desc()
        h = C.c_void_p()
        _ok(lib().orc_sys_create(C.byref(d), C.byref(h)), "orc_sys_create")
        self.h = h

    def close(self):
        if self.h:
            lib().orc_sys_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def energy_total(self) -> dict:
        t = A.EnergyTerms()
        _ok(lib().orc_energy_total(self.h, C.byref(t)), "orc_energy_total")
        return t.as_dict()

    def volume_move(self, new_volume, method, u) -> dict:
        r = A.TrialResult()
        rc = lib().orc_volume_move(self.h, float(new_volume), int(method), float(u), C.byref(r))
        out = r.as_dict()
        out["status"] = rc
        return out

    def box(self) -> np.ndarray:
        b = np.zeros(3)
        _ok(lib().orc_get_box(self.h, A.as_dptr(b)), "orc_get_box")
        return b

    def trial_atomic(self, i, dr, u) -> dict:
        r = A.TrialResult()
        rc = lib().orc_trial_atomic(self.h, int(i), (C.c_double * 3)(*dr), float(u), C.byref(r))
        out = r.as_dict()
        out["status"] = rc
        return out

    def trial_group(self, g, dr, quat, u) -> dict:
        r = A.TrialResult()
        rc = lib().orc_trial_group(self.h, int(g), (C.c_double * 3)(*dr), (C.c_double * 4)(*quat), float(u),
                                   C.byref(r))
        out = r.as_dict()
        out["status"] = rc
        return out

    def du_atomic(self, i, dr) -> dict:
        r = A.TrialResult()
        _ok(lib().orc_du_atomic(self.h, int(i), (C.c_double * 3)(*dr), C.byref(r)), "orc_du_atomic")
        return r.as_dict()

    def run_proposals(self, props):
        props = np.ascontiguousarray(props, dtype=A.PROPOSAL_DTYPE)
        n = len(props)
        acc = np.zeros(n, dtype=np.uint8)
        du = np.zeros(n, dtype=np.float64)
        st = A.RunStats()
        _ok(lib().orc_run_proposals(self.h, props.ctypes.data, n, acc.ctypes.data, A.as_dptr(du), C.byref(st)),
            "orc_run_proposals")
        return acc, du, st.as_dict()

    def run_detail(self, props):
        props = np.ascontiguousarray(props, dtype=A.PROPOSAL_DTYPE)
        out = np.zeros(len(props), dtype=A.TRIAL_DTYPE)
        _ok(lib().orc_run_proposals_detail(self.h, props.ctypes.data, len(props), out.ctypes.data),
            "orc_run_proposals_detail")
        return out

    def positions(self):
        out = np.zeros((self.spec.n, 3))
        _ok(lib().orc_get_positions(self.h, A.as_dptr(out)), "orc_get_positions")
        return out

    def mass_centers(self):
        out = np.zeros((self.spec.n_groups, 3))
        _ok(lib().orc_get_mass_centers(self.h, A.as_dptr(out)), "orc_get_mass_centers")
        return out

    def q(self):
        K = lib().orc_num_kvectors(self.h)
        out = np.zeros(2 * max(K, 1))
        lib().orc_get_q(self.h, A.as_dptr(out))
        return out[: 2 * K].view(np.complex128)

    def kvectors(self):
        K = lib().orc_num_kvectors(self.h)
        kv = np.zeros((max(K, 1), 3))
        ak = np.zeros(max(K, 1))
        lib().orc_kvectors(self.h, A.as_dptr(kv), A.as_dptr(ak))
        return kv[:K], ak[:K]


class OracleMoveGen:
    def __init__(self, osys: OracleSystem, moves, slump_seed=0, random_seed=0, default_seeds=True):
        from faunus_gb300.system import move_descs
        arr, self._keep = move_descs(osys.spec, moves)
        self._arr = arr
        h = C.c_void_p()
        _ok(lib().orc_movegen_create(osys.h, arr, len(moves), slump_seed, random_seed, 1 if default_seeds else 0,
                                     C.byref(h)), "orc_movegen_create")
        self.h = h
        self.osys = osys

    def generate(self, n):
        out = np.zeros(n, dtype=A.PROPOSAL_DTYPE)
        _ok(lib().orc_movegen_generate(self.h, out.ctypes.data, n), "orc_movegen_generate")
        return out

    def mc_run(self, n):
        acc = np.zeros(n, dtype=np.uint8)
        du = np.zeros(n)
        st = A.RunStats()
        _ok(lib().orc_mc_run(self.osys.h, self.h, n, acc.ctypes.data, A.as_dptr(du), C.byref(st)), "orc_mc_run")
        return acc, du, st.as_dict()

    def close(self):
        if self.h:
            lib().orc_movegen_destroy(self.h)
            self.h = None


def ewald_policy(pos, q, box, alpha, ncut, spherical, epss, lB, ipbc):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64)
    out = np.zeros(3)
    nk = C.c_int()
    _ok(lib().orc_ewald_policy(len(q), A.as_dptr(pos), A.as_dptr(q), A.as_dptr(box), alpha, ncut, int(spherical),
                               epss, lB, int(ipbc), A.as_dptr(out), C.byref(nk)), "orc_ewald_policy")
    return {"self": out[0], "surface": out[1], "reciprocal": out[2], "K": nk.value}


def pair_u(spec, ta, tb, qa, qb, r2) -> float:
    d, keep = spec.to_desc()
    u = C.c_double()
    _ok(lib().orc_pair_u(C.byref(d), ta, tb, qa, qb, r2, C.byref(u)), "orc_pair_u")
    return u.value


def geometry(box, a, b):
    """(boundary(a), vdist(a, b), sqdist(a, b)) of the oracle's cuboid Chameleon, per row."""
    box = np.ascontiguousarray(box, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = len(a)
    aw, vd, sq = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
    _ok(lib().orc_geometry(A.as_dptr(box), n, A.as_dptr(a.reshape(-1)), A.as_dptr(b.reshape(-1)),
                           A.as_dptr(aw.reshape(-1)), A.as_dptr(vd.reshape(-1)), A.as_dptr(sq)), "orc_geometry")
    return aw, vd, sq


def rdf_hist(pos, types, box, ta, tb, dr, n_bins):
    """AtomRDF pair histogram of one configuration: (n_bins,) counts and the count beyond."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    types = np.ascontiguousarray(types, dtype=np.int32)
    box = np.ascontiguousarray(box, dtype=np.float64)
    h = np.zeros(n_bins + 1, dtype=np.uint64)
    _ok(lib().orc_rdf(len(pos), A.as_dptr(pos.reshape(-1)), A.as_iptr(types), A.as_dptr(box), ta, tb, dr, n_bins,
                      h.ctypes.data), "orc_rdf")
    return h[:n_bins], int(h[n_bins])


def cell_bin(box, min_cell, pos):
    box = np.ascontiguousarray(box, dtype=np.float64)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    n = len(pos)
    cells = np.zeros(n, dtype=np.int32)
    dims = np.zeros(3, dtype=np.int32)
    omin = np.zeros(3, dtype=np.int32)
    omax = np.zeros(3, dtype=np.int32)
    _ok(lib().orc_cell_bin(A.as_dptr(box), min_cell, n, A.as_dptr(pos.reshape(-1)), A.as_iptr(cells), A.as_iptr(dims),
                           A.as_iptr(omin), A.as_iptr(omax)), "orc_cell_bin")
    return cells, tuple(dims), tuple(omin), tuple(omax)
