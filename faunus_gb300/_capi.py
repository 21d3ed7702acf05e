"""ctypes mirror of ``include/fau_gpu.h`` and the loader of the CUDA library.

The product path goes through ``libfau_gpu.so`` only: if the library is
missing, :func:`lib` raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIBPATH = Path(__file__).resolve().parent / "_lib" / "libfau_gpu.so"

# status codes
FAU_OK = 0
FAU_ERR_ARG = 1
FAU_ERR_OOM = 2
FAU_ERR_CUDA = 3
FAU_ERR_TIMEOUT = 4
FAU_ERR_NAN = 5
FAU_ERR_CAPACITY = 6
FAU_ERR_STATE = 7
FAU_ERR_NODEVICE = 8

# pair terms / coulomb types / flags / precision / moves
FAU_PAIR_COULOMB, FAU_PAIR_LJ, FAU_PAIR_WCA, FAU_PAIR_HS, FAU_PAIR_SPLINE = 1, 2, 4, 8, 16
FAU_COUL_PLAIN, FAU_COUL_CUT, FAU_COUL_EWALD, FAU_COUL_TRUNC = 0, 1, 2, 3
FAU_COUL_MAX_POLY = 16
FAU_VOLUME_ISOTROPIC, FAU_VOLUME_XY, FAU_VOLUME_Z, FAU_VOLUME_ISOCHORIC = 0, 1, 2, 3
FAU_GROUP_ATOMIC, FAU_GROUP_RIGID = 1, 2
FAU_PREC_FP32C, FAU_PREC_FP64 = 0, 1
FAU_MOVE_NONE, FAU_MOVE_ATOMIC, FAU_MOVE_MOLECULAR, FAU_MOVE_VOLUME = -1, 0, 1, 2

dptr = C.POINTER(C.c_double)
iptr = C.POINTER(C.c_int)


class EwaldDesc(C.Structure):
    _fields_ = [("enabled", C.c_int), ("alpha", C.c_double), ("ncutoff", C.c_double),
                ("spherical_sum", C.c_int), ("epss", C.c_double)]


class SysDesc(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int), ("box", C.c_double * 3),
        ("pos", dptr), ("charge", dptr), ("type", iptr),
        ("n_groups", C.c_int), ("group_begin", iptr), ("group_molid", iptr), ("group_flags", iptr),
        ("group_mass_center", dptr),
        ("n_types", C.c_int), ("type_mass", dptr), ("sigma2", dptr), ("eps4", dptr), ("hs_sigma2", dptr),
        ("pair_terms", C.c_int), ("coulomb_type", C.c_int),
        ("bjerrum_length", C.c_double), ("coulomb_cutoff", C.c_double), ("coulomb_alpha", C.c_double),
        ("pair_cutoff", C.c_double), ("cutoff_g2g", C.c_double),
        ("ewald", EwaldDesc), ("precision", C.c_int), ("cell_capacity", C.c_int),
        ("n_molids", C.c_int), ("cutoff_g2g_pairs", dptr),
        ("coulomb_poly_n", C.c_int), ("coulomb_erfc", C.c_double), ("coulomb_poly", C.c_double * 16),
        ("isobaric", C.c_int), ("pressure", C.c_double),
        ("spline_begin", iptr), ("spline_r2", dptr), ("spline_coef", dptr), ("spline_hs", iptr),
        ("maxenergy_set", C.c_int), ("maxenergy", C.c_double), ("cell_staging", C.c_int),
    ]


class SplineOpts(C.Structure):
    _fields_ = [("utol", C.c_double), ("ftol", C.c_double), ("u_at_rmin", C.c_double), ("u_at_rmax", C.c_double),
                ("rmax_start", C.c_double), ("hardsphere", C.c_int), ("pad", C.c_int)]


SCALAR_FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


class EnergyTerms(C.Structure):
    _fields_ = [("self", C.c_double), ("nonbonded", C.c_double), ("ewald_rec", C.c_double),
                ("ewald_surf", C.c_double), ("total", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class TrialResult(C.Structure):
    _fields_ = [("du", C.c_double), ("du_nonbonded", C.c_double), ("du_ewald", C.c_double),
                ("err_scale", C.c_double), ("accepted", C.c_int), ("new_inf", C.c_int),
                ("old_inf", C.c_int), ("pad", C.c_int)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class Proposal(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int32), ("dr", C.c_double * 3),
                ("quat", C.c_double * 4), ("u", C.c_double)]


PROPOSAL_DTYPE = np.dtype([("kind", "<i4"), ("index", "<i4"), ("dr", "<f8", (3,)),
                           ("quat", "<f8", (4,)), ("u", "<f8")])
assert PROPOSAL_DTYPE.itemsize == C.sizeof(Proposal) == 72

TRIAL_DTYPE = np.dtype([("du", "<f8"), ("du_nonbonded", "<f8"), ("du_ewald", "<f8"), ("err_scale", "<f8"),
                        ("accepted", "<i4"), ("new_inf", "<i4"), ("old_inf", "<i4"), ("pad", "<i4")])
assert TRIAL_DTYPE.itemsize == C.sizeof(TrialResult)


class RunStats(C.Structure):
    _fields_ = [("moves", C.c_int64), ("accepted", C.c_int64), ("pair_evals", C.c_int64),
                ("k_updates", C.c_int64), ("energy_change", C.c_double), ("energy", C.c_double),
                ("max_rel_err", C.c_double), ("device_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class BatchParams(C.Structure):
    _fields_ = [("moves", C.c_int64), ("moves_per_system", C.POINTER(C.c_int64)), ("seed", C.c_uint64),
                ("counter_base", C.c_uint64), ("dp", C.c_double), ("dprot", C.c_double),
                ("swap_interval_moves", C.c_int), ("n_swap_blocks", C.c_int),
                ("temperatures", dptr), ("threads", C.c_int), ("streams", C.POINTER(C.c_uint32)),
                ("counters", C.POINTER(C.c_uint64)), ("dp_per_system", dptr), ("dprot_per_system", dptr),
                ("cycles_out", C.POINTER(C.c_uint64)), ("sampler", C.c_void_p),
                ("sample_slots", iptr), ("sample_interval_moves", C.c_int), ("n_sample_blocks", C.c_int),
                ("time_budget_ns", C.c_uint64), ("moves_out", C.POINTER(C.c_int64)),
                ("swap_slots_out", iptr), ("swap_energy_out", dptr), ("no_audit", C.c_int),
                ("volume_interval_moves", C.c_int), ("n_volume_blocks", C.c_int), ("volume_dv", C.c_double),
                ("volume_method", C.c_int)]


class SamplerDesc(C.Structure):
    _fields_ = [("n_slots", C.c_int), ("rdf_type_a", C.c_int), ("rdf_type_b", C.c_int), ("rdf_dr", C.c_double),
                ("rdf_bins", C.c_int), ("energy", C.c_int)]


FAU_SAMPLER_MAX_BINS = 12000


class BatchStats(C.Structure):
    _fields_ = [("moves", C.c_int64), ("accepted", C.c_int64), ("pair_evals", C.c_int64),
                ("k_updates", C.c_int64), ("swaps_attempted", C.c_int64), ("swaps_accepted", C.c_int64),
                ("device_ms", C.c_double), ("du_err_scaled_max", C.c_double), ("du_err_rel_max", C.c_double),
                ("du_err_samples", C.c_int64), ("volume_attempted", C.c_int64), ("volume_accepted", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class MoveDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("repeat", C.c_double), ("dp", C.c_double), ("dprot", C.c_double),
                ("dir", C.c_double * 3), ("n_groups", C.c_int), ("groups", iptr),
                ("type_dp", dptr), ("type_dprot", dptr), ("volume_method", C.c_int)]


FAU_NOALLOC_MAX_PARTICLES = 65536


class NonbondedArgs(C.Structure):
    """fau_nonbonded_args: device pointers (as integers) for the allocation-free entry point."""
    _fields_ = [("n_particles", C.c_int), ("box", C.c_double * 3), ("pos", C.c_void_p), ("charge", C.c_void_p),
                ("type", C.c_void_p), ("n_types", C.c_int), ("sigma2", C.c_void_p), ("eps4", C.c_void_p),
                ("hs_sigma2", C.c_void_p), ("pair_terms", C.c_int), ("coulomb_type", C.c_int),
                ("bjerrum_length", C.c_double), ("coulomb_cutoff", C.c_double), ("coulomb_alpha", C.c_double),
                ("pair_cutoff", C.c_double)]


class FauError(RuntimeError):
    """A non-zero status returned by the C ABI."""

    def __init__(self, status: int, where: str, detail: str):
        self.status = status
        super().__init__(f"{where}: status {status} ({detail})")


_LIB = None


def _declare(lib: C.CDLL) -> None:
    P = C.c_void_p
    sig = {
        "fau_abi_version": ([], C.c_int),
        "fau_strerror": ([C.c_int], C.c_char_p),
        "fau_last_error": ([], C.c_char_p),
        "fau_ctx_create": ([C.c_int, C.c_size_t, C.POINTER(P)], C.c_int),
        "fau_ctx_destroy": ([P], C.c_int),
        "fau_ctx_hbm_used": ([P, C.POINTER(C.c_size_t)], C.c_int),
        "fau_sys_footprint": ([C.POINTER(SysDesc), C.POINTER(C.c_size_t)], C.c_int),
        "fau_sys_create": ([P, C.POINTER(SysDesc), C.POINTER(P)], C.c_int),
        "fau_sys_destroy": ([P], C.c_int),
        "fau_sys_clone": ([P, C.POINTER(P)], C.c_int),
        "fau_sys_num_kvectors": ([P, iptr], C.c_int),
        "fau_energy_total": ([P, C.POINTER(EnergyTerms)], C.c_int),
        "fau_trial_atomic": ([P, C.c_int, dptr, C.c_double, C.POINTER(TrialResult)], C.c_int),
        "fau_trial_group": ([P, C.c_int, dptr, dptr, C.c_double, C.POINTER(TrialResult)], C.c_int),
        "fau_run_proposals": ([P, P, C.c_int, P, dptr, C.POINTER(RunStats)], C.c_int),
        "fau_energy_change": ([P, C.POINTER(Proposal), C.POINTER(TrialResult)], C.c_int),
        "fau_commit_pending": ([P, C.c_int], C.c_int),
        "fau_run_batch": ([P, C.POINTER(P), C.c_int, C.POINTER(BatchParams), C.POINTER(BatchStats)], C.c_int),
        "fau_run_proposals_batch": ([P, C.POINTER(P), C.c_int, P, C.POINTER(C.c_int64), P, dptr,
                                     C.POINTER(BatchStats)], C.c_int),
        "fau_measure_fp32_peak": ([P, dptr], C.c_int),
        "fau_nonbonded_energy_noalloc": ([C.POINTER(NonbondedArgs), C.c_void_p, C.c_void_p], C.c_int),
        "fau_get_positions": ([P, dptr], C.c_int),
        "fau_get_mass_centers": ([P, dptr], C.c_int),
        "fau_get_cells": ([P, iptr], C.c_int),
        "fau_get_cell_grid": ([P, iptr], C.c_int),
        "fau_get_running_energy": ([P, dptr], C.c_int),
        "fau_get_counters": ([P, C.POINTER(C.c_int64)], C.c_int),
        "fau_get_box": ([P, dptr], C.c_int),
        "fau_refresh_energy": ([P, dptr], C.c_int),
        "fau_volume_move": ([P, C.c_double, C.c_int, C.c_double, C.POINTER(TrialResult)], C.c_int),
        "fau_sampler_create": ([P, C.POINTER(SamplerDesc), C.POINTER(P)], C.c_int),
        "fau_sampler_destroy": ([P], C.c_int),
        "fau_sampler_reset": ([P], C.c_int),
        "fau_sampler_sample": ([P, C.POINTER(P), C.c_int, iptr], C.c_int),
        "fau_sampler_read": ([P, P, dptr, P, dptr, dptr, P], C.c_int),
        "fau_set_temperature_scale": ([P, C.c_double], C.c_int),
        "fau_q_rebuild": ([P, dptr], C.c_int),
        "fau_get_q": ([P, dptr], C.c_int),
        "fau_get_kvectors": ([P, iptr, dptr, dptr], C.c_int),
        "fau_get_audit": ([P, dptr, C.POINTER(C.c_int64)], C.c_int),
        "fau_sys_state_size": ([P, C.POINTER(C.c_size_t)], C.c_int),
        "fau_sys_save_state": ([P, P, C.c_size_t], C.c_int),
        "fau_sys_load_state": ([P, P, C.c_size_t], C.c_int),
        "fau_movegen_create": ([C.POINTER(SysDesc), C.POINTER(MoveDesc), C.c_int, C.c_uint32, C.c_uint32, C.c_int,
                                C.POINTER(P)], C.c_int),
        "fau_movegen_destroy": ([P], C.c_int),
        "fau_andrea_generate": ([SCALAR_FN, P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, dptr, dptr,
                                 iptr], C.c_int),
        "fau_spline_tabulate": ([C.POINTER(SysDesc), C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                 C.POINTER(SplineOpts), C.c_int, dptr, dptr, iptr, iptr], C.c_int),
        "fau_movegen_generate": ([P, P, C.c_int], C.c_int),
        "fau_movegen_get_state": ([P, C.c_char_p, C.c_size_t], C.c_int),
        "fau_movegen_set_state": ([P, C.c_char_p], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res


def lib() -> C.CDLL:
    """Load ``libfau_gpu.so`` (built by ``__graft_entry__.build()``)."""
    global _LIB
    if _LIB is None:
        path = Path(os.environ.get("FAU_GPU_LIB", LIBPATH))
        if not path.exists():
            raise RuntimeError(f"{path} not found: build the CUDA library first (__graft_entry__.build())")
        _LIB = C.CDLL(str(path))
        _declare(_LIB)
    return _LIB


def check(status: int, where: str) -> None:
    if status != FAU_OK:
        L = lib()
        detail = (L.fau_last_error() or b"").decode() or L.fau_strerror(status).decode()
        raise FauError(status, where, detail)


def as_dptr(a: np.ndarray):
    return a.ctypes.data_as(dptr)


def as_iptr(a: np.ndarray):
    return a.ctypes.data_as(iptr)
