"""The allocation-free nonbonded energy entry point.

Callers that own all device memory (a host engine with its own pool, or a loop
that must not stall on cudaMalloc/cudaFree) pass device buffers in and out;
the library's only scratch is a fixed file-scope device array.  This file is
collected last so that a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O

pytestmark = pytest.mark.gpu


def _args(spec, torch):
    dev = "cuda"
    keep = {
        "pos": torch.tensor(spec.pos.reshape(-1), dtype=torch.float64, device=dev),
        "charge": torch.tensor(spec.charge, dtype=torch.float64, device=dev),
        "type": torch.tensor(spec.type, dtype=torch.int32, device=dev),
    }
    T = spec.n_types
    for key in ("sigma2", "eps4", "hs_sigma2"):
        v = getattr(spec, key)
        keep[key] = torch.tensor((np.zeros((T, T)) if v is None else v).reshape(-1), dtype=torch.float64, device=dev)
    a = A.NonbondedArgs()
    a.n_particles = spec.n
    a.box = (C.c_double * 3)(*map(float, spec.box))
    for key in ("pos", "charge", "type", "sigma2", "eps4", "hs_sigma2"):
        setattr(a, key, keep[key].data_ptr())
    a.n_types = T
    a.pair_terms = spec.pair_terms
    a.coulomb_type = spec.coulomb_type
    a.bjerrum_length = spec.bjerrum_length
    a.coulomb_cutoff = spec.coulomb_cutoff
    a.coulomb_alpha = spec.coulomb_alpha
    a.pair_cutoff = spec.pair_cutoff
    return a, keep


def _call(a, out, stream=None):
    A.check(A.lib().fau_nonbonded_energy_noalloc(C.byref(a), C.c_void_p(out.data_ptr()),
                                                 C.c_void_p(stream) if stream else None),
            "fau_nonbonded_energy_noalloc")


def _plain_coulomb_wca():
    spec = configs.primitive_model(n=200, hs=False)
    spec.coulomb_type = A.FAU_COUL_PLAIN
    spec.pair_cutoff = 0.0
    return spec


CASES = {
    "cut_coulomb_wca_hs": lambda: configs.primitive_model(n=200),
    "ewald_real_space_lj": lambda: configs.bulk_ewald(n_salt=1000),
    "plain_coulomb_wca": _plain_coulomb_wca,
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_noalloc_energy_matches_system_entry_point(ctx, case):
    """Two calls in a row (they share the scratch array) against the system entry point's
    FP64 total and the oracle's nonbonded energy."""
    torch = pytest.importorskip("torch")
    spec = CASES[case]()
    ref = ctx.create(spec).energy_total()["nonbonded"]
    ref_o = O.OracleSystem(spec).energy_total()["nonbonded"]
    assert abs(ref - ref_o) <= 1e-9 * max(1.0, abs(ref_o))
    a, keep = _args(spec, torch)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        _call(a, out)
        torch.cuda.synchronize()
        e = float(out.item())
        assert abs(e - ref) <= 1e-9 * max(1.0, abs(ref)), (e, ref)
        assert abs(e - ref_o) <= 1e-9 * max(1.0, abs(ref_o)), (e, ref_o)


def test_noalloc_on_a_caller_stream_with_unwrapped_positions(ctx):
    """The caller's stream carries the work; positions shifted by whole box lengths (an engine
    that does not wrap) give the energy of the wrapped configuration."""
    torch = pytest.importorskip("torch")
    spec = configs.bulk_ewald(n_salt=1000, seed=3)
    ref_o = O.OracleSystem(spec).energy_total()["nonbonded"]
    shifted = spec.copy()
    rng = np.random.default_rng(1)
    shifted.pos = spec.pos + spec.box * rng.integers(-2, 3, size=spec.pos.shape)
    a, keep = _args(shifted, torch)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    s.synchronize()
    _call(a, out, s.cuda_stream)
    s.synchronize()
    e = float(out.item())
    assert abs(e - ref_o) <= 1e-9 * max(1.0, abs(ref_o)), (e, ref_o)


def test_noalloc_rejects_bad_settings(ctx):
    torch = pytest.importorskip("torch")
    spec = configs.primitive_model(n=200)
    a, keep = _args(spec, torch)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    a.coulomb_cutoff = 0.0
    assert A.lib().fau_nonbonded_energy_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), None) == A.FAU_ERR_ARG
    a.coulomb_cutoff = spec.coulomb_cutoff
    a.pair_cutoff = float("nan")
    assert A.lib().fau_nonbonded_energy_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), None) == A.FAU_ERR_ARG


def test_noalloc_rejects_sizes_beyond_the_scratch(ctx):
    torch = pytest.importorskip("torch")
    spec = configs.primitive_model(n=200)
    a, keep = _args(spec, torch)
    a.n_particles = A.FAU_NOALLOC_MAX_PARTICLES + 1
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = A.lib().fau_nonbonded_energy_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), None)
    assert rc == A.FAU_ERR_ARG
    assert b"65536" in A.lib().fau_last_error()
