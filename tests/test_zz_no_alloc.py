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


@pytest.mark.parametrize("make", [lambda: configs.primitive_model(n=200),
                                  lambda: configs.bulk_ewald(n_salt=1000)])
def test_noalloc_energy_matches_system_entry_point(ctx, make):
    torch = pytest.importorskip("torch")
    spec = make()
    ref = ctx.create(spec).energy_total()["nonbonded"]
    a, keep = _args(spec, torch)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    lib = A.lib()
    for _ in range(2):  # two calls in a row share the scratch array
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        A.check(lib.fau_nonbonded_energy_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), None),
                "fau_nonbonded_energy_noalloc")
        torch.cuda.synchronize()
        e = float(out.item())
        assert abs(e - ref) <= 1e-9 * max(1.0, abs(ref)), (e, ref)


def test_noalloc_rejects_sizes_beyond_the_scratch(ctx):
    torch = pytest.importorskip("torch")
    spec = configs.primitive_model(n=200)
    a, keep = _args(spec, torch)
    a.n_particles = A.FAU_NOALLOC_MAX_PARTICLES + 1
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = A.lib().fau_nonbonded_energy_noalloc(C.byref(a), C.c_void_p(out.data_ptr()), None)
    assert rc == A.FAU_ERR_ARG
    assert b"65536" in A.lib().fau_last_error()
