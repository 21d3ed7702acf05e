"""The compiled C++ host adaptor (faunus_gb300/adaptor/fau_faunus.hpp).

tests/adaptor/adaptor_driver.cpp runs MetropolisMonteCarlo::performMove's loop
(reference src/montecarlo.cpp:139-187) with the adaptor's EnergyTerm in an accepted and a
trial Hamiltonian and its reference-stream Move.  Without a GPU it must compile against the
header and link against the library; on the GPU its accept sequence and energy changes must
equal the FP64 oracle's on the same proposals (to the parity tolerance, except at near ties).
"""
import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs
from faunus_gb300.system import move_descs

import oracle_lib as O

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "adaptor" / "adaptor_driver.cpp"


def build_driver(out_dir: Path) -> Path:
    A.lib()  # the library the driver links against
    libdir = Path(A.LIBPATH).parent
    out = out_dir / "libadaptor_driver.so"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-shared", "-fPIC", "-I", str(ROOT / "include"),
           "-I", str(ROOT / "faunus_gb300" / "adaptor"), str(SRC), "-o", str(out), "-L", str(libdir), "-lfau_gpu",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_adaptor_compiles_and_links(tmp_path):
    so = build_driver(tmp_path)
    nm = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True).stdout
    assert " adaptor_run" in nm


def _run(so: Path, spec, n, seeds=(17, 19), maxenergy=math.inf):
    lib = C.CDLL(str(so))
    lib.adaptor_run.restype = C.c_int
    d, keep = spec.to_desc()
    arr, keep2 = move_descs(spec, spec.extra["moves"])
    acc = np.zeros(n, np.uint8)
    du = np.zeros(n)
    en = np.zeros(2)
    err = C.create_string_buffer(512)
    rc = lib.adaptor_run(C.byref(d), arr, C.c_int(len(spec.extra["moves"])), C.c_uint32(seeds[0]),
                         C.c_uint32(seeds[1]), C.c_double(maxenergy), C.c_int(n), acc.ctypes.data_as(C.c_void_p),
                         du.ctypes.data_as(C.c_void_p), en.ctypes.data_as(C.c_void_p), err, C.c_int(512))
    assert rc == 0, err.value.decode()
    return acc, du, en


@pytest.mark.gpu
@pytest.mark.parametrize("make,n", [(lambda: configs.bulk_ewald(n_salt=1000, seed=4), 3000),
                                    (lambda: configs.primitive_model(n=200, seed=2), 5000),
                                    (lambda: configs.spce_water(n_mol=256, L=18.6, seed=3), 1500)])
def test_adaptor_loop_matches_oracle(ctx, tmp_path, make, n):
    spec = make()
    so = build_driver(tmp_path)
    acc, du, en = _run(so, spec, n)
    props = F.MoveGenerator(spec, spec.extra["moves"], 17, 19, default_seeds=False).generate(n)
    det = O.OracleSystem(spec).run_detail(props)
    acc_o, du_o, scale = det["accepted"].astype(np.uint8), det["du"], det["err_scale"]
    mism = np.nonzero(acc != acc_o)[0]
    first = int(mism[0]) if len(mism) else n
    sl = slice(0, first + 1 if first < n else first)
    moved = props["kind"][sl] != A.FAU_MOVE_NONE
    fin = np.isfinite(du_o[sl]) & moved
    assert np.array_equal(np.isfinite(du[sl]) | ~moved, np.isfinite(du_o[sl]) | ~moved)
    rep = O.du_errors(du[sl][fin], du_o[sl][fin], scale[sl][fin])
    print(f"PARITY adaptor {spec.name} moves={n} " + " ".join(f"{k}={v}" for k, v in rep.items()))
    assert rep["rel_scaled_max"] <= 1e-6
    if len(mism):  # a near tie: u between the two exponentials
        m = first
        lo, hi = sorted([math.exp(-min(du[m], 700)), math.exp(-min(du_o[m], 700))])
        assert lo - 1e-12 <= props["u"][m] <= hi + 1e-12
        assert first > n // 10
    assert acc[:first].sum() > 100
