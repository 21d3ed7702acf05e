"""Build the sm_103a shared library ``faunus_gb300/_lib/libfau_gpu.so``.

Every translation unit is compiled in parallel with nvcc (one ``-gencode``,
sm_103a only) and linked with the static CUDA runtime; the library has no
PyTorch dependency.  Host code is compiled without FMA contraction so its
FP64 arithmetic (trial positions, fixed-point conversion) is IEEE-exact.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIBNAME = "libfau_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["fau_kernels.cu", "fau_capi.cu", "fau_batch.cu", "fau_movegen.cpp", "fau_noalloc.cu",
           "fau_chain_128_host.cu", "fau_chain_128_ph.cu", "fau_chain_256_host.cu", "fau_chain_256_ph.cu",
           "fau_fast_2_ph.cu", "fau_fast_2_host.cu", "fau_fast_4_ph.cu", "fau_fast_4_host.cu", "fau_fast_8_ph.cu",
           "fau_fast_4s_ph.cu", "fau_fast_4s_host.cu", "fau_fast_8s_ph.cu", "fau_sampler.cu", "fau_mol_256.cu", "fau_mol_256_host.cu", "fau_mol_512.cu",
           "fau_spline.cpp", "fau_audit.cu", "fau_fp64.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build faunus_gb300")


def _compile(src: Path, obj: Path, extra: list[str], host: list[str] | None = None) -> None:
    """host: further host-compiler options, for the .cu and the .cpp sources alike."""
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(PKG.parent / "include")]
    hostx = [a for h in (host or []) for a in ("-Xcompiler", h)]
    if src.suffix == ".cu":
        cmd = [nvcc, *ARCH, "-lineinfo", *common, *hostx, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [nvcc, "-x", "c++", *common, *hostx, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile and link the library; returns its path."""
    extra = list(extra or [])
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    objs = [objdir / (s.name + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], extra), zip(srcs, objs)))
    out = LIBDIR / LIBNAME
    tmp = LIBDIR / (LIBNAME + ".tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    if verbose:
        print(f"built {out}")
    return out


def build_sanitized(verbose: bool = False) -> Path:
    """The library with its host code under AddressSanitizer and UndefinedBehaviorSanitizer, as
    ``_lib/libfau_gpu_san.so`` beside the product (never loaded by default): the CPU tests run
    against it with ``FAU_GPU_LIB`` pointing at it and the sanitizer runtimes preloaded, e.g.

        make -C oracle sanitize
        FAU_GPU_LIB=faunus_gb300/_lib/libfau_gpu_san.so FAU_ORACLE_LIB=oracle/_build/liboracle_san.so \
        LD_PRELOAD="$(gcc -print-file-name=libasan.so) $(gcc -print-file-name=libubsan.so)" \
        ASAN_OPTIONS=detect_leaks=0 python -m pytest tests -m "not gpu"
    """
    san = ["-fsanitize=address", "-fsanitize=undefined", "-fno-omit-frame-pointer"]
    objdir = PKG / "_build" / "san"
    objdir.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    objs = [objdir / (s.name + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], [], san), zip(srcs, objs)))
    out = LIBDIR / "libfau_gpu_san.so"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(out), *map(str, objs), *[a for h in san for a in ("-Xcompiler", h)],
           "-lasan", "-lubsan"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {out}")
    return out


def build_oracle() -> Path:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    odir = PKG.parent / "oracle"
    r = subprocess.run(["make", "-C", str(odir)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")
    return odir / "_build" / "liboracle.so"


if __name__ == "__main__":
    build(verbose=True)
    build_oracle()
