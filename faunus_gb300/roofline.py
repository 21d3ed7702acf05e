"""Algorithmic work per unit of the Metropolis MC hot path, in one place.

A *trial move* is one proposal through the Metropolis decision.  A *pair
interaction* is one u(r_ij) evaluation; a single-atom move counts two per
candidate j (its old and its new state), as the reference evaluates both
states (MetropolisMonteCarlo::performMove, src/montecarlo.cpp:139-187).  A
*k-vector update* is one Ewald k-vector for one moved atom
(PolicyIonIon::updateComplex, src/energy.cpp:219-247).

Counting: add, multiply, compare, select = 1 flop; FMA = 2.

  pair, primitive model (Coulomb + WCA + hard sphere)   24 flop + 1 MUFU (rsqrt)
  pair, LJ + Ewald real space (erfc)                     38 flop + 2 MUFU (rsqrt, exp)
  k-vector, per moved atom: two phase dot products (12),
      the delta Q(k) accumulation (8)                    20 flop + 4 MUFU (2 sincos)
  k-vector, per move: the reciprocal energy change        6 flop
      -> a single-atom move: 26 flop per k-vector

Bytes (the algorithmic traffic of the path, whatever level of the memory
hierarchy serves it):

  per candidate particle j: x, y, z, q (FP32) + type     20 B (FP32 form; 36 B in FP64)
  per k-vector and move: k-vector (12 B FP32) + A_k (4 B)
      + Q_k (16 B, FP64 complex) read                    32 B
  per k-vector and accepted move: Q_k written            16 B

The fractions the benchmark reports against these:

  hbm      algorithmic bytes / s  / measured HBM copy bandwidth (the contract's form)
  dram     DRAM bytes per move measured by ncu x moves/s / the same peak
  fp32     algorithmic flop / s   / measured FP32 FMA peak
  issue    warp instructions per move measured by ncu x moves/s
           / (SMs x 4 schedulers x SM clock): the instruction-issue ceiling
"""
from __future__ import annotations

import json
from pathlib import Path

FLOPS_PER_PAIR_PM = 24.0
FLOPS_PER_PAIR_LJ_EWALD = 38.0
FLOPS_PER_K_PER_ATOM = 20.0
FLOPS_PER_K_PER_MOVE = 6.0
FLOPS_PER_K_SINGLE_ATOM_MOVE = FLOPS_PER_K_PER_ATOM + FLOPS_PER_K_PER_MOVE  # 26
MUFU_PER_PAIR_PM = 1
MUFU_PER_PAIR_LJ_EWALD = 2
MUFU_PER_K_PER_ATOM = 4

BYTES_PER_CANDIDATE_FP32 = 20
BYTES_PER_CANDIDATE_FP64 = 36
BYTES_PER_K_READ = 32
BYTES_PER_K_WRITE = 16

SCHEDULERS_PER_SM = 4

ROOT = Path(__file__).resolve().parent.parent


def single_atom_flops(pair_evals: float, moves: float, kvectors: int, ewald_pair: bool = True) -> float:
    """Algorithmic flop of single-atom moves: pairs plus K k-vectors per move (one moved atom)."""
    per_pair = FLOPS_PER_PAIR_LJ_EWALD if ewald_pair else FLOPS_PER_PAIR_PM
    return per_pair * pair_evals + FLOPS_PER_K_SINGLE_ATOM_MOVE * kvectors * moves


def single_atom_bytes(pair_evals: float, moves: float, accepted: float, kvectors: int) -> float:
    """Algorithmic bytes of single-atom moves: every candidate once (its two pair interactions share
    the record), the k-vector table, A_k and Q(k) read every move, Q(k) written on acceptance."""
    return (BYTES_PER_CANDIDATE_FP32 * pair_evals / 2 + BYTES_PER_K_READ * kvectors * moves +
            BYTES_PER_K_WRITE * kvectors * accepted)


def measured_peaks() -> dict:
    """HBM copy bandwidth (GB/s) measured on the GB300s, or the fallback figure."""
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0))}
    except (OSError, ValueError, KeyError):
        return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s", "sm_max_mhz": 2070.0}


def kernel_profile(name: str) -> dict | None:
    """Per-move DRAM bytes and warp instructions of a kernel from its committed ncu summary
    (profiles/<name>.json), or None."""
    p = ROOT / "profiles" / f"{name}.json"
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return None


def fractions(moves_per_s: float, alg_bytes_per_move: float, flops_per_move: float, fp32_peak_tflops: float | None,
              sms: int, sm_mhz: float | None, profile: dict | None) -> dict:
    """Every roofline fraction of the kernel at a measured rate, and which one binds."""
    pk = measured_peaks()
    hbm = alg_bytes_per_move * moves_per_s / 1e9
    out = {"hbm": {"achieved_gbs": hbm, "peak_gbs": pk["hbm_gbs"], "frac": hbm / pk["hbm_gbs"],
                   "peak_source": pk["source"]}}
    if fp32_peak_tflops:
        tf = flops_per_move * moves_per_s / 1e12
        out["fp32"] = {"achieved_tflops": tf, "peak_tflops": fp32_peak_tflops, "frac": tf / fp32_peak_tflops,
                       "peak_source": "measured FP32 FMA probe (fau_measure_fp32_peak) in this run"}
    if profile:
        if profile.get("dram_bytes_per_move"):
            d = profile["dram_bytes_per_move"] * moves_per_s / 1e9
            out["dram"] = {"achieved_gbs": d, "peak_gbs": pk["hbm_gbs"], "frac": d / pk["hbm_gbs"],
                           "bytes_per_move": profile["dram_bytes_per_move"], "source": profile.get("source")}
        if profile.get("warp_instructions_per_move"):
            clk = (sm_mhz or pk["sm_max_mhz"]) * 1e6
            cap = sms * SCHEDULERS_PER_SM * clk
            ipm = profile["warp_instructions_per_move"]
            out["issue"] = {"warp_instructions_per_move": ipm, "achieved_per_s": ipm * moves_per_s,
                            "peak_per_s": cap, "frac": ipm * moves_per_s / cap,
                            "peak": f"{sms} SMs x {SCHEDULERS_PER_SM} schedulers x {clk / 1e6:.0f} MHz"}
    # what binds: the largest fraction of a hardware unit measured on the kernel itself (the
    # algorithmic-bytes form is the contract's yardstick, not a unit's utilisation)
    hw = [k for k in ("dram", "fp32", "issue") if k in out]
    out["binding"] = max(hw, key=lambda k: out[k]["frac"]) if hw else "hbm"
    return out
