"""Autotuner for the batched chain kernels.

For a system shape it measures the device throughput of ``fau_run_batch`` for
each kernel configuration (the ``threads`` parameter of fau_batch_params):

    96, 160, 288   pipelined kernel, 1 producer + 2, 4 or 8 compute warps
    128, 256       chain kernel of that CTA size

on ``replicas`` clones of the system (default: enough for four CTAs per SM),
and keeps the fastest.  Results are cached per (device name, SM count, system
shape) in a JSON file, so a shape is tuned once per machine.  The shape key
is what decides the kernel's cost: particle count, k-vector count, cell grid,
whether moves are molecular.
"""
from __future__ import annotations

import json
import os
from pathlib import Path
from typing import Callable, Dict, Optional, Sequence

CANDIDATES = (96, 160, 288, 128, 256)


def default_cache() -> Path:
    base = os.environ.get("FAU_AUTOTUNE_CACHE")
    if base:
        return Path(base)
    return Path(os.environ.get("XDG_CACHE_HOME", Path.home() / ".cache")) / "faunus_gb300" / "autotune.json"


def shape_key(system, device: str) -> str:
    spec = system.spec
    molecular = any(m.get("kind", 0) == 1 for m in spec.extra.get("moves", []))
    return (f"{device}|N={spec.n}|K={system.K}|cells={'x'.join(map(str, system.cell_grid()))}"
            f"|groups={spec.n_groups}|molecular={int(molecular)}")


def measure(ctx, system, threads: int, replicas: int, moves: int, seed: int = 1) -> float:
    """Device-timed moves/s of `replicas` clones advanced by `moves` moves each."""
    clones = [system.clone() for _ in range(replicas)]
    try:
        kw = dict(seed=seed, dp=float(system.spec.extra.get("moves", [{}])[0].get("dp", 1.0)),
                  dprot=float(system.spec.extra.get("moves", [{}])[0].get("dprot", 0.0)), threads=threads)
        ctx.run_batch(clones, max(1, moves // 10), **kw)  # warm-up (graph, caches)
        st = ctx.run_batch(clones, moves, counter_base=moves, **kw)
        return st["moves"] / (st["device_ms"] * 1e-3) if st["device_ms"] > 0 else 0.0
    finally:
        for c in clones:
            c.close()


def tune(ctx, system, *, replicas: Optional[int] = None, moves: int = 2000, candidates: Sequence[int] = CANDIDATES,
         cache: Optional[Path] = None, device: Optional[str] = None, force: bool = False,
         measure_fn: Callable = measure) -> Dict:
    """Best kernel configuration for `system`'s shape: {"threads", "moves_per_s", "table", "key"}."""
    if device is None or replicas is None:
        try:
            import torch
            prop = torch.cuda.get_device_properties(0)
            device = device or f"{prop.name}/{prop.multi_processor_count}"
            replicas = replicas or 4 * prop.multi_processor_count
        except Exception:
            device = device or "unknown"
            replicas = replicas or 4
    cache = cache or default_cache()
    key = shape_key(system, device)
    table_all = {}
    if cache.exists():
        try:
            table_all = json.loads(cache.read_text())
        except ValueError:
            table_all = {}
    if not force and key in table_all:
        return table_all[key]
    table = {}
    for t in candidates:
        try:
            table[str(t)] = measure_fn(ctx, system, t, replicas, moves)
        except Exception as e:  # a configuration the system cannot use (e.g. too little shared memory)
            table[str(t)] = 0.0
            table[f"{t}_error"] = str(e)
    best = max((t for t in candidates), key=lambda t: table[str(t)])
    out = {"threads": int(best), "moves_per_s": table[str(best)], "table": table, "key": key,
           "replicas": replicas, "moves": moves}
    table_all[key] = out
    try:
        cache.parent.mkdir(parents=True, exist_ok=True)
        cache.write_text(json.dumps(table_all, indent=1))
    except OSError:
        pass
    return out
