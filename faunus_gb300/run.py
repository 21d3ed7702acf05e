"""The Faunus MC loop on the device path, driven by an input file.

``simulate`` follows the reference executable's loop (src/faunus.cpp:226-243):
``macro`` x ``micro`` sweeps; one sweep is sum(repeat) moves drawn from the move
collection (MetropolisMonteCarlo::sweep, src/montecarlo.cpp:220-227); after each
sweep the analyses sample when their step count is a multiple of ``nstep``
(Analysis::sample, src/analysis.cpp:65-75).  Moves come from the reference's RNG
stream (``mode="reference"``: mt19937 on the host, every move kind including
volume moves, through fau_run_proposals) or from the device's counter-based RNG
(``mode="batch"``: fau_run_batch, single-atom or molecular moves, no volume moves).
SystemEnergy samples the running energy and AtomRDF the pair histogram on the
device (fau_sampler); savestate writes the reference's state file (JSON, or UBJSON for .ubj)
with the RNG engines and the exact device state, from which ``resume`` continues bit for bit.  The result
mirrors the reference's output JSON: per-move acceptance, energy statistics,
analysis sample counts and the relative energy drift
(MetropolisMonteCarlo::relativeEnergyDrift, src/montecarlo.cpp:85-98).
"""
from __future__ import annotations

import json
from pathlib import Path
from typing import Optional

import numpy as np

from . import _capi as A
from .input import Setup, resume_state, save_state
from .system import MoveGenerator, Sampler


def simulate(setup: Setup, ctx, *, out_dir=".", mode: str = "reference", seed: int = 1,
             macro: Optional[int] = None, micro: Optional[int] = None, resume=None, first_step: int = 0) -> dict:
    """resume: a state saved by an earlier run (dict or path; setup already carries its positions
    through apply_state) whose engines and exact device state continue the chain; first_step:
    the sweeps that run already made (the device RNG's counter and the analyses' step count
    continue from it)."""
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    spec = setup.spec
    system = ctx.create(spec)
    macro = setup.mcloop["macro"] if macro is None else macro
    micro = setup.mcloop["micro"] if micro is None else micro
    per_sweep = int(round(sum(m["repeat"] for m in setup.moves)))
    has_volume = any(m["kind"] == A.FAU_MOVE_VOLUME for m in setup.moves)
    batch_dp = batch_dprot = 0.0
    if mode == "batch":
        kinds = {m["kind"] for m in setup.moves}
        if has_volume or len(kinds) != 1:
            raise NotImplementedError("batch mode runs one kind of translate/rotate move (volume moves: reference mode)")
        m = setup.moves[0]
        batch_dp, batch_dprot = float(m.get("dp", 0.0)), float(m.get("dprot", 0.0))
        if m["kind"] == A.FAU_MOVE_ATOMIC and m.get("type_dp") is not None:
            used = {float(v) for v in np.asarray(m["type_dp"])[np.unique(spec.type)] if not np.isnan(v)}
            if len(used) > 1:
                raise NotImplementedError("batch mode needs one dp for every moved atom type")
            if used:
                batch_dp = used.pop()
    gen = None
    if mode == "reference":
        fixed = setup.seed in ("fixed", "default", None)
        gen = MoveGenerator(spec, setup.moves, seed, seed + 1, default_seeds=fixed)
    elif mode != "batch":
        raise ValueError(f"unknown mode '{mode}'")
    if resume is not None:
        resume_state(resume, system, gen)

    # analyses
    energy_an, rdf_an, saves = None, [], []
    for item in setup.analysis:
        (name, p), = item.items()
        p = p or {}
        if name == "systemenergy":
            energy_an = {"nstep": int(p.get("nstep", 1)), "file": p.get("file"), "samples": []}
        elif name == "atomrdf":
            a, b = setup.atoms.index(p["name1"]), setup.atoms.index(p["name2"])
            dr = float(p.get("dr", 0.1))
            rmax = 0.5 * float(np.sqrt((spec.box ** 2).sum())) * 1.5  # room for volume moves
            bins = min(A.FAU_SAMPLER_MAX_BINS, int(np.ceil(rmax / dr)))
            rdf_an.append({"nstep": int(p.get("nstep", 1)), "file": p.get("file"), "dr": dr,
                           "sampler": Sampler(ctx, 1, rdf=(a, b, dr, bins), energy=False), "name1": p["name1"],
                           "name2": p["name2"]})
        elif name == "savestate":
            saves.append(p.get("file"))
    e0 = system.energy_total()["total"]
    c0 = system.counters()
    step = first_step
    accepted = {}
    for _ in range(macro):
        for _ in range(micro):
            if mode == "reference":
                props = gen.generate(per_sweep)
                acc, _, _ = system.run_proposals(props)
                for k in np.unique(props["kind"]):
                    sel = props["kind"] == k
                    a, n = accepted.get(int(k), (0, 0))
                    accepted[int(k)] = (a + int(acc[sel].sum()), n + int(sel.sum()))
            else:
                ctx.run_batch([system], per_sweep, seed=seed, counter_base=step * per_sweep, dp=batch_dp,
                              dprot=batch_dprot)
            step += 1
            if not np.isfinite(system.running_energy()):  # left an infinite start: sum of changes undefined
                system.refresh_energy()
            if energy_an and step % energy_an["nstep"] == 0:
                energy_an["samples"].append(system.running_energy())
            for r in rdf_an:
                if step % r["nstep"] == 0:
                    r["sampler"].sample([system])

    # results
    e_total = system.energy_total()["total"]
    c1 = system.counters()
    du_sum = e_total - e0
    e_run = system.running_energy()  # initial energy + sum of accepted changes (refreshed after an infinite start)
    if not np.isfinite(du_sum):  # e.g. a start with hard-sphere overlaps (infinite energy)
        drift = float("nan")
    elif abs(du_sum) <= 2.220446049250313e-16:
        drift = 0.0
    else:
        drift = (e_total - e_run) / (e0 if abs(e0) > 2.220446049250313e-16 else e_total)
    result = {"moves": {"attempted": c1["moves"] - c0["moves"], "accepted": c1["accepted"] - c0["accepted"],
                        "acceptance": {str(k): a / n for k, (a, n) in accepted.items() if n}},
              "energy": {"initial": e0, "final": e_total, "change": du_sum},
              "relative drift": drift, "geometry": {"length": [float(x) for x in system.box()]},
              "analysis": []}
    if energy_an:
        s = np.array(energy_an["samples"])
        result["analysis"].append({"systemenergy": {"samples": len(s), "mean": float(s.mean()) if len(s) else None,
                                                    "final": float(e_total)}})
        if energy_an["file"]:
            (out / energy_an["file"]).write_text(
                "".join(f"{(k + 1) * energy_an['nstep']} {e:.12e}\n" for k, e in enumerate(s)))
    for r in rdf_an:
        d = r["sampler"].read()
        n = int(d["rdf_samples"][0])
        entry = {"name1": r["name1"], "name2": r["name2"], "dr": r["dr"], "samples": n}
        if n:
            rr, g = r["sampler"].g_of_r(d)
            if r["file"]:
                (out / r["file"]).write_text("".join(f"{x:.6E} {y:.6E}\n" for x, y in zip(rr, g)))
        result["analysis"].append({"atomrdf": entry})
        r["sampler"].close()
    for f in saves:
        if f and (f.endswith(".json") or f.endswith(".ubj")):
            save_state(setup, system, out / f, movegen=gen)
    (out / "out.json").write_text(json.dumps(result, indent=1))
    system.close()
    return result
