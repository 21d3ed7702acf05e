"""Faunus input files and state files at the boundary.

``load_input`` reads a Faunus input (JSON, or YAML through ``yason``) and builds
what the device path runs: a SystemSpec (Space + Hamiltonian), the move list for
MoveGenerator / run_batch, the MC loop and the analysis list.  ``state_json`` and
``apply_state`` write and read the reference's state-file schema (Space
to_json/from_json, src/space.cpp:449-500: geometry, groups {id, cm, atomic,
compressible, size}, particles {id, pos, q}), so a state saved by either side
restarts on the other.

Supported subset (anything else raises NotImplementedError naming the key):
  temperature, random {seed}, geometry {type: cuboid, length}, mcloop {macro, micro};
  atomlist (q, sigma or r, eps [kJ/mol], mw, dp, dprot) -- AtomData::from_json,
    src/atomdata.cpp:134-193;
  moleculelist (atoms + atomic, or structure [{atom: [x, y, z]}]; rigid) --
    src/molecule.cpp:395-470;
  insertmolecules ({name: {N | molarity, inactive}}) -- positions drawn with a seeded
    numpy generator (the reference's insertion draws from its own RNG, so initial
    states differ; a state file carries positions exactly);
  energy: nonbonded_coulomblj / _newcoulomblj / _coulombwca / _pm / _coulombhs / _pmwca
    (src/energy.cpp:1280-1327), nonbonded / nonbonded_exact (FunctorPotential:
    "default" and "A B" lists of coulomb / lennardjones / wca / hardsphere),
    nonbonded_splined (the same lists tabulated: utol, ftol, u_at_rmin, u_at_rmax, rmax,
    hardsphere; src/potentials.cpp:1513-1553),
    cutoff_g2g (number or per molecule pair), Ewald when coulomb type is ewald
    (src/energy.cpp:1134-1160), isobaric (P/atm, P/bar, P/kT, P/mM, P/Pa), maxenergy;
  moves: transrot, moltransrot, volume (src/move.cpp:190-222, 1580-1613, 986-993);
  analysis: kept as given (systemenergy, atomrdf and savestate drive ``simulate``).
"""
from __future__ import annotations

import base64
import json
import math
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any, Dict, List, Optional

import numpy as np

from . import _capi as A
from . import ubjson
from . import yason
from .system import (AVOGADRO, SystemSpec, bjerrum_length, coulomb_scheme, group_cutoff, kjmol_to_kt,
                     pressure_kt, splined)

NAN = float("nan")


@dataclass
class Setup:
    spec: SystemSpec
    moves: List[dict]
    mcloop: Dict[str, int]
    analysis: List[dict]
    atoms: List[str]
    molecules: List[str]
    temperature: float
    seed: Any
    source: dict = field(default_factory=dict)


def _items(lst, what: str):
    """[{name: props}, ...] -> [(name, props)] (one key per item, the reference's list form)."""
    out = []
    for it in lst or []:
        if not isinstance(it, dict) or len(it) != 1:
            raise ValueError(f"{what}: each item must be a single-key object, got {it!r}")
        (k, v), = it.items()
        out.append((k, v if v is not None else {}))
    return out


def _read(src) -> dict:
    if isinstance(src, dict):
        return src
    if isinstance(src, (bytes, bytearray)):
        return ubjson.loads(bytes(src))
    if isinstance(src, Path) or (isinstance(src, str) and "\n" not in src and Path(src).exists()):
        p = Path(src)
        if p.suffix == ".ubj":  # Universal Binary JSON state file (src/faunus.cpp:430-470)
            return ubjson.loads(p.read_bytes())
        text = p.read_text()
        return json.loads(text) if p.suffix == ".json" else yason.loads(text)
    text = str(src)
    try:
        return json.loads(text)
    except ValueError:
        return yason.loads(text)


# ------------------------------------------------------------------ pair potential pieces
def _mix(values: np.ndarray, rule: str) -> np.ndarray:
    a = values[:, None]
    b = values[None, :]
    if rule == "arithmetic":
        return 0.5 * (a + b)
    if rule == "geometric":
        return np.sqrt(a * b)
    raise NotImplementedError(f"mixing rule '{rule}'")


_RULES = {"LB": ("arithmetic", "geometric"), "lorentz_berthelot": ("arithmetic", "geometric"),
          "arithmetic": ("arithmetic", "arithmetic"), "geometric": ("geometric", "geometric")}


def _custom(block: dict, names: List[str]):
    for key, val in (block.get("custom") or {}).items():
        a, b = key.split()
        yield names.index(a), names.index(b), val


def _lj_tables(block: dict, sig: np.ndarray, eps_kjmol: np.ndarray, names, T: float):
    """LennardJones::initPairMatrices (src/potentials.cpp:671-690): sigma^2 and 4 eps (kT)."""
    rs, re = _RULES[block.get("mixing", "LB")]
    s = _mix(sig, rs)
    e = _mix(eps_kjmol, re)
    np.fill_diagonal(s, sig)
    np.fill_diagonal(e, eps_kjmol)
    for i, j, v in _custom(block, names):
        s[i, j] = s[j, i] = float(v.get("sigma", s[i, j]))
        e[i, j] = e[j, i] = float(v.get("eps", e[i, j]))
    return s * s, 4.0 * kjmol_to_kt(e, T)


def _hs_table(block: dict, sig: np.ndarray, names):
    """HardSphere::initPairMatrices (src/potentials.cpp:956-963): arithmetic by default."""
    s = _mix(sig, _RULES.get(block.get("mixing", "arithmetic"), ("arithmetic",))[0])
    np.fill_diagonal(s, sig)
    for i, j, v in _custom(block, names):
        s[i, j] = s[j, i] = float(v.get("sigma", s[i, j]))
    return s * s


def _coulomb(block: dict, T: float, plain_class: bool) -> dict:
    """Coulomb (plain class, src/potentials.h:463-479) or NewCoulombGalore::from_json
    (src/potentials.cpp:1628-1700) -> SystemSpec fields; Ewald adds its reciprocal part."""
    epsr = float(block["epsr"])
    if plain_class:
        return {"coulomb_type": A.FAU_COUL_PLAIN, "bjerrum_length": bjerrum_length(epsr, T)}
    typ = block.get("type")
    if typ is None:
        raise ValueError("coulomb needs a type")
    for key in ("debyelength", "molarity"):
        if key in block:
            raise NotImplementedError(f"coulomb '{key}' (screened electrostatics)")
    if typ == "yukawa":
        raise NotImplementedError("coulomb type 'yukawa'")
    kw = dict(epsr=epsr, cutoff=float(block.get("cutoff", 0.0)), alpha=float(block.get("alpha", 0.0)),
              temperature=T)
    if typ == "reactionfield":
        kw["epsrf"] = float(block["epsrf"])
    if typ == "poisson":
        kw["C"], kw["D"] = int(block.get("C", 3)), int(block.get("D", 3))
    if typ == "qpotential":
        kw["order"] = int(block["order"])
    f = coulomb_scheme(typ, **kw)
    if typ == "ewald":
        scheme = block.get("ewaldscheme", "PBC")
        if scheme not in ("PBC", "PBCEigen"):
            raise NotImplementedError(f"ewaldscheme '{scheme}'")
        f["ewald"] = {"alpha": float(block["alpha"]), "ncutoff": float(block.get("ncutoff", block.get("kcutoff"))),
                      "spherical_sum": int(bool(block.get("spherical_sum", True))),
                      "epss": float(block.get("epss", 0.0))}
    return f


# ------------------------------------------------------------------ configuration
def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _wrap(x: np.ndarray, L: np.ndarray) -> np.ndarray:
    out = x.copy()
    big = np.abs(out) > 0.5 * L
    t = out / L
    n = np.where(t > 0, np.trunc(t + 0.5), np.trunc(t - 0.5))
    return np.where(big, out - L * n, out)


def _mass_center(pos: np.ndarray, w: np.ndarray, L: np.ndarray) -> np.ndarray:
    """Group::updateMassCenter (src/group.cpp:136-157): shifted by the middle particle."""
    sh = -pos[len(pos) // 2]
    p = _wrap(pos + sh, L)
    c = (w[:, None] * p).sum(0) / w.sum() - sh
    return _wrap(c[None, :], L)[0]


def load_input(src, seed: int = 0) -> Setup:
    """Build a Setup from a Faunus input (dict, JSON/YAML text or file path).  `seed`
    seeds the random insertion of `insertmolecules`."""
    j = _read(src)
    base_dir = Path(src).parent if isinstance(src, Path) or (
        isinstance(src, str) and "\n" not in src and Path(src).exists()) else None
    known = {"temperature", "random", "geometry", "mcloop", "atomlist", "moleculelist", "insertmolecules",
             "energy", "moves", "analysis", "reactionlist", "groups", "particles", "implicit_reservoir"}
    extra = set(j) - known
    if extra:
        raise NotImplementedError(f"input section(s) {sorted(extra)}")
    T = float(j.get("temperature", 298.15))
    geo = j.get("geometry", {})
    if geo.get("type", "cuboid") != "cuboid":
        raise NotImplementedError(f"geometry type '{geo.get('type')}'")
    length = geo.get("length")
    box = np.array(length if isinstance(length, list) else [length] * 3, dtype=np.float64)

    # atoms (AtomData::from_json)
    atoms = _items(j.get("atomlist"), "atomlist")
    names = [a for a, _ in atoms]
    nt = len(names)
    q_t = np.array([float(p.get("q", 0.0)) for _, p in atoms])
    sig = np.array([float(p["sigma"]) if p.get("sigma") else 2.0 * float(p.get("r", 0.0)) for _, p in atoms])
    eps = np.array([float(p.get("eps", NAN)) for _, p in atoms])
    mw = np.array([float(p.get("mw", 1.0)) for _, p in atoms])
    type_dp = np.array([float(p["dp"]) if "dp" in p else NAN for _, p in atoms])
    type_dprot = np.array([float(p["dprot"]) if "dprot" in p else NAN for _, p in atoms])

    # molecules (MoleculeData::from_json)
    mols = _items(j.get("moleculelist"), "moleculelist")
    mnames = [m for m, _ in mols]
    mdefs = []
    for m, p in mols:
        atomic = bool(p.get("atomic", False))
        if "traj" in p:
            raise NotImplementedError(f"molecule '{m}': traj (conformation library)")
        if p.get("implicit"):  # a reaction's reservoir species, never in the space
            mdefs.append({"atomic": True, "rigid": False, "types": [], "xyz": None, "implicit": True})
            continue
        if "structure" in p and isinstance(p["structure"], dict):
            raise NotImplementedError(f"molecule '{m}': structure from {sorted(p['structure'])} (sequence input)")
        if "structure" in p and isinstance(p["structure"], str):
            # an .xyz file beside the input (MoleculeData::from_json: count, comment, name x y z)
            if base_dir is None or not p["structure"].endswith(".xyz"):
                raise NotImplementedError(f"molecule '{m}': structure file '{p['structure']}' "
                                          "(xyz files beside an input file are read)")
            lines = (base_dir / p["structure"]).read_text().split("\n")
            count = int(lines[0].split()[0])
            p = dict(p, structure=[{ln.split()[0]: [float(v) for v in ln.split()[1:4]]} for ln in lines[2:2 + count]])
        if "structure" in p:
            st = _items(p["structure"], f"molecule {m} structure")
            mdefs.append({"atomic": atomic, "rigid": bool(p.get("rigid", False)),
                          "types": [names.index(a) for a, _ in st],
                          "xyz": np.array([xyz for _, xyz in st], dtype=np.float64)})
        elif "atoms" in p:
            mdefs.append({"atomic": atomic, "rigid": bool(p.get("rigid", False)),
                          "types": [names.index(a) for a in p["atoms"]], "xyz": None})
        else:
            raise ValueError(f"molecule '{m}' needs atoms or a structure")

    # insertmolecules -> groups (InsertMoleculesInSpace; inactive groups are left out)
    rng = np.random.default_rng(seed)
    V = float(np.prod(box))
    pos_l, typ_l, gb, gflags, gmol = [], [], [0], [], []
    for m, p in _items(j.get("insertmolecules"), "insertmolecules"):
        if p.get("inactive"):
            continue
        mid = mnames.index(m)
        md = mdefs[mid]
        if md.get("implicit"):
            raise NotImplementedError(f"inserting implicit molecule '{m}'")
        n = int(p["N"]) if "N" in p else int(round(float(p["molarity"]) * V * AVOGADRO / 1e27))
        if md["atomic"]:
            t = np.tile(md["types"], n)
            pos_l.append((rng.random((len(t), 3)) - 0.5) * box)
            typ_l.append(t)
            gb.append(gb[-1] + len(t))
            gflags.append(A.FAU_GROUP_ATOMIC)
            gmol.append(mid)
        else:
            xyz, w = md["xyz"], mw[md["types"]]
            xyz = xyz - (w[:, None] * xyz).sum(0) / w.sum()
            for _ in range(n):
                c = (rng.random(3) - 0.5) * box
                pos_l.append(_wrap(c + xyz @ _random_rotation(rng).T, box))
                typ_l.append(np.array(md["types"]))
                gb.append(gb[-1] + len(md["types"]))
                gflags.append(A.FAU_GROUP_RIGID if md["rigid"] else 0)
                gmol.append(mid)
    pos = np.concatenate(pos_l) if pos_l else np.zeros((0, 3))
    types = np.concatenate(typ_l).astype(np.int32) if typ_l else np.zeros(0, np.int32)
    group_begin = np.array(gb, dtype=np.int32)
    group_flags = np.array(gflags, dtype=np.int32)
    group_molid = np.array(gmol, dtype=np.int32)

    # energy
    fields: Dict[str, Any] = {"pair_terms": 0}
    spline_opts: Optional[dict] = None
    for name, block in _items(j.get("energy"), "energy"):
        if name == "maxenergy":  # Hamiltonian's maximum_allowed_energy (src/energy.cpp:1189-1193)
            fields["maxenergy"] = float(block)
            continue
        if name == "isobaric":
            units = [k for k in block if k.startswith("P/")]
            if len(units) != 1:
                raise ValueError("isobaric needs exactly one pressure (P/atm, P/bar, P/kT, P/mM, P/Pa)")
            fields["isobaric_pressure"] = pressure_kt(float(block[units[0]]), units[0], T)
            continue
        if not name.startswith("nonbonded"):
            raise NotImplementedError(f"energy term '{name}'")
        if name == "nonbonded_cached":
            raise NotImplementedError("energy term 'nonbonded_cached' (FP32 group-pair energy cache)")
        if name in ("nonbonded", "nonbonded_exact", "nonbonded_splined"):
            _functor(block, fields, sig, eps, names, T)
            if name == "nonbonded_splined":  # SplinedPotential::from_json, src/potentials.cpp:1513-1553
                rmax = block.get("rmax")
                cg = block.get("cutoff_g2g")
                if isinstance(cg, (int, float)):
                    rmax = float(cg)
                elif isinstance(cg, dict):
                    if "default" not in cg:
                        raise ValueError("nonbonded_splined: an object cutoff_g2g needs a 'default' (the spline's rmax)")
                    rmax = float(cg["default"])
                spline_opts = {"utol": float(block.get("utol", 1e-3)), "ftol": float(block.get("ftol", 1e-2)),
                               "u_at_rmin": float(block.get("u_at_rmin", 20.0)),
                               "u_at_rmax": float(block.get("u_at_rmax", 1e-6)),
                               "rmax": rmax, "hardsphere": bool(block.get("hardsphere", False))}
        else:
            parts = {"nonbonded_coulomblj": ("coulomb", "lennardjones"),
                     "nonbonded_newcoulomblj": ("coulomb", "lennardjones"),
                     "nonbonded_coulombwca": ("coulomb", "wca"),
                     "nonbonded_pm": ("coulomb_plain", "hardsphere"),
                     "nonbonded_coulombhs": ("coulomb_plain", "hardsphere"),
                     "nonbonded_pmwca": ("coulomb_plain", "wca")}.get(name)
            if parts is None:
                raise NotImplementedError(f"energy term '{name}'")
            cblock = dict(block.get("coulomb", {}))
            fields.update(_coulomb(cblock, T, parts[0] == "coulomb_plain"))
            fields["pair_terms"] |= A.FAU_PAIR_COULOMB
            other = parts[1]
            sub = block.get(other) or {}
            if other == "hardsphere":
                fields["hs_sigma2"] = _hs_table(sub, sig, names)
                fields["pair_terms"] |= A.FAU_PAIR_HS
            else:
                fields["sigma2"], fields["eps4"] = _lj_tables(sub, sig, eps, names, T)
                fields["pair_terms"] |= A.FAU_PAIR_LJ if other == "lennardjones" else A.FAU_PAIR_WCA
        if "cutoff_g2g" in block:
            c = block["cutoff_g2g"]
            if isinstance(c, (int, float)):
                fields["cutoff_g2g"] = float(c)
            else:
                fields["cutoff_g2g_pairs"] = group_cutoff(c, mnames)

    spec = SystemSpec(box=box, pos=pos, charge=q_t[types], type=types, group_begin=group_begin,
                      group_flags=group_flags, group_molid=group_molid, n_types=nt, type_mass=mw,
                      temperature=T, name=str(Path(src).name) if isinstance(src, (str, Path)) and
                      "\n" not in str(src) and Path(str(src)).exists() else "input", **fields)
    if spline_opts is not None:
        spec = splined(spec, q_t, sig, **spline_opts)
    if spec.n_groups:
        cm = np.zeros((spec.n_groups, 3))
        for g in range(spec.n_groups):
            b, e = group_begin[g], group_begin[g + 1]
            if not group_flags[g] & A.FAU_GROUP_ATOMIC and e > b:
                cm[g] = _mass_center(pos[b:e], mw[types[b:e]], box)
        spec.mass_center = cm

    # moves
    moves = []
    for name, p in _items(j.get("moves"), "moves"):
        rep = p.get("repeat", 1)
        if name == "volume":
            moves.append({"kind": A.FAU_MOVE_VOLUME, "repeat": float(rep if rep != "N" else 1),
                          "dV": float(p["dV"]), "method": p.get("method", "isotropic")})
            continue
        if name not in ("transrot", "moltransrot"):
            raise NotImplementedError(f"move '{name}'")
        mid = mnames.index(p["molecule"])
        groups = [g for g in range(spec.n_groups) if group_molid[g] == mid]
        if name == "transrot":
            if rep == "N":  # AtomicTranslateRotate::_from_json: molecules x atoms of the first
                rep = len(groups) * (group_begin[groups[0] + 1] - group_begin[groups[0]]) if groups else 0
            moves.append({"kind": A.FAU_MOVE_ATOMIC, "repeat": float(rep), "dp": float(p.get("dp", 0.0)),
                          "dprot": float(p.get("dprot", 0.0)), "dir": tuple(p.get("dir", (1.0, 1.0, 1.0))),
                          "groups": groups, "type_dp": type_dp, "type_dprot": type_dprot})
        else:
            if mdefs[mid]["atomic"]:
                raise ValueError(f"molecule '{p['molecule']}' cannot be atomic")
            if rep == "N":  # TranslateRotate::_from_json: active molecules, at least 1
                rep = max(1, len(groups))
            moves.append({"kind": A.FAU_MOVE_MOLECULAR, "repeat": float(rep), "dp": float(p["dp"]),
                          "dprot": abs(float(p["dprot"])), "dir": tuple(p.get("dir", (1.0, 1.0, 1.0))),
                          "groups": groups})
    spec.extra["moves"] = moves
    mcloop = {"macro": int(j.get("mcloop", {}).get("macro", 10)), "micro": int(j.get("mcloop", {}).get("micro", 100))}
    setup = Setup(spec=spec, moves=moves, mcloop=mcloop, analysis=list(j.get("analysis", []) or []), atoms=names,
                  molecules=mnames, temperature=T, seed=(j.get("random") or {}).get("seed", "default"), source=j)
    if "groups" in j and "particles" in j:  # Space::from_json with a saved state merged in
        apply_state(setup, j)
    return setup


def _functor(block: dict, fields: dict, sig, eps, names, T: float) -> None:
    """FunctorPotential (src/potentials.cpp:1333-1368): per atom-pair lists of potentials.
    The descriptor's terms are global; a pair without a term gets a zero coefficient
    (eps4 = 0 for LJ/WCA, hs_sigma2 = 0 for hard spheres).  Coulomb must be the same
    for every pair that has it, and every pair must have it if any does."""
    nt = len(names)
    lists = {}
    default = block.get("default", [])
    for key, lst in block.items():
        if key in ("default", "cutoff_g2g", "selfenergy", "utol", "ftol", "u_at_rmin", "u_at_rmax", "rmax",
                   "hardsphere", "to_disk"):
            continue
        a, b = key.split()
        lists[(names.index(a), names.index(b))] = lst
        lists[(names.index(b), names.index(a))] = lst
    pairs = {(i, j): lists.get((i, j), default) for i in range(nt) for j in range(nt)}
    kinds = {}
    for (i, j), lst in pairs.items():
        for name, sub in _items(lst, "nonbonded pair list"):
            kinds.setdefault(name, {})[(i, j)] = sub or {}
    unknown = set(kinds) - {"coulomb", "lennardjones", "wca", "hardsphere"}
    if unknown:
        raise NotImplementedError(f"FunctorPotential term(s) {sorted(unknown)}")
    if "coulomb" in kinds:
        if len(kinds["coulomb"]) != nt * nt:
            raise NotImplementedError("Coulomb on some atom pairs only")
        first = next(iter(kinds["coulomb"].values()))
        if any(v != first for v in kinds["coulomb"].values()):
            raise NotImplementedError("different Coulomb schemes per atom pair")
        fields.update(_coulomb(first, T, False))
        fields["pair_terms"] |= A.FAU_PAIR_COULOMB
    if "lennardjones" in kinds and "wca" in kinds:
        raise NotImplementedError("LJ and WCA in one FunctorPotential")
    for name, bit in (("lennardjones", A.FAU_PAIR_LJ), ("wca", A.FAU_PAIR_WCA)):
        if name in kinds:
            sub = next(iter(kinds[name].values()))
            s2, e4 = _lj_tables(sub, sig, eps, names, T)
            mask = np.zeros((nt, nt), bool)
            for ij in kinds[name]:
                mask[ij] = True
            fields["sigma2"], fields["eps4"] = s2, np.where(mask, e4, 0.0)
            fields["pair_terms"] |= bit
    if "hardsphere" in kinds:
        sub = next(iter(kinds["hardsphere"].values()))
        hs = _hs_table(sub, sig, names)
        mask = np.zeros((nt, nt), bool)
        for ij in kinds["hardsphere"]:
            mask[ij] = True
        fields["hs_sigma2"] = np.where(mask, hs, 0.0)
        fields["pair_terms"] |= A.FAU_PAIR_HS


# ------------------------------------------------------------------ state files
def apply_state(setup: Setup, state) -> Setup:
    """Space::from_json (src/space.cpp:458-500): particles (id, pos, q), groups (id, size,
    cm, atomic) and geometry from a state (dict or JSON file) replace the setup's."""
    st = _read(state)
    spec = setup.spec
    parts = st["particles"]
    spec.pos = np.array([p.get("pos", [0.0, 0.0, 0.0]) for p in parts], dtype=np.float64)
    spec.charge = np.array([float(p.get("q", 0.0)) for p in parts])
    spec.type = np.array([int(p["id"]) for p in parts], dtype=np.int32)
    gb, fl, mol, cm = [0], [], [], []
    for g in st["groups"]:
        if int(g.get("capacity", g["size"])) != int(g["size"]):
            raise NotImplementedError("groups with capacity beyond their size (inactive particles)")
        gb.append(gb[-1] + int(g["size"]))
        mid = int(g["id"])
        mol.append(mid)
        atomic = bool(g.get("atomic", False))
        rigid = False
        src_mols = _items(setup.source.get("moleculelist"), "moleculelist")
        if mid < len(src_mols):
            rigid = bool(src_mols[mid][1].get("rigid", False))
        fl.append(A.FAU_GROUP_ATOMIC if atomic else (A.FAU_GROUP_RIGID if rigid else 0))
        cm.append(g.get("cm", [0.0, 0.0, 0.0]))
    if gb[-1] != len(parts):
        raise ValueError("load error: group sizes do not add up to the particle count")
    spec.group_begin = np.array(gb, dtype=np.int32)
    spec.group_flags = np.array(fl, dtype=np.int32)
    spec.group_molid = np.array(mol, dtype=np.int32)
    spec.mass_center = np.array(cm, dtype=np.float64).reshape(-1, 3)
    if "geometry" in st:
        length = st["geometry"].get("length")
        spec.box = np.array(length if isinstance(length, list) else [length] * 3, dtype=np.float64)
    for m in setup.moves:  # move groups follow the new group list
        if m["kind"] in (A.FAU_MOVE_ATOMIC, A.FAU_MOVE_MOLECULAR):
            mids = {int(spec.group_molid[g]) for g in m["groups"]} if m["groups"] else set()
            if mids:
                m["groups"] = [g for g in range(spec.n_groups) if int(spec.group_molid[g]) in mids]
    return setup


def state_json(setup: Setup, positions: np.ndarray, box: np.ndarray, mass_centers: np.ndarray) -> dict:
    """Space::to_json (src/space.cpp:449-456) of the given configuration."""
    spec = setup.spec
    groups = []
    for g in range(spec.n_groups):
        b, e = int(spec.group_begin[g]), int(spec.group_begin[g + 1])
        groups.append({"id": int(spec.group_molid[g]) if spec.group_molid is not None else 0,
                       "cm": [float(x) for x in mass_centers[g]],
                       "atomic": bool(spec.group_flags[g] & A.FAU_GROUP_ATOMIC), "compressible": False,
                       "size": e - b})
    parts = [{"id": int(t), "pos": [float(x) for x in p], "q": float(q)}
             for t, p, q in zip(spec.type, positions, spec.charge)]
    return {"geometry": {"type": "cuboid", "length": [float(x) for x in box]}, "groups": groups,
            "particles": parts, "reactionlist": [], "implicit_reservoir": []}


ENGINE_NAME = "Mersenne Twister (std::mt19937)"
DEVICE_STATE_KEY = "fau-device-state"


def save_state(setup: Setup, system, path, movegen=None, device_state: bool = True) -> dict:
    """SaveState (src/analysis.cpp:586-690): the state of a resident System -- positions, box,
    mass centres -- as JSON, or as Universal Binary JSON for a `.ubj` path.  With the move
    generator, its two mt19937 engines as "random-move" and "random-global" (saverandom: the
    reference's Random::to_json form, src/random.cpp:35-46).  device_state adds the system's
    exact device state (base64 of fau_sys_save_state, a key the reference ignores), from which
    resume_state continues the chain bit for bit."""
    st = state_json(setup, system.positions(), system.box(), system.mass_centers())
    if movegen is not None:
        slump, rnd = movegen.state().split("\n")
        st["random-move"] = {"seed": slump, "engine": ENGINE_NAME}
        st["random-global"] = {"seed": rnd, "engine": ENGINE_NAME}
    if device_state:
        st[DEVICE_STATE_KEY] = base64.b64encode(system.save_state()).decode("ascii")
    p = Path(path)
    if p.suffix == ".ubj":
        p.write_bytes(ubjson.dumps(st))
    else:
        p.write_text(json.dumps(st))
    return st


def resume_state(state, system=None, movegen=None) -> None:
    """The other half of a restart (MetropolisMonteCarlo::restore, src/montecarlo.cpp:116-137):
    the engines of "random-move" / "random-global" into the move generator, and the exact device
    state, when the file carries one, into a system made from the state's setup
    (apply_state)."""
    st = _read(state)
    if movegen is not None and "random-move" in st and "random-global" in st:
        movegen.set_state(st["random-move"]["seed"] + "\n" + st["random-global"]["seed"])
    if system is not None and DEVICE_STATE_KEY in st:
        system.load_state(base64.b64decode(st[DEVICE_STATE_KEY]))
