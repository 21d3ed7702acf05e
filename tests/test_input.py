"""Faunus input and state files at the boundary: the YAML subset reader, the input ->
SystemSpec mapping (atoms, molecules, energy terms, moves, MC loop), state-file round
trips, and the reference's own examples/bulk run as a golden case (its input, the state
its run saved, and the energies it reported for that state)."""
import json
import math
import os
from pathlib import Path

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import input as I
from faunus_gb300 import yason
from faunus_gb300.system import kjmol_to_kt

import oracle_lib as O

GOLDEN = Path(__file__).parent / "golden"


def test_yason_subset():
    text = """#!/usr/bin/env yason.py
temperature: 300   # K
flags: {a: true, b: no, c: null, d: ~}
list: [1, 2.5, -3e-2, Na+, "quoted: yes", 'it''s']
energy:
    - nonbonded_pm:
        coulomb: {epsr: 80}
        cutoff_g2g: {default: 13, "M Q": 14}
    - isobaric: {P/atm: 1}
moves:
- transrot: {molecule: salt, repeat: N}
-
  - 1
  - 2
empty:
nested:
  deeper:
    x: [[1, 2], {y: [3]}]
"""
    want = {"temperature": 300, "flags": {"a": True, "b": False, "c": None, "d": None},
            "list": [1, 2.5, -0.03, "Na+", "quoted: yes", "it's"],
            "energy": [{"nonbonded_pm": {"coulomb": {"epsr": 80}, "cutoff_g2g": {"default": 13, "M Q": 14}}},
                       {"isobaric": {"P/atm": 1}}],
            "moves": [{"transrot": {"molecule": "salt", "repeat": "N"}}, [1, 2]],
            "empty": None, "nested": {"deeper": {"x": [[1, 2], {"y": [3]}]}}}
    assert yason.loads(text) == want
    for bad in ("a: &anchor 1", "a:\n\t- 1", "a: [1, 2"):
        with pytest.raises(ValueError):
            yason.loads(bad)


PM = """
temperature: 300
random: {seed: fixed}
geometry: {type: cuboid, length: 60}
mcloop: {macro: 2, micro: 10}
energy:
    - nonbonded_pm:
        coulomb: {epsr: 80}
atomlist:
    - Na+: {q: 1.0, sigma: 4.0, dp: 20}
    - Cl-: {q: -1.0, r: 2.5, dp: 10}
moleculelist:
    - sodium: {atoms: [Na+], atomic: true}
    - chloride: {atoms: [Cl-], atomic: true}
    - ghost: {atoms: [Na+, Cl-], atomic: true}
insertmolecules:
    - sodium: {N: 30}
    - chloride: {N: 30}
    - ghost: {N: 1, inactive: 1}
moves:
    - transrot: {molecule: sodium, repeat: N}
    - transrot: {molecule: chloride, repeat: 5}
analysis:
    - systemenergy: {file: energy.dat, nstep: 10}
"""


def test_primitive_model_input():
    s = I.load_input(PM)
    spec = s.spec
    assert s.atoms == ["Na+", "Cl-"] and s.molecules == ["sodium", "chloride", "ghost"]
    assert spec.n == 60 and spec.n_groups == 2 and list(spec.group_begin) == [0, 30, 60]
    assert (spec.group_flags == A.FAU_GROUP_ATOMIC).all()
    assert spec.pair_terms == A.FAU_PAIR_COULOMB | A.FAU_PAIR_HS
    assert spec.coulomb_type == A.FAU_COUL_PLAIN
    assert spec.bjerrum_length == pytest.approx(F.bjerrum_length(80.0, 300.0), rel=1e-15)
    # sigma from r = 2.5 -> 5; hard-sphere arithmetic mixing
    assert np.allclose(spec.hs_sigma2, np.array([[16.0, 20.25], [20.25, 25.0]]))
    assert np.allclose(np.abs(spec.pos), np.abs(spec.pos).clip(max=30.0))
    assert list(spec.charge[:30]) == [1.0] * 30 and list(spec.charge[30:]) == [-1.0] * 30
    m0, m1 = s.moves
    assert m0["repeat"] == 30 and m1["repeat"] == 5 and m0["groups"] == [0] and m1["groups"] == [1]
    assert m0["dp"] == 0.0 and list(m0["type_dp"]) == [20.0, 10.0]
    assert s.mcloop == {"macro": 2, "micro": 10} and s.seed == "fixed"


WATER = """
temperature: 300
geometry: {type: cuboid, length: 18.6}
atomlist:
    - OW: {q: -0.8476, sigma: 3.166, eps: 0.650, mw: 15.999}
    - HW: {q: 0.4238,  sigma: 2, eps: 0, mw: 1.007}
moleculelist:
    - water:
        rigid: true
        structure:
            - OW: [2.30, 6.28, 1.13]
            - HW: [1.37, 6.26, 1.50]
            - HW: [2.31, 5.89, 0.21]
insertmolecules:
    - water: {N: 64}
energy:
    - isobaric: {P/atm: 1}
    - nonbonded_coulomblj:
        lennardjones: {mixing: LB}
        coulomb: {type: ewald, epsr: 1, cutoff: 9, ncutoff: 7.3, epss: 0, alpha: 0.2, ewaldscheme: PBCEigen}
        cutoff_g2g: 10
moves:
    - moltransrot: {molecule: water, dp: 0.4, dprot: 0.4, repeat: N}
    - volume: {dV: 0.03, method: isotropic}
"""


def test_water_npt_input():
    s = I.load_input(WATER)
    spec = s.spec
    assert spec.n == 192 and spec.n_groups == 64 and (spec.group_flags == A.FAU_GROUP_RIGID).all()
    assert spec.ewald == {"alpha": 0.2, "ncutoff": 7.3, "spherical_sum": 1, "epss": 0.0}
    assert spec.coulomb_type == A.FAU_COUL_EWALD and spec.coulomb_cutoff == 9.0 and spec.cutoff_g2g == 10.0
    assert spec.isobaric_pressure == pytest.approx(F.pressure_kt(1.0, "P/atm", 300.0), rel=1e-15)
    e_oo = 4 * kjmol_to_kt(0.65, 300.0)
    assert spec.eps4[0, 0] == pytest.approx(e_oo, rel=1e-15) and spec.eps4[0, 1] == 0.0
    assert spec.sigma2[0, 1] == pytest.approx(((3.166 + 2) / 2) ** 2, rel=1e-15)
    # rigid geometry kept: O-H distances of the structure
    oh = np.linalg.norm(np.array([1.37, 6.26, 1.50]) - np.array([2.30, 6.28, 1.13]))
    d = spec.pos[1::3] - spec.pos[0::3]
    d -= spec.box * np.round(d / spec.box)
    assert np.allclose(np.linalg.norm(d, axis=1), oh, atol=1e-12)
    mt, vol = s.moves
    assert mt["kind"] == A.FAU_MOVE_MOLECULAR and mt["repeat"] == 64 and mt["groups"] == list(range(64))
    assert vol == {"kind": A.FAU_MOVE_VOLUME, "repeat": 1.0, "dV": 0.03, "method": "isotropic"}
    # the oracle builds it and the move generator accepts the move list
    o = O.OracleSystem(spec)
    assert math.isfinite(o.energy_total()["total"])
    props = F.MoveGenerator(spec, s.moves, 1, 2, default_seeds=False).generate(500)
    assert set(np.unique(props["kind"])) <= {A.FAU_MOVE_MOLECULAR, A.FAU_MOVE_VOLUME}


def test_functor_potential_input():
    j = {"temperature": 298.15, "geometry": {"type": "cuboid", "length": 50},
         "atomlist": [{"A": {"q": 1.0, "sigma": 2.2, "eps": 0.1}}, {"B": {"q": -1.0, "sigma": 4.0, "eps": 0.05}},
                      {"C": {"sigma": 2.0}}],
         "moleculelist": [{"s": {"atoms": ["A", "B", "C"], "atomic": True}}],
         "insertmolecules": [{"s": {"N": 2}}],
         "energy": [{"nonbonded": {"default": [{"coulomb": {"type": "plain", "epsr": 80}}],
                                   "A B": [{"coulomb": {"type": "plain", "epsr": 80}}, {"wca": {"mixing": "LB"}}],
                                   "C C": [{"coulomb": {"type": "plain", "epsr": 80}}, {"hardsphere": {}}]}}],
         "moves": []}
    spec = I.load_input(j).spec
    assert spec.pair_terms == A.FAU_PAIR_COULOMB | A.FAU_PAIR_WCA | A.FAU_PAIR_HS
    nz = np.argwhere(spec.eps4 != 0).tolist()
    assert nz == [[0, 1], [1, 0]]
    assert np.argwhere(spec.hs_sigma2 != 0).tolist() == [[2, 2]]
    bad = json.loads(json.dumps(j))
    bad["energy"][0]["nonbonded"]["A B"] = [{"wca": {"mixing": "LB"}}]
    with pytest.raises(NotImplementedError):
        I.load_input(bad)
    with pytest.raises(NotImplementedError):
        I.load_input(dict(j, energy=[{"bonded": {}}]))


def test_state_round_trip():
    s = I.load_input(WATER)
    spec = s.spec
    st = I.state_json(s, spec.pos, spec.box, spec.mass_center)
    assert set(st) == {"geometry", "groups", "particles", "reactionlist", "implicit_reservoir"}
    assert st["groups"][0] == {"id": 0, "cm": list(spec.mass_center[0]), "atomic": False, "compressible": False,
                               "size": 3}
    assert st["particles"][1] == {"id": 1, "pos": list(spec.pos[1]), "q": 0.4238}
    s2 = I.load_input(WATER, seed=5)
    assert not np.array_equal(s2.spec.pos, spec.pos)
    I.apply_state(s2, json.loads(json.dumps(st)))
    assert np.array_equal(s2.spec.pos, spec.pos) and np.array_equal(s2.spec.mass_center, spec.mass_center)
    assert np.array_equal(s2.spec.group_flags, spec.group_flags)
    assert O.OracleSystem(s2.spec).energy_total() == O.OracleSystem(spec).energy_total()


def _bulk_example():
    fx = json.loads((GOLDEN / "bulk_example.json").read_text())
    z = np.load(GOLDEN / "bulk_example_state.npz")
    state = {"geometry": fx["geometry"], "groups": fx["groups"],
             "particles": [{"id": int(t), "pos": list(p), "q": float(q)} for t, p, q in zip(z["id"], z["pos"], z["q"])]}
    return fx, I.apply_state(I.load_input(fx["input"]), state)


def test_bulk_example_golden():
    """examples/bulk: fanourgakis Coulomb (epsr 1, Rc 14) + LB Lennard-Jones at 1100 K,
    2304 ions.  The Bjerrum length equals the reference's to the last digit; the
    nonbonded energy of the saved state agrees with the value the run reported to
    3.1e-4 (the reference splines S(q) with tolerance 0.005/lB per pair and this
    output comes from a 2019 build); the reported self energy is -lB q^2 / Rc per ion
    in that build, where the documented S'(0)/2 rule (src docs/_docs/energy.md:267-276)
    gives 7/8 of it for fanourgakis (S'(0) = -7/4)."""
    fx, s = _bulk_example()
    exp = fx["expected"]
    spec = s.spec
    assert spec.n == 2304 and spec.bjerrum_length == pytest.approx(exp["bjerrum_length"], rel=1e-15)
    e = O.OracleSystem(spec).energy_total()
    assert abs(e["nonbonded"] - exp["nonbonded"]) <= 5e-4 * abs(exp["nonbonded"])
    assert e["self"] == pytest.approx(7.0 / 8.0 * exp["self"], rel=1e-12)
    assert s.moves[0]["repeat"] == 1.0 and list(s.moves[0]["type_dp"]) == [1.0, 0.5]


def test_minimal_example_input():
    """examples/minimal: FunctorPotential default [LJ (LB), plain Coulomb epsr 80] on 20 NaCl
    at 300 K; the Bjerrum length equals the reference's reported value to the last digit."""
    fx = json.loads((GOLDEN / "minimal_example.json").read_text())
    s = I.load_input(fx["input"])
    assert s.spec.n == 40 and s.spec.pair_terms == A.FAU_PAIR_COULOMB | A.FAU_PAIR_LJ
    assert s.spec.coulomb_type == A.FAU_COUL_PLAIN
    assert s.spec.bjerrum_length == pytest.approx(fx["expected"]["bjerrum_length"], rel=1e-15)
    assert math.isfinite(O.OracleSystem(s.spec).energy_total()["total"])


_REFERENCE_EXAMPLES = Path(os.environ.get("FAUNUS_SOURCE", "")) / "examples"


@pytest.mark.skipif(not _REFERENCE_EXAMPLES.is_dir(), reason="set FAUNUS_SOURCE to a Faunus source tree")
def test_reference_example_inputs_load_or_name_what_is_missing():
    """Every example input of a Faunus tree that the YAML-subset reader parses either loads
    (its molecule .xyz structures read from beside it) or raises NotImplementedError naming
    the unsupported part -- never another error."""
    loaded, unsupported = [], []
    for f in sorted(_REFERENCE_EXAMPLES.rglob("*.yml")):
        try:
            yason.loads(f.read_text())
        except ValueError:
            continue  # templated (jinja) or block-scalar YAML: outside the reader's subset
        try:
            I.load_input(f)
            loaded.append(f.name)
        except NotImplementedError:
            unsupported.append(f.name)
    assert {"minimal.yml", "bulk.yml", "ewald.yml", "water.yml"} <= set(loaded)
    assert len(loaded) + len(unsupported) >= 30


def test_templates_rendered_as_the_reference_script_does():
    """The reference's yason.py renders inputs with jinja2 before YAML: `{% set %}` lines and
    `{{ expression }}` (arithmetic over the names set) render to Python's str() of the value."""
    text = "{% set N = 50 %}\n{% set eps = 0.05*2.5 %}\n{% set pH = 7.0 %}\n" \
           "a: {{2*N}}\nb: {{ eps }}\nc: [{{ 10**(-pH) }}, {{3/N}}]\nd: {N: {{ N }}}\n"
    assert yason.render(text).split("\n")[:2] == ["a: 100", "b: 0.125"]
    assert yason.loads(text) == {"a": 100, "b": 0.125, "c": [1e-07, 0.06], "d": {"N": 50}}
    with pytest.raises(ValueError):
        yason.loads("a: {{ undefined }}\n")
    with pytest.raises(ValueError):
        yason.loads("a: {% for i in range(3) %}Q{% endfor %}\n")
    with pytest.raises(ValueError):
        yason.loads("{% set x = __import__('os') %}\na: 1\n")
