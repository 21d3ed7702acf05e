"""Input files through the device path: the reference's examples/bulk state on the GPU
(total energy against the oracle and the reference's reported value), and ``simulate``
runs of input files -- the primitive model in both RNG modes and rigid water under
constant pressure (moltransrot + volume moves) in the reference-stream mode, whose
final state equals the oracle's run of the same move stream."""
import dataclasses
import json

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import input as I
from faunus_gb300.run import simulate

import oracle_lib as O
from test_input import PM, WATER, _bulk_example

pytestmark = pytest.mark.gpu


def test_bulk_example_on_device(ctx):
    fx, s = _bulk_example()
    g = ctx.create(s.spec)
    eg, eo = g.energy_total(), O.OracleSystem(s.spec).energy_total()
    for k in ("self", "nonbonded", "total"):
        assert abs(eg[k] - eo[k]) <= 1e-9 * abs(eo[k])
    assert abs(eg["nonbonded"] - fx["expected"]["nonbonded"]) <= 5e-4 * abs(fx["expected"]["nonbonded"])


@pytest.mark.parametrize("mode", ["reference", "batch"])
def test_simulate_primitive_model(ctx, tmp_path, mode):
    text = PM.replace("    - systemenergy: {file: energy.dat, nstep: 10}",
                      "    - systemenergy: {file: energy.dat, nstep: 2}\n"
                      "    - atomrdf: {name1: Na+, name2: Cl-, nstep: 2, file: rdf.dat, dr: 0.5}\n"
                      "    - savestate: {file: state.json}")
    text = text.replace("    - transrot: {molecule: chloride, repeat: 5}", "    - transrot: {molecule: chloride, repeat: N}")
    text = text.replace("r: 2.5, dp: 10", "r: 2.5, dp: 20")
    setup = I.load_input(text, seed=3)
    res = simulate(setup, ctx, out_dir=tmp_path, mode=mode, macro=2, micro=5)
    assert res["moves"]["attempted"] == 2 * 5 * 60
    if np.isfinite(res["energy"]["initial"]):
        assert abs(res["relative drift"]) < 1e-9
    else:  # random insertion left hard-sphere overlaps: the reference reports NaN too
        assert np.isnan(res["relative drift"]) and np.isfinite(res["energy"]["final"])
    en = res["analysis"][0]["systemenergy"]
    assert en["samples"] == 5 and np.isfinite(en["mean"])
    assert res["analysis"][1]["atomrdf"]["samples"] == 5
    rdf = np.loadtxt(tmp_path / "rdf.dat")
    assert rdf.shape[1] == 2 and (rdf[:, 1] >= 0).all()
    st = json.loads((tmp_path / "state.json").read_text())
    again = I.apply_state(I.load_input(text, seed=9), st)
    g = ctx.create(again.spec)
    assert g.energy_total()["total"] == pytest.approx(res["energy"]["final"], rel=1e-12)


def test_simulate_water_npt_matches_oracle(ctx, tmp_path):
    text = WATER + "analysis:\n    - savestate: {file: state.json}\n"
    setup = I.load_input(text, seed=4)
    res = simulate(setup, ctx, out_dir=tmp_path, mode="reference", seed=7, macro=1, micro=4)
    st = json.loads((tmp_path / "state.json").read_text())
    # the same stream through the oracle
    spec = setup.spec
    props = F.MoveGenerator(spec, setup.moves, 7, 8, default_seeds=True).generate(4 * 65)
    o = O.OracleSystem(spec)
    det = o.run_detail(props)
    assert res["moves"]["attempted"] == len(props)
    assert res["moves"]["accepted"] == int(det["accepted"].sum())
    assert np.array_equal(np.array(st["geometry"]["length"]), o.box())
    assert np.array_equal(np.array([p["pos"] for p in st["particles"]]), o.positions())
