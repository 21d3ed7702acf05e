"""fau_volume_move on the GPU against the FP64 oracle: the same accept sequence, bit-identical
boxes and positions (the scaling is IEEE-exact FP64 on both sides), dU within 1e-9 of the
Isobaric-inclusive energy scale, counters carried, and chains of trial moves after volume moves
(cell grids and k-vector amplitudes rebuilt for the new box) still at parity with the oracle."""
import dataclasses

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

import oracle_lib as O
from test_parity_gpu import TOL_FP32C, _compare_chain, _props

pytestmark = pytest.mark.gpu

METHODS = {"isotropic": 0, "xy": 1, "z": 2}


@pytest.mark.parametrize("kind", ["bulk", "pm", "water"])
def test_volume_moves_match_oracle(ctx, kind):
    if kind == "bulk":
        spec = configs.bulk_ewald(n_salt=1000, molar=1.0, seed=3)
    elif kind == "pm":
        spec = configs.primitive_model(n=200, seed=2)
    else:
        spec = configs.spce_water(n_mol=256, L=18.6, seed=5)
    spec = dataclasses.replace(spec, isobaric_pressure=F.pressure_kt(1.0, "P/atm"))
    g, o = ctx.create(spec), O.OracleSystem(spec)
    rng = np.random.default_rng(9)
    grids = {g.cell_grid()}
    n_acc = 0
    for k in range(12):
        v = float(np.prod(g.box()))
        v_new = float(np.exp(np.log(v) + (rng.random() - 0.5) * 0.3))
        method = ["isotropic", "xy", "z"][k % 3]
        u = float(rng.random())
        rg = g.volume_move(v_new, u, method=method)
        ro = o.volume_move(v_new, METHODS[method], u)
        assert rg["accepted"] == ro["accepted"]
        assert abs(rg["du"] - ro["du"]) <= 1e-9 * ro["err_scale"], (rg, ro)
        assert np.array_equal(g.box(), o.box())
        assert np.array_equal(g.positions(), o.positions())
        n_acc += rg["accepted"]
        grids.add(g.cell_grid())
        e_run = g.running_energy()
        assert abs(e_run - o.energy_total()["total"]) <= 1e-9 * max(1.0, abs(e_run))
    assert 0 < n_acc < 12
    c = g.counters()
    assert c["moves"] == 12 and c["accepted"] == n_acc
    # trial moves after the volume moves
    props = _props(spec, 1500, seeds=(5, 7))
    acc_g, du_g, _ = g.run_proposals(props)
    det = o.run_detail(props)
    first = int(np.argmax(acc_g != det["accepted"])) if (acc_g != det["accepted"]).any() else len(props)
    fin = np.isfinite(det["du"][:first])
    err = np.abs(du_g[:first][fin] - det["du"][:first][fin])
    den = np.maximum(np.abs(det["du"][:first][fin]), det["err_scale"][:first][fin])
    assert (err <= TOL_FP32C * np.where(den > 0, den, 1.0)).all()
    assert first > len(props) // 10
    if kind == "bulk":
        assert len(grids) > 1  # the cell grid followed the box


def test_rejected_volume_move_keeps_the_system(ctx):
    spec = dataclasses.replace(configs.bulk_ewald(n_salt=500, molar=1.0, seed=6), isobaric_pressure=1e3)
    g = ctx.create(spec)
    pos, box, e = g.positions(), g.box(), g.running_energy()
    r = g.volume_move(float(np.prod(box)) * 1.5, 0.5)
    assert r["accepted"] == 0
    assert np.array_equal(g.positions(), pos) and np.array_equal(g.box(), box) and g.running_energy() == e
    _compare_chain(g, spec, _props(spec, 1000), TOL_FP32C)


def test_volume_move_argument_errors(ctx):
    g = ctx.create(configs.primitive_model(n=50))
    with pytest.raises(F.FauError):
        g.volume_move(-1.0, 0.5)
    with pytest.raises(KeyError):
        g.volume_move(1e5, 0.5, method="sphere")


@pytest.mark.parametrize("precision", [0, 1])
def test_npt_reference_stream_matches_oracle(ctx, precision):
    """moltransrot + volume moves drawn from the reference stream (examples/water/ewald.yml's
    move set at a smaller size), run through fau_run_proposals: the stream is split at every
    volume move; accept sequence, dU, box and positions follow the oracle."""
    spec = configs.spce_water(n_mol=256, L=18.6, seed=5, precision=precision)
    spec = dataclasses.replace(spec, isobaric_pressure=F.pressure_kt(1.0, "P/atm", 300.0))
    spec.extra["moves"] = spec.extra["moves"] + [{"kind": 2, "repeat": 1, "dV": 0.03, "method": "isotropic"}]
    props = F.MoveGenerator(spec, spec.extra["moves"], 3, 4, default_seeds=False).generate(3000)
    vol = props["kind"] == 2
    assert vol.sum() > 3
    g, o = ctx.create(spec), O.OracleSystem(spec)
    acc_g, du_g, st = g.run_proposals(props)
    det = o.run_detail(props)
    mism = np.nonzero(acc_g != det["accepted"])[0]
    first = int(mism[0]) if len(mism) else len(props)
    sl = slice(0, first)
    tol = np.where(vol[sl], 1e-9, TOL_FP32C if precision == 0 else 1e-10)
    den = np.maximum(np.abs(det["du"][sl]), det["err_scale"][sl])
    fin = np.isfinite(det["du"][sl])
    assert (np.abs(du_g[sl] - det["du"][sl])[fin] <= (tol * np.where(den > 0, den, 1.0))[fin]).all()
    assert acc_g[vol].sum() > 0
    if first == len(props):
        assert np.array_equal(g.box(), o.box())
        assert np.array_equal(g.positions(), o.positions())
    else:
        assert first > len(props) // 10
