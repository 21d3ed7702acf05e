"""VolumeMove + Isobaric in the FP64 oracle (src/move.cpp:994-1006, src/energy.cpp:884-901,
src/space.cpp:249-301): the accepted state equals a system built afresh from positions scaled
as Space::scaleVolume (restated here with numpy), dU is the Hamiltonian change plus the
Isobaric change P dV - (N + 1) ln(V'/V), rigid molecules keep their geometry, and a rejected
move leaves the state untouched.  Pressure units follow src/units.h:162-190."""
import dataclasses
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O


def test_pressure_units():
    kT = 1.380658e-23 * 298.15
    assert F.pressure_kt(1.0, "P/kT") == 1.0
    assert F.pressure_kt(1.0, "P/Pa") == pytest.approx(1.0 / kT / 1e30, rel=1e-15)
    assert F.pressure_kt(2.0, "P/atm") == pytest.approx(2 * 101325.0 / kT / 1e30, rel=1e-15)
    assert F.pressure_kt(1.0, "P/bar") == pytest.approx(1e5 / kT / 1e30, rel=1e-15)
    assert F.pressure_kt(1.0, "P/mM") == pytest.approx(6.022137e23 * 1e-3 / 1e27, rel=1e-15)
    with pytest.raises(ValueError):
        F.pressure_kt(1.0, "P/psi")


def _wrap(p, L):
    out = p.copy()
    big = np.abs(out) > 0.5 * L
    t = out / L
    n = np.where(t > 0, np.trunc(t + 0.5), np.trunc(t - 0.5))
    return np.where(big, out - L * n, out)


def _scaled_spec(spec, pos, cm, L, method, v_new):
    """Space::scaleVolume restated: atomic groups scale positions, molecular groups move
    rigidly with their scaled mass centre; everything wrapped into the new box."""
    v_old = float(np.prod(L))
    a = {"isotropic": np.full(3, np.cbrt(v_new / v_old)), "xy": np.array([np.sqrt(v_new / v_old)] * 2 + [1.0]),
         "z": np.array([1.0, 1.0, v_new / v_old])}[method]
    Ln = L * a
    new_pos, new_cm = pos.copy(), cm.copy()
    gb = spec.group_begin
    for g in range(spec.n_groups):
        b, e = gb[g], gb[g + 1]
        if spec.group_flags[g] & A.FAU_GROUP_ATOMIC:
            new_pos[b:e] = _wrap(pos[b:e] * a, Ln)
        else:
            c = _wrap(cm[g] * a, Ln)
            d = pos[b:e] - cm[g]
            d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
            new_pos[b:e] = _wrap(cm[g] + d + (c - cm[g]), Ln)
            new_cm[g] = c
    return dataclasses.replace(spec, box=Ln, pos=new_pos, mass_center=new_cm), Ln


def _n_count(spec):
    return sum((spec.group_begin[g + 1] - spec.group_begin[g]) if spec.group_flags[g] & A.FAU_GROUP_ATOMIC else 1
               for g in range(spec.n_groups))


@pytest.mark.parametrize("kind,method", [("bulk", "isotropic"), ("pm", "xy"), ("water", "isotropic"),
                                         ("water", "z")])
def test_oracle_volume_move_equals_fresh_state(kind, method):
    if kind == "bulk":
        spec = configs.bulk_ewald(n_salt=200, molar=0.5, seed=3)
    elif kind == "pm":
        spec = configs.primitive_model(n=100, seed=2)
    else:
        spec = configs.spce_water(n_mol=64, L=12.4, seed=5)
    P = F.pressure_kt(1.0, "P/atm")
    spec = dataclasses.replace(spec, isobaric_pressure=P)
    o = O.OracleSystem(spec)
    pos, cm, L = o.positions(), o.mass_centers(), o.box()
    v_old = float(np.prod(L))
    v_new = v_old * 1.02
    e_old = o.energy_total()["total"]
    r = o.volume_move(v_new, {"isotropic": 0, "xy": 1, "z": 2}[method], 0.0)  # u = 0: always accepted
    assert r["status"] == 0 and r["accepted"] == 1
    fresh, Ln = _scaled_spec(spec, pos, cm, L, method, v_new)
    assert np.array_equal(o.box(), Ln)
    assert np.array_equal(o.positions(), fresh.pos)
    e_new = O.OracleSystem(fresh).energy_total()["total"]
    assert o.energy_total()["total"] == pytest.approx(e_new, rel=1e-12)
    N = _n_count(spec)
    iso = P * (np.prod(Ln) - v_old) - (N + 1) * math.log(np.prod(Ln) / v_old)
    assert r["du"] == pytest.approx((e_new - e_old) + iso, rel=1e-9, abs=1e-9 * abs(e_old))
    if kind == "water":  # rigid molecules keep their internal geometry
        p0, p1 = pos.reshape(-1, 3, 3), o.positions().reshape(-1, 3, 3)
        d0 = p0[:, 1:] - p0[:, :1]
        d1 = p1[:, 1:] - p1[:, :1]
        d0 -= L * np.round(d0 / L)
        d1 -= Ln * np.round(d1 / Ln)
        assert np.allclose(np.linalg.norm(d0, axis=-1), np.linalg.norm(d1, axis=-1), atol=1e-12)


def test_oracle_rejected_volume_move_leaves_state():
    spec = dataclasses.replace(configs.bulk_ewald(n_salt=100, molar=0.5, seed=4), isobaric_pressure=1e3)
    o = O.OracleSystem(spec)
    pos, L, e = o.positions(), o.box(), o.energy_total()["total"]
    r = o.volume_move(np.prod(L) * 1.5, 0, 0.5)  # P dV is huge: rejected
    assert r["accepted"] == 0 and r["du"] > 100
    assert np.array_equal(o.positions(), pos) and np.array_equal(o.box(), L)
    assert o.energy_total()["total"] == e


def test_without_isobaric_term_du_is_the_hamiltonian_change():
    spec = configs.primitive_model(n=100, seed=7)
    o = O.OracleSystem(spec)
    e0 = o.energy_total()["total"]
    r = o.volume_move(float(np.prod(o.box())) * 1.01, 0, 0.0)
    assert r["accepted"] == 1
    assert r["du"] == pytest.approx(o.energy_total()["total"] - e0, rel=1e-12, abs=1e-12)


def _npt_water(n_mol=64, L=12.4):
    spec = configs.spce_water(n_mol=n_mol, L=L, seed=5)
    spec = dataclasses.replace(spec, isobaric_pressure=F.pressure_kt(1.0, "P/atm", 300.0))
    moves = spec.extra["moves"] + [{"kind": A.FAU_MOVE_VOLUME, "repeat": 1, "dV": 0.03, "method": "isotropic"}]
    spec.extra["moves"] = moves
    return spec


def test_movegen_volume_stream_matches_oracle_generator():
    """fau_movegen and the oracle's generator draw volume moves in the same place of the
    reference stream (MoveCollection::sample, then one slump() for ln V, then the
    Metropolis uniform)."""
    spec = _npt_water()
    gen = F.MoveGenerator(spec, spec.extra["moves"], 3, 4, default_seeds=False)
    props = gen.generate(3000)
    vol = props["kind"] == A.FAU_MOVE_VOLUME
    assert 20 < vol.sum() < 100  # weight 1 against 64
    assert (np.abs(props["dr"][vol, 0]) <= 0.015).all()
    o = O.OracleSystem(spec)
    og = O.OracleMoveGen(o, spec.extra["moves"], 3, 4, default_seeds=False)
    assert np.array_equal(og.generate(3000), props)


def test_oracle_npt_loop_equals_proposal_replay():
    spec = _npt_water()
    a, b = O.OracleSystem(spec), O.OracleSystem(spec)
    ga = O.OracleMoveGen(a, spec.extra["moves"], 3, 4, default_seeds=False)
    acc_loop, _, _ = ga.mc_run(800)
    props = F.MoveGenerator(spec, spec.extra["moves"], 3, 4, default_seeds=False).generate(800)
    det = b.run_detail(props)
    assert np.array_equal(det["accepted"].astype(np.uint8), acc_loop)
    assert np.array_equal(a.positions(), b.positions()) and np.array_equal(a.box(), b.box())
    assert not np.array_equal(b.box(), spec.box)  # some volume move was accepted
