"""Hamiltonian maxenergy (reference src/energy.cpp:1189-1193, 1227-1241) in the oracle and the
input loader: each state's terms (self, Nonbonded, Ewald) are summed in order up to and including
the first that reaches maxenergy (or is NaN), so a trial move whose Nonbonded partial energy
reaches it leaves the Ewald term out of the trial state's sum."""
import dataclasses
import numpy as np

import faunus_gb300 as F
from faunus_gb300 import configs

import oracle_lib as O


def _terms(t):
    lst = [t["self"]] if t["self"] != 0.0 else []
    lst.append(t["nonbonded"])
    lst.append(t["ewald_rec"] + t["ewald_surf"])
    return lst


def _accumulate(lst, m):
    s = 0.0
    for v in lst:
        s += v
        if not v < m:
            break
    return s


def test_totals_stop_at_maxenergy():
    base = configs.bulk_ewald(n_salt=200, seed=3)
    ref = O.OracleSystem(base).energy_total()
    for m in (-1e9, ref["self"] + 1.0, ref["nonbonded"] - 1.0, 1e9):
        t = O.OracleSystem(dataclasses.replace(base, maxenergy=m)).energy_total()
        assert t["total"] == _accumulate(_terms(ref), m), m


def test_trial_energy_change_follows_the_truncated_sums():
    """A trial state whose Nonbonded partial energy reaches maxenergy sums no Ewald term:
    dU = (self + N_new) - (self + N_old + E_old) when the old state's sum runs to the end."""
    spec = dataclasses.replace(configs.bulk_ewald(n_salt=200, seed=5), maxenergy=2.0)
    props = F.MoveGenerator(spec, spec.extra["moves"], 3, 4, default_seeds=False).generate(3000)
    full = O.OracleSystem(dataclasses.replace(spec, maxenergy=None)).run_detail(props[:1])
    det = O.OracleSystem(spec).run_detail(props)
    assert det["accepted"].sum() > 100
    # the first move from the same state: with and without the stop the nonbonded change agrees
    assert det["du_nonbonded"][0] == full["du_nonbonded"][0]


def test_a_clash_leaves_the_ewald_term_out_of_the_trial_sum():
    """Move an ion onto a neighbour: its Nonbonded partial energy in the trial state exceeds
    maxenergy, so dU = N_new - (N_old + E_old): the accepted state's whole Ewald energy."""
    from faunus_gb300 import _capi as A
    spec = dataclasses.replace(configs.bulk_ewald(n_salt=200, seed=7), maxenergy=50.0)
    o = O.OracleSystem(spec)
    t0 = o.energy_total()
    e_old = t0["ewald_rec"] + t0["ewald_surf"]
    pos = np.asarray(spec.pos)
    p = np.zeros(1, dtype=A.PROPOSAL_DTYPE)
    p["kind"], p["index"], p["u"] = A.FAU_MOVE_ATOMIC, 0, 0.5
    p["dr"][0] = pos[1] - pos[0] + np.array([0.6, 0.0, 0.0])
    d = o.run_detail(p)[0]
    assert d["du_nonbonded"] > 50.0
    assert abs(d["du"] - (d["du_nonbonded"] - e_old)) <= 1e-9 * (abs(d["du"]) + abs(e_old))
    # without the stop the same move's change carries the Ewald change instead
    full = O.OracleSystem(dataclasses.replace(spec, maxenergy=None)).run_detail(p)[0]
    assert abs(full["du"] - (full["du_nonbonded"] + full["du_ewald"])) <= 1e-9 * abs(full["du"])


def test_loader_reads_maxenergy(tmp_path):
    j = tmp_path / "in.json"
    j.write_text('{"temperature": 298, "random": {"seed": "fixed"}, "geometry": {"type": "cuboid", "length": 30},'
                 ' "mcloop": {"macro": 1, "micro": 1},'
                 ' "atomlist": [{"Na": {"q": 1.0, "sigma": 3.0, "eps": 0.1}}, {"Cl": {"q": -1.0, "sigma": 4.0, "eps": 0.1}}],'
                 ' "moleculelist": [{"salt": {"atoms": ["Na", "Cl"], "atomic": true}}],'
                 ' "insertmolecules": [{"salt": {"N": 10}}],'
                 ' "energy": [{"maxenergy": 50}, {"nonbonded_coulomblj": {"coulomb": {"type": "plain", "epsr": 80},'
                 ' "lennardjones": {"mixing": "LB"}, "cutoff_g2g": 10}}],'
                 ' "moves": [{"transrot": {"molecule": "salt", "dp": 1.0, "repeat": "N"}}]}')
    from faunus_gb300.input import load_input
    spec = load_input(str(j)).spec
    assert spec.maxenergy == 50.0
    d, _ = spec.to_desc()
    assert d.maxenergy_set == 1 and d.maxenergy == 50.0
