"""GPU parity of the truncated Coulomb schemes (FAU_COUL_TRUNC: e erfc(alpha r) +
polynomial in q = r/Rc) against the FP64 oracle: total energies with the
S'(0) self energy, chains of single-atom moves in the chain kernel and in the
pipelined kernel (reference-stream host proposals), and rigid-water molecular
moves with a reaction field.  Tolerance as in test_parity_gpu: 1e-6 of
max(|dU|, S), S the sum of |summand| magnitudes (for these forms
|qq/r| (|e| erfc + sum |c_k| q^k))."""
import dataclasses

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

import oracle_lib as O
from test_parity_gpu import TOL_FP32C, _compare_chain, _props
from test_pipelined_gpu import _energy_consistent, _oracle_compare

pytestmark = pytest.mark.gpu

SCHEMES = {
    "wolf": dict(alpha=0.2),
    "fennell": dict(alpha=0.2),
    "zerodipole": dict(alpha=0.2),
    "zahn": dict(alpha=0.2),
    "fanourgakis": {},
    "qpotential": dict(order=3),
    "poisson": dict(C=3, D=3),
    "reactionfield": dict(epsrf=2000.0),
}


def _salt(name, seed=4):
    spec = configs.bulk_ewald(n_salt=1000, molar=1.0, seed=seed)
    f = F.coulomb_scheme(name, epsr=80.0, cutoff=12.0, **SCHEMES[name])
    return dataclasses.replace(spec, ewald=None, **f)


@pytest.mark.parametrize("name", sorted(SCHEMES))
def test_total_energy_matches_oracle(ctx, name):
    spec = _salt(name)
    eg = ctx.create(spec).energy_total()
    eo = O.OracleSystem(spec).energy_total()
    assert eo["self"] < 0.0  # S'(0) < 0 for every scheme here
    for key in ("self", "nonbonded", "total"):
        assert abs(eg[key] - eo[key]) <= 1e-9 * max(1.0, abs(eo[key])), (key, eg[key], eo[key])


@pytest.mark.parametrize("name", sorted(SCHEMES))
def test_chain_kernel_matches_oracle(ctx, name):
    spec = _salt(name)
    rep, _ = _compare_chain(ctx.create(spec), spec, _props(spec, 2000), TOL_FP32C)
    assert rep["accepted"] > 100


def test_pipelined_kernel_matches_oracle(ctx):
    names = sorted(SCHEMES)
    specs = [_salt(n, seed=10 + i) for i, n in enumerate(names)]
    systems = [ctx.create(s) for s in specs]
    M = 2000
    props = [F.MoveGenerator(s, s.extra["moves"], 41 + i, 43 + i, default_seeds=False).generate(M)
             for i, s in enumerate(specs)]
    allp = np.concatenate(props)
    off = np.arange(len(specs) + 1, dtype=np.int64) * M
    acc = np.zeros(len(allp), np.uint8)
    du = np.zeros(len(allp))
    st = ctx.run_proposals_batch(systems, allp, off, acc, du)
    assert st["moves"] == len(allp)
    for i, (s, spec) in enumerate(zip(systems, specs)):
        sl = slice(i * M, (i + 1) * M)
        assert _oracle_compare(s.positions(), acc[sl], du[sl], spec, props[i]) > 100
        _energy_consistent(s)


def test_water_reaction_field_molecular_moves(ctx):
    w = configs.spce_water(n_mol=256, L=18.6)
    f = F.coulomb_scheme("reactionfield", epsr=1.0, cutoff=9.0, epsrf=80.0, temperature=300.0)
    w = dataclasses.replace(w, ewald=None, **f)
    _compare_chain(ctx.create(w), w, _props(w, 2000), TOL_FP32C)
