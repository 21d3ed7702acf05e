"""A finite Hamiltonian maxenergy on the GPU (reference src/energy.cpp:1227-1241): systems with it
run in the chain kernel, which forms each state's term sums -- the trial state's Nonbonded
partial energy and the accepted state's Ewald energy beside the energy change -- and stops each
sum at the first term that reaches maxenergy.  The accept sequence and dU equal the FP64
oracle's, to the parity tolerance, on a bulk Ewald system where about half of the trial
states stop before their Ewald term; batched runs take the chain kernel for such systems."""
import dataclasses

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

import oracle_lib as O
from test_parity_gpu import TOL_FP32C, _compare_chain, _props

pytestmark = pytest.mark.gpu


def _spec(m=0.0):
    return dataclasses.replace(configs.bulk_ewald(n_salt=500, seed=8), maxenergy=m)


def test_maxenergy_chain_matches_oracle(ctx):
    spec = _spec()
    props = _props(spec, 3000, seeds=(21, 23))
    det = O.OracleSystem(spec).run_detail(props)
    fin = np.isfinite(det["du"])
    truncated = np.abs(det["du"] - (det["du_nonbonded"] + det["du_ewald"])) > 1e-6 * np.maximum(1.0, np.abs(det["du"]))
    assert truncated[fin].sum() > 100  # the stop matters in this run
    rep, _ = _compare_chain(ctx.create(spec), spec, props, TOL_FP32C, label="maxenergy bulk")
    assert rep["first_mismatch"] > 1000 and rep["accepted"] > 100


def test_batched_systems_with_maxenergy_take_the_chain_kernel(ctx):
    spec = _spec()
    a, b = ctx.create(spec), ctx.create(spec)
    ctx.run_batch([a], 2000, seed=4, dp=2.0, threads=0)
    ctx.run_batch([b], 2000, seed=4, dp=2.0, threads=256)
    assert np.array_equal(a.positions(), b.positions()) and a.running_energy() == b.running_energy()
    # the energy total follows the same stop
    t = a.energy_total()
    assert np.isfinite(t["total"])
