"""Statistical golden fixture: the reference's examples/minimal run (20 NaCl, FunctorPotential
[Lennard-Jones LB + plain Coulomb epsr 80], 50 A box, 300 K) reports a SystemEnergy mean of
-16.034 kT over 500 samples (one chain, 2e6 transrot moves).  The same input, loaded by
faunus_gb300.input, runs as 608 independent device chains (device RNG: a different stream,
the same ensemble) with SystemEnergy sampled on the device between blocks of 100 sweeps; the
ensemble mean must agree within the fixture's 2 % tolerance (the reference's own estimate comes
from one correlated chain)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import input as I

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).parent / "golden"


def test_minimal_example_mean_energy(ctx):
    fx = json.loads((GOLDEN / "minimal_example.json").read_text())
    setup = I.load_input(fx["input"], seed=1)
    R, sweep = 608, 40
    base = ctx.create(setup.spec)
    reps = [base] + [base.clone() for _ in range(R - 1)]
    dp = float(setup.moves[0]["type_dp"][0])
    ctx.run_batch(reps, 500 * sweep, seed=11, dp=dp)  # equilibration from the random insertion
    smp = F.Sampler(ctx, n_slots=R, energy=True)
    st = ctx.run_batch(reps, seed=11, dp=dp, counter_base=500 * sweep, sampler=smp, sample_interval=100 * sweep,
                       n_sample_blocks=40)
    assert st["moves"] == R * 40 * 100 * sweep
    d = smp.read()
    assert (d["energy_samples"] == 40).all()
    per_rep = d["energy_sum"] / d["energy_samples"]
    mean, se = per_rep.mean(), per_rep.std(ddof=1) / math.sqrt(R)
    ref = fx["expected"]["systemenergy_mean"]
    assert abs(mean - ref) <= 0.02 * abs(ref), (mean, se, ref)
    acc = st["accepted"] / st["moves"]
    assert abs(acc - fx["expected"]["acceptance"]) < 0.05, acc  # reference: 0.651
