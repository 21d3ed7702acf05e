"""Ensemble averages of the batched device chains against the FP64 oracle.

The device runs 64 independent replicas of the primitive model (200 hard-sphere
ions, Coulomb + WCA) with its counter-based RNG in the pipelined chain kernel;
the oracle runs one long chain with the reference's mt19937 move stream.  They
share no random numbers, only the Boltzmann distribution, so the test is
statistical (SystemEnergy / AtomRDF observables, src/analysis.cpp:339-357,
1570-1600): the mean energy and the radial distribution g(r) must agree within
their combined standard errors (4 sigma for <U>, a chi-square bound for g(r)).
"""
import math

import numpy as np
import pytest

from faunus_gb300 import configs

import oracle_lib as O

pytestmark = pytest.mark.gpu

EDGES = np.arange(4.0, 20.5, 1.0)  # angstrom


def _rdf(configs_xyz, L):
    """g(r) per configuration (rows), minimum image, ideal-gas normalisation
    (PairFunction::_to_disk: g = N <V> / (4 pi r^2 dr sum N))."""
    out = []
    for x in configs_xyz:
        n = len(x)
        d = x[:, None, :] - x[None, :, :]
        d -= L * np.round(d / L)
        r = np.sqrt((d * d).sum(-1))[np.triu_indices(n, 1)]
        h, _ = np.histogram(r, bins=EDGES)
        shell = 4.0 / 3.0 * math.pi * (EDGES[1:] ** 3 - EDGES[:-1] ** 3)
        out.append(h / (0.5 * n * (n - 1) * shell / L ** 3))
    return np.array(out)


def test_ensemble_energy_and_rdf_match_oracle(ctx):
    spec = configs.primitive_model(n=200, seed=11)
    L = float(spec.box[0])
    R, block, n_eq, n_samp = 64, 1000, 20, 40
    base = ctx.create(spec)
    systems = [base] + [base.clone() for _ in range(R - 1)]
    E = np.zeros((n_samp, R))
    g_dev = []
    for b in range(n_eq + n_samp):
        ctx.run_batch(systems, block, seed=5, streams=np.arange(R), counters=[b * block] * R, dp=2.0, threads=0)
        if b >= n_eq:
            E[b - n_eq] = [s.running_energy() for s in systems]
            if (b - n_eq) % 10 == 9:
                g_dev.append(_rdf([s.positions() for s in systems], L))
    rep_mean = E.mean(0)  # one mean per independent replica
    mu_d, se_d = rep_mean.mean(), rep_mean.std(ddof=1) / math.sqrt(R)
    g_rep = np.mean(g_dev, axis=0)  # (R, bins): per-replica g(r)
    gd, gd_se = g_rep.mean(0), g_rep.std(0, ddof=1) / math.sqrt(R)

    o = O.OracleSystem(spec)
    gen = O.OracleMoveGen(o, spec.extra["moves"], 3, 4, default_seeds=False)
    gen.mc_run(n_eq * block)
    n_blocks, per = 40, 20  # 800 samples in 40 blocks of 20 (100 sweeps each)
    e_blk, g_blk = [], []
    for _ in range(n_blocks):
        es, xs = [], []
        for k in range(per):
            gen.mc_run(block)
            es.append(o.energy_total()["total"])
            if k % 4 == 3:
                xs.append(o.positions())
        e_blk.append(np.mean(es))
        g_blk.append(_rdf(xs, L).mean(0))
    e_blk, g_blk = np.array(e_blk), np.array(g_blk)
    mu_o, se_o = e_blk.mean(), e_blk.std(ddof=1) / math.sqrt(n_blocks)
    go, go_se = g_blk.mean(0), g_blk.std(0, ddof=1) / math.sqrt(n_blocks)

    # <U>: the two estimates of the same ensemble average agree within 4 combined sigma
    z = (mu_d - mu_o) / math.sqrt(se_d ** 2 + se_o ** 2)
    assert abs(z) < 4.0, (mu_d, se_d, mu_o, se_o)
    # g(r): chi-square over the bins, well below a 3-sigma excess for this many bins
    chi2 = float((((gd - go) ** 2) / (gd_se ** 2 + go_se ** 2)).sum())
    nb = len(gd)
    assert chi2 < nb + 4 * math.sqrt(2 * nb) + 6, (chi2, gd, go)
    # the structure is not trivial: depletion at contact is resolved, long range tends to 1
    assert abs(go[-1] - 1.0) < 0.1 and abs(gd[-1] - 1.0) < 0.1
