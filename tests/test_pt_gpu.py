"""Parallel tempering on the device against its definition, decision by decision.

ParallelTempering::_move (reference src/move.cpp:883-923) with OddEvenPartner::generate
(src/mpicontroller.cpp:69-83): in each round the walkers at temperature slots (s, s + 1),
s = parity, parity + 2, ..., propose to exchange configurations; the exchange is accepted by
metropolisCriterion (src/montecarlo.cpp:17-34) on the sum of both walkers' energy changes,
each in its own kT.  The device exchanges temperatures instead of configurations.

The tests recompute every swap decision on the host from the record fau_run_batch returns
(each walker's running energy at the round, the slot order after it) with an independent
Philox4x32-10, and check that a walker's chain under tempering is, move for move, the chain
of the same walker run alone block by block at the temperatures the record gives it.
"""
import math

import numpy as np
import pytest

from faunus_gb300 import configs

pytestmark = pytest.mark.gpu

M32 = 0xFFFFFFFF


def philox4x32_10(ctr, k0, k1):
    """Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC'11) with its published constants."""
    c0, c1, c2, c3 = ctr
    for _ in range(10):
        p0 = 0xD2511F53 * c0
        p1 = 0xCD9E8D57 * c2
        hi0, lo0 = p0 >> 32, p0 & M32
        hi1, lo1 = p1 >> 32, p1 & M32
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & M32, lo1, (hi0 ^ c3 ^ k1) & M32, lo0
        k0 = (k0 + 0x9E3779B9) & M32
        k1 = (k1 + 0xBB67AE85) & M32
    return c0, c1, c2, c3


def u01_53(a, b):
    return float(((a >> 5) << 26) | (b >> 6)) * 2.0 ** -53


def recompute_swaps(slots_log, energy_log, temps, tref, seed, round0):
    """Replays every round from the record; returns (attempted, accepted)."""
    n = len(temps)
    key = seed ^ 0x5DEECE66D
    k0, k1 = key & M32, (key >> 32) & M32
    slots = list(range(n))
    attempted = accepted = 0
    for b in range(len(slots_log)):
        r = round0 + b
        parity = philox4x32_10((r & M32, r >> 32, M32, 7), k0, k1)[0] & 1
        E = energy_log[b]
        for s in range(parity, n - 1, 2):
            a, c = slots[s], slots[s + 1]
            x = (1.0 / temps[s] - 1.0 / temps[s + 1]) * (E[a] * tref[a] - E[c] * tref[c])
            w = philox4x32_10((r & M32, r >> 32, s, 8), k0, k1)
            u = u01_53(w[0], w[1])
            attempted += 1
            # metropolisCriterion on dU = -x: u <= exp(-dU)
            if x >= 0.0 or (not math.isnan(x) and u <= math.exp(x)):
                accepted += 1
                slots[s], slots[s + 1] = c, a
        assert slots == [int(v) for v in slots_log[b]], f"round {r}: device slots differ from the recomputed ones"
    return attempted, accepted


def _ladder(n_rep=8, n_min=100, n_max=300, seed=3):
    specs, temps = configs.pt_replicas(n_rep=n_rep, n_min=n_min, n_max=n_max, seed=seed)
    return specs, np.asarray(temps, dtype=np.float64)


@pytest.mark.parametrize("threads", [0, 128])
def test_every_swap_decision_recomputed(ctx, threads):
    specs, temps = _ladder()
    systems = [ctx.create(s) for s in specs]
    nblk = 12
    st = ctx.run_batch(systems, swap_interval=300, n_swap_blocks=nblk, temperatures=temps, seed=11, dp=2.0,
                       threads=threads, swap_log=True)
    att, acc = recompute_swaps(st["swap_slots"], st["swap_energy"], temps, temps, 11, 0)
    assert (att, acc) == (st["swaps_attempted"], st["swaps_accepted"])
    assert acc > 0 and att >= nblk * 3
    # the last round's energies are the walkers' final running energies (no moves after it)
    for i, s in enumerate(systems):
        assert st["swap_energy"][-1][i] == s.running_energy()


def test_sweep_blocks_equal_walkers_run_alone(ctx):
    """Block lengths in sweeps (moves_per_system = sweeps x N_i): each walker's PT chain equals
    the same walker run alone, block by block, at the temperature the record assigns it."""
    specs, temps = _ladder(n_rep=6, n_min=100, n_max=400, seed=5)
    sweeps = 3
    lens = np.array([sweeps * s.n for s in specs], np.int64)
    pt_sys = [ctx.create(s) for s in specs]
    nblk = 3
    mo = np.zeros(len(specs), np.int64)
    st = ctx.run_batch(pt_sys, moves_per_system=lens, swap_interval=1, n_swap_blocks=nblk, temperatures=temps,
                       seed=21, dp=2.0, threads=0, swap_log=True, moves_out=mo)
    assert st["moves"] == nblk * int(lens.sum())
    assert np.array_equal(mo, nblk * lens)
    recompute_swaps(st["swap_slots"], st["swap_energy"], temps, temps, 21, 0)
    # the same walkers alone: block b at the temperature of the slot the walker held after round b-1
    alone = [ctx.create(s) for s in specs]
    slot_of = {i: i for i in range(len(specs))}
    for b in range(nblk):
        for i, s in enumerate(alone):
            s.set_temperature_scale(temps[i] / temps[slot_of[i]])
            ctx.run_batch([s], int(lens[i]), seed=21, streams=[i], counters=[b * int(lens[i])], dp=2.0, threads=0)
        slot_of = {int(sysid): slot for slot, sysid in enumerate(st["swap_slots"][b])}
    for i in range(len(specs)):
        assert np.array_equal(pt_sys[i].positions(), alone[i].positions()), f"walker {i}"
        assert pt_sys[i].running_energy() == alone[i].running_energy()
