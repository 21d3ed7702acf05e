"""A chain split into several launches evolves exactly as in one launch: the accepted Q(k)
changes not yet flushed into the FP64 master (and the last accepted move's change) are kept
in device memory across launches, so each kernel resumes as its next move would.  Positions,
mass centres, acceptance counts, the running energy (the pipelined kernel's float-float
partial sum stays unfolded across launches too) and Q(k) are bit-identical between one launch
of 3,000 moves and launches of 1,000 + 500 + 1,500 moves, for the pipelined single-atom kernel,
the chain kernel and the molecular kernel."""
import numpy as np
import pytest

from faunus_gb300 import configs

pytestmark = pytest.mark.gpu

CASES = {
    "pipelined_bulk": (lambda: configs.bulk_ewald(n_salt=1000, seed=4), dict(dp=2.0, threads=160)),
    "chain_bulk": (lambda: configs.bulk_ewald(n_salt=1000, seed=5), dict(dp=2.0, threads=256)),
    # fixed widths: with threads 0 a launch of one molecular chain takes 512-thread CTAs and a
    # time-budgeted one 256, and the width sets the FP32 summation order
    "molecular_water": (lambda: configs.spce_water(n_mol=256, L=18.6, seed=6), dict(dp=0.5, dprot=0.5, threads=160)),
    "molecular_water_512": (lambda: configs.spce_water(n_mol=256, L=18.6, seed=6),
                            dict(dp=0.5, dprot=0.5, threads=512)),
    "chain_water": (lambda: configs.spce_water(n_mol=256, L=18.6, seed=7), dict(dp=0.5, dprot=0.5, threads=256)),
    # 4 x 4 x 4 mass-centre cells: the lists rebuilt at each launch equal the ones kept current
    "molecular_water_cells": (lambda: configs.spce_water(n_mol=4000, L=49.3, seed=8),
                              dict(dp=0.5, dprot=0.5, threads=160)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_launch_segmentation_is_invisible(ctx, case):
    make, kw = CASES[case]
    spec = make()
    a, b = ctx.create(spec), ctx.create(spec)
    ctx.run_batch([a], 3000, seed=9, **kw)
    c = 0
    for m in (1000, 500, 1500):
        ctx.run_batch([b], m, seed=9, counter_base=c, **kw)
        c += m
    assert a.counters()["accepted"] == b.counters()["accepted"]
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.mass_centers(), b.mass_centers())
    assert a.running_energy() == b.running_energy()
    assert np.array_equal(a.q(), b.q())  # fau_get_q folds the pending changes the same way for both


@pytest.mark.parametrize("name", sorted(CASES))
def test_time_budgeted_launches_are_invisible(ctx, name):
    """Launches cut short by a device-time budget continue exactly where they stopped:
    repeated until done, they end bit-identical to one launch; moves_out reports each
    system's moves."""
    make, kw = CASES[name]
    spec = make()
    a, b = ctx.create(spec), ctx.create(spec)
    ctx.run_batch([a], 3000, seed=9, **kw)
    done, launches = 0, 0
    while done < 3000:
        out = np.zeros(1, np.int64)
        ctx.run_batch([b], moves_per_system=[3000 - done], seed=9, counters=[done], time_budget_s=2e-4,
                      moves_out=out, **kw)
        assert 1 <= out[0] <= 3000 - done
        done += int(out[0])
        launches += 1
    assert launches > 1 and done == 3000
    assert np.array_equal(a.positions(), b.positions())
    assert a.running_energy() == b.running_energy()
    assert np.array_equal(a.q(), b.q())
    out = np.zeros(1, np.int64)
    ctx.run_batch([b], 500, seed=9, counter_base=3000, moves_out=out, **kw)
    assert out[0] == 500
