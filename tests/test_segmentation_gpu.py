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
    "molecular_water": (lambda: configs.spce_water(n_mol=256, L=18.6, seed=6), dict(dp=0.5, dprot=0.5, threads=0)),
    "chain_water": (lambda: configs.spce_water(n_mol=256, L=18.6, seed=7), dict(dp=0.5, dprot=0.5, threads=256)),
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
