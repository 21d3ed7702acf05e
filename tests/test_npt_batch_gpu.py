"""NPT in batched chains: fau_batch_params volume blocks.

Blocks of single-atom moves, each followed by one VolumeMove per system
(VolumeMove::_move / setNewVolume, reference src/move.cpp:994-1006: V' = exp(ln V + (u - 1/2) dV))
with the uniforms drawn from the counter-based generator.  A batch equals, system by system, the
explicit sequence -- the same block run alone, then fau_volume_move with the volume and the
uniform recomputed here with an independent Philox4x32-10 -- bit for bit; the move counts add up;
the argument checks hold.
"""
import dataclasses
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

from test_pt_gpu import M32, philox4x32_10, u01_53

pytestmark = pytest.mark.gpu


def _specs(kind):
    p = F.pressure_kt(1.0, "P/atm")
    if kind == "pm":
        base = [configs.primitive_model(n=200, seed=s) for s in (1, 2)]
    else:
        base = [configs.bulk_ewald(n_salt=500, molar=1.0, seed=s) for s in (3, 4)]
    return [dataclasses.replace(s, isobaric_pressure=p) for s in base]


@pytest.mark.parametrize("kind", ["pm", "bulk"])
def test_volume_blocks_equal_the_explicit_sequence(ctx, kind):
    specs = _specs(kind)
    seed, iv, nb, dv = 13, 300, 4, 0.2
    batch = [ctx.create(s) for s in specs]
    mo = np.zeros(len(specs), np.int64)
    st = ctx.run_batch(batch, seed=seed, dp=2.0, threads=160, volume_interval=iv, n_volume_blocks=nb, volume_dv=dv,
                       moves_out=mo)
    assert st["volume_attempted"] == nb * len(specs)
    assert np.array_equal(mo, np.full(len(specs), nb * (iv + 1)))
    assert st["moves"] == nb * len(specs) * (iv + 1)
    key = seed ^ 0x5DEECE66D
    k0, k1 = key & M32, (key >> 32) & M32
    alone = [ctx.create(s) for s in specs]
    n_acc = 0
    for i, a in enumerate(alone):
        for b in range(nb):
            ctx.run_batch([a], iv, seed=seed, streams=[i], counters=[b * iv], dp=2.0, threads=160)
            w = philox4x32_10((b & M32, b >> 32, i, 9), k0, k1)  # volume move number b of stream i
            ua, ub = u01_53(w[0], w[1]), u01_53(w[2], w[3])
            v = float(np.prod(a.box()))
            n_acc += a.volume_move(math.exp(math.log(v) + (ua - 0.5) * dv), ub, method="isotropic")["accepted"]
    assert n_acc == st["volume_accepted"]
    for x, y in zip(batch, alone):
        assert np.array_equal(x.box(), y.box())
        assert np.array_equal(x.positions(), y.positions())
        assert x.running_energy() == y.running_energy()
        cx, cy = x.counters(), y.counters()
        assert (cx["moves"], cx["accepted"]) == (cy["moves"], cy["accepted"])
        e_tot = x.energy_total()["total"]
        assert abs(x.running_energy() - e_tot) <= 1e-6 * max(1.0, abs(e_tot))


def test_volume_block_arguments(ctx):
    specs = _specs("pm")
    systems = [ctx.create(s) for s in specs]
    with pytest.raises(F.FauError):  # blocks without a length
        ctx.run_batch(systems, seed=1, volume_interval=0, n_volume_blocks=2, volume_dv=0.1)
    with pytest.raises(F.FauError):  # per-system move counts
        ctx.run_batch(systems, moves_per_system=[10, 20], seed=1, volume_interval=10, n_volume_blocks=2,
                      volume_dv=0.1)
    with pytest.raises(F.FauError):  # with parallel tempering
        ctx.run_batch(systems, seed=1, swap_interval=10, n_swap_blocks=2, temperatures=[298.0, 310.0],
                      volume_interval=10, n_volume_blocks=2, volume_dv=0.1)
    with pytest.raises(F.FauError):  # negative displacement
        ctx.run_batch(systems, seed=1, volume_interval=10, n_volume_blocks=2, volume_dv=-0.1)
    # dV = 0: blocks of moves only, as VolumeMove::_move does nothing without a displacement
    st = ctx.run_batch(systems, seed=1, dp=2.0, volume_interval=50, n_volume_blocks=2, volume_dv=0.0)
    assert st["volume_attempted"] == 0 and st["moves"] == 2 * 50 * len(specs)
