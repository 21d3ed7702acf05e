"""Checkpoint and resume: a chain stopped, saved and loaded into a fresh system continues
bit for bit -- the same accept sequence, energy changes, positions, Q(k) and running energy as
the chain that never stopped.

The saved state is the system's exact device state (fau_sys_save_state) plus the move
stream's position: the reference's two mt19937 engines (fau_movegen_get_state, as
SaveState's random-move / random-global, src/analysis.cpp:654-680) for host proposals, or
the next (seed, stream, counter) for device proposals.
"""
import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a.positions(), b.positions())
    assert a.running_energy() == b.running_energy()
    if a.K:
        assert np.array_equal(a.q(), b.q())
    if a.cell_grid() != (0, 0, 0):
        assert np.array_equal(a.cells(), b.cells())


@pytest.mark.parametrize("make", [lambda: configs.bulk_ewald(n_salt=500, seed=4),
                                  lambda: configs.bulk_ewald(n_salt=500, epss=1.0, seed=5),
                                  lambda: configs.spce_water(n_mol=256, L=18.6, seed=3)])
def test_host_stream_resumes_bit_for_bit(ctx, make):
    spec = make()
    gen = F.MoveGenerator(spec, spec.extra["moves"], 3, 4, default_seeds=False)
    a = ctx.create(spec)
    first = gen.generate(1500)
    off = np.array([0, len(first)], np.int64)
    ctx.run_proposals_batch([a], first, off)
    blob, rng = a.save_state(), gen.state()
    rest = gen.generate(1500)
    acc_a, du_a = np.zeros(len(rest), np.uint8), np.zeros(len(rest))
    ctx.run_proposals_batch([a], rest, off, acc_a, du_a)

    b = ctx.create(spec)
    b.load_state(blob)
    gen2 = F.MoveGenerator(spec, spec.extra["moves"], 0, 0, default_seeds=False)
    gen2.set_state(rng)
    rest2 = gen2.generate(1500)
    assert rest2.tobytes() == rest.tobytes()
    acc_b, du_b = np.zeros(len(rest), np.uint8), np.zeros(len(rest))
    ctx.run_proposals_batch([b], rest2, off, acc_b, du_b)
    assert np.array_equal(acc_a, acc_b) and np.array_equal(du_a, du_b)
    _same(a, b)


@pytest.mark.parametrize("make,dp,dprot", [(lambda: configs.bulk_ewald(n_salt=1000, seed=2), 2.0, 0.0),
                                           (lambda: configs.primitive_model(n=200, seed=1), 2.0, 0.0),
                                           (lambda: configs.spce_water(n_mol=256, L=18.6, seed=1), 0.5, 0.5)])
def test_device_stream_resumes_bit_for_bit(ctx, make, dp, dprot):
    spec = make()
    a = ctx.create(spec)
    ctx.run_batch([a], 2000, seed=9, streams=[4], counters=[0], dp=dp, dprot=dprot, threads=0)
    blob = a.save_state()
    ctx.run_batch([a], 3000, seed=9, streams=[4], counters=[2000], dp=dp, dprot=dprot, threads=0)
    b = ctx.create(spec)
    b.load_state(blob)
    ctx.run_batch([b], 3000, seed=9, streams=[4], counters=[2000], dp=dp, dprot=dprot, threads=0)
    _same(a, b)
    # and both equal one uninterrupted chain
    c = ctx.create(spec)
    ctx.run_batch([c], 5000, seed=9, streams=[4], counters=[0], dp=dp, dprot=dprot, threads=0)
    _same(a, c)


def test_state_of_another_system_is_rejected(ctx):
    a = ctx.create(configs.bulk_ewald(n_salt=500, seed=4))
    b = ctx.create(configs.bulk_ewald(n_salt=400, seed=4))
    with pytest.raises(F.FauError):
        b.load_state(a.save_state())
    with pytest.raises(F.FauError):
        a.load_state(b"not a state")


@pytest.mark.parametrize("mode,suffix", [("reference", ".ubj"), ("reference", ".json"), ("batch", ".ubj")])
def test_simulate_resumes_from_its_state_file(ctx, tmp_path, mode, suffix):
    """The MC loop's savestate file (JSON or UBJSON, with the RNG engines and the exact device
    state) restarts a run: 3 + 3 sweeps end where 6 uninterrupted sweeps end."""
    import json as _json

    from faunus_gb300 import input as I
    from faunus_gb300 import ubjson
    from faunus_gb300.run import simulate
    from test_input import PM

    text = PM.replace("    - systemenergy: {file: energy.dat, nstep: 10}", f"    - savestate: {{file: state{suffix}}}")
    # one dp for every moved atom type (what batch mode's device proposals take)
    text = text.replace("    - transrot: {molecule: chloride, repeat: 5}", "    - transrot: {molecule: chloride, repeat: N}")
    text = text.replace("r: 2.5, dp: 10", "r: 2.5, dp: 20")
    simulate(I.load_input(text, seed=3), ctx, out_dir=tmp_path / "a", mode=mode, macro=1, micro=6)
    simulate(I.load_input(text, seed=3), ctx, out_dir=tmp_path / "b", mode=mode, macro=1, micro=3)
    saved = tmp_path / "b" / f"state{suffix}"
    st = I._read(saved)
    assert "fau-device-state" in st
    if mode == "reference":
        assert {"random-move", "random-global"} <= set(st)
    resumed = I.apply_state(I.load_input(text, seed=3), st)
    simulate(resumed, ctx, out_dir=tmp_path / "c", mode=mode, macro=1, micro=3, resume=saved, first_step=3)

    def final(d):
        f = d / f"state{suffix}"
        return ubjson.loads(f.read_bytes()) if suffix == ".ubj" else _json.loads(f.read_text())

    a, c = final(tmp_path / "a"), final(tmp_path / "c")
    assert [p["pos"] for p in a["particles"]] == [p["pos"] for p in c["particles"]]
    if mode == "reference":
        assert a["random-move"] == c["random-move"] and a["random-global"] == c["random-global"]
