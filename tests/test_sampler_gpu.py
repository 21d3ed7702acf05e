"""Device analysis (fau_sampler) on the GPU: AtomRDF histograms identical to the
FP64 oracle's on the device's own positions (bins decided in FP32 from the
fixed-point records, FP64 near bin edges), SystemEnergy sums equal to the
running energies, and sampling fused between the blocks of one batched launch
equal to the same blocks launched one by one with a standalone sample after each."""
import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import configs

import oracle_lib as O

pytestmark = pytest.mark.gpu


def _replicas(ctx, spec, R, moves, dp):
    base = ctx.create(spec)
    reps = [base] + [base.clone() for _ in range(R - 1)]
    ctx.run_batch(reps, moves, seed=3, dp=dp)
    return reps


@pytest.mark.parametrize("kind,ta,tb,dr,nb", [("pm", 0, 0, 0.1, 400), ("pm", 0, 1, 0.05, 600),
                                             ("bulk", 1, 1, 0.2, 2000), ("bulk", 0, 1, 0.013, 12000)])
def test_rdf_histogram_identical_to_oracle(ctx, kind, ta, tb, dr, nb):
    spec = configs.primitive_model(n=200, seed=4) if kind == "pm" else configs.bulk_ewald(n_salt=1000, seed=2)
    reps = _replicas(ctx, spec, 3, 2000, 2.0)
    smp = F.Sampler(ctx, n_slots=3, rdf=(ta, tb, dr, nb))
    smp.sample(reps)
    smp.sample(reps, slots=[0, 0, 1])
    d = smp.read()
    want = np.zeros((3, nb), np.uint64)
    beyond = np.zeros(3, np.int64)
    for k, s in enumerate(reps):
        h, b = O.rdf_hist(s.positions(), spec.type, spec.box, ta, tb, dr, nb)
        for slot in (k, [0, 0, 1][k]):
            want[slot] += h.astype(np.uint64)
            beyond[slot] += b
    assert np.array_equal(d["rdf_hist"], want)
    assert np.array_equal(d["rdf_beyond"].astype(np.int64), beyond)
    assert list(d["rdf_samples"]) == [3, 2, 1]
    V = float(np.prod(spec.box))
    assert np.allclose(d["rdf_volume_sum"], np.array([3, 2, 1]) * V, rtol=1e-15)
    r, g = smp.g_of_r(d, slots=[2])
    assert len(r) == nb - 1 and np.isfinite(g).all()


def test_energy_sampling_equals_running_energy(ctx):
    reps = _replicas(ctx, configs.primitive_model(n=200, seed=6), 4, 3000, 2.0)
    smp = F.Sampler(ctx, n_slots=4)
    smp.sample(reps)
    d = smp.read()
    e = np.array([s.running_energy() for s in reps])
    assert np.array_equal(d["energy_sum"], e) and np.array_equal(d["energy_sum2"], e * e)
    assert list(d["energy_samples"]) == [1, 1, 1, 1]
    smp.reset()
    assert smp.read()["energy_samples"].sum() == 0


@pytest.mark.parametrize("threads", [0, 256])
def test_fused_sampling_equals_blockwise(ctx, threads):
    spec = configs.primitive_model(n=200, seed=8)
    R, B, I = 4, 3, 700
    a = _replicas(ctx, spec, R, 0, 2.0)
    b = [s.clone() for s in a]
    fa = F.Sampler(ctx, n_slots=R, rdf=(0, 1, 0.1, 300))
    fb = F.Sampler(ctx, n_slots=R, rdf=(0, 1, 0.1, 300))
    st = ctx.run_batch(a, seed=11, dp=2.0, threads=threads, sampler=fa, sample_interval=I, n_sample_blocks=B)
    assert st["moves"] == R * B * I
    for k in range(B):
        ctx.run_batch(b, I, seed=11, dp=2.0, threads=threads, counter_base=k * I)
        fb.sample(b)
    da, db = fa.read(), fb.read()
    for key in ("rdf_hist", "rdf_beyond", "rdf_samples", "energy_samples"):
        assert np.array_equal(da[key], db[key]), key
    assert list(da["energy_samples"]) == [B] * R
    assert np.allclose(da["energy_sum"], db["energy_sum"], rtol=1e-12)
    for x, y in zip(a, b):
        assert np.array_equal(x.positions(), y.positions())


def test_sampling_with_parallel_tempering(ctx):
    specs = [configs.primitive_model(n=200, seed=20 + k) for k in range(4)]
    systems = [ctx.create(s) for s in specs]
    smp = F.Sampler(ctx, n_slots=4)
    ctx.run_batch(systems, seed=5, dp=2.0, swap_interval=500, n_swap_blocks=5,
                  temperatures=[280.0, 300.0, 320.0, 340.0], sampler=smp)
    assert list(smp.read()["energy_samples"]) == [5] * 4


def test_sampler_argument_errors(ctx):
    with pytest.raises(F.FauError):
        F.Sampler(ctx, n_slots=0)
    with pytest.raises(F.FauError):
        F.Sampler(ctx, rdf=(0, 0, 0.0, 10))
    with pytest.raises(F.FauError):
        F.Sampler(ctx, rdf=(0, 0, 0.1, 20000))
    smp = F.Sampler(ctx, n_slots=2)
    s = ctx.create(configs.primitive_model(n=50))
    with pytest.raises(F.FauError):
        smp.sample([s], slots=[2])
    with pytest.raises(F.FauError):
        ctx.run_batch([s], moves_per_system=[10], sampler=smp, sample_interval=10, n_sample_blocks=2)
