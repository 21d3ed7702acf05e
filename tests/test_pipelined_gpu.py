"""GPU parity of the pipelined chain kernel (batched single-atom moves).

fau_run_batch (threads 0, 96, 160 or 288) and fau_run_proposals_batch run every system
whose proposals are single-atom translations in the pipelined kernel.  It must
reproduce:
  * the chain kernel (threads=128) under the same device proposals: the same
    accept sequence and bit-identical FP64 positions (barring a near tie, where
    u falls between the two FP32C energy changes' exponentials);
  * the FP64 oracle under reference-stream host proposals, to the tolerance of
    test_parity_gpu (1e-6 of max(|dU|, S));
  * its own running energy against an FP64 recomputation of the total.
Cases cover cell lists (union stencil box and the separate-stencil fallback of
a 3x3x3 grid), frequent commit/stencil conflicts (small box), all-pairs with
hard spheres, the Ewald surface term and batches mixing both kernels.
"""
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O

pytestmark = pytest.mark.gpu

TOL = 1e-6

CASES = {
    "primitive_model": lambda: configs.primitive_model(n=200, seed=3),
    "bulk_cells": lambda: configs.bulk_ewald(n_salt=1000, seed=4),
    "bulk_surface": lambda: configs.bulk_ewald(n_salt=1000, epss=1.0, seed=5),
    "bulk_small_box": lambda: configs.bulk_ewald(n_salt=100, seed=6),
    "bulk_3x3x3_cells": lambda: configs.bulk_ewald(n_salt=50, L=40.0, seed=7),
}


def _energy_consistent(s):
    e_run = s.running_energy()
    s.q_rebuild()
    e_tot = s.energy_total()["total"]
    assert abs(e_run - e_tot) <= 1e-6 * max(1.0, abs(e_tot)), (e_run, e_tot)


@pytest.mark.parametrize("case,threads", [(c, 160) for c in sorted(CASES)] +
                         [(c, t) for c in ("primitive_model", "bulk_cells", "bulk_small_box") for t in (96, 288)])
def test_pipelined_equals_chain_kernel(ctx, case, threads):
    spec = CASES[case]()
    a, b = ctx.create(spec), ctx.create(spec)
    if case == "bulk_3x3x3_cells":
        assert a.cell_grid() == (3, 3, 3)
    moves = 3000
    sa = ctx.run_batch([a], moves, seed=21, streams=[5], dp=2.0, threads=threads)
    sb = ctx.run_batch([b], moves, seed=21, streams=[5], dp=2.0, threads=128)
    assert sa["moves"] == sb["moves"] == moves
    assert sa["accepted"] == sb["accepted"] and sa["accepted"] > 100
    assert sa["pair_evals"] > 0
    assert np.array_equal(a.positions(), b.positions())
    ea, eb = a.running_energy(), b.running_energy()
    assert abs(ea - eb) <= 1e-6 * max(1.0, abs(eb))
    if a.cell_grid() != (0, 0, 0):
        assert np.array_equal(a.cells(), b.cells())
    if a.K:
        assert np.abs(a.q() - b.q()).max() < 1e-4
    _energy_consistent(a)


def _oracle_compare(g_pos, acc_g, du_g, spec, props, label="", median_tol=None):
    o = O.OracleSystem(spec)
    det = o.run_detail(props)
    acc_o, du_o, scale = det["accepted"].astype(np.uint8), det["du"], det["err_scale"]
    mism = np.nonzero(acc_g != acc_o)[0]
    first = int(mism[0]) if len(mism) else len(props)
    sl = slice(0, first + 1 if first < len(props) else first)
    fin = np.isfinite(du_o[sl])
    assert np.array_equal(np.isfinite(du_g[sl]), fin)
    rep = O.du_errors(du_g[sl][fin], du_o[sl][fin], scale[sl][fin])
    print(f"PARITY {label} moves={len(props)} " + " ".join(f"{k}={v:.3e}" if isinstance(v, float) else f"{k}={v}"
                                                          for k, v in rep.items()))
    assert rep["rel_scaled_max"] <= TOL, f"max rel err {rep['rel_scaled_max']:.3e}"
    if median_tol is not None:  # the benchmark forms: the median relative to |dU| itself too
        assert rep["rel_du_median"] <= median_tol, f"median err / |dU| {rep['rel_du_median']:.3e}"
    if len(mism):
        m = first
        lo, hi = sorted([math.exp(-min(du_g[m], 700)), math.exp(-min(du_o[m], 700))])
        assert lo <= props["u"][m] <= hi
        assert first > len(props) // 10
    else:
        assert np.array_equal(g_pos, o.positions())
    return int(acc_g.sum())


def test_pipelined_host_proposals_match_oracle(ctx):
    specs = [CASES["primitive_model"](), CASES["bulk_cells"](), CASES["bulk_surface"](),
             CASES["bulk_3x3x3_cells"]()]
    systems = [ctx.create(s) for s in specs]
    M = 3000
    props = [F.MoveGenerator(s, s.extra["moves"], 31 + i, 37 + i, default_seeds=False).generate(M)
             for i, s in enumerate(specs)]
    allp = np.concatenate(props)
    off = np.arange(len(specs) + 1, dtype=np.int64) * M
    acc = np.zeros(len(allp), np.uint8)
    du = np.zeros(len(allp))
    st = ctx.run_proposals_batch(systems, allp, off, acc, du)
    assert st["moves"] == len(allp)
    for i, (s, spec) in enumerate(zip(systems, specs)):
        sl = slice(i * M, (i + 1) * M)
        n_acc = _oracle_compare(s.positions(), acc[sl], du[sl], spec, props[i], label=f"host_batch_{i}",
                                median_tol=O.TOL_REL_DU_MEDIAN)
        assert n_acc > 100
        _energy_consistent(s)


def test_pipelined_full_size_bulk_matches_oracle(ctx):
    """The benchmarked kernel (fast_chain_kernel, host-proposal instance, 4 compute warps) on the
    benchmarked system: 20,000 ions, K = 1152, 45^3 cells, 2,500 reference-stream moves."""
    spec = configs.bulk_ewald(n_salt=10000, seed=1)
    g = ctx.create(spec)
    assert g.cell_grid() == (45, 45, 45) and g.K == 1152
    props = F.MoveGenerator(spec, spec.extra["moves"], 7, 11, default_seeds=False).generate(2500)
    off = np.array([0, len(props)], np.int64)
    acc = np.zeros(len(props), np.uint8)
    du = np.zeros(len(props))
    st = ctx.run_proposals_batch([g], props, off, acc, du)
    assert st["moves"] == len(props)
    n_acc = _oracle_compare(g.positions(), acc, du, spec, props, label="bulk_ewald_20000_fast",
                            median_tol=O.TOL_REL_DU_MEDIAN)
    assert n_acc > 1000
    _energy_consistent(g)


def test_pipelined_empty_moves_and_reference_move_counts(ctx):
    """FAU_MOVE_NONE proposals are skipped (not counted, never accepted)."""
    spec = CASES["bulk_cells"]()
    g = ctx.create(spec)
    props = F.MoveGenerator(spec, spec.extra["moves"], 3, 4, default_seeds=False).generate(500)
    props["kind"][::3] = A.FAU_MOVE_NONE
    acc = np.zeros(len(props), np.uint8)
    du = np.zeros(len(props))
    st = ctx.run_proposals_batch([g], props, np.array([0, len(props)], np.int64), acc, du)
    none = props["kind"] == A.FAU_MOVE_NONE
    assert st["moves"] == int((~none).sum())
    assert not acc[none].any() and not du[none].any()
    props_o = props.copy()
    _oracle_compare(g.positions(), acc, du, spec, props_o)


def test_pipelined_mixed_batch_with_molecular_systems(ctx):
    """Water (molecular moves) runs in the chain kernel beside the pipelined systems,
    on a forked stream inside the same graph."""
    specs = [configs.primitive_model(n=200, seed=1), configs.bulk_ewald(n_salt=1000, seed=2),
             configs.spce_water(n_mol=256, L=18.6, seed=3)]
    systems = [ctx.create(s) for s in specs]
    st = ctx.run_batch(systems, 3000, seed=7, dp=1.0, dprot=0.3, threads=0)
    assert st["moves"] == 9000 and st["accepted"] > 0
    for s in systems:
        _energy_consistent(s)


def test_pipelined_alone_equals_in_mix(ctx):
    a1 = ctx.create(configs.bulk_ewald(n_salt=500, seed=4))
    ctx.run_batch([a1], 2000, seed=3, streams=[42], counters=[0], threads=0)
    others = [ctx.create(configs.primitive_model(n=200, seed=s)) for s in range(3)]
    a2 = ctx.create(configs.bulk_ewald(n_salt=500, seed=4))
    ctx.run_batch(others[:1] + [a2] + others[1:], 2000, seed=3, streams=[1, 42, 2, 3], counters=[0] * 4, threads=0)
    assert np.array_equal(a1.positions(), a2.positions())
    assert a1.running_energy() == a2.running_energy()
    b1 = ctx.create(configs.bulk_ewald(n_salt=500, seed=8))
    ctx.run_batch([b1], 1000, seed=5, streams=[9], counters=[0], threads=0)
    ctx.run_batch([b1], 1000, seed=5, streams=[9], counters=[1000], threads=0)
    b2 = ctx.create(configs.bulk_ewald(n_salt=500, seed=8))
    ctx.run_batch([b2], 2000, seed=5, streams=[9], counters=[0], threads=0)
    assert np.array_equal(b1.positions(), b2.positions())


def test_whole_cell_body_is_the_same_in_either_instance(ctx):
    """A launch whose systems all stage whole cells (no cell list, or cell_staging=1) runs the
    kernel instance holding that body alone; beside a system staging occupied slots, the instance
    holding every body.  A chain is the same, bit for bit, in either; whole-cell and occupied-slot
    staging of one system agree to the energy tolerance."""
    import dataclasses
    bulk = configs.bulk_ewald(n_salt=500, seed=11)
    whole = dataclasses.replace(bulk, cell_staging=1)
    pm = configs.primitive_model(n=200, seed=12)
    alone = [ctx.create(whole), ctx.create(pm)]
    for i, s in enumerate(alone):
        ctx.run_batch([s], 3000, seed=9, streams=[i], counters=[0], dp=2.0, threads=160)
    mixed = [ctx.create(whole), ctx.create(pm), ctx.create(bulk)]
    ctx.run_batch(mixed, 3000, seed=9, streams=[0, 1, 2], counters=[0] * 3, dp=2.0, threads=160)
    for x, y in zip(alone, mixed):
        assert np.array_equal(x.positions(), y.positions()) and x.running_energy() == y.running_energy()
    occ = ctx.create(bulk)
    ctx.run_batch([occ], 3000, seed=9, streams=[0], counters=[0], dp=2.0, threads=160)
    if np.array_equal(occ.positions(), alone[0].positions()):  # barring a near tie, the same chain
        e = alone[0].energy_total()["total"]
        assert abs(occ.running_energy() - alone[0].running_energy()) <= 1e-6 * max(1.0, abs(e))
    for s in alone + mixed + [occ]:
        _energy_consistent(s)


def test_pipelined_parallel_tempering(ctx):
    specs, temps = configs.pt_replicas(n_rep=8, n_min=100, n_max=300)
    systems = [ctx.create(s) for s in specs]
    st = ctx.run_batch(systems, swap_interval=400, n_swap_blocks=6, temperatures=temps, seed=11, dp=2.0, threads=0)
    assert st["swaps_attempted"] >= 6 * 3 and st["moves"] == 8 * 400 * 6
    for s in systems:
        e_run = s.running_energy()
        e_tot = s.energy_total()["total"]
        assert abs(e_run - e_tot) <= 1e-6 * max(1.0, abs(e_tot))


def _pinned_copy(arr):
    torch = pytest.importorskip("torch")
    raw = np.ascontiguousarray(arr)
    t = torch.empty(raw.nbytes, dtype=torch.uint8).pin_memory()
    view = t.numpy().view(raw.dtype)
    view[:] = raw
    return view, t


def test_pipelined_reads_pinned_proposals_in_place(ctx):
    """Proposals in pinned host memory are read by the kernel directly (no staging copy);
    the result equals the staged run's bit for bit."""
    spec = CASES["bulk_cells"]()
    a, b = ctx.create(spec), ctx.create(spec)
    props = F.MoveGenerator(spec, spec.extra["moves"], 41, 43, default_seeds=False).generate(2000)
    off = np.array([0, len(props)], np.int64)
    acc_a, du_a = np.zeros(len(props), np.uint8), np.zeros(len(props))
    ctx.run_proposals_batch([a], props, off, acc_a, du_a)
    pinned, keep = _pinned_copy(props)
    acc_b, du_b = np.zeros(len(props), np.uint8), np.zeros(len(props))
    ctx.run_proposals_batch([b], pinned, off, acc_b, du_b)
    assert np.array_equal(acc_a, acc_b) and np.array_equal(du_a, du_b)
    assert np.array_equal(a.positions(), b.positions())


@pytest.mark.parametrize("kind", ["atomic_system", "molecular_system"])
def test_batch_proposals_checked_on_the_device(ctx, kind):
    """Out-of-range indices and unknown kinds end the chain with FAU_ERR_ARG (checked by the
    kernel as it reads each proposal), leaving the system usable."""
    spec = CASES["bulk_cells"]() if kind == "atomic_system" else configs.spce_water(n_mol=256, L=18.6, seed=3)
    g = ctx.create(spec)
    props = F.MoveGenerator(spec, spec.extra["moves"], 5, 6, default_seeds=False).generate(300)
    off = np.array([0, len(props)], np.int64)
    for field, value in (("index", 10 ** 6), ("kind", 7)):
        bad = props.copy()
        bad[field][150] = value
        with pytest.raises(F.FauError):
            ctx.run_proposals_batch([g], bad, off)
    st = ctx.run_proposals_batch([g], props, off)  # still usable afterwards
    assert st["moves"] == len(props)


def test_audit_reports_the_error_against_fp64(ctx):
    """Every launch's result carries its error against FP64: after its last move each chain
    evaluates a probe move that an FP64 re-evaluation then checks; the probe changes nothing
    (the chains equal unaudited ones bit for bit)."""
    specs = [configs.bulk_ewald(n_salt=1000, seed=2), configs.primitive_model(n=200, seed=1),
             configs.bulk_ewald(n_salt=500, epss=1.0, seed=5)]
    a = [ctx.create(s) for s in specs]
    b = [ctx.create(s) for s in specs]
    st = ctx.run_batch(a, 2000, seed=3, dp=2.0, threads=0)
    assert st["du_err_samples"] == len(specs)
    assert 0.0 < st["du_err_scaled_max"] <= TOL
    for s in a:
        au = s.audit()
        assert au["samples"] == 1 and au["rel_scaled_max"] <= TOL
    sb = ctx.run_batch(b, 2000, seed=3, dp=2.0, threads=0, audit=False)
    assert sb["du_err_samples"] == 0
    assert st["pair_evals"] == sb["pair_evals"]
    for x, y in zip(a, b):
        assert np.array_equal(x.positions(), y.positions()) and x.running_energy() == y.running_energy()
    # host streams are audited too (the probe repeats the last proposal on the final state)
    props = F.MoveGenerator(specs[0], specs[0].extra["moves"], 3, 4, default_seeds=False).generate(500)
    st2 = ctx.run_proposals_batch([a[0]], props, np.array([0, len(props)], np.int64))
    assert st2["du_err_samples"] == 1 and a[0].audit()["samples"] == 2


def test_launch_width_follows_the_chain_count(ctx):
    """threads=0 gives the pipelined chains CTAs of 8 compute warps when all of them fit on the GPU
    at once (two to an SM) and CTAs of 4 when there are more; each chain equals the same system run
    alone at that width (threads 288 or 160), bit for bit."""
    big, small = configs.primitive_model(n=2000, L=50.0 * 10 ** (1 / 3), seed=6), configs.bulk_ewald(n_salt=500, seed=7)
    mix = [ctx.create(big), ctx.create(small)]
    st = ctx.run_batch(mix, 1500, seed=5, streams=[1, 2], dp=2.0, threads=0)
    assert st["moves"] == 3000 and st["du_err_samples"] == 2
    alone_big, alone_small = ctx.create(big), ctx.create(small)
    ctx.run_batch([alone_big], 1500, seed=5, streams=[1], dp=2.0, threads=288)
    ctx.run_batch([alone_small], 1500, seed=5, streams=[2], dp=2.0, threads=288)
    for x, y in ((mix[0], alone_big), (mix[1], alone_small)):
        assert np.array_equal(x.positions(), y.positions()) and x.running_energy() == y.running_energy()
    _energy_consistent(mix[0])
    # more chains than two 8-warp CTAs per SM: CTAs of 4
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    spec = configs.primitive_model(n=100, seed=8)
    base = ctx.create(spec)
    many = [base] + [base.clone() for _ in range(2 * sms)]
    ctx.run_batch(many, 400, seed=5, streams=np.arange(len(many)), dp=2.0, threads=0)
    four = ctx.create(spec)
    ctx.run_batch([four], 400, seed=5, streams=[0], dp=2.0, threads=160)
    assert np.array_equal(many[0].positions(), four.positions()) and many[0].running_energy() == four.running_energy()
