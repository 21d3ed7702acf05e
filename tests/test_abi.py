"""C ABI checks that need no GPU: exported symbols, struct layouts, host-side
entry points (footprint, move generator) and their error behaviour."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def _declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fau_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = A.lib()
    names = _declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    nm = subprocess.run(["nm", "-D", "--defined-only", str(A.LIBPATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fau_\w+)", nm))
    assert set(names) <= exported


def test_abi_version_and_strerror():
    lib = A.lib()
    assert lib.fau_abi_version() == 1
    assert lib.fau_strerror(A.FAU_ERR_NAN) == b"Metropolis error: energy cannot be NaN"
    assert lib.fau_strerror(12345) == b"unknown status"


_PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "fau_gpu.h"
#define S(t) printf(#t " %zu\n", sizeof(t));
#define O(t, f) printf(#t "." #f " %zu\n", offsetof(t, f));
int main(void) {
  S(fau_ewald_desc) S(fau_sys_desc) S(fau_energy_terms) S(fau_trial_result) S(fau_proposal)
  S(fau_run_stats) S(fau_batch_params) S(fau_batch_stats) S(fau_move_desc) S(fau_sampler_desc)
  O(fau_sys_desc, ewald) O(fau_sys_desc, precision) O(fau_sys_desc, pair_cutoff) O(fau_sys_desc, n_types)
  O(fau_proposal, u) O(fau_batch_params, temperatures) O(fau_move_desc, groups) O(fau_trial_result, accepted)
  O(fau_sys_desc, cutoff_g2g_pairs) O(fau_sys_desc, coulomb_poly) O(fau_sys_desc, pressure)
  O(fau_batch_params, sampler) O(fau_batch_params, n_sample_blocks) O(fau_move_desc, volume_method)
  O(fau_sampler_desc, rdf_dr) O(fau_sampler_desc, energy) S(fau_spline_opts)
  O(fau_sys_desc, spline_begin) O(fau_sys_desc, spline_hs) O(fau_spline_opts, hardsphere)
  O(fau_batch_params, time_budget_ns) O(fau_batch_params, moves_out) O(fau_batch_params, swap_energy_out) O(fau_batch_params, no_audit) O(fau_batch_stats, du_err_samples)
  O(fau_batch_params, volume_dv) O(fau_batch_params, volume_method) O(fau_batch_stats, volume_accepted) O(fau_sys_desc, maxenergy)
  O(fau_sys_desc, cell_staging)
  return 0;
}
"""


def test_struct_layouts_match_header(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(_PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.split("\n") if line)
    sizes = {"fau_ewald_desc": A.EwaldDesc, "fau_sys_desc": A.SysDesc, "fau_energy_terms": A.EnergyTerms,
             "fau_trial_result": A.TrialResult, "fau_proposal": A.Proposal, "fau_run_stats": A.RunStats,
             "fau_batch_params": A.BatchParams, "fau_batch_stats": A.BatchStats, "fau_move_desc": A.MoveDesc,
             "fau_sampler_desc": A.SamplerDesc, "fau_spline_opts": A.SplineOpts}
    for name, cls in sizes.items():
        assert int(out[name]) == C.sizeof(cls), name
    offs = {"fau_sys_desc.ewald": A.SysDesc.ewald.offset, "fau_sys_desc.precision": A.SysDesc.precision.offset,
            "fau_sys_desc.pair_cutoff": A.SysDesc.pair_cutoff.offset, "fau_sys_desc.n_types": A.SysDesc.n_types.offset,
            "fau_proposal.u": A.Proposal.u.offset, "fau_batch_params.temperatures": A.BatchParams.temperatures.offset,
            "fau_move_desc.groups": A.MoveDesc.groups.offset, "fau_trial_result.accepted": A.TrialResult.accepted.offset,
            "fau_sys_desc.cutoff_g2g_pairs": A.SysDesc.cutoff_g2g_pairs.offset,
            "fau_sys_desc.coulomb_poly": A.SysDesc.coulomb_poly.offset, "fau_sys_desc.pressure": A.SysDesc.pressure.offset,
            "fau_batch_params.sampler": A.BatchParams.sampler.offset,
            "fau_batch_params.n_sample_blocks": A.BatchParams.n_sample_blocks.offset,
            "fau_move_desc.volume_method": A.MoveDesc.volume_method.offset,
            "fau_sampler_desc.rdf_dr": A.SamplerDesc.rdf_dr.offset, "fau_sampler_desc.energy": A.SamplerDesc.energy.offset,
            "fau_sys_desc.spline_begin": A.SysDesc.spline_begin.offset,
            "fau_sys_desc.spline_hs": A.SysDesc.spline_hs.offset,
            "fau_spline_opts.hardsphere": A.SplineOpts.hardsphere.offset,
            "fau_batch_params.time_budget_ns": A.BatchParams.time_budget_ns.offset,
            "fau_batch_params.moves_out": A.BatchParams.moves_out.offset,
            "fau_batch_params.volume_dv": A.BatchParams.volume_dv.offset,
            "fau_batch_params.volume_method": A.BatchParams.volume_method.offset,
            "fau_batch_stats.volume_accepted": A.BatchStats.volume_accepted.offset,
            "fau_sys_desc.maxenergy": A.SysDesc.maxenergy.offset,
            "fau_sys_desc.cell_staging": A.SysDesc.cell_staging.offset}
    for k, v in offs.items():
        assert int(out[k]) == v, k


def test_footprint_host_only():
    spec = configs.primitive_model(n=200)
    b = F.footprint(spec)
    assert 10_000 < b < 1_000_000
    big = configs.bulk_ewald(n_salt=10000)
    bb = F.footprint(big)
    assert bb > b
    bad = spec.copy()
    bad.pos = bad.pos.copy()
    bad.pos[0, 0] = 1e9
    with pytest.raises(F.FauError) as e:
        F.footprint(bad)
    assert e.value.status == A.FAU_ERR_ARG


def test_context_without_gpu_fails_cleanly():
    lib = A.lib()
    h = C.c_void_p()
    rc = lib.fau_ctx_create(0, 0, C.byref(h))
    if rc == A.FAU_OK:
        lib.fau_ctx_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == A.FAU_ERR_NODEVICE
    assert b"no CUDA device" in lib.fau_last_error()


# ---------------------------------------------------------------- move generator vs oracle
def _streams_equal(a, b):
    assert np.array_equal(a["kind"], b["kind"])
    assert np.array_equal(a["index"], b["index"])
    assert np.array_equal(a["dr"], b["dr"])  # bit-exact
    assert np.array_equal(a["quat"], b["quat"])
    assert np.array_equal(a["u"], b["u"])


@pytest.mark.parametrize("default_seeds", [True, False])
def test_movegen_transrot_matches_oracle(default_seeds):
    spec = configs.primitive_model(n=200)
    moves = spec.extra["moves"]
    g = F.MoveGenerator(spec, moves, 17, 29, default_seeds=default_seeds)
    o = O.OracleMoveGen(O.OracleSystem(spec), moves, 17, 29, default_seeds=default_seeds)
    _streams_equal(g.generate(5000), o.generate(5000))
    assert (g.generate(10)["kind"] == A.FAU_MOVE_ATOMIC).all()


def test_movegen_moltransrot_matches_oracle():
    spec = configs.spce_water(n_mol=64, L=12.4)
    moves = spec.extra["moves"]
    g = F.MoveGenerator(spec, moves, 3, 4, default_seeds=False)
    o = O.OracleMoveGen(O.OracleSystem(spec), moves, 3, 4, default_seeds=False)
    a, b = g.generate(3000), o.generate(3000)
    _streams_equal(a, b)
    q = a["quat"]
    assert np.allclose((q * q).sum(1), 1.0)
    assert (a["index"] < 64).all()


def test_movegen_mixed_collection_and_type_dp():
    """Two moves with weights (MoveCollection::sample), per-type dp override and a
    rotational dprot on isotropic atoms that only consumes draws."""
    spec = configs.primitive_model(n=40, L=30.0)
    moves = [
        {"kind": A.FAU_MOVE_ATOMIC, "repeat": 40, "dp": 1.0, "dprot": 0.3, "groups": [0],
         "type_dp": np.array([np.nan, 3.0])},
        {"kind": A.FAU_MOVE_ATOMIC, "repeat": 10, "dp": 0.0, "groups": [0]},
    ]
    g = F.MoveGenerator(spec, moves, 5, 6, default_seeds=False)
    o = O.OracleMoveGen(O.OracleSystem(spec), moves, 5, 6, default_seeds=False)
    a, b = g.generate(4000), o.generate(4000)
    _streams_equal(a, b)
    # the dp=0 move with no rotation yields empty changes (only the Metropolis draw)
    assert (a["kind"] == A.FAU_MOVE_NONE).sum() > 0
    # anions (type 1) move with the per-type dp = 3
    atomic = a[a["kind"] == A.FAU_MOVE_ATOMIC]
    r = np.linalg.norm(atomic["dr"], axis=1)
    types = spec.type[atomic["index"]]
    assert r[types == 1].max() > 1.5 and r[types == 0].max() <= 1.0 + 1e-12


def test_movegen_state_roundtrip():
    spec = configs.primitive_model(n=200)
    g = F.MoveGenerator(spec, spec.extra["moves"])
    g.generate(123)
    s = g.state()
    a = g.generate(500)
    g2 = F.MoveGenerator(spec, spec.extra["moves"])
    g2.set_state(s)
    _streams_equal(a, g2.generate(500))
    with pytest.raises(F.FauError):
        g2.set_state("not a state")


def test_movegen_invalid_arguments():
    spec = configs.primitive_model(n=20, L=20.0)
    with pytest.raises(F.FauError) as e:
        F.MoveGenerator(spec, [{"kind": A.FAU_MOVE_ATOMIC, "repeat": 1, "dp": 1.0, "groups": [5]}])
    assert e.value.status == A.FAU_ERR_ARG


def test_full_oracle_loop_equals_oracle_proposals():
    """The oracle's own draw-and-move loop equals generating the proposals first
    and then performing them: proposals are independent of the state."""
    spec = configs.primitive_model(n=60, L=30.0)
    o1 = O.OracleSystem(spec)
    g1 = O.OracleMoveGen(o1, spec.extra["moves"], 1, 2, default_seeds=False)
    acc1, du1, _ = g1.mc_run(3000)
    o2 = O.OracleSystem(spec)
    g2 = O.OracleMoveGen(o2, spec.extra["moves"], 1, 2, default_seeds=False)
    acc2, du2, _ = o2.run_proposals(g2.generate(3000))
    assert np.array_equal(acc1, acc2) and np.array_equal(du1, du2)
    assert np.array_equal(o1.positions(), o2.positions())


def test_configs_shapes():
    s = configs.bulk_ewald(n_salt=10000)
    assert s.n == 20000 and abs(s.box[0] - 549.65) < 0.01
    assert np.abs(s.pos).max() <= 0.5 * s.box[0]
    w = configs.spce_water()
    assert w.n == 3000 and w.n_groups == 1000
    specs, temps = configs.pt_replicas(n_rep=8)
    assert len(specs) == 8 and temps[0] == 250.0 and abs(temps[-1] - 400.0) < 1e-9
    assert all(100 <= sp.n <= 5000 for sp in specs)
