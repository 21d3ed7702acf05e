"""Autotuner on the device: every kernel configuration runs the system and the
choice is one of them."""
import pytest

from faunus_gb300 import autotune, configs

pytestmark = pytest.mark.gpu


def test_tune_primitive_model(ctx, tmp_path):
    s = ctx.create(configs.primitive_model(n=200, seed=2))
    r = autotune.tune(ctx, s, replicas=16, moves=300, cache=tmp_path / "t.json", device="test")
    assert r["threads"] in autotune.CANDIDATES
    assert all(r["table"][str(t)] > 0 for t in autotune.CANDIDATES), r["table"]
