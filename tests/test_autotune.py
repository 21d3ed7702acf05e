"""Autotuner: picks the fastest configuration, caches it per system shape, and
records configurations a system cannot use (host only, with a fake timer)."""
import json

from faunus_gb300 import autotune


class FakeSpec:
    def __init__(self, n, moves):
        self.n = n
        self.n_groups = 1
        self.extra = {"moves": moves}


class FakeSystem:
    def __init__(self, n=200, K=0, grid=(0, 0, 0), moves=({"kind": 0, "dp": 2.0},)):
        self.spec = FakeSpec(n, list(moves))
        self.K = K
        self._grid = grid

    def cell_grid(self):
        return self._grid


def test_picks_fastest_and_caches(tmp_path):
    calls = []

    def fake_measure(ctx, system, threads, replicas, moves):
        calls.append(threads)
        if threads == 256:
            raise RuntimeError("too many k-vectors for the chain kernel")
        return {96: 1.0, 160: 3.0, 288: 2.0, 128: 0.5}[threads]

    cache = tmp_path / "tune.json"
    s = FakeSystem(K=1152, grid=(45, 45, 45))
    r = autotune.tune(None, s, replicas=8, moves=100, cache=cache, device="dev", measure_fn=fake_measure)
    assert r["threads"] == 160 and r["moves_per_s"] == 3.0
    assert r["table"]["256"] == 0.0 and "too many" in r["table"]["256_error"]
    assert sorted(calls) == sorted(autotune.CANDIDATES)
    n = len(calls)
    r2 = autotune.tune(None, s, replicas=8, moves=100, cache=cache, device="dev", measure_fn=fake_measure)
    assert r2 == r and len(calls) == n  # cached: nothing measured again
    other = FakeSystem(n=400)
    autotune.tune(None, other, replicas=8, moves=100, cache=cache, device="dev", measure_fn=fake_measure)
    assert len(json.loads(cache.read_text())) == 2


def test_shape_key_distinguishes_molecular_moves():
    a = autotune.shape_key(FakeSystem(), "d")
    b = autotune.shape_key(FakeSystem(moves=({"kind": 1, "dp": 0.5, "dprot": 0.5},)), "d")
    assert a != b and "molecular=1" in b
