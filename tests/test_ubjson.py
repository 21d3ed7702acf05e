"""Universal Binary JSON state files (faunus_gb300/ubjson.py).

Pinned on a state file the reference itself wrote (examples/multipole/multipole.state.ubj,
saved by SaveState::saveBinaryJsonStateFile, src/analysis.cpp:654-667): it decodes to the
reference's state schema, and encoding the decoded value gives the same bytes back.
"""
import math
from pathlib import Path

import pytest

from faunus_gb300 import ubjson

GOLDEN = Path(__file__).resolve().parent / "golden" / "multipole.state.ubj"


def test_reference_state_file_decodes_and_reencodes_byte_for_byte():
    raw = GOLDEN.read_bytes()
    v = ubjson.loads(raw)
    assert set(v) >= {"geometry", "groups", "particles"}
    assert v["geometry"] == {"radius": 10.0, "type": "sphere"}
    assert len(v["particles"]) == sum(g["size"] for g in v["groups"]) == 6
    assert all(len(p["pos"]) == 3 and isinstance(p["id"], int) for p in v["particles"])
    assert ubjson.dumps(v) == raw


@pytest.mark.parametrize("value", [
    None, True, False, 0, 127, 128, 255, 256, -1, -128, -129, 32767, 32768, -32769, 2 ** 31, -(2 ** 31) - 1,
    2 ** 63 - 1, 2 ** 64, 1.5, -0.0, math.inf, "", "ångström", [], {}, [1, [2.5, "x"], {"b": None, "a": [True]}],
])
def test_round_trip(value):
    back = ubjson.loads(ubjson.dumps(value))
    if isinstance(value, float) and math.isnan(value):
        assert math.isnan(back)
    else:
        assert back == value and type(back) is type(value)


def test_integer_markers_are_the_smallest_that_fit():
    assert ubjson.dumps(5) == b"i\x05"
    assert ubjson.dumps(200) == b"U\xc8"
    assert ubjson.dumps(-200) == b"I\xff\x38"
    assert ubjson.dumps(70000) == b"l\x00\x01\x11\x70"
    assert ubjson.dumps({"b": 1, "a": 2}) == b"{i\x01ai\x02i\x01bi\x01}"  # keys sorted


def test_optimised_containers_are_read():
    # [$i#i\x03 1 2 3] and {#i\x01 i\x01 k S i\x01 v}
    assert ubjson.loads(b"[$i#i\x03\x01\x02\x03") == [1, 2, 3]
    assert ubjson.loads(b"{#i\x01i\x01kSi\x01v") == {"k": "v"}
    with pytest.raises(ValueError):
        ubjson.loads(b"[i\x01")
