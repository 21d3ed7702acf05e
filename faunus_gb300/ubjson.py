"""Universal Binary JSON, as Faunus reads and writes its `.ubj` state files.

The reference saves a state file with the JSON library's to_ubjson and reads it with
from_ubjson (SaveState::saveBinaryJsonStateFile, src/analysis.cpp:654-667; the `--state`
reader, src/faunus.cpp:430-470).  That encoding (UBJSON draft 12, big-endian) is written
here the same way, so a state saved by this package is read by the reference and the other
way round:

  null Z, true T, false F
  integers: the smallest of i (int8), U (uint8, non-negative only), I (int16), l (int32),
            L (int64) that holds the value; beyond int64, H (the decimal digits as a string)
  floats:   D (float64)
  strings:  S, then the length as an integer, then the UTF-8 bytes
  arrays:   [ values ]           objects: { (length, key bytes, value)... }
            with keys in sorted order (the reference's objects are sorted maps)

The reader also takes the optimised containers ($ type, # count), d (float32), C (char)
and the no-op N.
"""
from __future__ import annotations

import struct
from typing import Any

_INT_FORMATS = (("i", ">b", -(1 << 7), (1 << 7) - 1), ("U", ">B", 0, (1 << 8) - 1), ("I", ">h", -(1 << 15), (1 << 15) - 1),
                ("l", ">i", -(1 << 31), (1 << 31) - 1), ("L", ">q", -(1 << 63), (1 << 63) - 1))


def _int(v: int, out: bytearray) -> None:
    for marker, fmt, lo, hi in _INT_FORMATS:
        if lo <= v <= hi:
            out += marker.encode() + struct.pack(fmt, v)
            return
    digits = str(v).encode()
    out += b"H"
    _int(len(digits), out)
    out += digits


def _value(v: Any, out: bytearray, sort_keys: bool) -> None:
    if v is None:
        out += b"Z"
    elif v is True:
        out += b"T"
    elif v is False:
        out += b"F"
    elif isinstance(v, int):
        _int(int(v), out)
    elif isinstance(v, float):
        out += b"D" + struct.pack(">d", v)
    elif isinstance(v, str):
        b = v.encode("utf-8")
        out += b"S"
        _int(len(b), out)
        out += b
    elif isinstance(v, dict):
        out += b"{"
        for k in (sorted(v) if sort_keys else v):
            kb = str(k).encode("utf-8")
            _int(len(kb), out)
            out += kb
            _value(v[k], out, sort_keys)
        out += b"}"
    elif isinstance(v, (list, tuple)):
        out += b"["
        for x in v:
            _value(x, out, sort_keys)
        out += b"]"
    else:
        # numpy scalars and arrays
        if hasattr(v, "tolist"):
            _value(v.tolist(), out, sort_keys)
        else:
            raise TypeError(f"cannot encode {type(v).__name__} as UBJSON")


def dumps(obj: Any, sort_keys: bool = True) -> bytes:
    """Encode a JSON-like value (dict, list, str, int, float, bool, None)."""
    out = bytearray()
    _value(obj, out, sort_keys)
    return bytes(out)


class _Reader:
    def __init__(self, data: bytes):
        self.d = memoryview(data)
        self.p = 0

    def peek(self) -> str:
        if self.p >= len(self.d):
            raise ValueError("truncated UBJSON data")
        return chr(self.d[self.p])

    def marker(self) -> str:
        while True:
            c = self.peek()
            self.p += 1
            if c != "N":
                return c

    def take(self, n: int) -> bytes:
        b = bytes(self.d[self.p:self.p + n])
        if len(b) != n:
            raise ValueError("truncated UBJSON data")
        self.p += n
        return b

    def typed(self, m: str) -> Any:
        if m == "Z":
            return None
        if m == "T":
            return True
        if m == "F":
            return False
        for marker, fmt, _, _ in _INT_FORMATS:
            if m == marker:
                return struct.unpack(fmt, self.take(struct.calcsize(fmt)))[0]
        if m == "d":
            return struct.unpack(">f", self.take(4))[0]
        if m == "D":
            return struct.unpack(">d", self.take(8))[0]
        if m == "H":
            s = self.take(self.count()).decode()
            return float(s) if any(c in s for c in ".eE") else int(s)
        if m == "C":
            return self.take(1).decode()
        if m == "S":
            return self.take(self.count()).decode("utf-8")
        if m == "[":
            return self.array()
        if m == "{":
            return self.obj()
        raise ValueError(f"unknown UBJSON marker {m!r} at byte {self.p - 1}")

    def count(self) -> int:
        n = self.typed(self.marker())
        if not isinstance(n, int) or n < 0:
            raise ValueError("invalid UBJSON length")
        return n

    def _header(self):
        t = n = None
        if self.peek() == "$":
            self.p += 1
            t = self.marker()
        if self.peek() == "#":
            self.p += 1
            n = self.count()
        return t, n

    def array(self) -> list:
        t, n = self._header()
        out = []
        if n is not None:
            for _ in range(n):
                out.append(self.typed(t if t else self.marker()))
            return out
        while True:
            m = self.marker()
            if m == "]":
                return out
            out.append(self.typed(m))

    def obj(self) -> dict:
        t, n = self._header()
        out = {}
        if n is not None:
            for _ in range(n):
                k = self.take(self.count()).decode("utf-8")
                out[k] = self.typed(t if t else self.marker())
            return out
        while True:
            if self.peek() == "}":
                self.p += 1
                return out
            k = self.take(self.count()).decode("utf-8")
            out[k] = self.typed(self.marker())


def loads(data: bytes) -> Any:
    """Decode one UBJSON value."""
    r = _Reader(data)
    v = r.typed(r.marker())
    return v
