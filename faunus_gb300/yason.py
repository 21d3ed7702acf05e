"""A YAML subset reader for Faunus input files.

The reference reads JSON and converts YAML input with its ``yason.py`` script
(scripts/yason.py) through PyYAML.  This reader covers the YAML that Faunus
inputs use -- block mappings and sequences, sequence items that open a mapping
(``- nonbonded_pm:`` followed by indented keys), flow mappings and sequences
(``{q: 1.0, sigma: 4}``, ``[Na, Cl]``), plain and quoted scalars, comments and a
``#!`` first line -- and returns the same Python objects PyYAML would (int,
float, bool, None, str, list, dict).  Anchors, tags, multi-line scalars and
multiple documents are not supported and raise ValueError.

Like the reference script, which renders the file with jinja2 first
(scripts/yason.py:160-165), ``loads`` renders the template forms Faunus inputs
use: ``{% set name = expression %}`` lines and ``{{ expression }}`` with numbers,
the names set before, + - * / // % ** and parentheses; a value renders as
Python's str() of it, as jinja2 prints it.  Other template constructs raise
ValueError.
"""
from __future__ import annotations

import ast
import operator
import re
from typing import Any, List, Tuple

_INT = re.compile(r"^[-+]?(0|[1-9][0-9]*)$")
_FLOAT = re.compile(r"^[-+]?(\.[0-9]+|[0-9]+(\.[0-9]*)?)([eE][-+]?[0-9]+)?$")


def scalar(text: str) -> Any:
    """YAML 1.1 core scalars as PyYAML resolves them (bools, null, int, float, str)."""
    t = text.strip()
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "\"'":
        body = t[1:-1]
        return body.replace("\\\"", "\"").replace("\\\\", "\\") if t[0] == '"' else body.replace("''", "'")
    low = t.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    if low in ("null", "~", ""):
        return None
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t) and any(c.isdigit() for c in t):
        return float(t)
    if low in (".inf", "+.inf"):
        return float("inf")
    if low == "-.inf":
        return float("-inf")
    if low == ".nan":
        return float("nan")
    return t


def _strip_comment(line: str) -> str:
    out, quote, depth = [], None, 0
    for i, c in enumerate(line):
        if quote:
            if c == quote:
                quote = None
        elif c in "\"'" and (i == 0 or line[i - 1] in " \t[{,:"):
            quote = c
        elif c == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(c)
    return "".join(out).rstrip()


def _split_key(text: str):
    """(key, rest) if `text` is `key: rest` / `key:` outside quotes and brackets, else None."""
    quote, depth = None, 0
    for i, c in enumerate(text):
        if quote:
            if c == quote:
                quote = None
            continue
        if c in "\"'" and i == 0:
            quote = c
        elif c in "[{":
            depth += 1
        elif c in "]}":
            depth -= 1
        elif c == ":" and depth == 0 and (i + 1 == len(text) or text[i + 1] in " \t"):
            return text[:i].strip(), text[i + 1:].strip()
    return None


class _Flow:
    """Recursive-descent parser for flow collections."""

    def __init__(self, text: str):
        self.s, self.i = text, 0

    def ws(self):
        while self.i < len(self.s) and self.s[self.i] in " \t":
            self.i += 1

    def value(self) -> Any:
        self.ws()
        if self.i >= len(self.s):
            return None
        c = self.s[self.i]
        if c == "{":
            return self.mapping()
        if c == "[":
            return self.sequence()
        return scalar(self.token())

    def token(self) -> str:
        self.ws()
        st = self.i
        if self.i < len(self.s) and self.s[self.i] in "\"'":
            q = self.s[self.i]
            self.i += 1
            while self.i < len(self.s):
                if self.s[self.i] == q:
                    if q == "'" and self.s[self.i + 1:self.i + 2] == "'":  # '' inside '...'
                        self.i += 2
                        continue
                    break
                if q == '"' and self.s[self.i] == "\\":
                    self.i += 1
                self.i += 1
            self.i += 1
            return self.s[st:self.i]
        while self.i < len(self.s):
            c = self.s[self.i]
            if c in ",]}":
                break
            if c == ":" and (self.i + 1 == len(self.s) or self.s[self.i + 1] in " \t,]}"):
                break
            self.i += 1
        return self.s[st:self.i].strip()

    def expect(self, c: str):
        self.ws()
        if self.i >= len(self.s) or self.s[self.i] != c:
            raise ValueError(f"expected '{c}' at column {self.i} of {self.s!r}")
        self.i += 1

    def mapping(self) -> dict:
        self.expect("{")
        out = {}
        self.ws()
        if self.s[self.i:self.i + 1] == "}":
            self.i += 1
            return out
        while True:
            key = scalar(self.token())
            self.ws()
            if self.s[self.i:self.i + 1] == ":":
                self.i += 1
                out[key] = self.value()
            else:
                out[key] = None
            self.ws()
            if self.s[self.i:self.i + 1] == ",":
                self.i += 1
                continue
            self.expect("}")
            return out

    def sequence(self) -> list:
        self.expect("[")
        out = []
        self.ws()
        if self.s[self.i:self.i + 1] == "]":
            self.i += 1
            return out
        while True:
            out.append(self.value())
            self.ws()
            if self.s[self.i:self.i + 1] == ",":
                self.i += 1
                continue
            self.expect("]")
            return out


def _flow(text: str) -> Any:
    if text[:1] in "[{":
        f = _Flow(text)
        v = f.value()
        f.ws()
        if f.i != len(f.s):
            raise ValueError(f"trailing text after flow collection: {text!r}")
        return v
    if text[:1] in "&*!|>":
        raise ValueError(f"unsupported YAML construct: {text!r}")
    return scalar(text)


def _block(lines: List[Tuple[int, str]], i: int, indent: int) -> Tuple[Any, int]:
    ind, text = lines[i]
    if text == "-" or text.startswith("- "):
        out = []
        while i < len(lines) and lines[i][0] == indent and (lines[i][1] == "-" or lines[i][1].startswith("- ")):
            item = lines[i][1][1:].strip()
            if not item:
                if i + 1 < len(lines) and lines[i + 1][0] > indent:
                    v, i = _block(lines, i + 1, lines[i + 1][0])
                else:
                    v, i = None, i + 1
                out.append(v)
                continue
            if _split_key(item) is not None and item[:1] not in "[{":
                # the item opens a mapping: its first key sits two columns right of the dash
                sub = indent + (len(lines[i][1]) - len(lines[i][1][1:].lstrip()))
                lines[i] = (sub, item)
                v, i = _block(lines, i, sub)
                out.append(v)
                continue
            out.append(_flow(item))
            i += 1
        return out, i
    out = {}
    while i < len(lines) and lines[i][0] == indent:
        text = lines[i][1]
        kv = _split_key(text)
        if kv is None:
            raise ValueError(f"expected 'key: value', got {text!r}")
        key, rest = kv
        key = scalar(key)
        if rest:
            out[key] = _flow(rest)
            i += 1
            continue
        i += 1
        if i < len(lines) and (lines[i][0] > indent or
                               (lines[i][0] == indent and (lines[i][1] == "-" or lines[i][1].startswith("- ")))):
            out[key], i = _block(lines, i, lines[i][0])
        else:
            out[key] = None
    if i < len(lines) and lines[i][0] > indent:
        raise ValueError(f"unexpected indentation at {lines[i][1]!r}")
    return out, i


_SET = re.compile(r"^\{%-?\s*set\s+([A-Za-z_]\w*)\s*=\s*(.+?)\s*-?%\}$")
_EXPR = re.compile(r"\{\{\s*(.+?)\s*\}\}")
_BINOPS = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
           ast.FloorDiv: operator.floordiv, ast.Mod: operator.mod, ast.Pow: operator.pow}


def _evaluate(expr: str, names: dict) -> Any:
    """An arithmetic template expression over numbers and the names set so far."""
    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return node.value
        if isinstance(node, ast.Name):
            if node.id not in names:
                raise ValueError(f"template name {node.id!r} is not set")
            return names[node.id]
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
            v = ev(node.operand)
            return -v if isinstance(node.op, ast.USub) else v
        if isinstance(node, ast.BinOp) and type(node.op) in _BINOPS:
            return _BINOPS[type(node.op)](ev(node.left), ev(node.right))
        raise ValueError(f"unsupported template expression {expr!r}")
    try:
        tree = ast.parse(expr.strip(), mode="eval")
    except SyntaxError as e:
        raise ValueError(f"unsupported template expression {expr!r}") from e
    return ev(tree)


def render(text: str) -> str:
    """The jinja2 forms of Faunus inputs: `{% set %}` lines and `{{ expression }}`."""
    if "{%" not in text and "{{" not in text:
        return text
    names: dict = {}
    out = []
    for line in text.split("\n"):
        m = _SET.match(line.strip())
        if m:
            names[m.group(1)] = _evaluate(m.group(2), names)
            continue
        line = _EXPR.sub(lambda mm: str(_evaluate(mm.group(1), names)), line)
        if "{%" in line or "{{" in line:
            raise ValueError(f"unsupported template construct in {line.strip()!r}")
        out.append(line)
    return "\n".join(out)


def loads(text: str) -> Any:
    """Parse one YAML document of the supported subset (templates rendered first)."""
    text = render(text)
    lines = []
    for n, raw in enumerate(text.splitlines()):
        if n == 0 and raw.startswith("#!"):
            continue
        if "\t" in raw[: len(raw) - len(raw.lstrip())]:
            raise ValueError("tabs in indentation")
        s = _strip_comment(raw)
        if not s.strip():
            continue
        if s.strip() in ("---", "..."):
            continue
        lines.append((len(s) - len(s.lstrip()), s.strip()))
    if not lines:
        return None
    v, i = _block(lines, 0, lines[0][0])
    if i != len(lines):
        raise ValueError(f"could not parse from line {lines[i][1]!r}")
    return v
