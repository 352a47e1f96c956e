"""A YAML subset parser for SpinED configuration files.

SpinED reads its input with Data.Yaml (src/SpinED.hs:252-261); neither
libyaml nor PyYAML is available to this package, so this module parses the
part of YAML that the configuration format uses (template.yaml, the example
files):

* block mappings (``key: value``) and block sequences (``- item``), nested by
  indentation, including a mapping that starts on a sequence item's line;
* flow sequences and mappings (``[1, [2, 3]]``, ``{a: 1}``), which may span
  several lines;
* comments (``#`` at the start of a line or after whitespace);
* scalars: double- and single-quoted strings, integers, floats (``1.0e-6``,
  ``.5``, ``.inf``, ``.nan``), ``true``/``false``, ``null``/``~``/empty,
  anything else as a plain string.

Anchors, aliases, tags, block scalars (``|``, ``>``) and multi-document
streams are rejected with YamlError.
"""
from __future__ import annotations

import math
import re

__all__ = ["YamlError", "loads", "load"]


class YamlError(ValueError):
    pass


_INT = re.compile(r"[-+]?(0|[1-9][0-9_]*)$")
_HEX = re.compile(r"0x[0-9a-fA-F_]+$")
_FLOAT = re.compile(r"[-+]?(\.[0-9]+|[0-9][0-9_]*(\.[0-9]*)?)([eE][-+]?[0-9]+)?$")


def _scalar(text: str, line: int):
    t = text.strip()
    if t == "" or t in ("~", "null", "Null", "NULL"):
        return None
    if t[0] in "\"'":
        s, rest = _quoted(t, 0, line)
        if t[rest:].strip():
            raise YamlError(f"line {line}: unexpected text after string: {t[rest:]!r}")
        return s
    if t[0] in "&*!|>%@`":
        raise YamlError(f"line {line}: unsupported YAML construct {t[0]!r}")
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if _INT.match(t):
        return int(t.replace("_", ""))
    if _HEX.match(t):
        return int(t.replace("_", ""), 16)
    if _FLOAT.match(t):
        return float(t.replace("_", ""))
    low = t.lower()
    if low in (".inf", "+.inf"):
        return math.inf
    if low == "-.inf":
        return -math.inf
    if low == ".nan":
        return math.nan
    return t


def _quoted(t: str, i: int, line: int) -> tuple[str, int]:
    """String starting at t[i] (a quote); returns (value, index after it)."""
    q = t[i]
    out = []
    j = i + 1
    while j < len(t):
        ch = t[j]
        if q == "'" and ch == "'":
            if j + 1 < len(t) and t[j + 1] == "'":
                out.append("'")
                j += 2
                continue
            return "".join(out), j + 1
        if q == '"' and ch == "\\":
            if j + 1 >= len(t):
                break
            esc = t[j + 1]
            table = {"n": "\n", "t": "\t", "\\": "\\", '"': '"', "/": "/", "0": "\0", "r": "\r"}
            if esc in table:
                out.append(table[esc])
                j += 2
                continue
            if esc == "u" and j + 5 < len(t):
                out.append(chr(int(t[j + 2:j + 6], 16)))
                j += 6
                continue
            raise YamlError(f"line {line}: unknown escape \\{esc}")
        if q == '"' and ch == '"':
            return "".join(out), j + 1
        out.append(ch)
        j += 1
    raise YamlError(f"line {line}: unterminated string")


def _strip_comment(s: str) -> str:
    """Removes a comment that is not inside quotes."""
    q = None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            elif ch == "\\" and q == '"':
                continue
        elif ch in "\"'" and (i == 0 or s[i - 1] in " \t[{,:-"):
            q = ch
        elif ch == "#" and (i == 0 or s[i - 1] in " \t"):
            return s[:i]
    return s


def _depth(s: str) -> int:
    """Net count of open flow brackets outside quotes."""
    d, q = 0, None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
        elif ch in "\"'" and (i == 0 or s[i - 1] in " \t[{,:"):
            q = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
    return d


class _Flow:
    """Recursive-descent parser for a flow collection or scalar."""

    def __init__(self, text: str, line: int):
        self.t, self.i, self.line = text, 0, line

    def ws(self):
        while self.i < len(self.t) and self.t[self.i] in " \t\n":
            self.i += 1

    def value(self):
        self.ws()
        if self.i >= len(self.t):
            raise YamlError(f"line {self.line}: unexpected end of flow collection")
        ch = self.t[self.i]
        if ch == "[":
            return self.seq()
        if ch == "{":
            return self.map()
        if ch in "\"'":
            s, self.i = _quoted(self.t, self.i, self.line)
            return s
        j = self.i
        while j < len(self.t) and self.t[j] not in ",]}":
            if self.t[j] == ":" and (j + 1 >= len(self.t) or self.t[j + 1] in " \t"):
                break
            j += 1
        text = self.t[self.i:j]
        self.i = j
        return _scalar(text, self.line)

    def seq(self):
        self.i += 1
        out = []
        self.ws()
        if self.t[self.i:self.i + 1] == "]":
            self.i += 1
            return out
        while True:
            out.append(self.value())
            self.ws()
            if self.i >= len(self.t):
                raise YamlError(f"line {self.line}: unterminated [")
            ch = self.t[self.i]
            self.i += 1
            if ch == "]":
                return out
            if ch != ",":
                raise YamlError(f"line {self.line}: expected ',' or ']' in flow sequence, got {ch!r}")
            self.ws()
            if self.t[self.i:self.i + 1] == "]":  # trailing comma
                self.i += 1
                return out

    def map(self):
        self.i += 1
        out = {}
        self.ws()
        if self.t[self.i:self.i + 1] == "}":
            self.i += 1
            return out
        while True:
            k = self.value()
            self.ws()
            if self.t[self.i:self.i + 1] != ":":
                raise YamlError(f"line {self.line}: expected ':' in flow mapping")
            self.i += 1
            out[k] = self.value()
            self.ws()
            if self.i >= len(self.t):
                raise YamlError(f"line {self.line}: unterminated {{")
            ch = self.t[self.i]
            self.i += 1
            if ch == "}":
                return out
            if ch != ",":
                raise YamlError(f"line {self.line}: expected ',' or '}}' in flow mapping")


def _flow_value(text: str, line: int):
    text = text.strip()
    if text[:1] in "[{":
        p = _Flow(text, line)
        v = p.value()
        p.ws()
        if p.i != len(text):
            raise YamlError(f"line {line}: unexpected text after flow collection: {text[p.i:]!r}")
        return v
    return _scalar(text, line)


def _logical_lines(src: str) -> list[tuple[int, str, int]]:
    """(indent, content, line number) with comments removed and flow
    collections joined across lines."""
    out = []
    pending = None
    for n, raw in enumerate(src.splitlines(), 1):
        if "\t" in raw[: len(raw) - len(raw.lstrip())]:
            raise YamlError(f"line {n}: tabs are not allowed in indentation")
        s = _strip_comment(raw).rstrip()
        if pending is not None:
            pending[1] += " " + s.strip()
            if _depth(pending[1]) <= 0:
                out.append(tuple(pending))
                pending = None
            continue
        if not s.strip():
            continue
        if s.strip() in ("---", "..."):
            if out:
                raise YamlError(f"line {n}: multi-document streams are not supported")
            continue
        indent = len(s) - len(s.lstrip(" "))
        item = [indent, s.strip(), n]
        if _depth(s) > 0:
            pending = item
        else:
            out.append(tuple(item))
    if pending is not None:
        raise YamlError(f"line {pending[2]}: unterminated flow collection")
    return out


def _split_key(content: str, line: int):
    """'key: value' -> (key, value text) or None when content is not a mapping entry."""
    if content[:1] in "\"'":
        key, j = _quoted(content, 0, line)
        rest = content[j:].lstrip()
        if rest.startswith(":") and (len(rest) == 1 or rest[1] in " \t"):
            return key, rest[1:].strip()
        return None
    if content[:1] in "[{":
        return None
    m = re.match(r"([^:#]+?)\s*:(\s+|$)", content)
    if not m:
        return None
    return _scalar(m.group(1), line), content[m.end():]


class _Block:
    def __init__(self, lines):
        self.lines = lines
        self.i = 0

    def parse(self, indent: int):
        if self.i >= len(self.lines):
            return None
        ind, content, n = self.lines[self.i]
        if ind < indent:
            return None
        if content == "-" or content.startswith("- "):
            return self.seq(ind)
        if _split_key(content, n) is not None:
            return self.mapping(ind)
        self.i += 1
        return _flow_value(content, n)

    def seq(self, indent: int):
        out = []
        while self.i < len(self.lines):
            ind, content, n = self.lines[self.i]
            if ind != indent or not (content == "-" or content.startswith("- ")):
                if ind > indent:
                    raise YamlError(f"line {n}: bad indentation")
                break
            rest = content[1:].lstrip()
            if not rest:
                self.i += 1
                out.append(self.parse(indent + 1))
                continue
            # the item's content starts at this column; rewrite the line and parse it as a block
            col = indent + (len(content) - len(rest))
            self.lines[self.i] = (col, rest, n)
            out.append(self.parse(col))
        return out

    def mapping(self, indent: int):
        out = {}
        while self.i < len(self.lines):
            ind, content, n = self.lines[self.i]
            if ind != indent:
                if ind > indent:
                    raise YamlError(f"line {n}: bad indentation")
                break
            kv = _split_key(content, n)
            if kv is None:
                raise YamlError(f"line {n}: expected 'key: value'")
            key, rest = kv
            if key in out:
                raise YamlError(f"line {n}: duplicate key {key!r}")
            self.i += 1
            if rest:
                out[key] = _flow_value(rest, n)
                continue
            if self.i < len(self.lines):
                nind, ncontent, _ = self.lines[self.i]
                if nind > indent or (nind == indent and (ncontent == "-" or ncontent.startswith("- "))):
                    out[key] = self.parse(nind)
                    continue
            out[key] = None
        return out


def loads(src: str):
    """Parses a YAML document (the subset described in the module docstring)."""
    lines = _logical_lines(src)
    if not lines:
        return None
    b = _Block(lines)
    v = b.parse(lines[0][0])
    if b.i != len(b.lines):
        raise YamlError(f"line {b.lines[b.i][2]}: unexpected content")
    return v


def load(path: str):
    with open(path, encoding="utf-8") as f:
        return loads(f.read())
