"""Reader for the subset of YAML that rubix's configuration files use (PyYAML is not a
dependency of this package).

rubix reads its configurations with ``yaml.safe_load`` (rubix/utils.py:47-66).  This
module parses, with YAML 1.1 scalar rules as safe_load applies them: block mappings and
block sequences by indentation (sequence items may be mappings), flow sequences and
flow mappings (``[a, b]``, ``{a: 1}``), comments, single- and double-quoted strings,
null (``null``, ``~``, empty), booleans (``true``/``false``/``yes``/``no``/``on``/
``off`` in their three spellings), integers (decimal, ``0x``, ``0o``) and floats (with a
dot, an optional exponent, ``.inf``/``.nan``; ``1e-3`` without a dot stays a string in
YAML 1.1).  Anchors, aliases, tags, block scalars (``|``, ``>``) and multi-document
streams are refused by name.
"""

from __future__ import annotations

import re
from typing import Any, List, Tuple

__all__ = ["load", "load_file", "YAMLSubsetError"]


class YAMLSubsetError(ValueError):
    pass


_INT = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_HEX = re.compile(r"^[-+]?0x[0-9a-fA-F_]+$")
_OCT = re.compile(r"^[-+]?0o?[0-7_]+$")
_FLOAT = re.compile(r"^[-+]?([0-9][0-9_]*)?\.[0-9_]*([eE][-+][0-9]+)?$")
_BOOL = {"true": True, "True": True, "TRUE": True, "false": False, "False": False,
         "FALSE": False, "yes": True, "Yes": True, "YES": True, "no": False, "No": False,
         "NO": False, "on": True, "On": True, "ON": True, "off": False, "Off": False,
         "OFF": False}
_NULL = {"", "~", "null", "Null", "NULL"}


def _scalar(tok: str) -> Any:
    s = tok.strip()
    if not s:
        return None
    if s[0] == '"':
        return _double_quoted(s)
    if s[0] == "'":
        if len(s) < 2 or s[-1] != "'":
            raise YAMLSubsetError(f"unterminated string {s!r}")
        return s[1:-1].replace("''", "'")
    if s[0] in "&*!|>":
        raise YAMLSubsetError(f"YAML feature not supported (anchor/alias/tag/block scalar): "
                              f"{s!r}")
    if s in _NULL:
        return None
    if s in _BOOL:
        return _BOOL[s]
    if _INT.match(s):
        return int(s.replace("_", ""))
    if _HEX.match(s):
        return int(s.replace("_", ""), 16)
    if _OCT.match(s) and s.lstrip("+-") not in ("0",):
        body = s.lstrip("+-")
        body = body[2:] if body.startswith("0o") else body[1:]
        val = int(body.replace("_", "") or "0", 8)
        return -val if s.startswith("-") else val
    if _FLOAT.match(s) and any(c.isdigit() for c in s):
        return float(s.replace("_", ""))
    low = s.lower()
    if low in (".inf", "+.inf"):
        return float("inf")
    if low == "-.inf":
        return float("-inf")
    if low == ".nan":
        return float("nan")
    return s


_ESC = {"n": "\n", "t": "\t", '"': '"', "\\": "\\", "/": "/", "0": "\0", "r": "\r"}


def _double_quoted(s: str) -> str:
    if len(s) < 2 or s[-1] != '"':
        raise YAMLSubsetError(f"unterminated string {s!r}")
    out, i, body = [], 0, s[1:-1]
    while i < len(body):
        c = body[i]
        if c == "\\" and i + 1 < len(body):
            out.append(_ESC.get(body[i + 1], body[i + 1]))
            i += 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _strip_comment(line: str) -> str:
    quote = None
    for i, c in enumerate(line):
        if quote:
            if c == quote:
                quote = None
        elif c in "'\"":
            quote = c
        elif c == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def _split_flow(body: str) -> List[str]:
    """Top-level comma split of the inside of [...] or {...}."""
    parts, depth, quote, cur = [], 0, None, []
    for c in body:
        if quote:
            cur.append(c)
            if c == quote:
                quote = None
            continue
        if c in "'\"":
            quote = c
        elif c in "[{":
            depth += 1
        elif c in "]}":
            depth -= 1
        elif c == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(c)
    if "".join(cur).strip():
        parts.append("".join(cur))
    return parts


def _key_split(text: str):
    """(key, rest) when text is 'key: rest' / 'key:' outside quotes and brackets."""
    quote, depth = None, 0
    for i, c in enumerate(text):
        if quote:
            if c == quote:
                quote = None
            continue
        if c in "'\"":
            quote = c
        elif c in "[{":
            depth += 1
        elif c in "]}":
            depth -= 1
        elif c == ":" and depth == 0 and (i + 1 == len(text) or text[i + 1] in " \t"):
            return _scalar(text[:i].strip()), text[i + 1:].strip()
    return None


def _value(text: str) -> Any:
    s = text.strip()
    if s.startswith("["):
        if not s.endswith("]"):
            raise YAMLSubsetError(f"unterminated flow sequence {s!r}")
        return [_value(p) for p in _split_flow(s[1:-1])]
    if s.startswith("{"):
        if not s.endswith("}"):
            raise YAMLSubsetError(f"unterminated flow mapping {s!r}")
        out = {}
        for p in _split_flow(s[1:-1]):
            kv = _key_split(p.strip()) or (p.strip().rstrip(":"), "")
            out[kv[0]] = _value(kv[1])
        return out
    return _scalar(s)


def load(text: str) -> Any:
    """The document in ``text`` as Python objects (dict / list / scalars)."""
    lines: List[Tuple[int, str]] = []
    for raw in text.splitlines():
        if raw.strip() in ("---", "...") and not lines:
            continue
        if raw.strip() == "---":
            raise YAMLSubsetError("multi-document streams are not supported")
        if "\t" in raw[:len(raw) - len(raw.lstrip())]:
            raise YAMLSubsetError("tab indentation is not allowed in YAML")
        line = _strip_comment(raw).rstrip()
        if line.strip():
            lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    if not lines:
        return None
    value, pos = _block(lines, 0, lines[0][0])
    if pos != len(lines):
        raise YAMLSubsetError(f"unexpected indentation at {lines[pos][1]!r}")
    return value


def _block(lines, pos, indent):
    if lines[pos][1].startswith("- ") or lines[pos][1] == "-":
        return _sequence(lines, pos, indent)
    if _key_split(lines[pos][1]) is not None:
        return _mapping(lines, pos, indent)
    return _value(lines[pos][1]), pos + 1


def _mapping(lines, pos, indent):
    out = {}
    while pos < len(lines) and lines[pos][0] == indent:
        kv = _key_split(lines[pos][1])
        if kv is None:
            raise YAMLSubsetError(f"expected 'key: value' at {lines[pos][1]!r}")
        key, rest = kv
        pos += 1
        if rest:
            out[key] = _value(rest)
        elif pos < len(lines) and (lines[pos][0] > indent or (
                lines[pos][0] == indent and lines[pos][1].startswith("-"))):
            out[key], pos = _block(lines, pos, lines[pos][0])
        else:
            out[key] = None
    return out, pos


def _sequence(lines, pos, indent):
    out = []
    while pos < len(lines) and lines[pos][0] == indent and (
            lines[pos][1].startswith("- ") or lines[pos][1] == "-"):
        item = lines[pos][1][1:].strip()
        if not item:
            pos += 1
            if pos < len(lines) and lines[pos][0] > indent:
                v, pos = _block(lines, pos, lines[pos][0])
                out.append(v)
            else:
                out.append(None)
            continue
        if _key_split(item) is not None and not item.startswith(("[", "{", "'", '"')):
            # a mapping item: its first key sits after "- ", the rest are indented to it
            sub_indent = indent + 2 + (len(lines[pos][1][1:]) - len(lines[pos][1][1:].lstrip()) - 1)
            sub = [(sub_indent, item)]
            pos += 1
            while pos < len(lines) and lines[pos][0] > indent:
                sub.append(lines[pos])
                pos += 1
            v, used = _mapping(sub, 0, sub_indent)
            if used != len(sub):
                raise YAMLSubsetError(f"bad indentation in the sequence item {item!r}")
            out.append(v)
        else:
            out.append(_value(item))
            pos += 1
    return out, pos


def load_file(path: str) -> Any:
    """rubix/utils.py:47-66: the YAML file at ``path`` (errors re-raised as RuntimeError
    naming the file, as rubix's read_yaml does)."""
    try:
        with open(path, "r") as f:
            return load(f.read())
    except Exception as e:
        raise RuntimeError(f"Something went wrong while reading yaml file {str(path)}") from e
