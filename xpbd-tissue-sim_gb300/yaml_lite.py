"""A reader for the YAML subset the reference's configuration files use
(config/*.yaml, parsed there by yaml-cpp in include/config/Config.hpp).

Supported: block mappings (`key: value`), block sequences (`-` items, with
the item's mapping either on the dash line or indented below it), flow
sequences (`[a, "b", 1e-3]`, also over several lines), plain / single- /
double-quoted scalars, `#`
comments, and the scalar forms yaml-cpp converts for the reference's
parameter types: booleans (true/false/yes/no/on/off), integers, floats
(including `1e-3`, `.5`, `inf`) and null (`~`, `null`, empty). Anchors,
aliases, tags, multi-line scalars and flow mappings are not part of that
subset and raise ValueError.
"""
from __future__ import annotations

import re

_FLOAT = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$")
_INT = re.compile(r"^[-+]?\d+$")


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for i, ch in enumerate(line):
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def scalar(text: str):
    """Convert one scalar as yaml-cpp's `as<T>` would for the reference's
    parameter types (strings stay strings unless they read as numbers or
    booleans)."""
    t = text.strip()
    if not t or t in ("~", "null", "Null", "NULL"):
        return None
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "\"'":
        return t[1:-1]
    low = t.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t):
        return float(t)
    if low in (".inf", "inf", "+.inf", "+inf"):
        return float("inf")
    if low in ("-.inf", "-inf"):
        return float("-inf")
    if t[0] in "&*!|>{":
        raise ValueError(f"unsupported YAML construct: {t!r}")
    return t


def _depth(text: str) -> int:
    """Open '[' minus ']' outside quotes."""
    depth, quote = 0, None
    for ch in text:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
    return depth


def _flow_seq(text: str):
    inner = text.strip()[1:-1]
    items, cur, quote, depth = [], [], None, 0
    for ch in inner:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
        elif ch == "," and depth == 0:
            items.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    if "".join(cur).strip():
        items.append("".join(cur))
    return [_value(i) for i in items]


def _value(text: str):
    t = text.strip()
    if t.startswith("["):
        if not t.endswith("]"):
            raise ValueError(f"unterminated flow sequence: {t!r}")
        return _flow_seq(t)
    return scalar(t)


def _split_key(content: str):
    """`key: value` -> (key, value text) or None when the line is no mapping entry."""
    quote = None
    for i, ch in enumerate(content):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch == ":" and (i + 1 == len(content) or content[i + 1] in " \t"):
            key = content[:i].strip()
            if len(key) >= 2 and key[0] == key[-1] and key[0] in "\"'":
                key = key[1:-1]
            return key, content[i + 1:].strip()
    return None


def loads(text: str):
    lines = []
    for raw in text.splitlines():
        if "\t" in raw[: len(raw) - len(raw.lstrip())]:
            raise ValueError("tabs in indentation")
        s = _strip_comment(raw)
        if s.strip() in ("---", "..."):
            continue
        if s.strip():
            lines.append((len(s) - len(s.lstrip(" ")), s.strip()))
    # a flow sequence may continue over several lines: join until balanced
    merged = []
    for ind, content in lines:
        if merged and _depth(merged[-1][1]) > 0:
            merged[-1] = (merged[-1][0], merged[-1][1] + " " + content)
        else:
            merged.append((ind, content))
    lines = merged
    pos = 0

    def block(indent):
        nonlocal pos
        if pos >= len(lines):
            return None
        ind, content = lines[pos]
        if content.startswith("- ") or content == "-":
            return seq(ind)
        return mapping(ind)

    def seq(indent):
        nonlocal pos
        out = []
        while pos < len(lines):
            ind, content = lines[pos]
            if ind != indent or not (content.startswith("- ") or content == "-"):
                break
            rest = content[1:].strip()
            pos += 1
            if not rest:
                out.append(block(lines[pos][0]) if pos < len(lines) and lines[pos][0] > indent else None)
            elif _split_key(rest) is not None and not rest.startswith("["):
                # a mapping starting on the dash line: its keys align with rest
                key_indent = indent + (len(content) - len(rest))
                lines.insert(pos, (key_indent, rest))
                out.append(mapping(key_indent))
            else:
                out.append(_value(rest))
        return out

    def mapping(indent):
        nonlocal pos
        out = {}
        while pos < len(lines):
            ind, content = lines[pos]
            if ind < indent:
                break
            if ind > indent:
                raise ValueError(f"bad indentation at {content!r}")
            kv = _split_key(content)
            if kv is None:
                raise ValueError(f"expected 'key: value', got {content!r}")
            key, rest = kv
            pos += 1
            if rest:
                out[key] = _value(rest)
            elif pos < len(lines) and (lines[pos][0] > indent or
                                       (lines[pos][0] == indent and lines[pos][1].startswith("-"))):
                out[key] = block(lines[pos][0])
            else:
                out[key] = None
        return out

    result = block(0)
    if pos != len(lines):
        raise ValueError(f"unparsed content at {lines[pos][1]!r}")
    return result


def load(path: str):
    with open(path) as f:
        return loads(f.read())
