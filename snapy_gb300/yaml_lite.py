"""A small YAML-subset reader for snapy input decks.

PyYAML and yaml-cpp are not part of this stack, so the decks are read by this
module.  It covers what snapy's decks use: block mappings, block sequences
(``- name: dry``), flow mappings ``{a: b, c: d}``, flow sequences ``[a, b]``,
plain and quoted scalars, ``#`` comments, and the scalar types null, bool,
int, float and string (YAML 1.2 core schema plus the ``1.e5`` float forms the
decks write).  Anchors, tags and multi-line scalars are rejected.
"""
from __future__ import annotations

import re

__all__ = ["load", "loads", "YamlError"]


class YamlError(ValueError):
    pass


_INT = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_FLOAT = re.compile(
    r"^[-+]?(\.[0-9]+|[0-9][0-9_]*(\.[0-9_]*)?)([eE][-+]?[0-9]+)?$")


def _scalar(tok: str):
    t = tok.strip()
    if t == "" or t in ("~", "null", "Null", "NULL"):
        return None
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        body = t[1:-1]
        if t[0] == '"':
            body = bytes(body, "utf-8").decode("unicode_escape")
        else:
            body = body.replace("''", "'")
        return body
    if t in ("true", "True", "TRUE", "yes", "Yes", "on", "On"):
        return True
    if t in ("false", "False", "FALSE", "no", "No", "off", "Off"):
        return False
    if _INT.match(t):
        return int(t.replace("_", ""))
    if _FLOAT.match(t) and any(c.isdigit() for c in t):
        return float(t.replace("_", ""))
    if t in (".inf", "+.inf", ".Inf"):
        return float("inf")
    if t in ("-.inf", "-.Inf"):
        return float("-inf")
    if t in (".nan", ".NaN"):
        return float("nan")
    if t[0] in "&*!|>":
        raise YamlError(f"unsupported YAML construct: {t!r}")
    return t


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for i, ch in enumerate(line):
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _split_flow(body: str):
    """Split a flow collection body at top-level commas."""
    parts, depth, cur, quote = [], 0, [], None
    for ch in body:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur))
    return parts


def _split_key(text: str):
    """'key: value' -> (key, value) at the first top-level ': ' / trailing ':'."""
    depth, quote = 0, None
    for i, ch in enumerate(text):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == ":" and depth == 0 and (i + 1 == len(text) or text[i + 1] in " \t"):
            return text[:i].strip(), text[i + 1:].strip()
    return None


def _flow(text: str):
    t = text.strip()
    if t.startswith("{"):
        if not t.endswith("}"):
            raise YamlError(f"unterminated flow mapping: {t!r}")
        out = {}
        for item in _split_flow(t[1:-1]):
            kv = _split_key(item.strip())
            if kv is None:
                raise YamlError(f"flow mapping item without ':': {item!r}")
            out[_scalar(kv[0])] = _flow(kv[1])
        return out
    if t.startswith("["):
        if not t.endswith("]"):
            raise YamlError(f"unterminated flow sequence: {t!r}")
        return [_flow(x) for x in _split_flow(t[1:-1])]
    return _scalar(t)


class _Lines:
    def __init__(self, text: str):
        self.items = []
        for n, raw in enumerate(text.splitlines(), 1):
            if raw.strip() in ("---", "..."):
                continue
            if "\t" in raw[: len(raw) - len(raw.lstrip())]:
                raise YamlError(f"line {n}: tab indentation")
            line = _strip_comment(raw)
            if not line.strip():
                continue
            ind = len(line) - len(line.lstrip(" "))
            self.items.append((ind, line.strip(), n))
        self.pos = 0

    def peek(self):
        return self.items[self.pos] if self.pos < len(self.items) else None


def _parse_block(L: _Lines, indent: int):
    first = L.peek()
    if first is None or first[0] < indent:
        return None
    ind = first[0]
    if first[1].startswith("- ") or first[1] == "-":
        return _parse_seq(L, ind)
    return _parse_map(L, ind)


def _value_after(L: _Lines, rest: str, ind: int, lineno: int):
    if rest == "":
        nxt = L.peek()
        if nxt is not None and (nxt[0] > ind or (
                nxt[0] == ind and (nxt[1].startswith("- ") or nxt[1] == "-"))):
            return _parse_block(L, nxt[0])
        return None
    if rest[0] in "{[":
        # a flow collection may span lines: join until brackets balance
        text = rest
        while _depth(text) > 0:
            nxt = L.peek()
            if nxt is None:
                raise YamlError(f"line {lineno}: unterminated flow collection")
            text += " " + nxt[1]
            L.pos += 1
        return _flow(text)
    return _scalar(rest)


def _depth(text: str) -> int:
    d, quote = 0, None
    for ch in text:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch in "[{":
            d += 1
        elif ch in "]}":
            d -= 1
    return d


def _parse_map(L: _Lines, ind: int):
    out = {}
    while True:
        cur = L.peek()
        if cur is None or cur[0] < ind:
            return out
        if cur[0] > ind:
            raise YamlError(f"line {cur[2]}: bad indentation")
        text = cur[1]
        if text.startswith("- "):
            return out
        kv = _split_key(text)
        if kv is None:
            raise YamlError(f"line {cur[2]}: expected 'key: value', got {text!r}")
        L.pos += 1
        key = _scalar(kv[0])
        if key in out:
            raise YamlError(f"line {cur[2]}: duplicate key {key!r}")
        out[key] = _value_after(L, kv[1], ind, cur[2])


def _parse_seq(L: _Lines, ind: int):
    out = []
    while True:
        cur = L.peek()
        if cur is None or cur[0] < ind:
            return out
        text = cur[1]
        if cur[0] != ind or not (text.startswith("- ") or text == "-"):
            return out
        L.pos += 1
        rest = text[1:].strip()
        if rest == "":
            out.append(_parse_block(L, ind + 1))
            continue
        kv = _split_key(rest) if rest[0] not in "{[\"'" else None
        if kv is not None:
            # an inline mapping item: "- key: value" with more keys below
            child_ind = ind + 2
            item = {_scalar(kv[0]): _value_after(L, kv[1], child_ind, cur[2])}
            nxt = L.peek()
            if nxt is not None and nxt[0] > ind and not nxt[1].startswith("- "):
                more = _parse_map(L, nxt[0])
                for k, v in more.items():
                    if k in item:
                        raise YamlError(f"line {nxt[2]}: duplicate key {k!r}")
                    item[k] = v
            out.append(item)
        else:
            out.append(_value_after(L, rest, ind, cur[2]))


def loads(text: str):
    L = _Lines(text)
    if L.peek() is None:
        return None
    v = _parse_block(L, 0)
    if L.peek() is not None:
        raise YamlError(f"line {L.peek()[2]}: unexpected content")
    return v


def load(path: str):
    with open(path, "r", encoding="utf-8") as f:
        return loads(f.read())
