"""Minimal YAML-subset reader for Cantera-style mechanism files.

Neither pyyaml nor Cantera is available, so this reader covers the subset the
mechanism files use: block mappings and sequences (any indentation), flow
sequences ``[...]`` and flow mappings ``{...}`` that may span lines, plain and
quoted scalars, ``#`` comments, and ``|`` / ``|-`` block scalars (skipped into a
string).  It is host-side set-up code, not on the hot path.
"""
from __future__ import annotations

import ast
import re

_NUM_RE = re.compile(r"^[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)$")


def _scalar(tok: str):
    t = tok.strip()
    if not t:
        return None
    if (t[0] == t[-1]) and t[0] in "'\"" and len(t) >= 2:
        return t[1:-1]
    if _NUM_RE.match(t):
        if re.match(r"^[+-]?\d+$", t):
            return int(t)
        return float(t)
    low = t.lower()
    if low in ("true", "yes"):
        return True
    if low in ("false", "no"):
        return False
    if low in ("null", "~"):
        return None
    return t


def _strip_comment(line: str) -> str:
    out, q = [], None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            # a quote only opens a quoted scalar at the start of a token
            if i == 0 or line[i - 1] in " [{,:":
                q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _parse_flow(text: str, pos: int = 0):
    """Parse a flow collection or scalar starting at text[pos]; return (value, newpos)."""
    n = len(text)
    while pos < n and text[pos] in " \t\n":
        pos += 1
    if pos >= n:
        return None, pos
    ch = text[pos]
    if ch == "[":
        pos += 1
        items = []
        while True:
            while pos < n and text[pos] in " \t\n,":
                pos += 1
            if pos < n and text[pos] == "]":
                return items, pos + 1
            val, pos = _parse_flow(text, pos)
            items.append(val)
    if ch == "{":
        pos += 1
        d = {}
        while True:
            while pos < n and text[pos] in " \t\n,":
                pos += 1
            if pos < n and text[pos] == "}":
                return d, pos + 1
            # key up to ':' followed by space
            m = re.compile(r"([^:]+?):\s").match(text, pos)
            if not m:
                raise ValueError(f"bad flow mapping near {text[pos:pos + 40]!r}")
            key = _scalar(m.group(1))
            pos = m.end()
            val, pos = _parse_flow(text, pos)
            d[key] = val
    # plain or quoted scalar up to , ] }
    if ch in "'\"":
        end = text.index(ch, pos + 1)
        return text[pos + 1:end], end + 1
    start = pos
    while pos < n and text[pos] not in ",]}":
        pos += 1
    return _scalar(text[start:pos]), pos


def _balanced(s: str) -> bool:
    depth, q = 0, None
    for ch in s:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
    return depth <= 0


def _open_quote(content: str) -> bool:
    """True when the value of a `key: value` or `- value` line opens a quoted
    scalar that does not close on this line (it continues on the next)."""
    m = re.match(r"^(?:-\s+)?(?:[^'\"\s][^:]*:\s+)?(['\"])", content)
    if not m:
        return False
    q = m.group(1)
    body = content[m.end():]
    if q == "'":
        body = body.replace("''", "")
    else:
        body = body.replace('\\"', "")
    return q not in body


class _Lines:
    def __init__(self, text: str):
        raw = text.splitlines()
        self.items = []  # (indent, content, raw_line)
        i = 0
        while i < len(raw):
            line = raw[i]
            stripped = _strip_comment(line)
            if not stripped.strip():
                i += 1
                continue
            indent = len(stripped) - len(stripped.lstrip(" "))
            content = stripped.strip()
            # block scalar: swallow following more-indented (or blank) lines
            if re.search(r":\s*[|>][-+]?$", content) or content in ("|", "|-", ">", ">-"):
                body = []
                j = i + 1
                while j < len(raw) and (not raw[j].strip() or
                                        len(raw[j]) - len(raw[j].lstrip(" ")) > indent):
                    body.append(raw[j].strip())
                    j += 1
                content = re.sub(r"[|>][-+]?$", "", content).rstrip() + " " + repr("\n".join(body))
                self.items.append((indent, content))
                i = j
                continue
            # join multi-line flow collections and quoted scalars
            j = i
            while (not _balanced(content) or _open_quote(content)) and j + 1 < len(raw):
                j += 1
                content += " " + (raw[j].strip() if _open_quote(content) else _strip_comment(raw[j]).strip())
            self.items.append((indent, content))
            i = j + 1


def _split_key(content: str):
    """Split 'key: value' at the first ': ' (or trailing ':') outside brackets/quotes."""
    depth, q = 0, None
    for i, ch in enumerate(content):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"" and (i == 0 or content[i - 1] in " [{,:"):
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == ":" and depth == 0 and (i + 1 == len(content) or content[i + 1] == " "):
            return content[:i].strip(), content[i + 1:].strip()
    return None, content


def _value(text: str):
    text = text.strip()
    if text[:1] in "'\"":
        if len(text) >= 2 and text[-1] == text[0]:
            try:
                return ast.literal_eval(text)
            except (ValueError, SyntaxError):
                return text[1:-1]
        return text.strip("'\"")
    if text[:1] in "[{":
        return _parse_flow(text)[0]
    return _scalar(text)


def _parse_block(items, i, indent):
    """Parse a block node whose lines sit at column `indent`; return (value, next_i)."""
    if i >= len(items):
        return None, i
    ind, content = items[i]
    if content.startswith("- ") or content == "-":
        seq = []
        while i < len(items) and items[i][0] == indent and (items[i][1].startswith("- ") or items[i][1] == "-"):
            body = items[i][1][2:] if items[i][1] != "-" else ""
            if not body.strip():
                if i + 1 < len(items) and items[i + 1][0] > indent:
                    val, i = _parse_block(items, i + 1, items[i + 1][0])
                else:
                    val, i = None, i + 1
                seq.append(val)
                continue
            key, rest = _split_key(body)
            if key is None:
                seq.append(_value(body))
                i += 1
                continue
            # mapping inside a sequence item: first key is inline after "- "
            sub_indent = indent + (len(items[i][1]) - len(body))
            items[i] = (sub_indent, body)
            val, i = _parse_block(items, i, sub_indent)
            seq.append(val)
        return seq, i
    d = {}
    while i < len(items) and items[i][0] == indent and not items[i][1].startswith("- "):
        key, rest = _split_key(items[i][1])
        if key is None:
            raise ValueError(f"expected key at line {items[i][1]!r}")
        key = _scalar(key)
        if rest:
            d[key] = _value(rest)
            i += 1
        else:
            if i + 1 < len(items) and (items[i + 1][0] > indent or
                                       (items[i + 1][0] == indent and items[i + 1][1].startswith("- "))):
                val, i = _parse_block(items, i + 1, items[i + 1][0])
                d[key] = val
            else:
                d[key] = None
                i += 1
    return d, i


def loads(text: str):
    items = _Lines(text).items
    if not items:
        return None
    val, _ = _parse_block(items, 0, items[0][0])
    return val


def load(path: str):
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        return loads(f.read())
