"""Configuration files in the reference's schema (phrike/io.py:12-16 loads
them with yaml.safe_load).

PyYAML is used when it is installed.  Without it, ``load_yaml`` reads the
subset of YAML the reference's configs are written in: nested mappings by
indentation, ``key: value`` scalars (integers, floats such as ``1e-6``,
true/false, null/~, plain or quoted strings), flow lists ``[a, "b", 1.0]``
and empty flow mappings ``{}``, with ``#`` comments.  Anything else raises
ValueError rather than being read differently from PyYAML.
"""
from __future__ import annotations

import json
import re
from typing import Any, Dict, List, Optional, Tuple

_INT = re.compile(r"^[-+]?(0|[1-9][0-9]*)$")
_FLOAT = re.compile(r"^[-+]?(\d+\.\d*|\.\d+|\d+)([eE][-+]?\d+)?$")


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in ("'", '"'):
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        out.append(ch)
    return "".join(out).rstrip()


def _scalar(text: str) -> Any:
    s = text.strip()
    if s == "" or s in ("null", "Null", "NULL", "~"):
        return None
    if s in ("true", "True", "TRUE"):
        return True
    if s in ("false", "False", "FALSE"):
        return False
    if len(s) >= 2 and s[0] == s[-1] and s[0] in ("'", '"'):
        return s[1:-1]
    if _INT.match(s):
        return int(s)
    if _FLOAT.match(s) and any(c.isdigit() for c in s):
        return float(s)
    if s in (".inf", "+.inf"):
        return float("inf")
    if s == "-.inf":
        return float("-inf")
    if s[0] in "[{&*!|>%@`":
        raise ValueError(f"unsupported YAML value {s!r}")
    return s


def _split_flow(body: str) -> List[str]:
    items, cur, quote = [], [], None
    for ch in body:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
        elif ch in ("'", '"'):
            quote = ch
            cur.append(ch)
        elif ch == ",":
            items.append("".join(cur))
            cur = []
        elif ch in "[]{}":
            raise ValueError("nested flow collections are not supported")
        else:
            cur.append(ch)
    if "".join(cur).strip():
        items.append("".join(cur))
    return items


def _value(text: str) -> Any:
    s = text.strip()
    if s.startswith("["):
        if not s.endswith("]"):
            raise ValueError(f"unterminated flow list {s!r}")
        return [_scalar(t) for t in _split_flow(s[1:-1])]
    if s.startswith("{"):
        if s.replace(" ", "") != "{}":
            raise ValueError("only empty flow mappings are supported")
        return {}
    return _scalar(s)


def load_yaml(text: str) -> Dict[str, Any]:
    """Parse the YAML subset described in the module docstring."""
    lines: List[Tuple[int, str]] = []
    for raw in text.splitlines():
        if "\t" in raw[: len(raw) - len(raw.lstrip())]:
            raise ValueError("tab indentation is not supported")
        s = _strip_comment(raw)
        if not s.strip() or s.strip() == "---":
            continue
        if s.lstrip().startswith("- "):
            raise ValueError("block lists are not supported")
        lines.append((len(s) - len(s.lstrip()), s.strip()))
    root: Dict[str, Any] = {}
    stack: List[Tuple[int, Dict[str, Any]]] = [(0, root)]  # (indent of the keys, mapping)
    pending: Optional[Tuple[Dict[str, Any], Any, int]] = None  # key whose value may be a block
    for indent, s in lines:
        if pending is not None:
            pmap, pkey, pind = pending
            pending = None
            if indent > pind:
                child: Dict[str, Any] = {}
                pmap[pkey] = child
                stack.append((indent, child))
        while len(stack) > 1 and indent < stack[-1][0]:
            stack.pop()
        if indent != stack[-1][0]:
            raise ValueError(f"bad indentation at {s!r}")
        m = re.match(r"^([^:]+?):(\s+(.*)|)$", s)
        if not m:
            raise ValueError(f"cannot parse line {s!r}")
        key = _scalar(m.group(1))
        rest = (m.group(3) or "").strip()
        cur = stack[-1][1]
        if rest == "":
            cur[key] = None
            pending = (cur, key, indent)
        else:
            cur[key] = _value(rest)
    return root


def load_config(path: str) -> Dict[str, Any]:
    """A config file: YAML (PyYAML when installed, else ``load_yaml``) or JSON."""
    with open(path) as f:
        text = f.read()
    if path.endswith((".yaml", ".yml")):
        try:
            import yaml  # type: ignore
        except ImportError:
            return load_yaml(text)
        return yaml.safe_load(text) or {}
    return json.loads(text)
