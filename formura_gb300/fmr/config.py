"""Numerical config files (``<program>.yaml``, src/Formura/NumericalConfig.hs:17-34).

The files use a small YAML subset: ``key: value`` lines, flow lists
``[1, 2, 3]`` (numbers or quoted strings), and one level of nested maps
(``initial_walls:`` followed by indented ``x: [136]`` lines).  This reader
covers that subset without a YAML library.
"""
from __future__ import annotations

import ast
from pathlib import Path
from typing import Dict


def _value(text: str):
    t = text.strip()
    if not t:
        return None
    if t.startswith("[") or t[0].isdigit() or t[0] in "-+'\"":
        try:
            return ast.literal_eval(t)
        except (ValueError, SyntaxError):
            pass
    if t in ("true", "True"):
        return True
    if t in ("false", "False"):
        return False
    return t


def loads(text: str) -> Dict:
    out: Dict = {}
    current = None
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip()
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip())
        key, _, val = line.strip().partition(":")
        key = key.strip()
        if indent == 0:
            v = _value(val)
            if v is None:
                out[key] = {}
                current = out[key]
            else:
                out[key] = v
                current = None
        elif current is not None:
            current[key] = _value(val)
        else:
            raise ValueError("unexpected indentation: %r" % raw)
    return out


def load(path) -> Dict:
    return loads(Path(path).read_text(encoding="utf-8"))
