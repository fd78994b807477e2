"""Load the golden fixtures written by ``tests/golden/make_golden.py``."""

from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def _insert(tree, parts, value):
    head = parts[0]
    if len(parts) == 1:
        tree[head] = value
        return
    _insert(tree.setdefault(head, {}), parts[1:], value)


def _finish(node):
    if not isinstance(node, dict):
        return node
    if "__none__" in node:
        return None
    if "__len__" in node:
        return [_finish(node[str(i)]) for i in range(int(node["__len__"]))]
    return {key: _finish(value) for key, value in node.items()}


def load(name):
    """Return ``(inputs, outputs)`` nested as they were saved."""
    with np.load(GOLDEN / f"{name}.npz") as data:
        tree = {}
        for key in data.files:
            _insert(tree, key.split("/"), data[key])
    tree = _finish(tree)
    return tree["in"], tree["out"]


def scalar(value):
    return value.item() if isinstance(value, np.ndarray) else value
