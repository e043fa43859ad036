import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_npz(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def boundary_layer(brain):
    """Tissue cells with at least one non-tissue face neighbour (periodic)."""
    nb = np.zeros_like(brain)
    for ax in range(3):
        for s in (1, -1):
            nb |= ~np.roll(brain, s, axis=ax)
    return brain & nb


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
