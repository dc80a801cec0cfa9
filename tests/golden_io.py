"""Loading helpers for the golden vectors in tests/golden/*.npz."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["tgv16_lattice", "tgv24_jitter_wrap", "fourier20", "dambreak16"]


def load_case(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    cfg = json.loads(bytes(z["config_json"]).decode())
    state = {}
    for k in z.files:
        if k.startswith("in/"):
            _, part, key = k.split("/", 2)
            state.setdefault(part, {})[key] = z[k].copy()
    return z, cfg, state


def rel_max(a, b):
    """max |a - b| / max |b|: error relative to the field's magnitude."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-30))
