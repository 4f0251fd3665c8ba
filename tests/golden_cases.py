"""Loader for the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("ref_dambreak", "ref_hydrostatic_original", "ref_dambreak_fine", "dambreak_l0_01",
         "jitter_collide", "jitter_higher_order", "box3d")
STATE_KEYS = ("pos", "vel", "pressure", "min_pressure", "ndr", "type", "bc", "dirichlet")
NB_KEYS = ("nb_off", "nb_id", "nb_dist")
SYS_KEYS = ("source", "row_ptr", "col", "val")


def digest(arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def load(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d.pop("params_json")))
    d["meta"] = json.loads(str(d.pop("meta")))
    return d
