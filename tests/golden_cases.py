"""Loader of the golden fixtures (tests/golden/*.npz, made by make_golden.py)."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load(name):
    z = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    d = {k: z[k] for k in z.files if k != "meta"}
    d["meta"] = json.loads(str(z["meta"]))
    d["dt"] = float(d["dt"])
    d["SI"] = float(d["SI"])
    return d


def spacing(d):
    return {k: d[k] for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def modes(d):
    m = d["meta"]
    return dict(surface_mode=m["surface_mode"], bc=m["bc"], source_mode=m["source_mode"])


def matches(d, key, arr):
    """Bit-exact agreement with the reference output ``key``."""
    if key in d:
        return np.array_equal(np.asarray(arr, np.float64), d[key]) and digest(arr) == d["meta"][f"sha256_{key}"]
    return digest(arr) == d["meta"][f"sha256_{key}"]
