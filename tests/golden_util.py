"""Loads the golden vectors written by tests/golden/make_golden.py."""
import functools
import hashlib
import json
import os

import numpy as np

from tests.golden.cases import CASES, make_pairs

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@functools.lru_cache(maxsize=None)
def index() -> dict:
    with open(os.path.join(HERE, "golden.json")) as f:
        return json.load(f)


@functools.lru_cache(maxsize=None)
def arrays(name: str) -> dict:
    with np.load(os.path.join(HERE, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


@functools.lru_cache(maxsize=None)
def pairs(name: str) -> np.ndarray:
    a = arrays(name)
    if "pairs" in a:
        p = a["pairs"]
    else:
        case = next(c for c in CASES if c["name"] == name)
        p = make_pairs(case)
    p = np.ascontiguousarray(p, dtype=np.uint32).reshape(-1, 2)
    assert hashlib.sha256(p.tobytes()).hexdigest() == index()[name]["sha256"], f"{name}: edge list drifted"
    return p


def case_ks():
    """(case name, k, T) for every golden run."""
    out = []
    for c in CASES:
        for k in c["ks"]:
            out.append((c["name"], k, c["T"]))
    return out


def infos_equal(a, b) -> bool:
    """info records [T, n, m, density, ub] vs objects with n, m, density, ub (bit-exact)."""
    if len(a) != len(b):
        return False
    for x, y in zip(a, b):
        if (x[1], x[2]) != (y.n, y.m):
            return False
        if np.float64(x[3]).tobytes() != np.float64(y.density).tobytes():
            return False
        if np.float64(x[4]).tobytes() != np.float64(y.ub).tobytes():
            return False
    return True
