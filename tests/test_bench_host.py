"""Host-side pieces of bench.py, on the CPU.

* The reference arm's input: the oracle's restatement of the RMAT generator
  plus the kept set recorded from the reference program's own trim must give
  exactly the reference's trimmed edge list (tests/golden/rmat20_trim.json
  holds its SHA-256), at k = 4 and k = 5 -- the arm never loads the library.
  (The byte model of the roofline is checked in tests/test_host.py.)
* The committed ncu counters feed the roofline only on the workload they
  were measured on.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import bench
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "rmat20_trim.json")))


@pytest.fixture(scope="module")
def rmat20_pairs():
    P = O.rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    assert hashlib.sha256(np.ascontiguousarray(P, dtype="<u4").tobytes()).hexdigest() == GOLD["graph"]["sha256"]
    return P


@pytest.mark.parametrize("k", [k for k in (4, 5) if str(k) in GOLD])
def test_reference_arm_input_is_the_reference_trim(rmat20_pairs, k):
    g = GOLD[str(k)]
    pairs = bench.induce_kept(rmat20_pairs, g["kept_in_label_order"])
    assert len(pairs) == g["mtrim"]
    assert int(np.unique(pairs).size) == g["ntrim"]
    h = hashlib.sha256()
    h.update("".join(f"{u} {v}\n" for u, v in pairs.tolist()).encode())
    assert h.hexdigest() == g["trimmed_sha256"]
    assert bench.golden_trim(20, k, 1) == g
    assert bench.golden_trim(19, k, 1) is None


def test_committed_counters_apply_to_their_workload_only():
    import types

    a = types.SimpleNamespace(scale=20, seed=1, k=4)
    assert bench.profiled("warp_inst_per_pass", "seq", a) > 0
    for other in ({"k": 5}, {"scale": 18}, {"seed": 2}):
        b = types.SimpleNamespace(**{**vars(a), **other})
        assert bench.profiled("warp_inst_per_pass", "seq", b) is None
