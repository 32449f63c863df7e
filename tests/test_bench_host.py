"""Host-side pieces of bench.py, on the CPU.

* The reference arm's input: the oracle's restatement of the RMAT generator
  plus the kept set recorded from the reference program's own trim must give
  exactly the reference's trimmed edge list (tests/golden/rmat20_trim.json
  holds its SHA-256), at k = 4 and k = 5 -- the arm never loads the library.
* The reference-equivalent bytes of a pass (the per-root-edge gathers of the
  reference's MakeSubgraph, kCDensestNoAtom.c:86-113) against a direct count.
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


def test_reference_equivalent_bytes_match_a_direct_count():
    rng = np.random.default_rng(5)
    n = 300
    pairs = set()
    while len(pairs) < 3000:
        a, b = rng.integers(0, n, 2)
        if a != b:
            pairs.add((int(min(a, b)), int(max(a, b))))
    og = O.Graph(np.array(sorted(pairs), dtype=np.uint32))
    off, cols = og.csr()
    off = off.astype(np.int64)
    nv = len(off) - 1
    out = [set(cols[off[v]:off[v + 1]].tolist()) for v in range(nv)]
    deg = [len(o) for o in out]
    want = 8 * (nv + 1) + 16 * nv
    for s in range(nv):
        for t in out[s]:
            C = out[s] & out[t]
            want += 8 + 4 * (deg[s] + deg[t]) + 4 * sum(deg[x] for x in C) + 8 * (len(C) + 2)
    got = bench.dag_stats(off, cols, 4)["ref_equiv_bytes_per_pass"]
    assert got == want
