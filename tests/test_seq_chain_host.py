"""The Seq kernel's chain algorithm, restated lane by lane on the host
(tests/seq_chain_emul.c), against the oracle's per-root-edge pass bit for
bit: the word skip (every word whose least starting value is at least
c + |V| - 1 falls whole) and the per-word fixed point from the exact prefix
value are exact, at k = 3..5, from zero (ties everywhere), after a few
passes, from spread loads and from loads beyond the 32-bit form (the 64-bit
path).  The kernel itself is compared with the oracle on the GPU
(tests/test_gpu_parity.py, tests/test_headline_parity.py); this checks the
algorithm it implements on any machine."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_util as G

HERE = os.path.dirname(os.path.abspath(__file__))
GRAPHS = ["kat_complete10", "kat_clique_tree", "kat_disjoint_cliques", "er_1500", "cl_2000", "planted_3000",
          "rmat12", "config1_chung_lu_1e4"]


@pytest.fixture(scope="module")
def emul(tmp_path_factory):
    d = tmp_path_factory.mktemp("seq_chain")
    exe = str(d / "seq_chain_emul")
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-o", exe, os.path.join(HERE, "seq_chain_emul.c")])
    return exe, d


def run(emul, og, r, k):
    exe, d = emul
    off, cols = og.csr()
    np.ascontiguousarray(off, dtype="<u8").tofile(d / "off.bin")
    np.ascontiguousarray(cols, dtype="<u4").tofile(d / "cols.bin")
    np.ascontiguousarray(r, dtype="<u8").tofile(d / "r.bin")
    out = subprocess.run([exe, str(d / "off.bin"), str(d / "cols.bin"), str(d / "r.bin"), str(k), str(d / "out.bin")],
                         check=True, capture_output=True, text=True).stdout.split()
    stats = {out[i]: int(out[i + 1]) for i in range(0, len(out), 2)}
    return np.fromfile(d / "out.bin", dtype="<u8"), stats


@pytest.mark.parametrize("name", GRAPHS)
@pytest.mark.parametrize("k", [3, 4, 5])
def test_chain_restatement_matches_the_oracle(emul, name, k):
    og = O.Graph(G.pairs(name))
    n = og.n
    threads = max(1, min(8, O.max_threads()))
    rng = np.random.default_rng(k * 101 + len(name))
    r2 = og.seq_pass(k, og.seq_pass(k, np.zeros(n, np.uint64), O.SEQ_EDGE_STREAMS, threads), O.SEQ_EDGE_STREAMS,
                     threads)
    states = {
        "zero": np.zeros(n, np.uint64),
        "after two passes": r2,
        "spread": rng.integers(0, 40 * 10 ** (k - 1), size=n, dtype=np.uint64),
        "beyond 32 bits": rng.integers(0, 1 << 40, size=n, dtype=np.uint64),
    }
    for label, r0 in states.items():
        got, stats = run(emul, og, r0, k)
        want = og.seq_pass(k, r0.copy(), O.SEQ_EDGE_STREAMS, threads)
        assert np.array_equal(got, want), f"{name} k={k} {label}"
    # the skip decided whole chains in the runs above, and words went through
    # the fixed point: both parts of the algorithm were exercised
    assert stats["streams"] > 0
