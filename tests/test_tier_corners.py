"""Kernel corners the other parity tests do not reach, against the oracle:

* the Seq chain at k = 6, 7 on roots of out-degree above 256 (tier M's upper
  groups, where k >= 6 keeps 64-bit values per stream);
* tier L (out-degree 1025..2048, rows in a global slab) at k = 4 and 5.

Large out-degrees need a large degeneracy, which dense communities pay for
with enormous clique counts; a complete bipartite graph K_{a,a} has
degeneracy a and no triangle, so with sparse random edges added inside each
side its k-cliques are few (products of the small cliques of the two sides)
while its degeneracy DAG keeps out-degrees up to a.
"""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, O.max_threads()))


def bipartite_core(a: int, p_in: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    left, right = np.arange(a), np.arange(a, 2 * a)
    edges = [np.stack(np.meshgrid(left, right, indexing="ij"), -1).reshape(-1, 2)]
    for side in (left, right):
        iu = np.triu_indices(a, 1)
        keep = rng.random(len(iu[0])) < p_in
        edges.append(np.stack([side[iu[0][keep]], side[iu[1][keep]]], 1))
    e = np.sort(np.concatenate(edges).astype(np.int64), axis=1)
    return np.unique(e, axis=0).astype(np.uint32)


CASES = {
    "m_above_256": (bipartite_core(280, 0.05, seed=61), (6, 7), 256),
    "tier_l": (bipartite_core(1100, 0.002, seed=62), (4, 5), 1024),
}
PARAMS = [(name, k) for name, (_, ks, _) in CASES.items() for k in ks]


@pytest.mark.parametrize("name,k", PARAMS)
def test_seq_and_sim_on_large_roots(ctx, name, k):
    P, _, dmin = CASES[name]
    g = K.build_graph(ctx, K.EdgeList.from_pairs(P))
    assert g.core > dmin, g.core  # a root in the intended group
    og = O.Graph(P)
    tot, per = K.count_cliques(g, k)
    otot, oper = og.count_cliques(k)
    assert tot == otot and tot > 0 and np.array_equal(per, oper)
    rng = np.random.default_rng(k)
    for r0 in (np.zeros(g.n, np.uint64), rng.integers(0, 4, size=g.n, dtype=np.uint64) * np.uint64(3),
               np.where(rng.random(g.n) < 0.5, np.uint64(2**40), np.uint64(5)).astype(np.uint64)):
        r = K.seq_passes(g, k, 2, r0)
        ro = og.seq_pass(k, og.seq_pass(k, r0, O.SEQ_EDGE_STREAMS, THREADS), O.SEQ_EDGE_STREAMS, THREADS)
        assert np.array_equal(r, ro)
    rho = rng.integers(0, 3, size=g.n).astype(np.float64) * 0.5
    assert np.array_equal(K.sim_counts(g, k, rho), og.sim_counts(k, rho, THREADS))
    g.close()
