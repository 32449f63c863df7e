"""kclpp_certify_densest: the exact algorithm's certificate (kCDensestMem.c:
329-432, PAVA + stability + Goldberg-type test) restated with GPU passes.

A certified candidate must be a densest subgraph: its density m / n equals
the optimum found by trying every vertex subset (small graphs) and by the
library's max-flow (kclpp_densest_exact) on larger ones, exactly as
rationals.  A candidate that is not densest must never be certified: the
last test hands the certifier loads that rank a sparse part of the graph
first.
"""
import numpy as np
import pytest

import kclistpp_gb300 as K
from tests.test_certify import _cliques, _rho_star, _small_graphs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("i,k", [(i, k) for i in range(len(_small_graphs())) for k in (3, 4)])
def test_certificate_on_exhaustive_optimum(ctx, i, k):
    n, pairs = _small_graphs()[i]
    masks = _cliques(n, pairs, k)
    if len(masks) == 0:
        pytest.skip("no k-clique")
    num, den = _rho_star(n, masks)
    g = K.build_graph(ctx, K.EdgeList.from_pairs(pairs))
    _, r = K.seq_main(g, k, 64)
    info, mem = K.certify_densest(g, k, r, 1 << 14)
    assert info.certified and info.inside_method == 1, info.as_dict()  # the loads alone decide
    assert info.cliques * den == num * info.n  # exactly the optimum
    g.close()


def graphs():
    return {
        "config1": K.chung_lu(10000, 20.0, 2.5, seed=1),
        "planted": K.planted(6000, 8.0, 2.2, 3, 60, 140, 0.6, seed=41),
        "rmat_planted": K.rmat_planted(12, 12, 3, 40, 90, 0.5, seed=42),
    }


GRAPHS = graphs()


@pytest.mark.parametrize("name,k", [(n, k) for n in GRAPHS for k in (3, 4)])
def test_certificate_matches_max_flow(ctx, name, k):
    el = GRAPHS[name]
    ex, _ = K.densest_exact(el, k)
    g = K.build_graph(ctx, el)
    _, r = K.seq_main(g, k, 64, K.SEQ_SHARED)
    info, mem = K.certify_densest(g, k, r, 256)
    assert info.certified, info.as_dict()
    assert info.cliques * ex.den == ex.num * info.n
    g.close()


def test_a_sparse_candidate_is_not_certified(ctx):
    """Loads that put a sparse path first make the first PAVA block a set that
    is not densest; the certificate must refuse it."""
    pairs = [(u, v) for u in range(8) for v in range(u + 1, 8)]  # K_8: 56 triangles, density 7
    pairs += [(7 + i, 8 + i) for i in range(40)]                  # a path hanging on it (8..47)
    pairs += [(20, 48), (21, 48)]                                  # a triangle on the path
    el = K.EdgeList.from_pairs(np.array(pairs, dtype=np.uint32))
    g = K.build_graph(ctx, el)
    rank = K.core_order(el)  # the DAG's vertex ids are the core ranks
    assert g.n == el.n  # no isolated vertex
    r = np.zeros(g.n, np.uint64)
    for v in range(8, g.n):
        r[rank[v]] = 1000 + v
    info, _ = K.certify_densest(g, 3, r, 64)
    assert info.cliques * 8 < 56 * info.n  # a worse candidate than K_8
    assert not info.certified
    g.close()
