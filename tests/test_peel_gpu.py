"""The k-clique core peel (kcliquecore / oneshortpass, kClistCoreTrim.c:577-666)
with its recounts on the GPU in speculative batches, against the oracle's
restatement of the reference's sequential loop and the library's own host
loop (TRIM_EXACT_HOST): core numbers, the peel order (the ckcore file's line
order), ckrho / rho / size, the trimmed set and its counts must all be equal.

The graphs make the popped vertices' live-neighbour lists fall in every GPU
group (up to 64, 65..1024, 1025..2048 members) and beyond 2048 (the host
recursion), and make the heap's ties matter (many equal k-clique degrees).
"""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def hub_graph(fan: int, extra: int, seed: int) -> np.ndarray:
    """A hub adjacent to `fan` vertices, each of which sits in its own K6 with
    five further vertices (so it keeps a high k-clique degree), plus `extra`
    random edges and triangles among the hub's neighbours: the hub has few
    k-cliques, is popped early with all `fan` neighbours live, and its recount
    is not empty."""
    rng = np.random.default_rng(seed)
    edges = []
    hub = 0
    nxt = 1
    nbrs = []
    for _ in range(fan):
        grp = list(range(nxt, nxt + 6))
        nxt += 6
        nbrs.append(grp[0])
        edges += [(a, b) for i, a in enumerate(grp) for b in grp[i + 1:]]
        edges.append((hub, grp[0]))
    nb = np.array(nbrs)
    for _ in range(extra):
        a, b, c = rng.choice(nb, size=3, replace=False)
        edges += [(a, b), (b, c), (a, c)]
    e = np.array(edges, dtype=np.int64)
    e = np.sort(e, axis=1)
    e = np.unique(e, axis=0)
    return e.astype(np.uint32)


def graphs():
    return {
        "cl_ties": K.chung_lu(3000, 12.0, 2.4, seed=31).pairs(),
        "planted_m": K.planted(4000, 6.0, 2.2, 2, 250, 500, 0.35, seed=32).pairs(),
        "rmat_planted": K.rmat_planted(12, 12, 3, 40, 120, 0.5, seed=33).pairs(),
        "hub_l": hub_graph(1500, 2, seed=34),   # a 1500-member recount (1025..2048)
        "hub_host": hub_graph(2600, 2, seed=35),  # a 2600-member recount (host)
    }


GRAPHS = graphs()
CASES = [(n, k) for n in GRAPHS for k in (3, 4, 5)] + [("planted_m", 6), ("rmat_planted", 6)]


def same_trim(t, o):
    assert t.info.n2 == o["n2"] and t.info.e2 == o["e2"] and t.info.total == o["total"]
    assert np.array_equal(t.map, o["map"]) and np.array_equal(t.nck, o["nck"])
    assert np.array_equal(t.order, o["order"]), "peel order differs"
    assert np.array_equal(t.core_num, o["core_num"]), "core numbers differ"
    assert t.info.ckcore == o["ckcore"]
    assert np.float64(t.info.ckrho).view(np.uint64) == np.float64(o["ckrho"]).view(np.uint64)
    assert np.float64(t.info.rho).view(np.uint64) == np.float64(o["rho"]).view(np.uint64)
    assert (t.info.size, t.info.ntrim, t.info.ncktrim, t.info.mtrim) == (o["size"], o["ntrim"], o["ncktrim"],
                                                                        o["mtrim"])
    assert np.array_equal(t.edges.pairs(), o["trimmed"])


@pytest.mark.parametrize("name,k", CASES)
def test_gpu_peel_matches_oracle(ctx, name, k):
    P = GRAPHS[name]
    el = K.EdgeList.from_pairs(P)
    t = K.trim(ctx, el, k, K.TRIM_EXACT)
    same_trim(t, O.trim(P, k))
    st = t.peel
    assert st.committed == max(t.info.n2 - 1, 0)
    assert st.predicted >= st.committed and st.batches >= 1
    if name == "hub_host":
        assert st.host_roots >= 1  # the hub's 2600 live neighbours
    if name == "hub_l":
        assert st.gpu_roots >= 1


@pytest.mark.parametrize("name,k", [("planted_m", 4), ("hub_host", 3), ("rmat_planted", 5)])
def test_gpu_peel_matches_host_loop(ctx, name, k):
    el = K.EdgeList.from_pairs(GRAPHS[name])
    a = K.trim(ctx, el, k, K.TRIM_EXACT)
    b = K.trim(ctx, el, k, K.TRIM_EXACT_HOST)
    assert np.array_equal(a.order, b.order) and np.array_equal(a.core_num, b.core_num)
    assert (a.info.ckrho, a.info.rho, a.info.size, a.info.ntrim, a.info.ncktrim, a.info.mtrim) == (
        b.info.ckrho, b.info.rho, b.info.size, b.info.ntrim, b.info.ncktrim, b.info.mtrim)
    assert np.array_equal(a.edges.pairs(), b.edges.pairs())
    assert b.peel.gpu_roots == 0 and b.peel.committed == a.peel.committed


def test_core_numbers_are_order_free(ctx):
    """The core number of a vertex is the largest c such that it lies in a
    subgraph whose every vertex is in at least c k-cliques of it: check the
    peel's numbers against that definition by recounting each c-core."""
    P = GRAPHS["planted_m"]
    k = 4
    t = K.trim(ctx, K.EdgeList.from_pairs(P), k, K.TRIM_EXACT)
    core = np.empty(t.info.n2, np.uint64)
    core[t.order] = t.core_num
    orig = t.map
    for c in np.unique(core)[-3:]:
        keep = set(orig[core >= c].tolist())
        sub = np.array([e for e in P.tolist() if e[0] in keep and e[1] in keep], dtype=np.uint32)
        og = O.Graph(sub)
        _, per = og.count_cliques(k)
        rank = O.sort_by_core(sub)
        ids = np.unique(sub)
        assert per[rank[ids]].min() >= c
