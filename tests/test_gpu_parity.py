"""GPU path against the oracle and the reference's golden vectors.

Integer results (clique counts, k-clique degrees, Seq-kClist++ r, PAVA
counts, densest-prefix n/m/cliques, trim outputs) must be bit-exact; FP64
results (Sim-kClist++ rho, density, upper bound) are compared bit for bit as
well, which is stricter than the 1e-9 relative tolerance the path allows.
"""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O
from tests import golden_util as G

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, O.max_threads()))


def bits(x):
    return np.ascontiguousarray(x, dtype=np.float64).view(np.uint64)


def dev_graph(ctx, pairs):
    return K.build_graph(ctx, K.EdgeList.from_pairs(pairs))


@pytest.mark.parametrize("name", sorted(G.index()))
def test_dag_matches_oracle(ctx, name):
    P = G.pairs(name)
    g = dev_graph(ctx, P)
    og = O.Graph(P)
    assert (g.n, g.m, g.core) == (og.n, og.m, og.core)
    off, cols = g.csr()
    ooff, ocols = og.csr()
    assert np.array_equal(off, ooff) and np.array_equal(cols, ocols)


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_count_cliques(ctx, name, k, T):
    P = G.pairs(name)
    g = dev_graph(ctx, P)
    tot, per = K.count_cliques(g, k)
    otot, oper = O.Graph(P).count_cliques(k)
    assert tot == otot
    assert np.array_equal(per, oper)
    tr = G.index()[name]["runs"][str(k)].get("trim")
    if tr:
        assert tot == tr["total"]


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_seq_main_matches_reference(ctx, name, k, T):
    """CDF_Main of kCDensestNoAtom with per-root-edge streams: every power-of-two
    report and the final r equal the reference's own functions' output."""
    g = dev_graph(ctx, G.pairs(name))
    infos, r = K.seq_main(g, k, T)
    assert G.infos_equal(G.index()[name]["runs"][str(k)]["seq_edge"], infos)
    assert np.array_equal(r, G.arrays(name)[f"k{k}_seq_edge_rho"])


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_sim_main_matches_reference(ctx, name, k, T):
    g = dev_graph(ctx, G.pairs(name))
    infos, rho = K.sim_main(g, k, T)
    assert G.infos_equal(G.index()[name]["runs"][str(k)]["sim"], infos)
    assert np.array_equal(bits(rho), G.arrays(name)[f"k{k}_sim_rho_bits"])


TRIM_RUNS = [(n, k, T) for (n, k, T) in G.case_ks() if "trim" in G.index()[n]["runs"][str(k)]]


@pytest.mark.parametrize("name,k,T", TRIM_RUNS)
def test_trim_exact_matches_reference(ctx, name, k, T):
    ref = G.index()[name]["runs"][str(k)]["trim"]
    arr = G.arrays(name)
    t = K.trim(ctx, K.EdgeList.from_pairs(G.pairs(name)), k, K.TRIM_EXACT)
    deg = arr[f"k{k}_trim_ckdeg"]
    assert np.array_equal(deg[:, 0], t.map) and np.array_equal(deg[:, 1], t.nck)
    core = arr[f"k{k}_trim_ckcore"]
    assert np.array_equal(core[:, 0], t.map[t.order]) and np.array_equal(core[:, 1], t.core_num)
    ck = ref["ckdens"]
    assert ("%f" % t.info.ckrho, "%f" % t.info.rho, int(ck[2])) == (ck[0], ck[1], t.info.size)
    assert (t.info.ntrim, t.info.mtrim, t.info.ncktrim, t.info.total) == (
        ref["ntrim"], ref["mtrim"], ref["ncktrim"], ref["total"])
    assert np.array_equal(t.edges.pairs(), arr[f"k{k}_trim_trimmed"].reshape(-1, 2))


@pytest.mark.parametrize("name,k,T", TRIM_RUNS)
def test_trim_fast_is_a_valid_core(ctx, name, k, T):
    """FAST ends on a rho-core for its own best density (a valid lower bound):
    recounting the kept graph, every kept vertex has k-clique degree >= ckrho
    and the kept clique count is the one reported."""
    el = K.EdgeList.from_pairs(G.pairs(name))
    f = K.trim(ctx, el, k, K.TRIM_FAST)
    x = K.trim(ctx, el, k, K.TRIM_EXACT)
    assert f.info.total == x.info.total and f.info.n2 == x.info.n2
    assert f.info.ckrho >= f.info.total / f.info.n2
    kept = f.edges.pairs()
    if len(kept):
        og = O.Graph(kept)
        tot, per = og.count_cliques(k)
        assert tot == f.info.ncktrim
        rank = O.sort_by_core(kept)
        ids = np.unique(kept)
        assert np.all(per[rank[ids]].astype(np.float64) >= f.info.ckrho)


# ---- live comparisons on graphs that exercise every tier ---------------------------

def _tier_graphs():
    return {
        # tier S only
        "cl_5000": K.chung_lu(5000, 14.0, 2.3, seed=11).pairs(),
        # tier M (out-degrees 64..512)
        "planted_m": K.planted(4000, 6.0, 2.2, 2, 300, 400, 0.5, seed=12).pairs(),
        # tier M, largest shared-memory bucket (512..1024)
        "planted_m3": K.planted(3000, 4.0, 2.2, 1, 1400, 1400, 0.4, seed=13).pairs(),
        # tier L (1024..2048, rows in a global slab)
        "planted_l": K.planted(3000, 4.0, 2.2, 1, 2000, 2000, 0.6, seed=14).pairs(),
    }


TIERS = _tier_graphs()
TIER_KS = {"cl_5000": [3, 4, 5, 6], "planted_m": [3, 4, 5], "planted_m3": [3, 4], "planted_l": [3]}
TIER_CASES = [(n, k) for n in TIERS for k in TIER_KS[n]]


@pytest.mark.parametrize("name,k", TIER_CASES)
def test_tiers_count(ctx, name, k):
    P = TIERS[name]
    g = dev_graph(ctx, P)
    tot, per = K.count_cliques(g, k)
    otot, oper = O.Graph(P).count_cliques(k)
    assert tot == otot and np.array_equal(per, oper)


@pytest.mark.parametrize("name,k", TIER_CASES)
def test_tiers_seq_pass_from_nonzero_r(ctx, name, k):
    """One pass from a random r with many ties: the in-place chain's tie rules
    (strict <, cached argmin) matter most here."""
    P = TIERS[name]
    g = dev_graph(ctx, P)
    og = O.Graph(P)
    rng = np.random.default_rng(k)
    r0 = rng.integers(0, 4, size=g.n, dtype=np.uint64) * np.uint64(1000)
    r = K.seq_passes(g, k, 1, r0)
    ro = og.seq_pass(k, r0, mode=O.SEQ_EDGE_STREAMS, threads=THREADS)
    assert np.array_equal(r, ro)
    r2 = K.seq_passes(g, k, 1, r)
    assert np.array_equal(r2, og.seq_pass(k, ro, mode=O.SEQ_EDGE_STREAMS, threads=THREADS))


@pytest.mark.parametrize("name,k", TIER_CASES)
def test_tiers_seq_pass_wide_values(ctx, name, k):
    """Values whose spread inside a root exceeds 2^31 (the kernel then keeps
    64-bit values; otherwise it works on 32-bit values relative to the root's
    minimum) and values near the top of the u64 range."""
    P = TIERS[name]
    g = dev_graph(ctx, P)
    og = O.Graph(P)
    rng = np.random.default_rng(300 + k)
    choices = np.array([0, 1, 2, 7, 2**31 - 5, 2**31 + 3, 2**40, 2**62], dtype=np.uint64)
    r0 = choices[rng.integers(0, len(choices), size=g.n)] + rng.integers(0, 3, size=g.n, dtype=np.uint64)
    r = K.seq_passes(g, k, 1, r0)
    assert np.array_equal(r, og.seq_pass(k, r0, mode=O.SEQ_EDGE_STREAMS, threads=THREADS))
    # near the 32-bit boundary for every root: a spread just under and just over
    r1 = (np.uint64(2**31 - 2**22) * (np.arange(g.n, dtype=np.uint64) % np.uint64(2))).astype(np.uint64)
    assert np.array_equal(K.seq_passes(g, k, 1, r1), og.seq_pass(k, r1, mode=O.SEQ_EDGE_STREAMS, threads=THREADS))


@pytest.mark.parametrize("name,k", TIER_CASES)
@pytest.mark.parametrize("waves", [16, 5])
def test_tiers_seq_waves(ctx, name, k, waves):
    """Wave-ordered passes: each wave's chains start from r as the earlier
    waves left it, so the result depends on the wave hash and the ordering of
    waves -- both must match the oracle's restatement bit for bit."""
    P = TIERS[name]
    g = dev_graph(ctx, P)
    sp = K.get_schedule(g)
    sp.seq_waves = waves
    K.set_schedule(g, sp)
    og = O.Graph(P)
    r0 = np.random.default_rng(200 + k).integers(0, 4, size=g.n, dtype=np.uint64) * np.uint64(1000)
    r = K.seq_passes(g, k, 2, r0, det_mode=K.SEQ_WAVES)
    ro = og.seq_pass_waves(k, og.seq_pass_waves(k, r0, waves, THREADS), waves, THREADS)
    assert np.array_equal(r, ro)
    # a pass adds exactly one unit per k-clique
    tot, _ = og.count_cliques(k)
    assert int((r - r0).sum()) == 2 * tot


@pytest.mark.parametrize("name,k", TIER_CASES)
def test_tiers_sim_counts_with_ties(ctx, name, k):
    P = TIERS[name]
    g = dev_graph(ctx, P)
    og = O.Graph(P)
    rng = np.random.default_rng(100 + k)
    rho = rng.integers(0, 3, size=g.n).astype(np.float64) * 0.5
    assert np.array_equal(K.sim_counts(g, k, rho), og.sim_counts(k, rho, threads=THREADS))
    rho2 = K.sim_passes(g, k, 2, rho, t_first=3)
    orho = og.sim_pass(k, 4, og.sim_pass(k, 3, rho, THREADS), THREADS)
    assert np.array_equal(bits(rho2), bits(orho))


@pytest.mark.parametrize("name,k", TIER_CASES)
def test_tiers_pava(ctx, name, k):
    P = TIERS[name]
    g = dev_graph(ctx, P)
    level = np.random.default_rng(7).permutation(g.n).astype(np.uint32)
    assert np.array_equal(K.pava(g, k, level), O.Graph(P).pava(k, level, THREADS))


def test_extract_matches_oracle(ctx):
    P = TIERS["planted_m"]
    g = dev_graph(ctx, P)
    og = O.Graph(P)
    r = K.seq_passes(g, 4, 3)
    info, re = K.extract_densest_seq(g, 4, 3, r)
    oinfo, ore = og.seq_find_densest(4, 3, r, THREADS)
    assert info.as_tuple() == oinfo.as_tuple() and np.array_equal(re, ore)
    rho = K.sim_passes(g, 4, 3)
    info, re = K.extract_densest_sim(g, 4, rho)
    oinfo, ore = og.sim_find_densest(4, rho, THREADS)
    assert info.as_tuple() == oinfo.as_tuple() and np.array_equal(re, ore)


def test_sort_and_count_edges(ctx):
    P = TIERS["cl_5000"]
    g = dev_graph(ctx, P)
    og = O.Graph(P)
    rng = np.random.default_rng(3)
    r = rng.integers(0, 50, size=g.n, dtype=np.uint64)
    re, lv = K.sort_by_r_u64(r)
    assert np.array_equal(re, O.sort_by_r_u64(r)) and np.array_equal(lv[re], np.arange(g.n))
    rho = rng.random(g.n) * 30
    re, _ = K.sort_by_r_f64(rho)
    assert np.array_equal(re, O.sort_by_r_f64(rho))
    nodes = re[:700]
    assert K.count_edges(g, nodes) == og.count_edges(nodes)


def test_one_shot_csr_calls(ctx):
    P = TIERS["planted_m"]
    g = dev_graph(ctx, P)
    off, cols = g.csr()
    r = np.zeros(g.n, dtype=np.uint64)
    K.seq_passes_csr(ctx, off, cols, 4, 2, r)
    assert np.array_equal(r, K.seq_passes(g, 4, 2))
    rho = np.zeros(g.n)
    K.sim_passes_csr(ctx, off, cols, 4, 2, rho)
    assert np.array_equal(bits(rho), bits(K.sim_passes(g, 4, 2)))


def test_edge_cases(ctx):
    # no edges at all
    el = K.EdgeList.from_pairs(np.zeros((0, 2), np.uint32))
    g = K.build_graph(ctx, el)
    assert g.n == 0 and K.count_cliques(g, 3)[0] == 0
    infos, r = K.seq_main(g, 4, 8)
    assert len(infos) == 4 and all(i.n == 0 for i in infos)
    # n < k and triangle-free graphs: no clique, r stays 0
    for name, k in (("kat_triangle_k4", 4), ("kat_star", 3)):
        g = dev_graph(ctx, G.pairs(name))
        assert K.count_cliques(g, k)[0] == 0
        assert not K.seq_passes(g, k, 3).any()
    # non-simple input is rejected, not miscounted
    with pytest.raises(K.KclppError) as ei:
        K.build_graph(ctx, K.EdgeList.from_pairs([[0, 1], [1, 0], [1, 2]]))
    assert ei.value.status == K.ERR_INVALID
    with pytest.raises(K.KclppError) as ei:
        K.build_graph(ctx, K.EdgeList.from_pairs([[0, 0], [1, 2]]))
    assert ei.value.status == K.ERR_INVALID
    # k outside the compiled range
    g = dev_graph(ctx, G.pairs("kat_complete10"))
    for bad in (2, K.MAX_K + 1):
        with pytest.raises(K.KclppError) as ei:
            K.seq_passes(g, bad, 1)
        assert ei.value.status == K.ERR_UNSUPPORTED
    # Sim accepts k = 2: every root edge is a clique (kCDensestCmpSync.c:189-192)
    cnt = K.sim_counts(g, 2, np.zeros(g.n))
    assert cnt.sum() == g.m


def test_complete_graph_known_answers(ctx):
    from math import comb

    g = dev_graph(ctx, G.pairs("kat_complete10"))
    for k in range(3, 9):
        tot, per = K.count_cliques(g, k)
        assert tot == comb(10, k) and np.all(per == comb(9, k - 1))
        r = K.seq_passes(g, k, 1)
        assert int(r.sum()) == comb(10, k)
        infos, _ = K.sim_main(g, k, 4)
        assert infos[-1].n == 10 and infos[-1].cliques == comb(10, k)


def test_sim_k2_matches_reference(ctx):
    """Sim-kClist++ at k = 2 (kCDensestCmpSync.c:189-192): reports and FP64 rho
    bit-identical to the reference's on every golden graph."""
    import json
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    index = json.load(open(os.path.join(here, "sim2.json")))
    arrays = np.load(os.path.join(here, "sim2.npz"))
    for name, meta in index.items():
        g = dev_graph(ctx, G.pairs(name))
        infos, rho = K.sim_main(g, 2, meta["T"])
        want = [[i[0], i[1], i[2], float.fromhex(i[3]), float.fromhex(i[4])] for i in meta["infos"]]
        assert G.infos_equal(want, infos), name
        assert np.array_equal(bits(rho), arrays[f"{name}_rho_bits"]), name
