"""The CPU oracle against the golden vectors produced by the reference itself.

This pins the oracle: every number below was printed by the reference's own
functions (kCDensestNoAtom.c, kCDensestCmpSync.c, kClistCoreTrim.c,
kCDensestSamplingKclistpp.c compiled from source), and the oracle must
reproduce it bit for bit.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_util as G


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_seq_sequential_matches_reference(name, k, T):
    """The reference at p = 1 (one in-place chain over all root edges)."""
    meta = G.index()[name]
    g = O.Graph(G.pairs(name))
    assert [g.n, g.m, g.core] == meta["graph"]
    infos, r = g.seq_main(k, T, mode=O.SEQ_SEQUENTIAL)
    assert G.infos_equal(meta["runs"][str(k)]["seq_p1"], infos)
    assert np.array_equal(r, G.arrays(name)[f"k{k}_seq_p1_rho"])


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_seq_edge_streams_matches_reference(name, k, T):
    """Per-root-edge streams, run through the reference's own MakeSubgraph and
    CDF_CliqueEnumThread by the harness."""
    meta = G.index()[name]
    g = O.Graph(G.pairs(name))
    infos, r = g.seq_main(k, T, mode=O.SEQ_EDGE_STREAMS, threads=2)
    assert G.infos_equal(meta["runs"][str(k)]["seq_edge"], infos)
    assert np.array_equal(r, G.arrays(name)[f"k{k}_seq_edge_rho"])


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_sim_matches_reference(name, k, T):
    """Sim-kClist++: FP64 rho bit-exact, infos bit-exact."""
    meta = G.index()[name]
    g = O.Graph(G.pairs(name))
    infos, rho = g.sim_main(k, T, threads=2)
    assert G.infos_equal(meta["runs"][str(k)]["sim"], infos)
    assert np.array_equal(rho.view(np.uint64), G.arrays(name)[f"k{k}_sim_rho_bits"])


TRIM_RUNS = [(n, k, T) for (n, k, T) in G.case_ks() if "trim" in G.index()[n]["runs"][str(k)]]


@pytest.mark.parametrize("name,k,T", TRIM_RUNS)
def test_trim_matches_reference(name, k, T):
    ref = G.index()[name]["runs"][str(k)]["trim"]
    arr = G.arrays(name)
    o = O.trim(G.pairs(name), k)
    deg = arr[f"k{k}_trim_ckdeg"]
    assert np.array_equal(deg[:, 0], o["map"]) and np.array_equal(deg[:, 1], o["nck"])
    core = arr[f"k{k}_trim_ckcore"]
    assert np.array_equal(core[:, 0], o["map"][o["order"]])
    assert np.array_equal(core[:, 1], o["core_num"])
    ck = ref["ckdens"]
    assert ("%f" % o["ckrho"], "%f" % o["rho"], int(ck[2])) == (ck[0], ck[1], o["size"])
    # printdensest (kClistCoreTrim.c:680) walks i from n-1 while i > n-size-1 in
    # unsigned arithmetic: when the best suffix is the whole graph the bound
    # wraps and no vertex is listed.
    listed = [] if o["size"] == o["n2"] else [str(x) for x in o["map"][o["order"][::-1][: o["size"]]]]
    assert list(ck[3:]) == listed
    assert (o["ntrim"], o["mtrim"], o["ncktrim"], o["total"]) == (ref["ntrim"], ref["mtrim"], ref["ncktrim"], ref["total"])
    assert np.array_equal(arr[f"k{k}_trim_trimmed"].reshape(-1, 2), o["trimmed"])


def test_known_answers():
    """K_10: C(10, k) cliques, densest prefix = the whole clique."""
    from math import comb

    g = O.Graph(G.pairs("kat_complete10"))
    for k in range(3, 9):
        tot, per = g.count_cliques(k)
        assert tot == comb(10, k)
        assert np.all(per == comb(9, k - 1))
        infos, _ = g.seq_main(k, 4)
        assert infos[-1].n == 10 and infos[-1].cliques == comb(10, k)
    star = O.Graph(G.pairs("kat_star"))
    assert star.count_cliques(3)[0] == 0


@pytest.mark.parametrize("name,k,T", G.case_ks())
def test_seq_waves_restatement(name, k, T):
    """The wave ordering has no reference counterpart; pin it to what it is
    built from.  One wave is exactly the per-root-edge-stream pass (which the
    reference pins above); with several waves each wave's increment is the
    masked per-root-edge delta from r as the earlier waves left it, and every
    pass still hands out one unit per k-clique."""
    g = O.Graph(G.pairs(name))
    tot, _ = g.count_cliques(k)
    rng = np.random.default_rng(k)
    r0 = rng.integers(0, 3, size=g.n, dtype=np.uint64)
    assert np.array_equal(g.seq_pass_waves(k, r0, 1), g.seq_pass(k, r0, mode=O.SEQ_EDGE_STREAMS))
    for waves in (3, 16):
        r = r0.copy()
        ids = np.arange(g.n, dtype=np.uint64)
        wave = ((ids * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) % np.uint64(waves)
        for w in range(waves):
            r = r + g.seq_delta_masked(k, r, (wave == w).astype(np.uint8))
        got = g.seq_pass_waves(k, r0, waves)
        assert np.array_equal(got, r)
        assert int((got - r0).sum()) == tot


def test_sim_k2_matches_reference():
    """Sim-kClist++ at k = 2 (the edge branch, kCDensestCmpSync.c:189-192): the
    oracle's reports and FP64 rho equal the reference's, bit for bit, on every
    golden graph (tests/golden/make_golden_sim2.py)."""
    import json
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    index = json.load(open(os.path.join(here, "sim2.json")))
    arrays = np.load(os.path.join(here, "sim2.npz"))
    for name, meta in index.items():
        g = O.Graph(G.pairs(name))
        infos, rho = g.sim_main(2, meta["T"])
        want = [[i[0], i[1], i[2], float.fromhex(i[3]), float.fromhex(i[4])] for i in meta["infos"]]
        assert G.infos_equal(want, infos), name
        assert np.array_equal(rho.view(np.uint64), arrays[f"{name}_rho_bits"]), name


def _sampling_cases():
    import json
    import os

    with open(os.path.join(G.HERE, "sampling.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("key", sorted(_sampling_cases()))
def test_sampling_matches_reference(key):
    """Seq-Sampling++ (kCDensestSamplingKclistpp.c): the reference's clique
    list at p = 1, its InMemoryFrankWolfe update in the order its own shuffle
    drew, ExtractDensest bit for bit, and Solve's printed report line -- all
    reproduced by the oracle from the stored order (tests/golden/
    make_golden_sampling.py)."""
    from tests.golden.make_golden_sampling import check_line, rows_digest

    meta = _sampling_cases()[key]
    k = meta["k"]
    with np.load(os.path.join(G.HERE, "sampling.npz")) as z:
        order, rho_ref = z[f"{key}_order"], z[f"{key}_rho"]
    g = O.Graph(G.pairs(meta["case"]))
    total = g.count_cliques(k)[0]
    assert total == meta["total"]
    full, _ = g.sampling_collect(k, meta["sample_seed"], 0, True, meta["waves"])
    assert rows_digest(full) == meta["all_digest"]
    all_, prob, thr = O.sampling_threshold(meta["target"], total)
    assert prob.hex() == meta["prob"]
    rows, _ = g.sampling_collect(k, meta["sample_seed"], thr, all_, meta["waves"])
    assert len(rows) == meta["sampled"]
    rho = O.sampling_pass_order(k, rows, order, np.zeros(g.n, np.uint32))
    assert np.array_equal(rho, rho_ref)
    info, _ = O.sampling_extract(g.n, k, rows, rho, 1)
    want = meta["info"]
    assert [info.n, info.m, info.density.hex(), info.ub.hex()] == want
    check_line(O.sampling_report(g, k, rows, rho, 1, prob), meta["line"])
