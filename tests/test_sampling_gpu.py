"""Seq-Sampling++ on the GPU (kclistpp_gb300/csrc/kclpp_sample.cu) against the
oracle (oracle/kclpp_oracle.c, pinned to the reference program by
tests/test_oracle_golden.py::test_sampling_matches_reference): the kept
cliques and their waves, the wave passes, every figure of the reports and the
whole Solve loop, bit for bit -- on graphs whose roots use every launch group
of the sampling kernel (rows in shared memory and rows in a global slab)."""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O
from tests import golden_util as G
from tests.test_sampling_host import bipartite_with_clique, sort_rows

pytestmark = pytest.mark.gpu


def _graphs():
    return {
        "cl_2000": G.pairs("cl_2000"),
        "planted_3000": G.pairs("planted_3000"),
        "kat_complete10": G.pairs("kat_complete10"),
        "kat_star": G.pairs("kat_star"),
        "bipartite_mid": bipartite_with_clique(200, 200, 10),  # roots of out-degree 129..200
    }


def _same_report(rep, want) -> None:
    for f in ("T", "n", "m", "sub_n", "sub_e", "sub_core", "sub_cliques"):
        assert getattr(rep, f) == want[f], (f, getattr(rep, f), want[f])
    for f in ("density", "ub", "edge_density", "clique_density", "upper_bound"):
        a, b = np.float64(getattr(rep, f)), np.float64(want[f])
        assert (np.isnan(a) and np.isnan(b)) or a.tobytes() == b.tobytes(), (f, a, b)


@pytest.mark.parametrize("k", [3, 4, 5])
def test_sample_equals_oracle(ctx, k):
    for name, pairs in _graphs().items():
        g = K.build_graph(ctx, K.EdgeList.from_pairs(pairs))
        og = O.Graph(pairs)
        total = og.count_cliques(k)[0]
        for target, seed, waves in [(total + 1, 5, 4), (max(total // 5, 1), 77, 8), (max(total // 50, 1), 3, 256)]:
            s = K.Sampling(g, k, target, seed, waves)
            info = s.info()
            all_, prob, thr = O.sampling_threshold(target, total)
            assert (info.cliques_total, bool(info.all), info.threshold) == (total, all_, thr), name
            assert np.float64(info.prob).tobytes() == np.float64(prob).tobytes()
            want = sort_rows(*og.sampling_collect(k, seed, thr, all_, waves))
            rows, wave = s.cliques()
            assert info.sampled == len(want[0]), (name, k, target)
            assert np.array_equal(rows, want[0]) and np.array_equal(wave, want[1]), (name, k, target)
            s.close()


def test_sample_wide_roots(ctx):
    """Roots of out-degree 1500 (rows beyond shared memory: the slab group) and
    of 128 < out-degree <= the shared-memory bound, in one graph."""
    pairs = bipartite_with_clique(1500, 1500, 14)
    mid = bipartite_with_clique(300, 300, 12).astype(np.int64) + 3000
    pairs = np.concatenate([pairs.astype(np.int64), mid]).astype(np.uint32)
    g = K.build_graph(ctx, K.EdgeList.from_pairs(pairs))
    og = O.Graph(pairs)
    assert g.core == 1500
    for k, div in ((3, 1), (4, 7)):
        total = og.count_cliques(k)[0]
        target = total // div
        s = K.Sampling(g, k, target, 21, 4)
        all_, prob, thr = O.sampling_threshold(target, total)
        want = sort_rows(*og.sampling_collect(k, 21, thr, all_, 4))
        rows, wave = s.cliques()
        assert np.array_equal(rows, want[0]) and np.array_equal(wave, want[1]), (k, target)
        s.close()


@pytest.mark.parametrize("waves", [1, 8])
def test_passes_and_reports_equal_oracle(ctx, waves):
    pairs = G.pairs("planted_3000")
    g = K.build_graph(ctx, K.EdgeList.from_pairs(pairs))
    og = O.Graph(pairs)
    k = 4
    total = og.count_cliques(k)[0]
    target = total // 3
    s = K.Sampling(g, k, target, 9, waves)
    all_, prob, thr = O.sampling_threshold(target, total)
    rows, wave = og.sampling_collect(k, 9, thr, all_, waves)
    rho = np.zeros(og.n, np.uint32)
    done = 0
    for T in (1, 2, 4, 8):
        s.passes(T - done)
        for _ in range(T - done):
            rho = O.sampling_pass(og.n, k, rows, wave, waves, rho)
        done = T
        assert np.array_equal(s.rho(), rho), T
        rep, order = s.extract(T)
        want = O.sampling_report(og, k, rows, rho, T, prob)
        assert np.array_equal(order, want["order"])
        _same_report(rep, want)
    # from a given state
    rng = np.random.default_rng(4)
    r0 = rng.integers(0, 50, size=og.n).astype(np.uint32)
    s.set_rho(r0, 3)
    s.passes(2)
    want = O.sampling_pass(og.n, k, rows, wave, waves, O.sampling_pass(og.n, k, rows, wave, waves, r0))
    assert np.array_equal(s.rho(), want)
    assert s.info().passes == 5
    s.close()


@pytest.mark.parametrize("name,k", [("cl_2000", 3), ("planted_3000", 5), ("kat_complete10", 4),
                                    ("kat_star", 3), ("kat_triangle_k4", 4)])
def test_sampling_main_equals_oracle(ctx, name, k):
    pairs = G.pairs(name)
    g = K.build_graph(ctx, K.EdgeList.from_pairs(pairs))
    og = O.Graph(pairs)
    reps = K.sampling_main(g, k, 20, 500, 13, 8)
    want = O.sampling_main(og, k, 20, 500, 13, 8)["reports"]
    assert len(reps) == len(want) == 5
    for rep, w in zip(reps, want):
        _same_report(rep, w)


def test_full_size_properties(ctx):
    """A larger graph, checked by what holds at any size: the sample size is
    binomial around the target, every pass adds one unit per kept clique, the
    reported subgraph's density is its exact count over its size, and a
    second sample with the same seed is the same set."""
    el = K.rmat(15, 16, seed=71)
    g = K.build_graph(ctx, el)
    k = 4
    s = K.Sampling(g, k, 200_000, 5, 8)
    info = s.info()
    sd = (info.cliques_total * info.prob * (1 - info.prob)) ** 0.5
    assert abs(info.sampled - 200_000) < 6 * sd + 1
    s.passes(16)
    assert int(s.rho().astype(np.int64).sum()) == 16 * info.sampled
    rep, order = s.extract(16)
    assert rep.clique_density == rep.sub_cliques / rep.sub_n
    assert sorted(order.tolist()) == list(range(g.n))
    a = s.cliques()
    s2 = K.Sampling(g, k, 200_000, 5, 8)
    b = s2.cliques()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    s.close()
    s2.close()


def test_sampling_rejects_bad_arguments(ctx):
    g = K.build_graph(ctx, K.EdgeList.from_pairs(G.pairs("kat_complete10")))
    for k, target, waves, status in [(2, 10, 1, K.ERR_UNSUPPORTED), (9, 10, 1, K.ERR_UNSUPPORTED),
                                     (3, 0, 1, K.ERR_INVALID), (3, 10, 0, K.ERR_INVALID),
                                     (3, 10, 257, K.ERR_INVALID), (3, 2**31, 1, K.ERR_INVALID)]:
        with pytest.raises(K.KclppError) as e:
            K.Sampling(g, k, target, 1, waves)
        assert e.value.status == status
    s = K.Sampling(g, 3, 10, 1, 1)
    with pytest.raises(K.KclppError):
        s.extract(0)
    s.close()


def test_cli_prints_the_reference_lines(tmp_path):
    """The drop-in program: the reference's argv and printed report lines,
    with figures equal to the oracle's Solve loop."""
    import os
    import re
    import subprocess

    from tests.golden.make_golden_sampling import LINE, check_line

    pairs = G.pairs("planted_3000")
    path = tmp_path / "g.txt"
    path.write_text("".join(f"{s} {t}\n" for s, t in pairs))
    exe = os.path.join(os.path.dirname(K.LIB_PATH), "bin", "kCDensestSamplingKclistpp")
    env = dict(os.environ, KCLPP_SEED="13", KCLPP_WAVES="8", KCLPP_SAMPLE_TARGET="500")
    out = subprocess.run([exe, "4", "20", "4", str(path)], check=True, capture_output=True, text=True,
                         env=env).stdout
    og = O.Graph(pairs)
    want = O.sampling_main(og, 4, 20, 500, 13, 8)
    assert re.search(r"Number of 4-cliques: %d\n" % want["total"], out)
    assert re.search(r"Number of sampled 4-cliques: %d\n" % len(want["rows"]), out)
    lines = [m for m in (LINE.match(x) for x in out.splitlines()) if m]
    assert len(lines) == 5
    for m, rep in zip(lines, want["reports"]):
        check_line(rep, [int(m.group(1)), int(m.group(2)), m.group(3), m.group(4), m.group(5)])
