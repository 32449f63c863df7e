"""Batched runs (many graphs, several k, one captured CUDA graph) and the
schedule autotuner.  Every slice of the batch's result must equal the
single-graph run bit for bit (and, for k = 6, 7 of the batched
configuration's shape, the oracle's passes), and a tuned schedule must not
change any result."""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _graphs():
    return [
        K.chung_lu(3000, 12.0, 2.4, seed=41),
        K.erdos_renyi(2000, 24.0, seed=42),
        K.planted(4000, 6.0, 2.2, 1, 200, 200, 0.5, seed=43),
        K.EdgeList.from_pairs([[0, 1], [1, 2], [0, 2], [2, 3]]),
        K.rmat(11, 16, seed=44),
        K.chung_lu(1500, 30.0, 2.1, seed=45),
    ]


@pytest.mark.parametrize("kernel", [K.KERNEL_SEQ, K.KERNEL_ORDER])
def test_batch_equals_single_runs(ctx, kernel):
    els = _graphs()
    b = K.Batch(ctx, els)
    ks = [3, 4, 5]
    passes = 3
    out = b.run(kernel, ks, passes)
    again = b.run(kernel, ks, passes)  # replays the captured graph
    assert np.array_equal(out.view(np.uint64), again.view(np.uint64))
    for gi, el in enumerate(els):
        g = K.build_graph(ctx, el)
        sl = b.slice(gi)
        assert sl.stop - sl.start == g.n
        for ki, k in enumerate(ks):
            if kernel == K.KERNEL_SEQ:
                ref = K.seq_passes(g, k, passes)
                assert np.array_equal(out[ki, sl], ref), f"graph {gi} k={k}"
            else:
                ref = K.sim_passes(g, k, passes)
                assert np.array_equal(out[ki, sl].view(np.uint64), ref.view(np.uint64)), f"graph {gi} k={k}"
    b.close()


@pytest.mark.parametrize("kernel,k", [(K.KERNEL_SEQ, 4), (K.KERNEL_ORDER, 5)])
def test_autotune_keeps_results(ctx, kernel, k):
    el = K.planted(4000, 8.0, 2.2, 2, 250, 600, 0.5, seed=46)
    g = K.build_graph(ctx, el)
    before = K.seq_passes(g, k, 2) if kernel == K.KERNEL_SEQ else K.sim_passes(g, k, 2)
    res = K.autotune(g, k, kernel)
    assert res.candidates > 1 and res.best_ms <= res.default_ms + 1e-9
    assert K.get_schedule(g).as_dict() == res.best.as_dict()
    after = K.seq_passes(g, k, 2) if kernel == K.KERNEL_SEQ else K.sim_passes(g, k, 2)
    assert np.array_equal(before.view(np.uint64), after.view(np.uint64))
    tot, per = K.count_cliques(g, k)
    sp = K.get_schedule(g)
    sp.steal_count = 1
    K.set_schedule(g, sp)
    tot2, per2 = K.count_cliques(g, k)  # counting with stealing on: same degrees
    assert tot == tot2 and np.array_equal(per, per2)


def test_batch_of_config4_shape(ctx):
    """A scaled-down batch with the shape of the batched configuration: uneven
    Erdos-Renyi and Chung-Lu graphs, k = 3..7, T passes, one launch."""
    rng = np.random.default_rng(47)
    els = []
    for i in range(24):
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(2e4))))
        d = float(rng.uniform(8, 64))
        els.append(K.erdos_renyi(n, d, seed=100 + i) if i % 2 else K.chung_lu(n, d, 2.5, seed=100 + i))
    b = K.Batch(ctx, els)
    ks = [3, 4, 5, 6, 7]
    out = b.run(K.KERNEL_SEQ, ks, 4)
    for gi in (0, 7, 23):
        g = K.build_graph(ctx, els[gi])
        for ki, k in enumerate(ks):
            assert np.array_equal(out[ki, b.slice(gi)], K.seq_passes(g, k, 4))
    # k = 6, 7 slices against the oracle itself (the reference's chain, one
    # stream per root edge), not only against the library's own single runs
    threads = max(1, min(16, O.max_threads()))
    for gi in (0, 7):
        og = O.Graph(els[gi].pairs())
        for ki, k in enumerate(ks):
            if k < 6:
                continue
            r = np.zeros(og.n, np.uint64)
            for _ in range(4):
                r = og.seq_pass(k, r, O.SEQ_EDGE_STREAMS, threads)
            assert np.array_equal(out[ki, b.slice(gi)], r), f"graph {gi} k={k}"


def _knob_graph():
    # many small roots (stealing among them) next to a few dense ones (all
    # tier M groups in use)
    els = [K.chung_lu(4000, 20.0, 2.3, seed=51), K.erdos_renyi(3000, 30.0, seed=52),
           K.planted(3000, 6.0, 2.2, 1, 1400, 1400, 0.5, seed=53)]
    pairs, base = [], 0
    for el in els:
        p = el.pairs().astype(np.int64)
        pairs.append(p + base)
        base += el.n
    return K.EdgeList.from_pairs(np.concatenate(pairs))


def test_schedule_knobs_change_no_result(ctx):
    """Tier bounds, group splits, CTA widths, work stealing and concurrent
    groups decide only where and when work runs: every combination gives the
    default schedule's r / counts bit for bit."""
    g = K.build_graph(ctx, _knob_graph())
    rng = np.random.default_rng(9)
    r0 = rng.integers(0, 5, size=g.n, dtype=np.uint64) * np.uint64(7)
    rho0 = rng.integers(0, 3, size=g.n).astype(np.float64) * 0.5
    want = {k: (K.seq_passes(g, k, 2, r0), K.sim_counts(g, k, rho0)) for k in (4, 5)}
    base = K.get_schedule(g)
    combos = [dict(steal_seq=s, steal_count=s, concurrent_tiers=c, concurrent_count=c, seq_warps=[w] * 4,
                   count_warps=[cw] * 4, tier_s_max=ts, tier_s_max_seq=tq, seq_split1=a, seq_split2=b,
                   m_split1=a, m_split2=b)
              for s, c, w, cw, ts, tq, a, b in [(0, 0, 8, 8, 64, 8, 128, 256), (1, 1, 24, 32, 32, 32, 256, 512),
                                                (1, 0, 16, 16, 64, 16, 384, 768), (0, 1, 20, 24, 16, 64, 512, 1024),
                                                (1, 1, 2, 8, 64, 8, 128, 256), (0, 0, 4, 16, 32, 16, 256, 512)]]
    for cb in combos:
        sp = K.Schedule(**{**base.as_dict(), **cb})
        K.set_schedule(g, sp)
        for k, (r_want, c_want) in want.items():
            assert np.array_equal(K.seq_passes(g, k, 2, r0), r_want), (cb, k)
            assert np.array_equal(K.sim_counts(g, k, rho0), c_want), (cb, k)


def test_batch_tuned_schedule_keeps_results(ctx):
    """Tuning the union graph after a run makes the next run capture its CUDA
    graph again with the new schedule; the results stay the single runs'."""
    els = _graphs()[:3]
    b = K.Batch(ctx, els)
    ks = [4, 6]
    before = b.run(K.KERNEL_SEQ, ks, 2)
    res = K.autotune(b.union_graph(), 6, K.KERNEL_SEQ)
    assert res.candidates > 1
    after = b.run(K.KERNEL_SEQ, ks, 2)
    assert np.array_equal(before, after)
    b.close()
