"""Batched runs (many graphs, several k, one captured CUDA graph) and the
schedule autotuner.  The oracle for a batch is each graph run on its own:
every slice of the batch's result must equal the single-graph run bit for
bit, and a tuned schedule must not change any result."""
import numpy as np
import pytest

import kclistpp_gb300 as K

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
