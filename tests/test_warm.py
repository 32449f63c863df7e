"""Learned warm start: the library's MLP kernels against an FP64 restatement,
training on the method's own r vectors, and what the trained network gains
over the plain zero-start run (passes to a certified 1% density gap)."""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import warm_oracle as WO

pytestmark = pytest.mark.gpu


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 6, size=(n, 4)).astype(np.float32)
    Y = (0.3 * X[:, 0] + 0.5 * X[:, 2] - 0.2 * X[:, 1] + rng.normal(0, 0.1, n)).astype(np.float32)
    return X, Y


def test_forward_and_gradient_match_fp64(ctx):
    torch = pytest.importorskip("torch")
    from kclistpp_gb300 import warm as W

    m = W.WarmModel(ctx, seed=3)
    X, Y = _data(20000, 1)
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    p = m.params()
    yh = m.predict(Xd).cpu().numpy()
    yo = WO.forward(p, X)
    assert np.allclose(yh, yo, rtol=1e-4, atol=1e-4 * np.abs(yo).max())
    g, loss = m.grad(Xd, Yd)
    go, lo = WO.grad(p, X, Y)
    # fp32 accumulation vs fp64: relative error of the whole gradient vector
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
    assert abs(loss - lo) <= 1e-4 * abs(lo)
    # a step of training changes the parameters in the descent direction
    before = m.params()
    m.train(Xd, Yd, steps=1, lr=1e-3)
    delta = m.params() - before
    assert np.dot(delta, go) < 0


def test_training_fits(ctx):
    torch = pytest.importorskip("torch")
    from kclistpp_gb300 import warm as W

    m = W.WarmModel(ctx, seed=4)
    X, Y = _data(50000, 2)
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    _, l0 = m.grad(Xd, Yd)
    l1 = m.train(Xd, Yd, steps=400, lr=1e-2)
    assert l1 < 0.1 * l0 and l1 < 0.05


def _community_graph(seed, n=6000):
    return K.planted(n, 8.0, 2.2, 3, 60, 160, 0.6, seed=seed)


def test_warm_start_reaches_the_gap_in_fewer_passes(ctx):
    """Train on zero-start runs of seeded planted-community graphs (k = 5), then
    compare passes to a certified 1% gap on held-out graphs of the same kind:
    the warm start must need fewer passes in total, and its answers must be
    certified (upper bound from its own increments >= the best density found
    by a long zero-start run)."""
    torch = pytest.importorskip("torch")
    from kclistpp_gb300 import warm as W

    k = 5
    train = [_community_graph(100 + i) for i in range(12)]
    X, Y = W.training_set(ctx, train, k, passes=64)
    m = W.WarmModel(ctx, seed=5)
    m.train(X, Y, steps=600, lr=1e-2)
    zero_p = warm_p = 0
    for s in (900, 901, 902):
        g = K.build_graph(ctx, _community_graph(s))
        z = W.time_to_gap(g, k, 0.01, 512)
        w = W.time_to_gap(g, k, 0.01, 512, model=m, t0=16.0)
        assert z["reached"] and w["reached"]
        best_density = max(z["density"], w["density"])
        assert w["ub"] >= best_density * (1 - 1e-12) and z["ub"] >= best_density * (1 - 1e-12)
        zero_p += z["passes"]
        warm_p += w["passes"]
    assert warm_p < zero_p, (warm_p, zero_p)
