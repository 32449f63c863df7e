"""Graphs built from the bin-sort core order (KCLPP_ORDER_FAST) on the GPU:
the same size, degeneracy and clique counts as from SortByCore's order, and
a Seq pass over the fast order's DAG equal to the oracle's over the same
orientation.  (Kept in its own file, run after the other GPU tests.)"""
import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_fast_order_graph(ctx):
    """KCLPP_ORDER_FAST: the DAG of the bin-sort peel has the exact order's
    size and degeneracy and the same k-clique counts, and a Seq pass over it
    equals the oracle's over the same orientation."""
    el = K.chung_lu(5000, 16.0, 2.3, seed=33)
    ge = K.build_graph(ctx, el)
    gf = K.build_graph(ctx, el, order=K.ORDER_FAST)
    assert (gf.n, gf.m, gf.core) == (ge.n, ge.m, ge.core)
    for k in (3, 4, 5):
        assert K.count_cliques(gf, k)[0] == K.count_cliques(ge, k)[0]
    og = O.Graph(el.pairs(), rank=K.core_order(el, K.ORDER_FAST))
    assert np.array_equal(K.seq_passes(gf, 4, 1), og.seq_pass(4, np.zeros(og.n, np.uint64)))
