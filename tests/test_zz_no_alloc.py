"""kclpp_count_cliques_noalloc: k-clique degrees for callers that cannot
allocate device memory (a pool or arena owns it, or the pipeline must not
enter the allocator).  The entry point's working memory is a static device
array; the test checks, through the C ABI, that it gives the same degrees
and total as the allocating entry point, twice in a row (the array keeps the
previous call's contents, so the second call also checks that the call clears
what must start at zero).

This file is the last one pytest collects (its name sorts after every other
test file), so that under -x a failure here comes after every other test has
run; it also passes on its own in a fresh process.  The test allocates its
own buffers with torch; the entry point under test allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

import kclistpp_gb300 as K

pytestmark = pytest.mark.gpu


def test_noalloc_degrees_match_the_allocating_entry_point():
    torch = pytest.importorskip("torch")
    ctx = K.Context(0)
    # tier S (out-degree <= 64) and tier M roots, and a tier-M root with
    # out-degree above 256
    big = K.build_graph(ctx, K.planted(6000, 8.0, 2.2, 1, 700, 700, 0.55, seed=21))
    assert big.core > 256
    # k = 7, 8 on a smaller community (the counts grow quickly with k)
    small = K.build_graph(ctx, K.planted(3000, 8.0, 2.2, 2, 90, 130, 0.6, seed=23))
    for g, ks in ((big, (3, 4, 5, 6)), (small, (6, 7, 8))):
        off, cols = g.csr()
        d_off = torch.from_numpy(off.view(np.int64).copy()).cuda()
        d_cols = torch.from_numpy(cols.view(np.int32).copy()).cuda()
        d_nck = torch.empty(g.n, dtype=torch.int64, device="cuda")
        for k in ks:
            tot, per = K.count_cliques(g, k)
            for call in range(2):
                d_nck.fill_(-1)  # garbage: the call must clear its output
                torch.cuda.synchronize()
                total = C.c_uint64(0)
                st = K._lib.kclpp_count_cliques_noalloc(None, g.n, g.m, C.c_void_p(d_off.data_ptr()),
                                                        C.c_void_p(d_cols.data_ptr()), k,
                                                        C.c_void_p(d_nck.data_ptr()), C.byref(total))
                assert st == K.OK, K._lib.kclpp_last_error()
                got = d_nck.cpu().numpy().view(np.uint64)
                assert np.array_equal(got, per), f"k={k} call {call}: degrees differ"
                assert total.value == tot, f"k={k} call {call}: total {total.value} != {tot}"
        g.close()
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_limit():
    st = K._lib.kclpp_count_cliques_noalloc(None, (1 << 21) + 1, 0, C.c_void_p(16), None, 4,
                                            C.c_void_p(16), None)
    assert st == K.ERR_UNSUPPORTED
    assert b"limit" in K._lib.kclpp_last_error()


def test_noalloc_refuses_a_capturing_stream():
    """The call reads its status back and synchronises, which a capture does
    not allow: on a stream being captured it returns KCLPP_ERR_INVALID and
    leaves the capture intact."""
    torch = pytest.importorskip("torch")
    ctx = K.Context(0)
    g = K.build_graph(ctx, K.planted(500, 6.0, 2.2, 1, 40, 40, 0.6, seed=3))
    off, cols = g.csr()
    d_off = torch.from_numpy(off.view(np.int64).copy()).cuda()
    d_cols = torch.from_numpy(cols.view(np.int32).copy()).cuda()
    d_nck = torch.zeros(g.n, dtype=torch.int64, device="cuda")
    x = torch.zeros(4, device="cuda")
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=s):
        x.add_(1)
        st = K._lib.kclpp_count_cliques_noalloc(C.c_void_p(s.cuda_stream), g.n, g.m, C.c_void_p(d_off.data_ptr()),
                                                C.c_void_p(d_cols.data_ptr()), 4, C.c_void_p(d_nck.data_ptr()),
                                                None)
    assert st == K.ERR_INVALID
    assert b"capture" in K._lib.kclpp_last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert x.tolist() == [1.0] * 4
    assert int(d_nck.abs().sum()) == 0
    # outside the capture the same call runs
    tot, per = K.count_cliques(g, 4)
    total = C.c_uint64(0)
    st = K._lib.kclpp_count_cliques_noalloc(C.c_void_p(s.cuda_stream), g.n, g.m, C.c_void_p(d_off.data_ptr()),
                                            C.c_void_p(d_cols.data_ptr()), 4, C.c_void_p(d_nck.data_ptr()),
                                            C.byref(total))
    assert st == K.OK, K._lib.kclpp_last_error()
    assert total.value == tot
    assert np.array_equal(d_nck.cpu().numpy().view(np.uint64), per)
    g.close()
    ctx.close()
