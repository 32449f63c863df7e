"""Seq-Sampling++ without a GPU: the sampling kernels' per-thread code
(kclistpp_gb300/csrc/kclpp_sample.cuh) compiled for the host by
tests/sample_emul.cpp and run root by root as a CTA runs it, against the
oracle's independent restatement (oracle/kclpp_oracle.c, pinned to the
reference by tests/test_oracle_golden.py::test_sampling_matches_reference).

The kept set, every kept row and its wave, one wave pass and the max-rank
push must agree exactly, for k = 3..8, for the whole clique set and for
samples, on graphs with roots of small and of wide rows (out-degree up to
1320, rows of 42 words).
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O
from tests import golden_util as G

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def emul(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    so = str(tmp_path_factory.mktemp("emul") / "sample_emul.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so, os.path.join(HERE, "sample_emul.cpp")],
                   check=True)
    L = C.CDLL(so)
    u32p, u64p, u8p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_uint8)
    L.emul_sample.restype = C.c_uint64
    L.emul_sample.argtypes = [C.c_uint32, u64p, u32p, C.c_int, C.c_uint32, C.c_uint64, C.c_uint64, C.c_int,
                              C.c_uint32, u32p, u8p, C.c_uint64]
    L.emul_pass.restype = None
    L.emul_pass.argtypes = [C.c_uint32, C.c_int, C.c_uint64, u32p, u8p, C.c_uint32, u32p]
    L.emul_push.restype = None
    L.emul_push.argtypes = [C.c_int, C.c_uint64, u32p, u32p, u32p]
    return L


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def emul_sample(L, g: O.Graph, k, seed, thr, all_, waves):
    off, cols = g.csr()
    off = np.ascontiguousarray(off, np.uint64)
    cols = np.ascontiguousarray(cols if len(cols) else np.zeros(1, np.uint32), np.uint32)
    dmax = max(g.core, 1)
    args = (g.n, _p(off, C.c_uint64), _p(cols, C.c_uint32), k, dmax, seed, thr, int(all_), waves)
    cnt = int(L.emul_sample(*args, C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint8)(), 0))
    rows = np.zeros((max(cnt, 1), k), np.uint32)
    wave = np.zeros(max(cnt, 1), np.uint8)
    got = int(L.emul_sample(*args, _p(rows, C.c_uint32), _p(wave, C.c_uint8), cnt))
    assert got == cnt
    return rows[:cnt], wave[:cnt]


def sort_rows(rows, wave):
    """Rows by (largest member, next largest, ...), the order the library returns."""
    if not len(rows):
        return rows, wave
    idx = np.lexsort(rows.T)
    return rows[idx], wave[idx]


def bipartite_with_clique(a: int, b: int, c: int) -> np.ndarray:
    """K_{a,b} (out-degrees near min(a, b) in the core order, no triangle) plus
    every edge among the first c vertices of each side."""
    pairs = [(i, a + j) for i in range(a) for j in range(b)]
    pairs += [(i, j) for i in range(c) for j in range(i + 1, c)]
    pairs += [(a + i, a + j) for i in range(c) for j in range(i + 1, c)]
    return np.asarray(pairs, dtype=np.uint32)


GRAPHS = {
    "cl_2000": lambda: G.pairs("cl_2000"),
    "planted_3000": lambda: G.pairs("planted_3000"),
    "kat_complete10": lambda: G.pairs("kat_complete10"),
    "kat_star": lambda: G.pairs("kat_star"),
    "dense_block": lambda: np.asarray([(i, j) for i in range(40) for j in range(i + 1, 40) if (i * 7 + j * 3) % 5],
                                      dtype=np.uint32),
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
@pytest.mark.parametrize("k", [3, 4, 5, 6])
def test_sample_equals_oracle(emul, name, k):
    g = O.Graph(GRAPHS[name]())
    total = g.count_cliques(k)[0]
    for target, seed, waves in [(total + 5, 3, 1), (max(total // 3, 1), 11, 4), (max(total // 17, 1), 2**63 + 5, 256)]:
        all_, prob, thr = O.sampling_threshold(target, total)
        want = sort_rows(*g.sampling_collect(k, seed, thr, all_, waves))
        got = sort_rows(*emul_sample(emul, g, k, seed, thr, all_, waves))
        assert np.array_equal(want[0], got[0]), (name, k, target)
        assert np.array_equal(want[1], got[1]), (name, k, target)
        if all_:
            assert len(got[0]) == total


@pytest.mark.parametrize("k", [7, 8])
def test_sample_large_k(emul, k):
    g = O.Graph(G.pairs("kat_complete10"))
    total = g.count_cliques(k)[0]
    all_, prob, thr = O.sampling_threshold(total // 2, total)
    want = sort_rows(*g.sampling_collect(k, 5, thr, all_, 8))
    got = sort_rows(*emul_sample(emul, g, k, 5, thr, all_, 8))
    assert np.array_equal(want[0], got[0]) and np.array_equal(want[1], got[1])


def test_sample_wide_rows(emul):
    """Roots of out-degree 1320 (rows of 42 words; on a GB300 such rows exceed
    shared memory and the kernel keeps them in a global slab) next to a dense
    part with cliques."""
    g = O.Graph(bipartite_with_clique(1320, 1320, 12))
    assert g.core == 1320
    for k in (3, 4):
        total = g.count_cliques(k)[0]
        assert total > 0
        all_, prob, thr = O.sampling_threshold(total // 3, total)
        want = sort_rows(*g.sampling_collect(k, 9, thr, all_, 4))
        got = sort_rows(*emul_sample(emul, g, k, 9, thr, all_, 4))
        assert np.array_equal(want[0], got[0]) and np.array_equal(want[1], got[1])


def test_pass_and_push_equal_oracle(emul):
    g = O.Graph(G.pairs("planted_3000"))
    k = 4
    total = g.count_cliques(k)[0]
    all_, prob, thr = O.sampling_threshold(total // 4, total)
    rows, wave = g.sampling_collect(k, 17, thr, all_, 8)
    rho = np.zeros(g.n, np.uint32)
    mine = rho.copy()
    for _ in range(5):
        rho = O.sampling_pass(g.n, k, rows, wave, 8, rho)
        emul.emul_pass(g.n, k, len(rows), _p(rows, C.c_uint32), _p(wave, C.c_uint8), 8, _p(mine, C.c_uint32))
    assert np.array_equal(rho, mine)
    assert int(rho.sum()) == 5 * len(rows)
    info, ordered = O.sampling_extract(g.n, k, rows, rho, 5)
    rank = np.empty(g.n, np.uint32)
    rank[ordered] = np.arange(g.n, dtype=np.uint32)
    push = np.zeros(g.n, np.uint32)
    emul.emul_push(k, len(rows), _p(rows, C.c_uint32), _p(rank, C.c_uint32), _p(push, C.c_uint32))
    c = np.cumsum(push.astype(np.int64))
    assert int(c[info.n - 1]) == info.m


def test_sample_size_follows_probability():
    """The counter-based rule keeps about p of the cliques (binomial spread)."""
    g = O.Graph(G.pairs("rmat12"))
    k = 3
    total = g.count_cliques(k)[0]
    for target, seed in [(20000, 1), (5000, 2), (100000, 3)]:
        all_, prob, thr = O.sampling_threshold(target, total)
        rows, wave = g.sampling_collect(k, seed, thr, all_, 16)
        sd = (total * prob * (1 - prob)) ** 0.5
        assert abs(len(rows) - target) < 5 * sd + 1, (len(rows), target, sd)
        counts = np.bincount(wave, minlength=16)
        assert counts.min() > 0.8 * len(rows) / 16


def test_more_waves_approach_the_sequential_update():
    """The wave count trades launches for fidelity to the reference's update
    (one clique at a time, a fresh random order each pass): on a planted RMAT
    graph the sampled bound's gap after 8 passes shrinks as the waves double,
    and at 256 waves it is within 3x of the sequential order's.  For powers of
    two the waves nest: the wave at W is the wave at 256 shifted right."""
    el = K.rmat_planted(13, 16, 4, 60, 150, 0.5, seed=79)
    g = O.Graph(el.pairs())
    k = 4
    total = g.count_cliques(k)[0]
    all_, prob, thr = O.sampling_threshold(100_000, total)
    rows, w256 = g.sampling_collect(k, 5, thr, all_, 256)
    _, w8 = g.sampling_collect(k, 5, thr, all_, 8)
    assert np.array_equal(w8, w256 >> 5)

    def gap(rho, T):
        info, _ = O.sampling_extract(g.n, k, rows, rho, T)
        return info.ub / info.density - 1

    gaps = {}
    for W in (1, 8, 64, 256):
        wave = (w256 >> (8 - int(np.log2(W)))).astype(np.uint8)
        rho = np.zeros(g.n, np.uint32)
        for _ in range(8):
            rho = O.sampling_pass(g.n, k, rows, wave, W, rho)
        gaps[W] = gap(rho, 8)
    rng = np.random.default_rng(1)
    rho = np.zeros(g.n, np.uint32)
    for _ in range(8):
        rho = O.sampling_pass_order(k, rows, rng.permutation(len(rows)).astype(np.uint32), rho)
    seq = gap(rho, 8)
    assert gaps[1] > gaps[8] > gaps[64] > gaps[256] > 0
    assert gaps[256] < 3 * seq + 1e-9, (gaps, seq)
