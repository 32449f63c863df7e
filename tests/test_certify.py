"""The certificates the extraction reports, against the exact optimum.

For graphs small enough to try every vertex subset, the densest k-clique
density rho* is computed exactly; every report of the Seq and Sim runs must
satisfy density <= rho* <= ub (the upper bounds of kCDensestNoAtom.c:352-369
and kCDensestCmpSync.c:365-381 are valid bounds), and so must the bound a
warm-started run uses (the loads its own passes added).  The density is also
an exact rational: cliques / n of the reported prefix, recounted here.
"""
import itertools

import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O


def _small_graphs():
    out = []
    for seed in range(6):
        rng = np.random.default_rng(seed)
        n = int(rng.integers(10, 17))
        p = float(rng.uniform(0.35, 0.75))
        pairs = [(u, v) for u in range(n) for v in range(u + 1, n) if rng.random() < p]
        if pairs:
            out.append((n, np.array(pairs, dtype=np.uint32)))
    # two dense groups joined by a path: the optimum is one group
    a = [(u, v) for u in range(7) for v in range(u + 1, 7)]
    b = [(u + 8, v + 8) for u in range(6) for v in range(u + 1, 6) if (u + v) % 5]
    out.append((14, np.array(a + b + [(6, 7), (7, 8)], dtype=np.uint32)))
    return out


def _cliques(n, pairs, k):
    adj = np.zeros((n, n), dtype=bool)
    adj[pairs[:, 0], pairs[:, 1]] = adj[pairs[:, 1], pairs[:, 0]] = True
    masks = []
    for c in itertools.combinations(range(n), k):
        if all(adj[x, y] for x, y in itertools.combinations(c, 2)):
            masks.append(sum(1 << x for x in c))
    return np.array(masks, dtype=np.int64)


def _rho_star(n, masks):
    """max over vertex subsets S of (k-cliques inside S) / |S|, as a fraction."""
    best = (0, 1)
    subsets = np.arange(1, 1 << n, dtype=np.int64)
    size = np.array([bin(int(s)).count("1") for s in subsets])
    for lo in range(0, len(subsets), 8192):
        S = subsets[lo:lo + 8192]
        inside = ((masks[None, :] & ~S[:, None]) == 0).sum(axis=1)
        for c, sz in zip(inside, size[lo:lo + 8192]):
            if c * best[1] > best[0] * sz:
                best = (int(c), int(sz))
    return best


def _ub_from_loads(loads, T, k):
    # kCDensestNoAtom.c:352-369 on loads sorted in descending order
    b = np.sort(np.asarray(loads, dtype=np.float64))[::-1]
    s = ub = 0.0
    ip1ck = 1.0
    for i in range(len(b)):
        s += b[i]
        if i + 1 == k:
            ip1ck = 1.0
        elif i + 1 > k:
            ip1ck = ip1ck * (i + 1) / (i + 1 - k)
        if ip1ck < s / T:
            ub = ip1ck / (i + 1)
        else:
            ub = max(ub, s / T / (i + 1))
            break
    return ub


CASES = [(i, k) for i in range(len(_small_graphs())) for k in (3, 4)]


@pytest.mark.parametrize("gi,k", CASES)
def test_reports_bracket_the_optimum(gi, k):
    n, pairs = _small_graphs()[gi]
    masks = _cliques(n, pairs, k)
    if len(masks) == 0:
        pytest.skip("no k-clique")
    num, den = _rho_star(n, masks)
    rho = num / den
    og = O.Graph(pairs)
    rank = O.sort_by_core(pairs)
    for infos, _ in (og.seq_main(k, 64, mode=O.SEQ_EDGE_STREAMS), og.seq_main(k, 64, mode=O.SEQ_SEQUENTIAL)):
        for j, info in enumerate(infos):
            assert info.density <= rho * (1 + 1e-12)
            assert info.density == info.cliques / info.n  # the exact rational, as a double
            assert info.ub >= rho * (1 - 1e-12), (1 << j, info.ub, rho)
        assert infos[-1].density >= 0.5 * rho
    # Sim-kClist++: the reference's reports are reproduced bit for bit, but
    # their upper bound is not a certificate: it scans the vertices in the
    # order of the truncated (unsigned long long)rho (kCDensestCmpSync.c:
    # 334-349), not of the loads, and rho after T passes from zero holds only
    # 1 - 2 / ((T + 1)(T + 2)) of the clique mass (the zero start keeps that
    # weight in the Frank-Wolfe average).  Sorted by the loads themselves and
    # rescaled by that factor, rho gives a valid bound.
    T = 64
    infos, rho_sim = og.sim_main(k, T)
    for info in infos:
        assert info.density <= rho * (1 + 1e-12)
    assert _ub_from_loads(rho_sim, 1, k) / (1.0 - 2.0 / ((T + 1) * (T + 2))) >= rho * (1 - 1e-12)
    # the warm-start bound: the loads that T passes added to any start vector
    inv = np.empty_like(rank)
    inv[rank] = np.arange(len(rank))
    r0 = np.random.default_rng(gi).integers(0, 50, size=og.n, dtype=np.uint64)
    r = r0.copy()
    for T in range(1, 9):
        r = og.seq_pass(k, r, mode=O.SEQ_EDGE_STREAMS)
        assert _ub_from_loads((r - r0).astype(np.float64), T, k) >= rho * (1 - 1e-12)
    # the waves ordering gives feasible loads as well
    r = np.zeros(og.n, dtype=np.uint64)
    for T in range(1, 9):
        r = og.seq_pass_waves(k, r, 3)
        assert _ub_from_loads(r.astype(np.float64), T, k) >= rho * (1 - 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("gi", range(len(_small_graphs())))
def test_library_certificates_bracket_the_optimum(ctx, gi):
    n, pairs = _small_graphs()[gi]
    k = 4
    masks = _cliques(n, pairs, k)
    if len(masks) == 0:
        pytest.skip("no k-clique")
    num, den = _rho_star(n, masks)
    rho = num / den
    g = K.build_graph(ctx, K.EdgeList.from_pairs(pairs))
    r0 = np.random.default_rng(gi).integers(0, 50, size=g.n, dtype=np.uint64)
    for T in (1, 2, 4, 8):
        r = K.seq_passes(g, k, T, r0)
        info = K.extract_densest_seq_warm(g, k, T, r, r0)
        assert info.density <= rho * (1 + 1e-12) and info.ub >= rho * (1 - 1e-12)
        info, _ = K.extract_densest_seq(g, k, T, K.seq_passes(g, k, T))
        assert info.density <= rho * (1 + 1e-12) and info.ub >= rho * (1 - 1e-12)


@pytest.mark.parametrize("gi,k", [(i, k) for i in range(len(_small_graphs())) for k in (2, 3, 4)])
def test_exact_densest_matches_every_subset(gi, k):
    """kclpp_densest_exact (host max-flow) against trying every vertex subset:
    the same optimum as a fraction, and a vertex set that attains it."""
    from fractions import Fraction

    n, pairs = _small_graphs()[gi]
    masks = _cliques(n, pairs, k)
    el = K.EdgeList.from_pairs(pairs)
    info, members = K.densest_exact(el, k)
    if len(masks) == 0:
        assert info.cliques_total == 0
        return
    num, den = _rho_star(n, masks)
    assert Fraction(info.num, info.den) == Fraction(num, den)
    assert info.cliques_total == len(masks)
    S = sum(1 << int(v) for v in np.nonzero(members)[0])
    inside = int(((masks & ~S) == 0).sum())
    assert members.sum() == info.size and inside == info.cliques
    assert Fraction(inside, int(members.sum())) == Fraction(num, den)


@pytest.mark.parametrize("name,k", [("config1_chung_lu_1e4", 3), ("config1_chung_lu_1e4", 4), ("planted_3000", 4),
                                    ("cl_2000", 3), ("cl_2000", 4)])
def test_seq_result_is_the_certified_optimum(name, k):
    """On the golden graphs (config 1: Chung-Lu n = 1e4, average degree 20,
    exponent 2.5, seed 1), the densest prefix Seq-kClist++ reports after 64
    passes is the exact optimum that the max-flow certifier proves, and the
    reported upper bound lies above it."""
    from fractions import Fraction

    from tests import golden_util as Gu

    P = Gu.pairs(name)
    info, members = K.densest_exact(K.EdgeList.from_pairs(P), k)
    infos, _ = O.Graph(P).seq_main(k, 64, mode=O.SEQ_EDGE_STREAMS)
    last = infos[-1]
    assert Fraction(last.cliques, last.n) == Fraction(info.num, info.den)
    assert last.ub >= info.density
    assert info.iterations >= 1 and members.sum() == info.size


def test_random_graphs_certificates_hold():
    """Random small graphs (hypothesis): the max-flow optimum equals the
    exhaustive one, and every Seq report brackets it."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from fractions import Fraction

    @hyp.settings(max_examples=60, deadline=None, derandomize=True)
    @hyp.given(st.integers(5, 12), st.floats(0.2, 0.9), st.integers(2, 4), st.integers(0, 2**31 - 1))
    def check(n, p, k, seed):
        rng = np.random.default_rng(seed)
        pairs = np.array([(u, v) for u in range(n) for v in range(u + 1, n) if rng.random() < p], dtype=np.uint32)
        if len(pairs) == 0:
            return
        masks = _cliques(n, pairs, k)
        info, _ = K.densest_exact(K.EdgeList.from_pairs(pairs), k)
        if len(masks) == 0:
            assert info.cliques_total == 0
            return
        num, den = _rho_star(n, masks)
        assert Fraction(info.num, info.den) == Fraction(num, den)
        if k >= 3:
            infos, _ = O.Graph(pairs).seq_main(k, 16, mode=O.SEQ_EDGE_STREAMS)
            for inf in infos:
                assert inf.density <= num / den * (1 + 1e-12) and inf.ub >= num / den * (1 - 1e-12)

    check()
