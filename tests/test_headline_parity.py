"""Parity on the headline workload itself: RMAT scale 20 (0.57, 0.19, 0.19,
0.05), edge factor 16, seed 1, k-clique-core trimmed, at k = 4 and k = 5.

* The trim (kClistCoreTrim.c:707-775) against the reference program's own
  output on this graph (tests/golden/rmat20_trim.json, made by
  make_golden_rmat20.py, for each k it holds): its statistics, the SHA-256
  of its ckdeg, ckcore and ckdens files and of the trimmed edge list, all
  rebuilt here from the library's result in the reference's formats.
* One Seq-kClist++ pass (per-root-edge streams, kCDensestNoAtom.c:270-295)
  and one Sim-kClist++ pass (kCDensestCmpSync.c:298-325, 399-404) on the
  trimmed core, from zero and from a spread state, against the oracle bit for
  bit, and the extraction (sort by r, PAVA pass, densest prefix, bound).  At
  k = 5 a whole oracle pass takes minutes on the host, so the passes are
  compared on two root shards of the library's partition (the shards of one
  pass sum to the pass, tests/test_shard.py): the GPU shard's increments and
  Sim counts against the oracle's restricted to the same roots.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "rmat20_trim.json")))
KS_TRIM = [k for k in (4, 5) if str(k) in GOLD]  # where the reference's own trim was recorded
THREADS = max(1, min(16, O.max_threads()))


def sha_lines(lines) -> str:
    h = hashlib.sha256()
    buf = []
    for ln in lines:
        buf.append(ln)
        if len(buf) >= 65536:
            h.update("".join(buf).encode())
            buf = []
    h.update("".join(buf).encode())
    return h.hexdigest()


@pytest.fixture(scope="module")
def rmat20():
    el = K.rmat(20, 16, 0.57, 0.19, 0.19, seed=1)
    P = el.pairs()
    assert hashlib.sha256(np.ascontiguousarray(P, dtype="<u4").tobytes()).hexdigest() == GOLD["graph"]["sha256"]
    return el


@pytest.fixture(scope="module")
def trims(ctx, rmat20):
    return {k: K.trim(ctx, rmat20, k, K.TRIM_EXACT) for k in (4, 5)}


@pytest.mark.parametrize("k", KS_TRIM)
def test_trim_matches_the_reference_program(trims, k):
    t, g = trims[k], GOLD[str(k)]
    i = t.info
    assert (i.n2, i.e2, i.total, i.ckcore, i.size, i.ntrim, i.mtrim, i.ncktrim) == (
        g["n2"], g["e2"], g["total"], g["ckcore"], g["size"], g["ntrim"], g["mtrim"], g["ncktrim"])
    assert ("%f" % i.ckrho, "%f" % i.rho) == (g["ckrho"], g["rho"])
    mp = t.map.tolist()
    assert sha_lines(f"{v} {c}\n" for v, c in zip(mp, t.nck.tolist())) == g["ckdeg_sha256"]
    assert sha_lines(f"{mp[u]} {c}\n" for u, c in zip(t.order.tolist(), t.core_num.tolist())) == g["ckcore_sha256"]
    n = i.n2
    dens = "%f %f %u" % (i.ckrho, i.rho, i.size) + "".join(
        f" {mp[t.order[j]]}" for j in range(n - 1, n - i.size - 1, -1)) + "\n"
    assert hashlib.sha256(dens.encode()).hexdigest() == g["ckdens_sha256"]
    pairs = t.edges.pairs()
    assert sha_lines(f"{u} {v}\n" for u, v in pairs.tolist()) == g["trimmed_sha256"]
    assert t.peel.committed == n - 1


def spread_state(n, k, seed):
    """A load vector as after some passes (distinct, spread values)."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, 40 * 10 ** (k - 1), size=n, dtype=np.uint64)


@pytest.mark.parametrize("k", [4])
def test_passes_match_oracle_k4(ctx, trims, k):
    P = trims[k].edges.pairs()
    g = K.build_graph(ctx, K.EdgeList.from_pairs(P))
    og = O.Graph(P)
    assert (g.n, g.m) == (og.n, og.m)
    for r0 in (np.zeros(g.n, np.uint64), spread_state(g.n, k, 3)):
        got = K.seq_passes(g, k, 1, r0.copy())
        want = og.seq_pass(k, r0.copy(), O.SEQ_EDGE_STREAMS, THREADS)
        assert np.array_equal(got, want), "Seq pass differs"
        info, re = K.extract_densest_seq(g, k, 1, got)
        oinfo, ore = og.seq_find_densest(k, 1, want, THREADS)
        assert np.array_equal(re, ore)
        assert (info.n, info.m, info.cliques) == (oinfo.n, oinfo.m, oinfo.cliques)
        assert np.float64(info.density).view(np.uint64) == np.float64(oinfo.density).view(np.uint64)
        assert np.float64(info.ub).view(np.uint64) == np.float64(oinfo.ub).view(np.uint64)
    rho0 = np.zeros(g.n)
    got = K.sim_passes(g, k, 2, rho0.copy())
    want = og.sim_pass(k, 2, og.sim_pass(k, 1, rho0.copy(), THREADS), THREADS)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), "Sim passes differ"
    info, re = K.extract_densest_sim(g, k, got)
    oinfo, ore = og.sim_find_densest(k, want, THREADS)
    assert np.array_equal(re, ore)
    assert (info.n, info.m, info.cliques) == (oinfo.n, oinfo.m, oinfo.cliques)
    assert np.float64(info.ub).view(np.uint64) == np.float64(oinfo.ub).view(np.uint64)
    g.close()


@pytest.mark.parametrize("k", [5])
def test_passes_match_oracle_on_root_shards_k5(ctx, trims, k):
    torch = pytest.importorskip("torch")
    P = trims[k].edges.pairs()
    g = K.build_graph(ctx, K.EdgeList.from_pairs(P))
    og = O.Graph(P)
    off, _ = g.csr()
    world = 48
    owner = K.shard_plan(off, world)
    n = g.n
    for r0 in (np.zeros(n, np.uint64), spread_state(n, k, 5)):
        rho0 = (r0 % 1000).astype(np.float64) * 0.5
        r_d = torch.from_numpy(r0.view(np.int64).copy()).cuda()
        rho_d = torch.from_numpy(rho0.copy()).cuda()
        part = torch.empty(n, dtype=torch.int64, device="cuda")
        for rank in (0, 29):
            mask = (owner == rank).astype(np.uint8)
            torch.cuda.synchronize()
            K.graph_shard(g, rank, world)
            K.seq_delta_dev(g, k, r_d.data_ptr(), part.data_ptr())
            ctx.synchronize()
            got = part.cpu().numpy().view(np.uint64).copy()
            want = og.seq_delta_masked(k, r0, mask, THREADS)
            assert np.array_equal(got, want), f"Seq shard {rank} differs"
            K.sim_counts_dev(g, k, rho_d.data_ptr(), part.data_ptr())
            ctx.synchronize()
            got = part.cpu().numpy().view(np.uint64).copy()
            want = og.sim_counts_masked(k, rho0, mask, THREADS)
            assert np.array_equal(got, want), f"Sim shard {rank} differs"
            K.graph_shard(g, 0, 1)
    g.close()
