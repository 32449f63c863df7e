"""Host-side logic of the library (no GPU needed): the C ABI's exports, the
edge-list reader and writer, the seeded generators and the exact degeneracy
order.  The compute entry points are exercised by the GPU tests."""
import hashlib
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O
from tests import golden_util as G
from tests.conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions() -> list[str]:
    src = open(os.path.join(ROOT, "include", "kclpp.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kclpp_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert len(names) >= 40
    out = subprocess.run(["nm", "-D", "--defined-only", K.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (kclpp_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    # and the Python binding covers every one of them
    assert set(names) <= set(K.EXPORTED), set(names) - set(K.EXPORTED)


def test_version_and_status_strings():
    assert "sm_103a" in K.version()
    for s in range(0, 8):
        assert K._lib.kclpp_status_string(s)


@pytest.mark.skipif(gpu_available(), reason="a GPU is present")
def test_no_device_is_reported():
    with pytest.raises(K.KclppError) as ei:
        K.Context(0)
    assert ei.value.status == K.ERR_NODEVICE


def test_generators_are_deterministic():
    a = K.chung_lu(3000, 12.0, 2.4, seed=9).pairs()
    b = K.chung_lu(3000, 12.0, 2.4, seed=9).pairs()
    c = K.chung_lu(3000, 12.0, 2.4, seed=10).pairs()
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    # canonical form: u < v, sorted, no repeats
    assert np.all(a[:, 0] < a[:, 1])
    keys = (a[:, 0].astype(np.uint64) << 32) | a[:, 1]
    assert np.all(np.diff(keys.astype(np.int64)) > 0)


def test_generator_shapes():
    r = K.rmat(14, 16, seed=2).pairs()
    assert r.max() < (1 << 14) and 150_000 < len(r) < 16 * (1 << 14)
    e = K.erdos_renyi(4000, 10.0, seed=1).pairs()
    assert abs(len(e) - 20000) < 200
    p = K.planted(5000, 6.0, 2.2, 4, 40, 120, 0.7, seed=3).pairs()
    assert len(p) > 15000


def test_golden_graph_hashes_are_stable():
    """The generated golden graphs are the ones the reference was run on."""
    for name in G.index():
        G.pairs(name)


def test_edge_list_roundtrip(tmp_path):
    P = K.erdos_renyi(500, 8.0, seed=4).pairs()
    el = K.EdgeList.from_pairs(P)
    f = tmp_path / "g.txt"
    el.write(str(f))
    back = K.read_edge_list(str(f))
    assert np.array_equal(back.pairs(), P)
    assert back.n == int(P.max()) + 1


def test_read_edge_list_semantics(tmp_path):
    """ReadEdgeList (Graph.c:34-53): n = max id + 1, reading stops at the first
    token that is not a number, a trailing half pair is dropped."""
    f = tmp_path / "a.txt"
    f.write_text("0 5\n3 2\n\n7 1\n9")
    el = K.read_edge_list(str(f))
    assert el.n == 8 and el.e == 3
    f.write_text("1 2\n2 3\n# comment\n4 5\n")
    el = K.read_edge_list(str(f))
    assert el.e == 2
    f.write_text("")
    el = K.read_edge_list(str(f))
    assert el.n == 1 and el.e == 0
    with pytest.raises(K.KclppError) as ei:
        K.read_edge_list(str(tmp_path / "missing.txt"))
    assert ei.value.status == K.ERR_IO


@pytest.mark.parametrize("maker", [
    lambda: K.chung_lu(10000, 20.0, 2.5, seed=1),
    lambda: K.rmat(13, 16, seed=7),
    lambda: K.planted(8000, 6.0, 2.1, 3, 50, 150, 0.5, seed=2),
    lambda: K.EdgeList.from_pairs(G.pairs("kat_clique_tree")),
])
def test_core_order_matches_oracle(maker):
    """SortByCore's rank permutation, including the heap's tie order."""
    el = maker()
    assert np.array_equal(K.core_order(el), O.sort_by_core(el.pairs(), el.n))


def _out_degrees(el, rank):
    """Out-degree of every vertex (by id) in the DAG the rank orients."""
    P = el.pairs().astype(np.int64)
    by_rank = np.bincount(np.maximum(rank[P[:, 0]], rank[P[:, 1]]), minlength=el.n)
    return by_rank[rank]


def _core_numbers(el, rank):
    """Core numbers along a peel: the running maximum of the out-degree (the
    degree each vertex had when it was peeled) in peel order (rank descending)."""
    od = _out_degrees(el, rank)
    order = np.argsort(-rank.astype(np.int64), kind="stable")
    out = np.empty(el.n, dtype=np.int64)
    out[order] = np.maximum.accumulate(od[order]) if el.n else od
    return out


@pytest.mark.parametrize("maker", [
    lambda: K.chung_lu(10000, 20.0, 2.5, seed=1),
    lambda: K.rmat(13, 16, seed=7),
    lambda: K.planted(8000, 6.0, 2.1, 3, 50, 150, 0.5, seed=2),
    lambda: K.EdgeList.from_pairs(G.pairs("kat_clique_tree")),
    lambda: K.EdgeList.from_pairs(G.pairs("kat_star")),
    lambda: K.EdgeList.from_pairs([[0, 5], [5, 9]]),
])
def test_fast_order_is_a_degeneracy_order(maker):
    """KCLPP_ORDER_FAST: a permutation whose peel has the exact order's core
    numbers and degeneracy (the DAG's largest out-degree), with the core
    numbers also equal to networkx's."""
    el = maker()
    fast, exact = K.core_order(el, K.ORDER_FAST), K.core_order(el)
    assert np.array_equal(np.sort(fast), np.arange(el.n, dtype=np.uint32))
    assert _out_degrees(el, fast).max() == _out_degrees(el, exact).max()
    cf = _core_numbers(el, fast)
    assert np.array_equal(cf, _core_numbers(el, exact))
    nx = pytest.importorskip("networkx")
    g = nx.Graph()
    g.add_nodes_from(range(el.n))
    g.add_edges_from(el.pairs().tolist())
    want = nx.core_number(g)
    assert all(cf[v] == want[v] for v in range(el.n))


def test_order_mode_rejects_unknown():
    el = K.EdgeList.from_pairs([[0, 1]])
    with pytest.raises(K.KclppError) as e:
        K.core_order(el, 7)
    assert e.value.status == K.ERR_INVALID


def test_oracle_pins_config1_hash():
    p = G.pairs("config1_chung_lu_1e4")
    assert len(p) == 96552
    assert hashlib.sha256(p.tobytes()).hexdigest() == G.index()["config1_chung_lu_1e4"]["sha256"]


def test_bench_byte_model_matches_brute_force():
    """bench.py's roofline bytes: the per-root-edge gathers of the reference's
    MakeSubgraph, 8 + 4(d+s + d+t) + 4 sum_{x in C(s,t)} d+x + 8(|C(s,t)| + 2)
    per root edge plus 8(n+1) + 16n per pass, checked against a direct count."""
    import importlib.util
    import os

    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py")
    spec = importlib.util.spec_from_file_location("kclpp_bench", path)
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    og = O.Graph(K.planted(1500, 6.0, 2.2, 1, 80, 80, 0.5, seed=61).pairs())
    off, cols = og.csr()
    off = off.astype(np.int64)
    cols = cols.astype(np.int64)
    n = len(off) - 1
    deg = np.diff(off)
    want = 8 * (n + 1) + 16 * n
    for s in range(n):
        Ns = set(cols[off[s]:off[s + 1]].tolist())
        for t in cols[off[s]:off[s + 1]]:
            C = Ns & set(cols[off[t]:off[t + 1]].tolist())
            want += 8 + 4 * (deg[s] + deg[t]) + 4 * sum(deg[x] for x in C) + 8 * (len(C) + 2)
    st = bench.dag_stats(off.astype(np.uint64), cols.astype(np.uint32), 4)
    assert st["ref_equiv_bytes_per_pass"] == want
    # the per-tier figures partition the per-root-edge part
    assert sum(v["bytes"] for v in st["tiers"].values()) == want - 8 * (n + 1) - 16 * n


def test_checkpoint_roundtrip_and_damage(tmp_path):
    """kclpp_save_state / kclpp_load_state: the vector, pass count, k and input
    hash come back bit for bit; a truncated, altered or foreign file is
    reported (KCLPP_ERR_IO), never loaded."""
    el = K.chung_lu(500, 6.0, 2.5, seed=71)
    h = el.hash()
    assert h == K.chung_lu(500, 6.0, 2.5, seed=71).hash() and h != K.chung_lu(500, 6.0, 2.5, seed=72).hash()
    rng = np.random.default_rng(3)
    r = rng.integers(0, 2**63, size=el.n, dtype=np.uint64)
    rho = rng.random(el.n) * 1e6
    for kern, vec in ((K.KERNEL_SEQ, r), (K.KERNEL_ORDER, rho)):
        path = str(tmp_path / f"state{kern}.bin")
        K.save_state(path, kern, 5, 37, vec, h)
        info, back = K.load_state(path)
        assert (info.kind, info.k, info.passes, info.n, info.graph_hash) == (kern, 5, 37, el.n, h)
        assert back.dtype == vec.dtype and np.array_equal(back.view(np.uint64), vec.view(np.uint64))
    raw = open(path, "rb").read()
    for bad in (raw[:-3], raw[:40], raw[:16] + bytes([raw[16] ^ 1]) + raw[17:], b"NOTKCLPP" + raw[8:]):
        p = str(tmp_path / "bad.bin")
        open(p, "wb").write(bad)
        with pytest.raises(K.KclppError) as e:
            K.load_state(p)
        assert e.value.status == K.ERR_IO
    with pytest.raises(K.KclppError):
        K.load_state(str(tmp_path / "missing.bin"))


def _read_ref(text: str):
    """The one-pass reading rule of ReadEdgeList (fscanf("%u %u") until it fails)."""
    nums, cur, innum, bad = [], 0, False, False
    for ch in text:
        if "0" <= ch <= "9":
            cur = cur * 10 + ord(ch) - 48
            if cur > 0xFFFFFFFF:
                bad = True
                break
            innum = True
        elif ch in " \n\t\r":
            if innum:
                nums.append(cur)
            cur, innum = 0, False
        else:
            bad = True
            break
    if innum and not bad:
        nums.append(cur)
    return nums[: 2 * (len(nums) // 2)]


def test_threaded_reader_matches_one_pass(tmp_path):
    """kclpp_read_edge_list_mt gives the one-pass result for every thread
    count, whatever stops the file: a stray character, a number above 2^32-1,
    an unpaired last number, a number the end of the file ends."""
    rng = np.random.default_rng(11)
    seps = [" ", "\n", "\t", "\r\n", "  ", "\n\n"]
    for case in range(40):
        m = int(rng.integers(0, 3000))
        toks = [str(int(x)) for x in rng.integers(0, 1 << 20, size=2 * m)]
        text = "".join(t + seps[int(rng.integers(0, len(seps)))] for t in toks)
        kind = case % 5
        if kind == 1 and text:
            p = int(rng.integers(0, len(text)))
            text = text[:p] + "#" + text[p:]
        elif kind == 2 and text:
            p = int(rng.integers(0, len(text)))
            text = text[:p] + " 99999999999 " + text[p:]
        elif kind == 3:
            text = text + "17"
        elif kind == 4:
            text = text.rstrip() + " 5 6"
        f = tmp_path / f"e{case}.txt"
        f.write_bytes(text.encode())
        want = np.array(_read_ref(text), dtype=np.uint32).reshape(-1, 2)
        for th in (1, 2, 3, 7, 16):
            el = K.read_edge_list(str(f), threads=th)
            got = el.pairs()
            assert np.array_equal(got, want), (case, th)
            assert el.n == (int(want.max()) + 1 if len(want) else 1)


def test_binary_edge_list_cache(tmp_path):
    """A parsed edge list written in binary reads back identical (n and the
    pairs in input order); a damaged file is refused."""
    el = K.rmat(12, 16, seed=5)
    p = str(tmp_path / "g.bin")
    el.write_bin(p)
    back = K.EdgeList.read_bin(p)
    assert back.n == el.n and np.array_equal(back.pairs(), el.pairs())
    raw = open(p, "rb").read()
    for bad in (raw[:-1], raw[:30], raw[:25] + bytes([raw[25] ^ 4]) + raw[26:], b"X" + raw[1:]):
        q = str(tmp_path / "bad.bin")
        open(q, "wb").write(bad)
        with pytest.raises(K.KclppError) as e:
            K.EdgeList.read_bin(q)
        assert e.value.status == K.ERR_IO


def _fnv1a(data: bytes) -> int:
    h = 0xCBF29CE484222325
    for b in data:
        h = ((h ^ b) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def test_binary_edge_list_ids_checked_against_n(tmp_path):
    """A binary edge list whose stored n is too small for its ids is refused,
    even when its checksum is consistent (the checksum only detects damage)."""
    import struct

    pairs = np.array([[0, 1], [1, 5], [2, 3]], dtype=np.uint32)
    for n, ok in ((6, True), (5, False), (1, False)):
        body = b"KCLPPEL1" + struct.pack("<IQ", n, len(pairs)) + pairs.astype("<u4").tobytes()
        q = str(tmp_path / f"n{n}.bin")
        open(q, "wb").write(body + struct.pack("<Q", _fnv1a(body)))
        if ok:
            back = K.EdgeList.read_bin(q)
            assert back.n == n and np.array_equal(back.pairs(), pairs)
        else:
            with pytest.raises(K.KclppError) as e:
                K.EdgeList.read_bin(q)
            assert e.value.status == K.ERR_IO
            assert b"not below" in K._lib.kclpp_last_error()


def test_trim_k2_matches_reference():
    """k = 2 (NormalGraphCoreTrim.c): vertices kept, edges kept and the trimmed
    edge list, in input order, equal to the reference program's output files
    on every golden graph (tests/golden/make_golden_trim2.py); host only."""
    import json

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    index = json.load(open(os.path.join(here, "trim2.json")))
    arrays = np.load(os.path.join(here, "trim2.npz"))
    graphs = {name: G.pairs(name) for name in G.index()}
    graphs["planted_k2"] = K.planted(4000, 6.0, 2.2, 2, 40, 90, 0.5, seed=21).pairs()
    graphs["chung_lu_k2"] = K.chung_lu(5000, 12.0, 2.2, seed=22).pairs()
    assert set(index) == set(graphs)
    for name, meta in index.items():
        pairs = np.ascontiguousarray(graphs[name], dtype=np.uint32)
        assert hashlib.sha256(pairs.tobytes()).hexdigest() == meta["sha256"], name
        tr = K.trim(None, K.EdgeList.from_pairs(pairs), 2)
        assert (tr.info.ntrim, tr.info.mtrim, tr.info.ncktrim) == (meta["ntrim"], meta["mtrim"], meta["ncktrim"]), name
        assert np.array_equal(tr.edges.pairs(), arrays[f"{name}_trimmed"]), name


def test_normal_graph_core_trim_cli(tmp_path):
    """The drop-in NormalGraphCoreTrim program writes the reference's two files
    (trimmed edges, statistics) for a golden graph; no GPU is used."""
    import json

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    meta = json.load(open(os.path.join(here, "trim2.json")))["cl_2000"]
    want = np.load(os.path.join(here, "trim2.npz"))["cl_2000_trimmed"]
    exe = os.path.join(os.path.dirname(K.LIB_PATH), "bin", "NormalGraphCoreTrim")
    edges = tmp_path / "g.txt"
    edges.write_text("".join(f"{s} {t}\n" for s, t in G.pairs("cl_2000")))
    subprocess.run([exe, str(edges), "x"], cwd=tmp_path, check=True, capture_output=True)
    got = np.loadtxt(tmp_path / "trimmed_x_2.txt", dtype=np.uint32, ndmin=2).reshape(-1, 2)
    assert np.array_equal(got, want)
    stat = (tmp_path / "stat_trim_x_2.txt").read_text().split("\n")
    assert stat[0].startswith("[Number of Nodes]")
    assert [int(x) for x in stat[1].split("\t")[:3]] == [meta["ntrim"], meta["mtrim"], meta["ncktrim"]]


C_CLIENT = r"""
#include <stdio.h>
#include <string.h>
#include "kclpp.h"

int main(void) {
  /* K_4 plus a pendant edge */
  const uint32_t pairs[] = {0, 1, 0, 2, 0, 3, 1, 2, 1, 3, 2, 3, 3, 4};
  kclpp_edge_list *el = NULL;
  uint32_t n = 0, exact[5], fast[5];
  uint64_t e = 0;
  if (kclpp_edge_list_create(pairs, 7, &el) != KCLPP_OK) return 1;
  if (kclpp_edge_list_info(el, &n, &e) != KCLPP_OK || n != 5 || e != 7) return 2;
  if (kclpp_core_order(el, exact) != KCLPP_OK) return 3;
  if (kclpp_core_order_mode(el, KCLPP_ORDER_FAST, fast) != KCLPP_OK) return 4;
  if (kclpp_core_order_mode(el, 9, fast) != KCLPP_ERR_INVALID) return 5;
  kclpp_exact_info info;
  if (kclpp_densest_exact(el, 4, &info, NULL) != KCLPP_OK || info.num != 1 || info.den != 4) return 6;
  kclpp_sampling *s = NULL;
  if (kclpp_sampling_create(NULL, NULL, 4, 10, 1, 1, &s) != KCLPP_ERR_INVALID || s) return 7;
  if (kclpp_sampling_info_get(NULL, NULL) != KCLPP_ERR_INVALID) return 8;
  printf("%u %u %u %u %u\n", exact[0], exact[1], exact[2], exact[3], exact[4]);
  kclpp_edge_list_free(el);
  return strlen(kclpp_version()) ? 0 : 9;
}
"""


def test_c_client_compiles_links_and_runs(tmp_path):
    """The header is plain C (C99, -pedantic -Werror) and a C program links
    the library and calls its host-only entry points."""
    import shutil

    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    libdir = os.path.dirname(K.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lkclpp", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    rank = [int(x) for x in r.stdout.split()]
    el = K.EdgeList.from_pairs([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3], [3, 4]])
    assert rank == K.core_order(el).tolist()


def test_schedule_cache_round_trip(tmp_path):
    """A stored schedule comes back field for field under its key; another
    graph, k or kernel, a damaged or truncated file are refused."""
    el = K.chung_lu(2000, 10.0, 2.3, seed=4)
    h = el.hash()
    sp = K.Schedule(tier_s_max=32, tier_s_max_seq=16, m_split1=320, m_split2=640, steal_seq=1, steal_count=1,
                    seq_waves=8, seq_warps=[8, 12, 16, 24], concurrent_tiers=0, count_warps=[8, 16, 24, 32],
                    seq_split1=384, seq_split2=768, concurrent_count=1)
    path = tmp_path / "tuned.sched"
    K.save_schedule(str(path), h, 4, K.KERNEL_SEQ, sp)
    assert K.load_schedule(str(path), h, 4, K.KERNEL_SEQ).as_dict() == sp.as_dict()
    for key in [(h ^ 1, 4, K.KERNEL_SEQ), (h, 5, K.KERNEL_SEQ), (h, 4, K.KERNEL_ORDER)]:
        with pytest.raises(K.KclppError) as e:
            K.load_schedule(str(path), *key)
        assert e.value.status == K.ERR_INVALID
    raw = path.read_bytes()
    for bad in (raw[:-1], raw[:30] + bytes([raw[30] ^ 0x40]) + raw[31:], b"not a schedule"):
        path.write_bytes(bad)
        with pytest.raises(K.KclppError) as e:
            K.load_schedule(str(path), h, 4, K.KERNEL_SEQ)
        assert e.value.status == K.ERR_IO
    with pytest.raises(K.KclppError) as e:
        K.load_schedule(str(tmp_path / "missing"), h, 4, K.KERNEL_SEQ)
    assert e.value.status == K.ERR_IO


NULL_PROBE = r"""
import ctypes as C, sys
sys.path.insert(0, sys.argv[1])
import kclistpp_gb300 as K
skip = {"kclpp_status_string", "kclpp_last_error", "kclpp_version", "kclpp_launch_count", "kclpp_create",
        "kclpp_count_cliques_noalloc"}
ok = {K.OK, K.ERR_INVALID, K.ERR_NODEVICE, None}
for name in K.EXPORTED:
    if name in skip:
        continue
    f = getattr(K._lib, name)
    args = [0 if t in (C.c_int, C.c_uint32, C.c_uint64, C.c_float, C.c_double) else None for t in f.argtypes]
    r = f(*args)
    if r not in ok:
        print("unexpected", name, r)
        sys.exit(3)
print("ok")
"""


def test_null_arguments_never_crash():
    """Every entry point called with null handles and pointers (zero sizes)
    returns a status -- KCLPP_ERR_INVALID, or OK where there is nothing to do --
    instead of faulting.  Run in a child process so that a crash fails the
    test instead of the session."""
    r = subprocess.run([sys.executable, "-c", NULL_PROBE, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.returncode, r.stdout[-500:], r.stderr[-500:])


def test_oracle_rmat_is_the_library_generator():
    """The CPU legs build the benchmark graph with the oracle's restatement of
    the library's RMAT generator (so that they load no library code); it must
    give the library's graph exactly."""
    for scale, ef, seed, (a, b, c) in ((6, 4, 2, (0.57, 0.19, 0.19)), (12, 16, 5, (0.57, 0.19, 0.19)),
                                       (13, 8, 9, (0.45, 0.15, 0.15))):
        want = K.rmat(scale, ef, a, b, c, seed=seed).pairs()
        assert np.array_equal(O.rmat(scale, ef, a, b, c, seed=seed), want), (scale, ef, seed)
