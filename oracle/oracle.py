"""ctypes binding of the CPU oracle (oracle/kclpp_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, always as the checker or the CPU timing, never
as part of the shipped path.  The oracle restates the reference algorithms
(btsun/kclistpp) on the CPU; see kclpp_oracle.h for the file:line citations.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkclpp_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

SEQ_SEQUENTIAL, SEQ_EDGE_STREAMS, SEQ_THREADS, SEQ_VERTEX_STREAMS = 0, 1, 2, 3


# Where the reference's C sources are read from when the reference programs
# are compiled (the golden-vector generators and build()); KCLPP_REFERENCE_SRC
# overrides it.  Only that compile step reads there; nothing at test or bench
# time does.
_REFERENCE_SRC_DEFAULT = "/root/reference"


def reference_sources() -> str | None:
    """The directory holding the reference's sources, or None where it is absent."""
    d = os.environ.get("KCLPP_REFERENCE_SRC", _REFERENCE_SRC_DEFAULT)
    return d if os.path.isdir(d) else None


def build(ref: bool = False, ref_if_present: bool = False) -> None:
    """make the oracle library; with ref=True also the reference programs
    (which must then be present), with ref_if_present=True wherever they are."""
    targets = ["all"]
    src = reference_sources()
    if ref and not src:
        raise RuntimeError("the reference sources are not present (set KCLPP_REFERENCE_SRC)")
    if (ref or ref_if_present) and src:
        targets += ["ref", "REF=" + src]
    r = subprocess.run(["make", "-s", "-C", HERE] + targets, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


class OrcEdge(C.Structure):
    _fields_ = [("s", C.c_uint32), ("t", C.c_uint32)]


class OrcGraph(C.Structure):
    _fields_ = [("n", C.c_uint32), ("e", C.c_uint64), ("edges", C.POINTER(OrcEdge)),
                ("cd", C.POINTER(C.c_uint64)), ("adj", C.POINTER(C.c_uint32)), ("core", C.c_uint32)]


class OrcInfo(C.Structure):
    _fields_ = [("n", C.c_uint32), ("m", C.c_uint32), ("cliques", C.c_uint64),
                ("density", C.c_double), ("ub", C.c_double)]

    def as_tuple(self):
        return (self.n, self.m, self.cliques, self.density, self.ub)


class OrcSamplingInfo(C.Structure):
    _fields_ = [("n", C.c_uint32), ("m", C.c_uint64), ("density", C.c_double), ("ub", C.c_double)]


class OrcTrim(C.Structure):
    _fields_ = [("n", C.c_uint32), ("e", C.c_uint64), ("n2", C.c_uint32), ("e2", C.c_uint64),
                ("core", C.c_uint32), ("map", C.POINTER(C.c_uint32)), ("nck", C.POINTER(C.c_uint64)),
                ("total", C.c_uint64), ("order", C.POINTER(C.c_uint32)), ("core_num", C.POINTER(C.c_uint64)),
                ("ckcore", C.c_uint64), ("ckrho", C.c_double), ("rho", C.c_double), ("size", C.c_uint32),
                ("ntrim", C.c_uint32), ("ncktrim", C.c_uint64), ("mtrim", C.c_uint64),
                ("trimmed", C.POINTER(OrcEdge))]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        u32p, u64p, f64p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_double)
        G = C.POINTER(OrcGraph)
        sig = {
            "orc_sort_by_core": (None, [C.c_uint32, C.c_uint64, C.POINTER(OrcEdge), u32p]),
            "orc_make_graph": (G, [C.c_uint32, C.c_uint64, C.POINTER(OrcEdge), u32p]),
            "orc_free_graph": (None, [G]),
            "orc_count_edges": (C.c_uint32, [G, C.c_uint32, u32p]),
            "orc_count_cliques": (C.c_uint64, [G, C.c_int, u64p]),
            "orc_seq_pass": (C.c_int, [G, C.c_int, u64p, C.c_int, C.c_int]),
            "orc_seq_pass_sample": (C.c_uint64, [G, C.c_int, u64p, C.c_int, C.c_int, C.c_uint64]),
            "orc_seq_pava": (None, [G, C.c_int, u32p, u64p, C.c_int]),
            "orc_seq_find_densest": (OrcInfo, [G, C.c_int, C.c_uint32, u64p, u32p, u32p, C.c_int]),
            "orc_sort_by_r_u64": (None, [C.c_uint32, u64p, u32p]),
            "orc_sim_counts": (None, [G, C.c_int, f64p, u64p, C.c_int]),
            "orc_sim_counts_sample": (C.c_uint64, [G, C.c_int, f64p, u64p, C.c_int, C.c_uint64]),
            "orc_sim_update": (None, [C.c_uint32, C.c_uint32, f64p, u64p]),
            "orc_sim_pava": (None, [G, C.c_int, u32p, u64p, C.c_int]),
            "orc_sim_find_densest": (OrcInfo, [G, C.c_int, f64p, u32p, u32p, C.c_int]),
            "orc_sort_by_r_f64": (None, [C.c_uint32, f64p, u32p]),
            "orc_trim": (C.c_int, [C.c_uint32, C.c_uint64, C.POINTER(OrcEdge), C.c_int, C.POINTER(OrcTrim)]),
            "orc_free_trim": (None, [C.POINTER(OrcTrim)]),
            "orc_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                   C.POINTER(u32p), u64p, u32p]),
            "orc_free": (None, [C.c_void_p]),
            "orc_seq_main": (C.c_int, [G, C.c_int, C.c_uint32, C.c_int, C.c_int, u64p, C.POINTER(OrcInfo), C.c_int]),
            "orc_sim_main": (C.c_int, [G, C.c_int, C.c_uint32, C.c_int, f64p, C.POINTER(OrcInfo), C.c_int]),
            "orc_seq_pass_waves": (C.c_int, [G, C.c_int, u64p, C.c_uint32, C.c_int]),
            "orc_seq_delta_masked": (C.c_int, [G, C.c_int, u64p, C.POINTER(C.c_uint8), C.c_int, u64p]),
            "orc_sim_counts_masked": (None, [G, C.c_int, f64p, C.POINTER(C.c_uint8), C.c_int, u64p]),
            "orc_sample_key": (C.c_uint64, [C.c_uint64, C.c_uint32]),
            "orc_sampling_collect": (C.c_uint64, [G, C.c_int, C.c_uint64, C.c_uint64, C.c_int, C.c_uint32, u32p,
                                                  C.POINTER(C.c_uint8), C.c_uint64]),
            "orc_sampling_pass_order": (None, [C.c_int, C.c_uint64, u32p, u32p, u32p]),
            "orc_sampling_pass": (None, [C.c_uint32, C.c_int, C.c_uint64, u32p, C.POINTER(C.c_uint8), C.c_uint32,
                                         u32p]),
            "orc_sampling_extract": (OrcSamplingInfo, [C.c_uint32, C.c_int, C.c_uint64, u32p, u32p, C.c_uint32,
                                                       u32p]),
            "orc_wtime": (C.c_double, []),
            "orc_max_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _edges(pairs: np.ndarray):
    a = np.ascontiguousarray(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))
    return a, a.ctypes.data_as(C.POINTER(OrcEdge))


def n_of(pairs: np.ndarray) -> int:
    """ReadEdgeList's n: max id + 1 (1 for no edges)."""
    a = np.asarray(pairs, dtype=np.uint32)
    return int(a.max()) + 1 if a.size else 1


def sort_by_core(pairs: np.ndarray, n: int | None = None) -> np.ndarray:
    a, ep = _edges(pairs)
    n = n_of(a) if n is None else n
    rank = np.empty(n, dtype=np.uint32)
    lib().orc_sort_by_core(n, a.shape[0], ep, _p(rank, C.c_uint32))
    return rank


class Graph:
    """Oracle DAG built exactly as SortByCore + Relabel + MakeGraph."""

    def __init__(self, pairs: np.ndarray, n: int | None = None, rank: np.ndarray | None = None):
        a, ep = _edges(pairs)
        n = n_of(a) if n is None else n
        if rank is None:
            rank = sort_by_core(a, n)
        rank = np.ascontiguousarray(rank, dtype=np.uint32)
        self._g = lib().orc_make_graph(n, a.shape[0], ep, _p(rank, C.c_uint32))
        g = self._g.contents
        self.n, self.m, self.core = g.n, g.e, g.core

    @property
    def ptr(self):
        return self._g

    def csr(self):
        g = self._g.contents
        off = np.ctypeslib.as_array(g.cd, shape=(self.n + 1,)).copy() if self.n else np.zeros(1, np.uint64)
        cols = np.ctypeslib.as_array(g.adj, shape=(self.m,)).copy() if self.m else np.zeros(0, np.uint32)
        return off, cols

    def edges(self):
        g = self._g.contents
        if not self.m:
            return np.zeros((0, 2), np.uint32)
        return np.ctypeslib.as_array(C.cast(g.edges, C.POINTER(C.c_uint32)), shape=(self.m * 2,)).reshape(-1, 2).copy()

    def __del__(self):
        if getattr(self, "_g", None):
            lib().orc_free_graph(self._g)
            self._g = None

    # ---- passes ----
    def count_cliques(self, k: int):
        per = np.zeros(self.n + 1, dtype=np.uint64)
        tot = lib().orc_count_cliques(self._g, k, _p(per, C.c_uint64))
        return int(tot), per[: self.n]

    def seq_pass(self, k: int, r: np.ndarray, mode: int = SEQ_EDGE_STREAMS, threads: int = 1) -> np.ndarray:
        r = np.array(r, dtype=np.uint64, copy=True)
        if lib().orc_seq_pass(self._g, k, _p(r, C.c_uint64), mode, threads) != 0:
            raise ValueError("oracle seq pass: unsupported k")
        return r

    def seq_pass_sample(self, k: int, r: np.ndarray, mode: int, threads: int, stride: int) -> int:
        return int(lib().orc_seq_pass_sample(self._g, k, _p(r, C.c_uint64), mode, threads, stride))

    def sim_counts(self, k: int, rho: np.ndarray, threads: int = 1) -> np.ndarray:
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        cnt = np.zeros(self.n + 1, dtype=np.uint64)
        lib().orc_sim_counts(self._g, k, _p(rho, C.c_double), _p(cnt, C.c_uint64), threads)
        return cnt[: self.n]

    def sim_counts_sample(self, k: int, rho: np.ndarray, threads: int, stride: int) -> int:
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        cnt = np.zeros(self.n + 1, dtype=np.uint64)
        return int(lib().orc_sim_counts_sample(self._g, k, _p(rho, C.c_double), _p(cnt, C.c_uint64), threads, stride))

    def sim_pass(self, k: int, t: int, rho: np.ndarray, threads: int = 1) -> np.ndarray:
        rho = np.array(rho, dtype=np.float64, copy=True)
        cnt = self.sim_counts(k, rho, threads)
        cnt = np.ascontiguousarray(np.concatenate([cnt, [0]]).astype(np.uint64))
        lib().orc_sim_update(self.n, t, _p(rho, C.c_double), _p(cnt, C.c_uint64))
        return rho

    def pava(self, k: int, level: np.ndarray, threads: int = 1) -> np.ndarray:
        level = np.ascontiguousarray(level, dtype=np.uint32)
        tent = np.zeros(self.n + 1, dtype=np.uint64)
        lib().orc_seq_pava(self._g, k, _p(level, C.c_uint32), _p(tent, C.c_uint64), threads)
        return tent[: self.n]

    def seq_pass_waves(self, k: int, r: np.ndarray, waves: int, threads: int = 1) -> np.ndarray:
        r = np.array(r, dtype=np.uint64, copy=True)
        if lib().orc_seq_pass_waves(self._g, k, _p(r, C.c_uint64), waves, threads) != 0:
            raise ValueError("oracle: unsupported k")
        return r

    def seq_delta_masked(self, k: int, r: np.ndarray, mask: np.ndarray, threads: int = 1) -> np.ndarray:
        """Increments of one shard's root edges (EDGE_STREAMS order)."""
        r = np.ascontiguousarray(r, dtype=np.uint64)
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        d = np.zeros(self.n + 1, dtype=np.uint64)
        if lib().orc_seq_delta_masked(self._g, k, _p(r, C.c_uint64), _p(m, C.c_uint8), threads, _p(d, C.c_uint64)):
            raise ValueError("oracle: unsupported k")
        return d[: self.n]

    def sim_counts_masked(self, k: int, rho: np.ndarray, mask: np.ndarray, threads: int = 1) -> np.ndarray:
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        cnt = np.zeros(self.n + 1, dtype=np.uint64)
        lib().orc_sim_counts_masked(self._g, k, _p(rho, C.c_double), _p(m, C.c_uint8), threads, _p(cnt, C.c_uint64))
        return cnt[: self.n]

    def count_edges(self, nodes: np.ndarray) -> int:
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        return int(lib().orc_count_edges(self._g, len(nodes), _p(nodes, C.c_uint32)))

    def seq_find_densest(self, k: int, T: int, r: np.ndarray, threads: int = 1):
        r = np.ascontiguousarray(r, dtype=np.uint64)
        re = np.empty(max(self.n, 1), dtype=np.uint32)
        lv = np.empty(max(self.n, 1), dtype=np.uint32)
        info = lib().orc_seq_find_densest(self._g, k, T, _p(r, C.c_uint64), _p(re, C.c_uint32),
                                          _p(lv, C.c_uint32), threads)
        return info, re[: self.n]

    def sim_find_densest(self, k: int, rho: np.ndarray, threads: int = 1):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        re = np.empty(max(self.n, 1), dtype=np.uint32)
        lv = np.empty(max(self.n, 1), dtype=np.uint32)
        info = lib().orc_sim_find_densest(self._g, k, _p(rho, C.c_double), _p(re, C.c_uint32),
                                          _p(lv, C.c_uint32), threads)
        return info, re[: self.n]

    def seq_main(self, k: int, num_iter: int, mode: int = SEQ_EDGE_STREAMS, threads: int = 1):
        cap = 40
        infos = (OrcInfo * cap)()
        r = np.zeros(self.n + 1, dtype=np.uint64)
        c = lib().orc_seq_main(self._g, k, num_iter, mode, threads, _p(r, C.c_uint64), infos, cap)
        if c < 0:
            raise ValueError("oracle seq_main: unsupported k")
        return [infos[i] for i in range(min(c, cap))], r[: self.n]

    # ---- Seq-Sampling++ ----
    def sampling_collect(self, k: int, seed: int, threshold: int, all_: bool, waves: int):
        """Kept cliques in enumeration order: rows (S, k) of ascending ids, waves (S,)."""
        L = lib()
        kept = int(L.orc_sampling_collect(self._g, k, seed, threshold, int(all_), waves,
                                          C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint8)(), 0))
        rows = np.zeros((max(kept, 1), k), dtype=np.uint32)
        wave = np.zeros(max(kept, 1), dtype=np.uint8)
        got = int(L.orc_sampling_collect(self._g, k, seed, threshold, int(all_), waves, _p(rows, C.c_uint32),
                                         _p(wave, C.c_uint8), kept))
        assert got == kept
        return rows[:kept], wave[:kept]

    def sim_main(self, k: int, num_iter: int, threads: int = 1):
        cap = 40
        infos = (OrcInfo * cap)()
        rho = np.zeros(self.n + 1, dtype=np.float64)
        c = lib().orc_sim_main(self._g, k, num_iter, threads, _p(rho, C.c_double), infos, cap)
        if c < 0:
            raise ValueError("oracle sim_main: unsupported k")
        return [infos[i] for i in range(min(c, cap))], rho[: self.n]


def sort_by_r_u64(r: np.ndarray) -> np.ndarray:
    r = np.ascontiguousarray(r, dtype=np.uint64)
    re = np.empty(max(len(r), 1), dtype=np.uint32)
    lib().orc_sort_by_r_u64(len(r), _p(r, C.c_uint64), _p(re, C.c_uint32))
    return re[: len(r)]


def sort_by_r_f64(r: np.ndarray) -> np.ndarray:
    r = np.ascontiguousarray(r, dtype=np.float64)
    re = np.empty(max(len(r), 1), dtype=np.uint32)
    lib().orc_sort_by_r_f64(len(r), _p(r, C.c_double), _p(re, C.c_uint32))
    return re[: len(r)]


def trim(pairs: np.ndarray, k: int, n: int | None = None) -> dict:
    a, ep = _edges(pairs)
    n = n_of(a) if n is None else n
    res = OrcTrim()
    if lib().orc_trim(n, a.shape[0], ep, k, C.byref(res)) != 0:
        raise ValueError("oracle trim: unsupported k")
    n2 = res.n2

    def arr(ptr, cnt, dt):
        return np.ctypeslib.as_array(ptr, shape=(cnt,)).astype(dt, copy=True) if cnt else np.zeros(0, dt)

    out = {
        "n": res.n, "e": res.e, "n2": n2, "e2": res.e2, "core": res.core, "total": res.total,
        "ckcore": res.ckcore, "ckrho": res.ckrho, "rho": res.rho, "size": res.size, "ntrim": res.ntrim,
        "ncktrim": res.ncktrim, "mtrim": res.mtrim,
        "map": arr(res.map, n2, np.uint32), "nck": arr(res.nck, n2, np.uint64),
        "order": arr(res.order, n2, np.uint32), "core_num": arr(res.core_num, n2, np.uint64),
        "trimmed": (np.ctypeslib.as_array(C.cast(res.trimmed, C.POINTER(C.c_uint32)), shape=(res.mtrim * 2,))
                    .reshape(-1, 2).copy() if res.mtrim else np.zeros((0, 2), np.uint32)),
    }
    lib().orc_free_trim(C.byref(res))
    return out


def rmat(scale: int, edge_factor: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1) -> np.ndarray:
    """The library's seeded RMAT graph, restated (kclpp_oracle.h, orc_rmat):
    canonical (u < v) pairs, sorted and deduplicated, as an (e, 2) array."""
    P = C.POINTER(C.c_uint32)()
    e = C.c_uint64()
    n = C.c_uint32()
    if lib().orc_rmat(scale, edge_factor, a, b, c, seed, C.byref(P), C.byref(e), C.byref(n)) != 0:
        raise ValueError("oracle rmat: bad parameters")
    try:
        out = np.ctypeslib.as_array(P, shape=(2 * e.value,)).reshape(-1, 2).copy() if e.value else \
            np.zeros((0, 2), np.uint32)
    finally:
        lib().orc_free(P)
    return out


def wtime() -> float:
    return lib().orc_wtime()


def max_threads() -> int:
    return lib().orc_max_threads()


# ---- Seq-Sampling++ (kCDensestSamplingKclistpp.c) ----------------------------
def sampling_key(seed: int, v: int) -> int:
    return int(lib().orc_sample_key(seed, v))


def sampling_threshold(target: int, total: int):
    """(all, prob, threshold) as the library derives them from p = target / total
    (kCDensestSamplingKclistpp.c:272)."""
    import math
    if target >= total:
        return True, 1.0, 0
    prob = target / total
    return False, prob, int(math.ldexp(prob, 64))


def sampling_pass(n: int, k: int, rows: np.ndarray, wave: np.ndarray, waves: int, rho: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    wave = np.ascontiguousarray(wave, dtype=np.uint8)
    rho = np.array(rho, dtype=np.uint32, copy=True)
    rho = np.concatenate([rho, np.zeros(1, np.uint32)])
    lib().orc_sampling_pass(n, k, len(wave), _p(rows, C.c_uint32), _p(wave, C.c_uint8), waves, _p(rho, C.c_uint32))
    return rho[:n]


def sampling_pass_order(k: int, rows: np.ndarray, order: np.ndarray, rho: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    order = np.ascontiguousarray(order, dtype=np.uint32)
    rho = np.array(rho, dtype=np.uint32, copy=True)
    lib().orc_sampling_pass_order(k, len(order), _p(rows, C.c_uint32), _p(order, C.c_uint32), _p(rho, C.c_uint32))
    return rho


def sampling_extract(n: int, k: int, rows: np.ndarray, rho: np.ndarray, T: int):
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    rho = np.ascontiguousarray(rho, dtype=np.uint32)
    ordered = np.zeros(max(n, 1), dtype=np.uint32)
    info = lib().orc_sampling_extract(n, k, rows.shape[0], _p(rows, C.c_uint32), _p(rho, C.c_uint32), T,
                                      _p(ordered, C.c_uint32))
    return info, ordered[:n]


def sampling_report(g: Graph, k: int, rows: np.ndarray, rho: np.ndarray, T: int, prob: float) -> dict:
    """One report line of Solve (kCDensestSamplingKclistpp.c:460-478): the
    densest prefix of the loads, the exact count in its induced subgraph
    (MakeDensestSubgraphEdgeList, :420-435, then SortByCore, Relabel, MakeGraph
    and the COUNT_IN_SUBGRAPH task) and the figures of the printed line."""
    import math
    info, ordered = sampling_extract(g.n, k, rows, rho, T)
    rank = np.empty(g.n, dtype=np.int64)
    rank[ordered] = np.arange(g.n)
    E = g.edges().astype(np.int64)
    keep = (rank[E[:, 0]] < info.n) & (rank[E[:, 1]] < info.n) if len(E) else np.zeros(0, bool)
    sub = np.stack([rank[E[keep, 0]], rank[E[keep, 1]]], axis=1).astype(np.uint32) if keep.any() else None
    if sub is None:
        sub_n, sub_e, sub_core, cliques = 0, 0, 0, 0
    else:
        sg = Graph(sub, n=info.n)
        sub_n, sub_e, sub_core = sg.n, sg.m, sg.core
        cliques = sg.count_cliques(k)[0]
    with np.errstate(all="ignore"):
        edge_density = float(np.float64(sub_e) * 2.0 / np.float64(sub_n) / np.float64((sub_n - 1) & 0xFFFFFFFF))
        clique_density = float(np.float64(cliques) / np.float64(sub_n))
        ub = np.float64(info.ub)
        upper = float(ub / np.float64(prob) / (1 - np.sqrt(6 * np.float64(math.log(g.n)) / ub)))
    return {"T": T, "n": info.n, "m": info.m, "density": info.density, "ub": info.ub, "sub_n": sub_n,
            "sub_e": sub_e, "sub_core": sub_core, "sub_cliques": cliques, "edge_density": edge_density,
            "clique_density": clique_density, "upper_bound": upper, "order": ordered}


def sampling_main(g: Graph, k: int, num_iter: int, target: int, seed: int, waves: int):
    """Solve (:446-489) with the library's sample and wave passes: one report per power of two."""
    total = g.count_cliques(k)[0]
    all_, prob, thr = sampling_threshold(target, total)
    rows, wave = g.sampling_collect(k, seed, thr, all_, waves)
    rho = np.zeros(g.n, dtype=np.uint32)
    reps, done, T = [], 0, 1
    while T <= num_iter:
        for _ in range(T - done):
            rho = sampling_pass(g.n, k, rows, wave, waves, rho)
        done = T
        reps.append(sampling_report(g, k, rows, rho, T, prob))
        T <<= 1
    return {"total": total, "prob": prob, "threshold": thr, "all": all_, "rows": rows, "wave": wave,
            "rho": rho, "reports": reps}
