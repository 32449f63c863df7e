"""How the pass ordering of Seq-kClist++ sets the number of passes to a
certified density gap -- the study behind the ordering tables of the design
notes.  CPU only, on the oracle (oracle/kclpp_oracle.c, pinned to the
reference) and the orderings of oracle/ordering_study.c.

TEST INFRASTRUCTURE ONLY: an analysis script, not part of the library.

    python oracle/ordering_study.py            # all three tables (about 6 minutes on 8 cores)
    python oracle/ordering_study.py --table b  # the shared-load simulation on a small graph only

Table A (k = 5, RMAT scale 13 with 4 planted G(n_c, 0.5) communities): the
reference's sequential order, the library's per-root-edge streams and waves,
the reference's own 8-thread schedule, per-root-vertex streams, root-order
waves, a sequential dense core with parallel streams elsewhere, and streams
started from extrapolated loads.

Table B (k = 4, RMAT scale 11 with 2 planted communities): P streams in lock
step, each clique giving its unit to its member of smallest load (ties to the
earlier member in (s, t, ...) order) against the loads every earlier step
left -- the ordering a GPU pass gets when its warps read and add to one
shared load vector instead of private copies.  "chunked" reads the shared
loads once per 32 cliques of a stream (the stream sees only its own
increments inside a chunk).  The same number of cliques per pass; every
clique still gives one unit to one member, so r / T stays a feasible load
and the bound a certificate.

Table C: the shared-load simulation of table B, in C, on the graph of table
A (1e8 cliques per pass), up to a GB300's 7,296 resident warps as streams.
"""
from __future__ import annotations

import argparse
import ctypes as C
import heapq
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, this folder would shadow the `oracle` package with oracle.py
sys.path = [os.path.dirname(HERE)] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]

import kclistpp_gb300 as K  # noqa: E402  (generators and the core order only: host code)
from oracle import oracle as O  # noqa: E402

GAP = 0.01


def study_lib() -> C.CDLL:
    subprocess.run(["make", "-s", "-C", HERE, "study"], check=True)
    L = C.CDLL(os.path.join(HERE, "_build", "libordering_study.so"))
    G = C.POINTER(O.OrcGraph)
    u32p, u64p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)
    sig = {
        "orc_make_graph": (G, [C.c_uint32, C.c_uint64, C.POINTER(O.OrcEdge), u32p]),
        "orc_seq_pass": (C.c_int, [G, C.c_int, u64p, C.c_int, C.c_int]),
        "orc_seq_pass_waves": (C.c_int, [G, C.c_int, u64p, C.c_uint32, C.c_int]),
        "orc_seq_pass_extrap": (None, [G, C.c_int, u64p, u64p, C.c_double, C.c_int]),
        "orc_seq_pass_rootwaves": (None, [G, C.c_int, u64p]),
        "orc_seq_pass_hybrid": (None, [G, C.c_int, u64p, C.c_uint32, C.c_int]),
        "orc_seq_find_densest": (O.OrcInfo, [G, C.c_int, C.c_uint32, u64p, u32p, u32p, C.c_int]),
        "orc_list_cliques": (C.c_uint64, [G, C.c_int, u32p, C.c_uint64, u64p]),
        "orc_sim_shared_pass": (None, [C.c_int, u32p, u64p, u32p, u64p, C.c_uint32, C.c_uint32, u64p, C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    return L


class Study:
    def __init__(self, L, el, k):
        self.L, self.k = L, k
        P = np.ascontiguousarray(el.pairs().astype(np.uint32))
        rank = np.ascontiguousarray(K.core_order(el), dtype=np.uint32)
        self.g = L.orc_make_graph(el.n, P.shape[0], P.ctypes.data_as(C.POINTER(O.OrcEdge)),
                                  rank.ctypes.data_as(C.POINTER(C.c_uint32)))
        self.n, self.e = self.g.contents.n, self.g.contents.e

    def gap(self, r, T) -> float:
        rr = np.ascontiguousarray(np.concatenate([np.asarray(r, np.int64), [0]]).astype(np.uint64))
        re = np.empty(max(self.n, 1), np.uint32)
        lv = np.empty(max(self.n, 1), np.uint32)
        info = self.L.orc_seq_find_densest(self.g, self.k, T, rr.ctypes.data_as(C.POINTER(C.c_uint64)),
                                           re.ctypes.data_as(C.POINTER(C.c_uint32)),
                                           lv.ctypes.data_as(C.POINTER(C.c_uint32)), 8)
        return info.ub / info.density - 1

    def passes(self, step, max_passes) -> str:
        """Passes until the certified gap is at most GAP; step(r, T) runs pass T in place."""
        r = np.zeros(self.n + 1, np.uint64)
        for T in range(1, max_passes + 1):
            step(r, T)
            gp = self.gap(r[: self.n], T)
            if gp <= GAP:
                return str(T)
        return f"> {max_passes} (gap {100 * gp:.2f} %)"

    def ptr(self, r):
        return r.ctypes.data_as(C.POINTER(C.c_uint64))


def list_cliques(L, S):
    cnt = L.orc_list_cliques(S.g, S.k, None, 0, None)
    cl = np.zeros((cnt, S.k), np.uint32)
    ef = np.zeros(S.e + 1, np.uint64)
    L.orc_list_cliques(S.g, S.k, cl.ctypes.data_as(C.POINTER(C.c_uint32)), cnt,
                       ef.ctypes.data_as(C.POINTER(C.c_uint64)))
    return cl, ef


def stream_schedule(ef, e, P, by_work=False):
    """Root edges in (s, t) order -- or by decreasing clique count, the order
    the kernels take roots in -- each to the stream that frees first (a GPU's
    dynamic schedule), as CSR: stream_first[P + 1], stream_edges."""
    sizes = np.diff(ef).astype(np.int64)
    heap = [(0, j) for j in range(P)]
    lists = [[] for _ in range(P)]
    order = np.argsort(-sizes, kind="stable") if by_work else range(e)
    for i in order:
        i = int(i)
        if sizes[i] == 0:
            continue
        t, j = heapq.heappop(heap)
        lists[j].append(i)
        heapq.heappush(heap, (t + int(sizes[i]), j))
    first = np.zeros(P + 1, np.uint64)
    first[1:] = np.cumsum([len(x) for x in lists])
    edges = np.array([i for x in lists for i in x], dtype=np.uint32)
    return edges, first


def shared_step(L, S, cl, ef, P, chunk, by_work=False):
    edges, first = stream_schedule(ef, S.e, P, by_work)
    edges = edges if len(edges) else np.zeros(1, np.uint32)

    def step(r, T):
        L.orc_sim_shared_pass(S.k, cl.ctypes.data_as(C.POINTER(C.c_uint32)),
                              ef.ctypes.data_as(C.POINTER(C.c_uint64)),
                              edges.ctypes.data_as(C.POINTER(C.c_uint32)),
                              first.ctypes.data_as(C.POINTER(C.c_uint64)), P, chunk, S.ptr(r), 8)

    return step


def table_a(L) -> None:
    el = K.rmat_planted(13, 16, 4, 60, 150, 0.5, seed=79)
    S = Study(L, el, 5)
    print(f"Table A: k = 5, {S.n} vertices, {S.e} root edges")
    rows = [
        ("sequential (the reference at p = 1)", lambda r, T: L.orc_seq_pass(S.g, 5, S.ptr(r), O.SEQ_SEQUENTIAL, 1)),
        ("per-root-edge streams", lambda r, T: L.orc_seq_pass(S.g, 5, S.ptr(r), O.SEQ_EDGE_STREAMS, 8)),
    ]
    for W in (4, 16, 64):
        rows.append((f"waves, W = {W}", lambda r, T, W=W: L.orc_seq_pass_waves(S.g, 5, S.ptr(r), W, 8)))
    rows += [
        ("the reference's 8-thread schedule", lambda r, T: L.orc_seq_pass(S.g, 5, S.ptr(r), O.SEQ_THREADS, 8)),
        ("per-root-vertex streams", lambda r, T: L.orc_seq_pass(S.g, 5, S.ptr(r), O.SEQ_VERTEX_STREAMS, 8)),
        ("every root its own wave, in root order", lambda r, T: L.orc_seq_pass_rootwaves(S.g, 5, S.ptr(r))),
    ]
    for cut in (100, 300, 600):
        rows.append((f"roots below {cut} in one sequential chain, the rest streams",
                     lambda r, T, cut=cut: L.orc_seq_pass_hybrid(S.g, 5, S.ptr(r), cut, 8)))
    prev = {"d": np.zeros(S.n + 1, np.uint64)}

    def extrap(r, T):
        before = r.copy()
        if T == 1:
            L.orc_seq_pass(S.g, 5, S.ptr(r), O.SEQ_EDGE_STREAMS, 8)
        else:
            d = np.ascontiguousarray(prev["d"])
            L.orc_seq_pass_extrap(S.g, 5, S.ptr(r), d.ctypes.data_as(C.POINTER(C.c_uint64)), 1.0, 8)
        prev["d"] = r - before

    rows.append(("streams from extrapolated loads", extrap))
    for name, step in rows:
        t0 = time.time()
        print(f"  {name:62s} {S.passes(step, 200):>24s}   ({time.time() - t0:.0f} s)", flush=True)


def table_b(L) -> None:
    el = K.rmat_planted(11, 16, 2, 40, 100, 0.5, seed=7)
    k = 4
    S = Study(L, el, k)
    cnt = L.orc_list_cliques(S.g, k, None, 0, None)
    cl = np.zeros((cnt, k), np.uint32)
    ef = np.zeros(S.e + 1, np.uint64)
    L.orc_list_cliques(S.g, k, cl.ctypes.data_as(C.POINTER(C.c_uint32)), cnt,
                       ef.ctypes.data_as(C.POINTER(C.c_uint64)))
    sizes = np.diff(ef).astype(np.int64)
    print(f"Table B: k = {k}, {S.n} vertices, {S.e} root edges, {cnt} cliques per pass")

    def schedule(P):
        """Root edges in order, each to the stream that frees first (a GPU's dynamic schedule)."""
        heap = [(0, j) for j in range(P)]
        seqs = [[] for _ in range(P)]
        for i in range(S.e):
            if sizes[i] == 0:
                continue
            t, j = heapq.heappop(heap)
            seqs[j].append(np.arange(ef[i], ef[i + 1], dtype=np.int64))
            heapq.heappush(heap, (t + int(sizes[i]), j))
        seqs = [np.concatenate(s) if s else np.zeros(0, np.int64) for s in seqs]
        M = np.full((P, max(len(s) for s in seqs)), -1, np.int64)
        for j, s in enumerate(seqs):
            M[j, : len(s)] = s
        return M

    def lockstep(P, chunk):
        M = schedule(P)
        streams = np.arange(P)

        def step(r, T):
            loads = r[: S.n].astype(np.int64)
            for c0 in range(0, M.shape[1], chunk):
                D = np.zeros((P, S.n), np.int64) if chunk > 1 else None
                for c in range(c0, min(c0 + chunk, M.shape[1])):
                    idx = M[:, c]
                    act = idx >= 0
                    if not act.any():
                        continue
                    mem = cl[idx[act]]
                    if D is None:
                        vals = loads[mem]
                    else:
                        j = streams[act]
                        vals = loads[mem] + D[j[:, None], mem]
                    ch = mem[np.arange(len(mem)), np.argmin(vals, axis=1)]
                    if D is None:
                        np.add.at(loads, ch, 1)
                    else:
                        np.add.at(D, (streams[act], ch), 1)
                if D is not None:
                    loads += D.sum(0)
            r[: S.n] = loads.astype(np.uint64)

        return step

    rows = [
        ("sequential (the reference at p = 1)", lambda r, T: L.orc_seq_pass(S.g, k, S.ptr(r), O.SEQ_SEQUENTIAL, 1)),
        ("per-root-edge streams", lambda r, T: L.orc_seq_pass(S.g, k, S.ptr(r), O.SEQ_EDGE_STREAMS, 8)),
    ]
    for P in (16, 256, 4096):
        rows.append((f"{P} streams in lock step, shared loads", lockstep(P, 1)))
    for P in (256, 1024, 4096):
        rows.append((f"{P} streams, shared loads read every 32 cliques", lockstep(P, 32)))
    rows.append(("256 streams, every 32 cliques (the C simulation of table C)",
                 shared_step(L, S, cl, ef, 256, 32)))
    for name, step in rows:
        t0 = time.time()
        print(f"  {name:62s} {S.passes(step, 300):>24s}   ({time.time() - t0:.0f} s)", flush=True)


def table_c(L) -> None:
    """Shared loads at a larger scale: the graph of table A (1.0e8 5-cliques per
    pass), with up to a GB300's resident warps (152 SMs x 48) as streams."""
    el = K.rmat_planted(13, 16, 4, 60, 150, 0.5, seed=79)
    S = Study(L, el, 5)
    cl, ef = list_cliques(L, S)
    print(f"Table C: k = 5, {S.n} vertices, {S.e} root edges, {len(cl)} cliques per pass")
    for P, by_work in ((1024, False), (7296, False), (32768, False), (7296, True)):
        t0 = time.time()
        res = S.passes(shared_step(L, S, cl, ef, P, 32, by_work), 200)
        order = "by decreasing work" if by_work else "in (s, t) order"
        print(f"  {P:6d} streams, shared loads every 32 cliques, root edges {order:18s} {res:>8s}"
              f"   ({time.time() - t0:.0f} s)", flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--table", choices=["a", "b", "c", "all"], default="all")
    a = ap.parse_args()
    L = study_lib()
    print(f"passes to a certified {100 * GAP:.0f} % gap (ub / density - 1)")
    if a.table in ("a", "all"):
        table_a(L)
    if a.table in ("b", "all"):
        table_b(L)
    if a.table in ("c", "all"):
        table_c(L)


if __name__ == "__main__":
    main()
