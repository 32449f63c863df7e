"""GB300-native KClist++: k-clique listing fused with the "++" updates.

Python binding of the C ABI in include/kclpp.h (libkclpp.so, built in-tree by
kclistpp_gb300.build).  The functions mirror the reference programs' C
functions (btsun/kclistpp):

    read_edge_list      ReadEdgeList            Graph.c:34-53
    core_order          SortByCore              Graph.c:57-91
    build_graph         SortByCore+Relabel+MakeGraph  Graph.c:57-156
    count_cliques       onepass (k-clique degrees)    kClistCoreTrim.c:394-416
    seq_passes          CDF_CliqueEnum(FRANK_WOLFE)   kCDensestNoAtom.c:270-295
    sim_counts          CDF_CliqueEnum(FRANK_WOLFE)   kCDensestCmpSync.c:298-325
    sim_passes          + rho update                  kCDensestCmpSync.c:396-404
    sort_by_r_*         CDF_NodeCmp + qsort           kCDensestNoAtom.c:322-337
    pava                CDF_CliqueEnum(PAVA_PREPROCESS) kCDensestNoAtom.c:296-309
    extract_densest_*   CDF_FindDensestSubset         kCDensestNoAtom.c:330-371
    seq_main/sim_main   CDF_Main                      kCDensestNoAtom.c:373-402
    trim                kClistCoreTrim main           kClistCoreTrim.c:707-775
    Sampling            SampleCliques / InMemoryFrankWolfe / ExtractDensest
                                                  kCDensestSamplingKclistpp.c:345-444
    sampling_main       Solve                         kCDensestSamplingKclistpp.c:446-489

Every call runs through the CUDA library; there is no CPU fallback.  If the
library has not been built (or cannot be loaded) the import fails.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libkclpp.so")

OK = 0
ERR_INVALID, ERR_IO, ERR_NOMEM, ERR_CUDA, ERR_UNSUPPORTED, ERR_OVERFLOW, ERR_NODEVICE = 1, 2, 3, 4, 5, 6, 7
MAX_K = 8
SEQ_EDGE_STREAMS = 1
SEQ_WAVES = 2
SEQ_SHARED = 3  # shared load vector, not deterministic (invariants only)
TRIM_EXACT, TRIM_FAST, TRIM_EXACT_HOST = 0, 1, 2
ORDER_EXACT, ORDER_FAST = 0, 1
SAMPLE_TARGET = 10_000_000  # the reference's CLIQUES_TO_SAMPLE
GEN_CHUNG_LU, GEN_RMAT, GEN_ER, GEN_PLANTED, GEN_RMAT_PLANTED = 1, 2, 3, 4, 5


class KclppError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"kclpp status {status}: {msg}")
        self.status = status


class DensestInfo(C.Structure):
    _fields_ = [("n", C.c_uint32), ("m", C.c_uint32), ("cliques", C.c_uint64),
                ("density", C.c_double), ("ub", C.c_double)]

    def as_tuple(self):
        return (self.n, self.m, self.cliques, self.density, self.ub)

    def __repr__(self):
        return (f"DensestInfo(n={self.n}, m={self.m}, cliques={self.cliques}, "
                f"density={self.density!r}, ub={self.ub!r})")


class TrimInfo(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n2", C.c_uint32), ("e", C.c_uint64), ("e2", C.c_uint64),
                ("core", C.c_uint32), ("total", C.c_uint64), ("ckcore", C.c_uint64),
                ("ckrho", C.c_double), ("rho", C.c_double), ("size", C.c_uint32),
                ("ntrim", C.c_uint32), ("mtrim", C.c_uint64), ("ncktrim", C.c_uint64)]


class PeelStats(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("predicted", C.c_uint64), ("committed", C.c_uint64),
                ("gpu_roots", C.c_uint64), ("host_roots", C.c_uint64), ("seconds", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class CertifyInfo(C.Structure):
    _fields_ = [("n", C.c_uint32), ("cliques", C.c_uint64), ("density", C.c_double), ("inside", C.c_int),
                ("inside_method", C.c_int), ("outside", C.c_int), ("certified", C.c_int),
                ("passes_inside", C.c_uint32),
                ("passes_outside", C.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class StateInfo(C.Structure):
    _fields_ = [("kind", C.c_int), ("k", C.c_int), ("passes", C.c_uint32), ("n", C.c_uint32),
                ("graph_hash", C.c_uint64)]


class ExactInfo(C.Structure):
    _fields_ = [("num", C.c_uint64), ("den", C.c_uint64), ("density", C.c_double), ("size", C.c_uint32),
                ("cliques", C.c_uint64), ("cliques_total", C.c_uint64), ("iterations", C.c_int)]


class SamplingInfo(C.Structure):
    _fields_ = [("cliques_total", C.c_uint64), ("sampled", C.c_uint64), ("prob", C.c_double),
                ("threshold", C.c_uint64), ("all", C.c_int), ("waves", C.c_uint32), ("passes", C.c_uint32)]


class SamplingReport(C.Structure):
    _fields_ = [("T", C.c_uint32), ("n", C.c_uint32), ("m", C.c_uint64), ("density", C.c_double),
                ("ub", C.c_double), ("sub_n", C.c_uint32), ("sub_e", C.c_uint64), ("sub_core", C.c_uint32),
                ("sub_cliques", C.c_uint64), ("edge_density", C.c_double), ("clique_density", C.c_double),
                ("upper_bound", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class KernelTime(C.Structure):
    _fields_ = [("mode", C.c_int), ("tier", C.c_int), ("dmax", C.c_uint32), ("launches", C.c_uint32),
                ("ms", C.c_double)]


KERNEL_NAMES = {0: "count", 1: "order", 2: "seq"}
TIER_NAMES = {0: "S", 1: "M", 2: "L"}


class Schedule(C.Structure):
    _fields_ = [("tier_s_max", C.c_uint32), ("tier_s_max_seq", C.c_uint32), ("m_split1", C.c_uint32),
                ("m_split2", C.c_uint32), ("steal_seq", C.c_int), ("steal_count", C.c_int),
                ("seq_waves", C.c_uint32), ("seq_warps", C.c_uint32 * 4),
                ("concurrent_tiers", C.c_int), ("count_warps", C.c_uint32 * 4),
                ("seq_split1", C.c_uint32), ("seq_split2", C.c_uint32), ("concurrent_count", C.c_int)]

    def __init__(self, **kw):
        arr = {f: t for f, t in self._fields_ if issubclass(t, C.Array)}
        super().__init__(**{f: (arr[f](*v) if f in arr and not isinstance(v, C.Array) else v) for f, v in kw.items()})

    def as_dict(self):
        return {f: (list(getattr(self, f)) if issubclass(t, C.Array) else getattr(self, f)) for f, t in self._fields_}


class TuneResult(C.Structure):
    _fields_ = [("best", Schedule), ("best_ms", C.c_double), ("default_ms", C.c_double), ("candidates", C.c_int)]


KERNEL_COUNT, KERNEL_ORDER, KERNEL_SEQ = 0, 1, 2


class GenParams(C.Structure):
    _fields_ = [("kind", C.c_int), ("n", C.c_uint32), ("avg_degree", C.c_double),
                ("gamma", C.c_double), ("scale", C.c_uint32), ("edge_factor", C.c_uint32),
                ("a", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("communities", C.c_uint32), ("comm_min", C.c_uint32), ("comm_max", C.c_uint32),
                ("p_in", C.c_double), ("seed", C.c_uint64)]


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python kclistpp_gb300/build.py`")
    return C.CDLL(LIB_PATH)


_lib = _load()

_P = C.c_void_p
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_f64p = C.POINTER(C.c_double)

_SIGS = {
    "kclpp_status_string": (C.c_char_p, [C.c_int]),
    "kclpp_last_error": (C.c_char_p, []),
    "kclpp_version": (C.c_char_p, []),
    "kclpp_create": (C.c_int, [C.c_int, _P, C.POINTER(_P)]),
    "kclpp_destroy": (C.c_int, [_P]),
    "kclpp_synchronize": (C.c_int, [_P]),
    "kclpp_launch_count": (C.c_uint64, [_P]),
    "kclpp_profile_enable": (C.c_int, [_P, C.c_int]),
    "kclpp_profile_read": (C.c_int, [_P, C.POINTER(KernelTime), C.c_int, C.POINTER(C.c_int)]),
    "kclpp_read_edge_list": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "kclpp_read_edge_list_mt": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
    "kclpp_write_edge_list_bin": (C.c_int, [_P, C.c_char_p]),
    "kclpp_read_edge_list_bin": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "kclpp_edge_list_create": (C.c_int, [_u32p, C.c_uint64, C.POINTER(_P)]),
    "kclpp_edge_list_info": (C.c_int, [_P, _u32p, _u64p]),
    "kclpp_edge_list_copy": (C.c_int, [_P, _u32p]),
    "kclpp_write_edge_list": (C.c_int, [_P, C.c_char_p]),
    "kclpp_densest_exact": (C.c_int, [_P, C.c_int, _P, _P]),
    "kclpp_save_state": (C.c_int, [C.c_char_p, _P, _P]),
    "kclpp_load_state": (C.c_int, [C.c_char_p, _P, _P, C.c_uint32]),
    "kclpp_edge_list_hash": (C.c_int, [_P, _u64p]),
    "kclpp_edge_list_free": (None, [_P]),
    "kclpp_generate": (C.c_int, [C.POINTER(GenParams), C.POINTER(_P)]),
    "kclpp_core_order": (C.c_int, [_P, _u32p]),
    "kclpp_make_graph": (C.c_int, [_P, _P, _u32p, C.POINTER(_P)]),
    "kclpp_build_graph": (C.c_int, [_P, _P, C.POINTER(_P)]),
    "kclpp_core_order_mode": (C.c_int, [_P, C.c_int, _u32p]),
    "kclpp_build_graph_mode": (C.c_int, [_P, _P, C.c_int, C.POINTER(_P)]),
    "kclpp_graph_from_csr": (C.c_int, [_P, C.c_uint32, C.c_uint64, _u64p, _u32p, C.POINTER(_P)]),
    "kclpp_graph_info": (C.c_int, [_P, _u32p, _u64p, _u32p]),
    "kclpp_graph_copy_csr": (C.c_int, [_P, _u64p, _u32p]),
    "kclpp_graph_free": (None, [_P]),
    "kclpp_count_edges": (C.c_int, [_P, _P, C.c_uint32, _u32p, _u32p]),
    "kclpp_count_cliques": (C.c_int, [_P, _P, C.c_int, _u64p, _u64p]),
    "kclpp_graph_get_schedule": (C.c_int, [_P, C.POINTER(Schedule)]),
    "kclpp_graph_set_schedule": (C.c_int, [_P, _P, C.POINTER(Schedule)]),
    "kclpp_autotune": (C.c_int, [_P, _P, C.c_int, C.c_int, C.POINTER(TuneResult)]),
    "kclpp_schedule_save": (C.c_int, [C.c_char_p, C.c_uint64, C.c_int, C.c_int, C.POINTER(Schedule)]),
    "kclpp_schedule_load": (C.c_int, [C.c_char_p, C.c_uint64, C.c_int, C.c_int, C.POINTER(Schedule)]),
    "kclpp_batch_create": (C.c_int, [_P, C.POINTER(_P), C.c_uint32, C.POINTER(_P)]),
    "kclpp_batch_info": (C.c_int, [_P, _u32p, _u32p, _u64p, C.POINTER(_P)]),
    "kclpp_batch_vertex_offsets": (C.c_int, [_P, _u32p]),
    "kclpp_batch_run": (C.c_int, [_P, _P, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_uint32, _P]),
    "kclpp_batch_free": (None, [_P]),
    "kclpp_count_cliques_noalloc": (C.c_int, [_P, C.c_uint32, C.c_uint64, _P, _P, C.c_int, _P, _u64p]),
    "kclpp_seq_passes": (C.c_int, [_P, _P, C.c_int, C.c_uint32, C.c_int, _u64p]),
    "kclpp_seq_passes_dev": (C.c_int, [_P, _P, C.c_int, C.c_uint32, C.c_int, _P]),
    "kclpp_seq_passes_csr": (C.c_int, [_P, C.c_uint32, C.c_uint64, _u64p, _u32p, C.c_int, C.c_uint32,
                                       C.c_int, _u64p]),
    "kclpp_sim_counts": (C.c_int, [_P, _P, C.c_int, _f64p, _u64p]),
    "kclpp_sim_passes": (C.c_int, [_P, _P, C.c_int, C.c_uint32, C.c_uint32, _f64p]),
    "kclpp_sim_passes_dev": (C.c_int, [_P, _P, C.c_int, C.c_uint32, C.c_uint32, _P]),
    "kclpp_sim_passes_csr": (C.c_int, [_P, C.c_uint32, C.c_uint64, _u64p, _u32p, C.c_int, C.c_uint32,
                                       C.c_uint32, _f64p]),
    "kclpp_shard_plan": (C.c_int, [C.c_uint32, _u64p, C.c_uint32, _u32p]),
    "kclpp_graph_shard": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32]),
    "kclpp_seq_delta_dev": (C.c_int, [_P, _P, C.c_int, _P, _P]),
    "kclpp_sim_counts_dev": (C.c_int, [_P, _P, C.c_int, _P, _P]),
    "kclpp_sim_update_dev": (C.c_int, [_P, C.c_uint32, C.c_uint32, _P, _P]),
    "kclpp_sort_by_r_u64": (C.c_int, [_P, C.c_uint32, _u64p, _u32p, _u32p]),
    "kclpp_sort_by_r_f64": (C.c_int, [_P, C.c_uint32, _f64p, _u32p, _u32p]),
    "kclpp_pava": (C.c_int, [_P, _P, C.c_int, _u32p, _u64p]),
    "kclpp_extract_densest_seq": (C.c_int, [_P, _P, C.c_int, C.c_uint32, _u64p, C.POINTER(DensestInfo), _u32p]),
    "kclpp_extract_densest_sim": (C.c_int, [_P, _P, C.c_int, _f64p, C.POINTER(DensestInfo), _u32p]),
    "kclpp_seq_main": (C.c_int, [_P, _P, C.c_int, C.c_uint32, C.c_int, _u64p, C.POINTER(DensestInfo),
                                 C.c_int, C.POINTER(C.c_int)]),
    "kclpp_sim_main": (C.c_int, [_P, _P, C.c_int, C.c_uint32, _f64p, C.POINTER(DensestInfo), C.c_int,
                                 C.POINTER(C.c_int)]),
    "kclpp_warm_create": (C.c_int, [_P, C.c_uint64, C.POINTER(_P)]),
    "kclpp_warm_free": (None, [_P]),
    "kclpp_warm_get_params": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "kclpp_warm_set_params": (C.c_int, [_P, _P, C.POINTER(C.c_float)]),
    "kclpp_warm_features": (C.c_int, [_P, _P, _P]),
    "kclpp_warm_features_dev": (C.c_int, [_P, C.c_uint32, _P, _P, _P, _P, _P]),
    "kclpp_warm_predict_dev": (C.c_int, [_P, _P, _P, C.c_uint32, _P]),
    "kclpp_warm_grad_dev": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "kclpp_warm_train": (C.c_int, [_P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_float, C.POINTER(C.c_float)]),
    "kclpp_warm_r0_dev": (C.c_int, [_P, _P, C.c_uint32, C.c_float, _P]),
    "kclpp_warm_start_r": (C.c_int, [_P, _P, _P, C.c_float, _P]),
    "kclpp_extract_densest_seq_warm": (C.c_int, [_P, _P, C.c_int, C.c_uint32, _u64p, _u64p, C.POINTER(DensestInfo)]),
    "kclpp_trim": (C.c_int, [_P, _P, C.c_int, C.c_int, C.POINTER(_P)]),
    "kclpp_trim_info_get": (C.c_int, [_P, C.POINTER(TrimInfo)]),
    "kclpp_trim_copy": (C.c_int, [_P, _u32p, _u64p, _u32p, _u64p]),
    "kclpp_trim_edges": (C.c_int, [_P, C.POINTER(_P)]),
    "kclpp_trim_peel_stats": (C.c_int, [_P, C.POINTER(PeelStats)]),
    "kclpp_certify_densest": (C.c_int, [_P, _P, C.c_int, _u64p, C.c_uint32, C.POINTER(CertifyInfo), _u32p]),
    "kclpp_trim_free": (None, [_P]),
    "kclpp_sampling_create": (C.c_int, [_P, _P, C.c_int, C.c_uint64, C.c_uint64, C.c_uint32, C.POINTER(_P)]),
    "kclpp_sampling_info_get": (C.c_int, [_P, C.POINTER(SamplingInfo)]),
    "kclpp_sampling_cliques": (C.c_int, [_P, _P, _u32p, C.POINTER(C.c_uint8)]),
    "kclpp_sampling_passes": (C.c_int, [_P, _P, C.c_uint32]),
    "kclpp_sampling_get_rho": (C.c_int, [_P, _P, _u32p]),
    "kclpp_sampling_set_rho": (C.c_int, [_P, _P, _u32p, C.c_uint32]),
    "kclpp_sampling_extract": (C.c_int, [_P, _P, C.c_uint32, C.POINTER(SamplingReport), _u32p]),
    "kclpp_sampling_free": (None, [_P]),
    "kclpp_sampling_main": (C.c_int, [_P, _P, C.c_int, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint32,
                                      C.POINTER(SamplingReport), C.c_int, C.POINTER(C.c_int)]),
}
for _name, (_res, _args) in _SIGS.items():
    _f = getattr(_lib, _name)
    _f.restype = _res
    _f.argtypes = _args

#: Every function the header declares (checked by the tests).
EXPORTED = tuple(_SIGS)


def _check(status: int) -> None:
    if status != OK:
        raise KclppError(status, _lib.kclpp_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def version() -> str:
    return _lib.kclpp_version().decode()


class Context:
    """One device and one CUDA stream (the caller's, if `stream` is given)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        h = _P()
        _check(_lib.kclpp_create(device, _P(stream) if stream else None, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def synchronize(self) -> None:
        _check(_lib.kclpp_synchronize(self._h))

    def launches(self) -> int:
        return int(_lib.kclpp_launch_count(self._h))

    def profile(self, on: bool = True) -> None:
        _check(_lib.kclpp_profile_enable(self._h, int(on)))

    def profile_read(self) -> list[dict]:
        """Per-(kernel, tier) launches and summed event time since the last read."""
        cap = 64
        buf = (KernelTime * cap)()
        cnt = C.c_int()
        _check(_lib.kclpp_profile_read(self._h, buf, cap, C.byref(cnt)))
        return [dict(kernel=KERNEL_NAMES.get(b.mode, str(b.mode)), tier=TIER_NAMES.get(b.tier, str(b.tier)),
                     dmax=b.dmax, launches=b.launches, ms=b.ms) for b in buf[: min(cnt.value, cap)]]

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.kclpp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class EdgeList:
    """Host edge list; n = max id + 1 as ReadEdgeList computes it."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_pairs(cls, pairs) -> "EdgeList":
        a = np.ascontiguousarray(np.asarray(pairs, dtype=np.uint32).reshape(-1, 2))
        h = _P()
        _check(_lib.kclpp_edge_list_create(_ptr(a, C.c_uint32), a.shape[0], C.byref(h)))
        return cls(h)

    def info(self) -> tuple[int, int]:
        n, e = C.c_uint32(), C.c_uint64()
        _check(_lib.kclpp_edge_list_info(self._h, C.byref(n), C.byref(e)))
        return n.value, e.value

    @property
    def n(self) -> int:
        return self.info()[0]

    @property
    def e(self) -> int:
        return self.info()[1]

    def pairs(self) -> np.ndarray:
        n, e = self.info()
        out = np.empty((e, 2), dtype=np.uint32)
        if e:
            _check(_lib.kclpp_edge_list_copy(self._h, _ptr(out, C.c_uint32)))
        return out

    def write(self, path: str) -> None:
        _check(_lib.kclpp_write_edge_list(self._h, os.fsencode(path)))

    def write_bin(self, path: str) -> None:
        _check(_lib.kclpp_write_edge_list_bin(self._h, os.fsencode(path)))

    @classmethod
    def read_bin(cls, path: str) -> "EdgeList":
        h = _P()
        _check(_lib.kclpp_read_edge_list_bin(os.fsencode(path), C.byref(h)))
        return cls(h)

    def hash(self) -> int:
        """FNV-1a of n and the pairs: the graph_hash of a checkpoint."""
        h = C.c_uint64()
        _check(_lib.kclpp_edge_list_hash(self._h, C.byref(h)))
        return h.value

    def close(self):
        if getattr(self, "_h", None):
            _lib.kclpp_edge_list_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


def read_edge_list(path: str, threads: int | None = None) -> EdgeList:
    """ReadEdgeList semantics; `threads` host threads (None: automatic)."""
    h = _P()
    if threads is None:
        _check(_lib.kclpp_read_edge_list(os.fsencode(path), C.byref(h)))
    else:
        _check(_lib.kclpp_read_edge_list_mt(os.fsencode(path), threads, C.byref(h)))
    return EdgeList(h)


def generate(kind: int, *, n=0, avg_degree=0.0, gamma=0.0, scale=0, edge_factor=0, a=0.0, b=0.0, c=0.0,
             communities=0, comm_min=0, comm_max=0, p_in=0.0, seed=1) -> EdgeList:
    p = GenParams(kind, n, avg_degree, gamma, scale, edge_factor, a, b, c, communities, comm_min,
                  comm_max, p_in, seed)
    h = _P()
    _check(_lib.kclpp_generate(C.byref(p), C.byref(h)))
    return EdgeList(h)


def chung_lu(n: int, avg_degree: float, gamma: float, seed: int = 1) -> EdgeList:
    return generate(GEN_CHUNG_LU, n=n, avg_degree=avg_degree, gamma=gamma, seed=seed)


def rmat(scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1) -> EdgeList:
    return generate(GEN_RMAT, scale=scale, edge_factor=edge_factor, a=a, b=b, c=c, seed=seed)


def rmat_planted(scale: int, edge_factor: int, communities: int, comm_min: int, comm_max: int, p_in: float,
                 a=0.57, b=0.19, c=0.19, seed: int = 1) -> EdgeList:
    """RMAT graph plus planted G(n_c, p_in) communities (sizes log-uniform)."""
    return generate(GEN_RMAT_PLANTED, scale=scale, edge_factor=edge_factor, a=a, b=b, c=c, communities=communities,
                    comm_min=comm_min, comm_max=comm_max, p_in=p_in, seed=seed)


def erdos_renyi(n: int, avg_degree: float, seed: int = 1) -> EdgeList:
    return generate(GEN_ER, n=n, avg_degree=avg_degree, seed=seed)


def planted(n: int, avg_degree: float, gamma: float, communities: int, comm_min: int, comm_max: int,
            p_in: float, seed: int = 1) -> EdgeList:
    return generate(GEN_PLANTED, n=n, avg_degree=avg_degree, gamma=gamma, communities=communities,
                    comm_min=comm_min, comm_max=comm_max, p_in=p_in, seed=seed)


def core_order(el: EdgeList, mode: int = ORDER_EXACT) -> np.ndarray:
    """rank[v] of every vertex: SortByCore's order (ORDER_EXACT) or the bin-sort
    peel (ORDER_FAST: same core numbers, other ties)."""
    rank = np.empty(el.n, dtype=np.uint32)
    if mode == ORDER_EXACT:
        _check(_lib.kclpp_core_order(el._h, _ptr(rank, C.c_uint32)))
    else:
        _check(_lib.kclpp_core_order_mode(el._h, mode, _ptr(rank, C.c_uint32)))
    return rank


class Graph:
    """Degeneracy-oriented DAG resident on the device."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self._h = handle
        n, m, core = C.c_uint32(), C.c_uint64(), C.c_uint32()
        _check(_lib.kclpp_graph_info(handle, C.byref(n), C.byref(m), C.byref(core)))
        self.n, self.m, self.core = n.value, m.value, core.value

    def csr(self) -> tuple[np.ndarray, np.ndarray]:
        off = np.empty(self.n + 1, dtype=np.uint64)
        cols = np.empty(self.m, dtype=np.uint32)
        _check(_lib.kclpp_graph_copy_csr(self._h, _ptr(off, C.c_uint64), _ptr(cols, C.c_uint32)))
        return off, cols

    def close(self):
        if getattr(self, "_h", None) and not getattr(self, "_borrowed", False):
            _lib.kclpp_graph_free(self._h)
        self._h = None

    def __del__(self):
        self.close()


def build_graph(ctx: Context, el: EdgeList, rank: np.ndarray | None = None, order: int = ORDER_EXACT) -> Graph:
    h = _P()
    if rank is None and order == ORDER_EXACT:
        _check(_lib.kclpp_build_graph(ctx.handle, el._h, C.byref(h)))
    elif rank is None:
        _check(_lib.kclpp_build_graph_mode(ctx.handle, el._h, order, C.byref(h)))
    else:
        rank = np.ascontiguousarray(rank, dtype=np.uint32)
        _check(_lib.kclpp_make_graph(ctx.handle, el._h, _ptr(rank, C.c_uint32), C.byref(h)))
    return Graph(ctx, h)


def graph_from_csr(ctx: Context, offsets: np.ndarray, cols: np.ndarray) -> Graph:
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    cl = np.ascontiguousarray(cols, dtype=np.uint32)
    h = _P()
    _check(_lib.kclpp_graph_from_csr(ctx.handle, len(off) - 1, len(cl), _ptr(off, C.c_uint64),
                                     _ptr(cl, C.c_uint32), C.byref(h)))
    return Graph(ctx, h)


def get_schedule(g: Graph) -> Schedule:
    sp = Schedule()
    _check(_lib.kclpp_graph_get_schedule(g._h, C.byref(sp)))
    return sp


def set_schedule(g: Graph, sp: Schedule) -> None:
    _check(_lib.kclpp_graph_set_schedule(g.ctx.handle, g._h, C.byref(sp)))


def save_schedule(path: str, graph_hash: int, k: int, kernel: int, sp: Schedule) -> None:
    """Store a tuned schedule for the graph of that edge-list hash, k and kernel."""
    _check(_lib.kclpp_schedule_save(os.fsencode(path), graph_hash, k, kernel, C.byref(sp)))


def load_schedule(path: str, graph_hash: int, k: int, kernel: int) -> Schedule:
    """A stored schedule; raises if the file is damaged or was tuned for another key."""
    sp = Schedule()
    _check(_lib.kclpp_schedule_load(os.fsencode(path), graph_hash, k, kernel, C.byref(sp)))
    return sp


def autotune(g: Graph, k: int, kernel: int = KERNEL_SEQ) -> TuneResult:
    """Time one pass under each candidate schedule and keep the fastest on g."""
    r = TuneResult()
    _check(_lib.kclpp_autotune(g.ctx.handle, g._h, k, kernel, C.byref(r)))
    return r


class Batch:
    """Many graphs as one device union, run for several k values in one captured CUDA graph."""

    def __init__(self, ctx: Context, edge_lists: list[EdgeList]):
        self.ctx = ctx
        arr = (_P * max(1, len(edge_lists)))(*[e._h for e in edge_lists])
        h = _P()
        _check(_lib.kclpp_batch_create(ctx.handle, arr, len(edge_lists), C.byref(h)))
        self._h = h
        gs, n, m, ug = C.c_uint32(), C.c_uint32(), C.c_uint64(), _P()
        _check(_lib.kclpp_batch_info(h, C.byref(gs), C.byref(n), C.byref(m), C.byref(ug)))
        self.graphs, self.n, self.m = gs.value, n.value, m.value
        self._union = ug
        self.offsets = np.empty(self.graphs + 1, dtype=np.uint32)
        _check(_lib.kclpp_batch_vertex_offsets(h, _ptr(self.offsets, C.c_uint32)))

    def union_graph(self) -> "Graph":
        """The union DAG (borrowed; valid while the batch lives)."""
        g = Graph.__new__(Graph)
        g.ctx, g._h, g.n, g.m, g.core = self.ctx, self._union, self.n, self.m, 0
        g._borrowed = True
        return g

    def run(self, kernel: int, ks: list[int], passes: int) -> np.ndarray:
        """(len(ks), n) array: Seq r (uint64) or Sim rho (float64) after `passes` passes."""
        dt = np.uint64 if kernel == KERNEL_SEQ else np.float64
        out = np.empty((len(ks), self.n), dtype=dt)
        kk = (C.c_int * len(ks))(*ks)
        _check(_lib.kclpp_batch_run(self.ctx.handle, self._h, kernel, kk, len(ks), passes,
                                    out.ctypes.data_as(_P)))
        return out

    def slice(self, i: int) -> slice:
        return slice(int(self.offsets[i]), int(self.offsets[i + 1]))

    def close(self):
        if getattr(self, "_h", None):
            _lib.kclpp_batch_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


def count_edges(g: Graph, nodes: np.ndarray) -> int:
    nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
    m = C.c_uint32()
    _check(_lib.kclpp_count_edges(g.ctx.handle, g._h, len(nodes), _ptr(nodes, C.c_uint32), C.byref(m)))
    return m.value


def count_cliques(g: Graph, k: int) -> tuple[int, np.ndarray]:
    per = np.empty(g.n, dtype=np.uint64)
    tot = C.c_uint64()
    _check(_lib.kclpp_count_cliques(g.ctx.handle, g._h, k, _ptr(per, C.c_uint64), C.byref(tot)))
    return tot.value, per


def seq_passes(g: Graph, k: int, passes: int, r: np.ndarray | None = None,
               det_mode: int = SEQ_EDGE_STREAMS) -> np.ndarray:
    r = np.zeros(g.n, dtype=np.uint64) if r is None else np.array(r, dtype=np.uint64, copy=True)
    _check(_lib.kclpp_seq_passes(g.ctx.handle, g._h, k, passes, det_mode, _ptr(r, C.c_uint64)))
    return r


def seq_passes_dev(g: Graph, k: int, passes: int, r_ptr: int, det_mode: int = SEQ_EDGE_STREAMS) -> None:
    """Enqueue `passes` Seq passes on a device r (u64[n] at r_ptr); no synchronisation."""
    _check(_lib.kclpp_seq_passes_dev(g.ctx.handle, g._h, k, passes, det_mode, _P(r_ptr)))


def sim_passes_dev(g: Graph, k: int, t_first: int, passes: int, rho_ptr: int) -> None:
    """Enqueue Sim passes t_first.. on a device rho (f64[n] at rho_ptr); no synchronisation."""
    _check(_lib.kclpp_sim_passes_dev(g.ctx.handle, g._h, k, t_first, passes, _P(rho_ptr)))


def seq_passes_csr(ctx: Context, offsets, cols, k: int, passes: int, r: np.ndarray,
                   det_mode: int = SEQ_EDGE_STREAMS) -> None:
    """One-shot host call (upload DAG + passes + download); r is updated in place."""
    _check(_lib.kclpp_seq_passes_csr(ctx.handle, len(offsets) - 1, len(cols), _ptr(offsets, C.c_uint64),
                                     _ptr(cols, C.c_uint32), k, passes, det_mode, _ptr(r, C.c_uint64)))


def shard_plan(offsets: np.ndarray, world: int) -> np.ndarray:
    """owner[v]: the rank that processes root v when a pass is split over `world` devices."""
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    n = len(off) - 1
    owner = np.empty(max(n, 1), dtype=np.uint32)
    _check(_lib.kclpp_shard_plan(n, _ptr(off, C.c_uint64), world, _ptr(owner, C.c_uint32)))
    return owner[:n]


def graph_shard(g: Graph, rank: int, world: int) -> None:
    _check(_lib.kclpp_graph_shard(g.ctx.handle, g._h, rank, world))


def seq_delta_dev(g: Graph, k: int, r_ptr: int, delta_ptr: int) -> None:
    _check(_lib.kclpp_seq_delta_dev(g.ctx.handle, g._h, k, _P(r_ptr), _P(delta_ptr)))


def sim_counts_dev(g: Graph, k: int, rho_ptr: int, cnt_ptr: int) -> None:
    _check(_lib.kclpp_sim_counts_dev(g.ctx.handle, g._h, k, _P(rho_ptr), _P(cnt_ptr)))


def sim_update_dev(ctx: Context, n: int, t: int, rho_ptr: int, cnt_ptr: int) -> None:
    _check(_lib.kclpp_sim_update_dev(ctx.handle, n, t, _P(rho_ptr), _P(cnt_ptr)))


def sim_counts(g: Graph, k: int, rho: np.ndarray) -> np.ndarray:
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    cnt = np.empty(g.n, dtype=np.uint64)
    _check(_lib.kclpp_sim_counts(g.ctx.handle, g._h, k, _ptr(rho, C.c_double), _ptr(cnt, C.c_uint64)))
    return cnt


def sim_passes(g: Graph, k: int, passes: int, rho: np.ndarray | None = None, t_first: int = 1) -> np.ndarray:
    rho = np.zeros(g.n, dtype=np.float64) if rho is None else np.array(rho, dtype=np.float64, copy=True)
    _check(_lib.kclpp_sim_passes(g.ctx.handle, g._h, k, t_first, passes, _ptr(rho, C.c_double)))
    return rho


def sim_passes_csr(ctx: Context, offsets, cols, k: int, passes: int, rho: np.ndarray, t_first: int = 1) -> None:
    _check(_lib.kclpp_sim_passes_csr(ctx.handle, len(offsets) - 1, len(cols), _ptr(offsets, C.c_uint64),
                                     _ptr(cols, C.c_uint32), k, t_first, passes, _ptr(rho, C.c_double)))


def sort_by_r_u64(r: np.ndarray, ctx: Context | None = None) -> tuple[np.ndarray, np.ndarray]:
    r = np.ascontiguousarray(r, dtype=np.uint64)
    n = len(r)
    re, lv = np.empty(n, dtype=np.uint32), np.empty(n, dtype=np.uint32)
    _check(_lib.kclpp_sort_by_r_u64(ctx.handle if ctx else None, n, _ptr(r, C.c_uint64),
                                    _ptr(re, C.c_uint32), _ptr(lv, C.c_uint32)))
    return re, lv


def sort_by_r_f64(r: np.ndarray, ctx: Context | None = None) -> tuple[np.ndarray, np.ndarray]:
    r = np.ascontiguousarray(r, dtype=np.float64)
    n = len(r)
    re, lv = np.empty(n, dtype=np.uint32), np.empty(n, dtype=np.uint32)
    _check(_lib.kclpp_sort_by_r_f64(ctx.handle if ctx else None, n, _ptr(r, C.c_double),
                                    _ptr(re, C.c_uint32), _ptr(lv, C.c_uint32)))
    return re, lv


def pava(g: Graph, k: int, level: np.ndarray) -> np.ndarray:
    level = np.ascontiguousarray(level, dtype=np.uint32)
    tent = np.empty(g.n, dtype=np.uint64)
    _check(_lib.kclpp_pava(g.ctx.handle, g._h, k, _ptr(level, C.c_uint32), _ptr(tent, C.c_uint64)))
    return tent


def extract_densest_seq(g: Graph, k: int, T: int, r: np.ndarray) -> tuple[DensestInfo, np.ndarray]:
    r = np.ascontiguousarray(r, dtype=np.uint64)
    info = DensestInfo()
    re = np.empty(g.n, dtype=np.uint32)
    _check(_lib.kclpp_extract_densest_seq(g.ctx.handle, g._h, k, T, _ptr(r, C.c_uint64), C.byref(info),
                                          _ptr(re, C.c_uint32)))
    return info, re


def extract_densest_seq_warm(g: Graph, k: int, T: int, r: np.ndarray, r0: np.ndarray) -> DensestInfo:
    """Densest prefix in the order of r; upper bound from the increments r - r0 of T passes."""
    r = np.ascontiguousarray(r, dtype=np.uint64)
    r0 = np.ascontiguousarray(r0, dtype=np.uint64)
    info = DensestInfo()
    _check(_lib.kclpp_extract_densest_seq_warm(g.ctx.handle, g._h, k, T, _ptr(r, C.c_uint64), _ptr(r0, C.c_uint64),
                                               C.byref(info)))
    return info


def extract_densest_sim(g: Graph, k: int, rho: np.ndarray) -> tuple[DensestInfo, np.ndarray]:
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    info = DensestInfo()
    re = np.empty(g.n, dtype=np.uint32)
    _check(_lib.kclpp_extract_densest_sim(g.ctx.handle, g._h, k, _ptr(rho, C.c_double), C.byref(info),
                                          _ptr(re, C.c_uint32)))
    return info, re


def _n_infos(num_iter: int) -> int:
    c, T = 0, 1
    while T <= num_iter:
        c += 1
        T <<= 1
    return c


def seq_main(g: Graph, k: int, num_iter: int, det_mode: int = SEQ_EDGE_STREAMS):
    cap = max(1, _n_infos(num_iter))
    infos = (DensestInfo * cap)()
    r = np.zeros(g.n, dtype=np.uint64)
    made = C.c_int()
    _check(_lib.kclpp_seq_main(g.ctx.handle, g._h, k, num_iter, det_mode, _ptr(r, C.c_uint64), infos, cap,
                               C.byref(made)))
    return [infos[i] for i in range(made.value)], r


def sim_main(g: Graph, k: int, num_iter: int):
    cap = max(1, _n_infos(num_iter))
    infos = (DensestInfo * cap)()
    rho = np.zeros(g.n, dtype=np.float64)
    made = C.c_int()
    _check(_lib.kclpp_sim_main(g.ctx.handle, g._h, k, num_iter, _ptr(rho, C.c_double), infos, cap,
                               C.byref(made)))
    return [infos[i] for i in range(made.value)], rho


@dataclass
class TrimResult:
    info: TrimInfo
    map: np.ndarray        # new label -> original id
    nck: np.ndarray        # k-clique degree per new label
    order: np.ndarray      # peel order (new labels)
    core_num: np.ndarray   # core number along the peel order
    edges: EdgeList        # trimmed graph, original ids, input order
    peel: PeelStats | None = None  # how the EXACT peel's recounts ran


def trim(ctx: Context | None, el: EdgeList, k: int, mode: int = TRIM_EXACT) -> TrimResult:
    """The k-clique core trim; k = 2 runs on the host alone (ctx may be None)."""
    h = _P()
    _check(_lib.kclpp_trim(ctx.handle if ctx is not None else None, el._h, k, mode, C.byref(h)))
    try:
        info = TrimInfo()
        _check(_lib.kclpp_trim_info_get(h, C.byref(info)))
        n2 = info.n2
        mp = np.empty(n2, dtype=np.uint32)
        nck = np.empty(n2, dtype=np.uint64)
        order = np.empty(n2, dtype=np.uint32)
        core = np.empty(n2, dtype=np.uint64)
        _check(_lib.kclpp_trim_copy(h, _ptr(mp, C.c_uint32), _ptr(nck, C.c_uint64), _ptr(order, C.c_uint32),
                                    _ptr(core, C.c_uint64)))
        eh = _P()
        _check(_lib.kclpp_trim_edges(h, C.byref(eh)))
        ps = PeelStats()
        _check(_lib.kclpp_trim_peel_stats(h, C.byref(ps)))
        return TrimResult(info, mp, nck, order, core, EdgeList(eh), ps)
    finally:
        _lib.kclpp_trim_free(h)


def save_state(path: str, kernel: int, k: int, passes: int, vec: np.ndarray, graph_hash: int = 0) -> None:
    """Checkpoint of a run: Seq r (uint64, kernel=KERNEL_SEQ) or Sim rho
    (float64, kernel=KERNEL_ORDER) after `passes` passes."""
    dt = np.uint64 if kernel == KERNEL_SEQ else np.float64
    v = np.ascontiguousarray(vec, dtype=dt)
    info = StateInfo(kernel, k, passes, len(v), graph_hash)
    _check(_lib.kclpp_save_state(os.fsencode(path), C.byref(info), v.ctypes.data_as(_P)))


def load_state(path: str) -> tuple[StateInfo, np.ndarray]:
    """(header, vector) of a checkpoint; a truncated or altered file raises."""
    info = StateInfo()
    _check(_lib.kclpp_load_state(os.fsencode(path), C.byref(info), None, 0))
    v = np.empty(info.n, dtype=np.uint64 if info.kind == KERNEL_SEQ else np.float64)
    _check(_lib.kclpp_load_state(os.fsencode(path), C.byref(info), v.ctypes.data_as(_P), info.n))
    return info, v


def certify_densest(g: Graph, k: int, r: np.ndarray, max_passes: int = 4096) -> tuple[CertifyInfo, np.ndarray]:
    """Exact certificate of the densest prefix of r (kCDensestMem.c:329-432,
    restated with GPU passes): (info, the candidate's vertices)."""
    r = np.ascontiguousarray(r, dtype=np.uint64)
    info = CertifyInfo()
    mem = np.zeros(max(g.n, 1), dtype=np.uint32)
    _check(_lib.kclpp_certify_densest(g.ctx.handle, g._h, k, _ptr(r, C.c_uint64), max_passes, C.byref(info),
                                      _ptr(mem, C.c_uint32)))
    return info, mem[: info.n].copy()


def densest_exact(el: EdgeList, k: int) -> tuple[ExactInfo, np.ndarray]:
    """Exact k-clique densest subgraph of a small graph (host max-flow): the
    optimum as a fraction, and a boolean mask of one densest vertex set."""
    info = ExactInfo()
    mask = np.zeros(max(el.n, 1), dtype=np.uint8)
    _check(_lib.kclpp_densest_exact(el._h, k, C.byref(info), mask.ctypes.data_as(_P)))
    return info, mask[: el.n].astype(bool)


class Sampling:
    """Seq-Sampling++ (kCDensestSamplingKclistpp.c): a sample of the graph's
    k-cliques kept on the device, "++" passes over it, and reports.  The graph
    must stay open while the sampling object is in use."""

    def __init__(self, g: Graph, k: int, target: int = SAMPLE_TARGET, seed: int = 1, waves: int = 8):
        self.g, self.k = g, k
        self._h = _P()
        _check(_lib.kclpp_sampling_create(g.ctx.handle, g._h, k, target, seed, waves, C.byref(self._h)))

    def info(self) -> SamplingInfo:
        i = SamplingInfo()
        _check(_lib.kclpp_sampling_info_get(self._h, C.byref(i)))
        return i

    def cliques(self) -> tuple[np.ndarray, np.ndarray]:
        """Kept cliques as (rows (S, k) of ascending ids, lexicographic by the
        largest member first; each row's wave)."""
        S = self.info().sampled
        rows = np.zeros((max(S, 1), self.k), dtype=np.uint32)
        wave = np.zeros(max(S, 1), dtype=np.uint8)
        _check(_lib.kclpp_sampling_cliques(self.g.ctx.handle, self._h, _ptr(rows, C.c_uint32),
                                           _ptr(wave, C.c_uint8)))
        return rows[:S], wave[:S]

    def passes(self, count: int) -> None:
        _check(_lib.kclpp_sampling_passes(self.g.ctx.handle, self._h, count))

    def rho(self) -> np.ndarray:
        r = np.zeros(max(self.g.n, 1), dtype=np.uint32)
        _check(_lib.kclpp_sampling_get_rho(self.g.ctx.handle, self._h, _ptr(r, C.c_uint32)))
        return r[: self.g.n]

    def set_rho(self, rho: np.ndarray, passes: int) -> None:
        r = np.ascontiguousarray(rho, dtype=np.uint32)
        _check(_lib.kclpp_sampling_set_rho(self.g.ctx.handle, self._h, _ptr(r, C.c_uint32), passes))

    def extract(self, T: int) -> tuple[SamplingReport, np.ndarray]:
        """Report for loads that stand for T passes, and the vertices by decreasing load."""
        rep = SamplingReport()
        order = np.zeros(max(self.g.n, 1), dtype=np.uint32)
        _check(_lib.kclpp_sampling_extract(self.g.ctx.handle, self._h, T, C.byref(rep), _ptr(order, C.c_uint32)))
        return rep, order[: self.g.n]

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.kclpp_sampling_free(self._h)
        self._h = None

    def __del__(self):
        self.close()


def sampling_main(g: Graph, k: int, num_iter: int, target: int = SAMPLE_TARGET, seed: int = 1,
                  waves: int = 8) -> list[SamplingReport]:
    """Solve: sample, then one report per power of two up to num_iter passes."""
    cap = max(1, num_iter.bit_length())
    reps = (SamplingReport * cap)()
    cnt = C.c_int()
    _check(_lib.kclpp_sampling_main(g.ctx.handle, g._h, k, num_iter, target, seed, waves, reps, cap,
                                    C.byref(cnt)))
    return [reps[i] for i in range(cnt.value)]
