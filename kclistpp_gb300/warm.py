"""Learned warm start for Seq-kClist++ (no counterpart in the reference).

The device work -- features, the MLP's forward/backward/Adam kernels, r0 --
runs in libkclpp; this module only holds the device tensors (PyTorch is used
as the device-memory allocator) and strings the calls together:

    X, Y = training_set(ctx, graphs, k, passes)   # features, log1p(r / T) of zero-start runs
    model = WarmModel(ctx, seed); model.train(X, Y, steps, lr)
    r0 = model.start_r(g, t0)                      # predicted loads x t0
    report = time_to_gap(g, k, gap=0.01, model=model, t0=t0)

The plain zero-start run (`time_to_gap(..., model=None)`) is the fallback and
the reference point; a warm-started run's upper bound uses only the loads its
own passes added (kclpp_extract_densest_seq_warm), so both report a certified
gap between the density they found and an upper bound on the optimum.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import (Context, DensestInfo, EdgeList, Graph, _check, _lib, build_graph, extract_densest_seq,
               extract_densest_seq_warm, seq_passes, seq_passes_dev, SEQ_EDGE_STREAMS)

NPARAMS = 64 * 4 + 64 + 64 + 1


def _torch():
    import torch

    return torch


# The library runs on its context's stream and torch on its own: every hand-over
# of a tensor between the two waits for the producer.
def _after_torch():
    _torch().cuda.synchronize()


def features(g: Graph):
    """(n, 4) float32 device tensor of the model's inputs for g."""
    torch = _torch()
    X = torch.empty((g.n, 4), dtype=torch.float32, device="cuda")
    _check(_lib.kclpp_warm_features(g.ctx.handle, g._h, C.c_void_p(X.data_ptr())))  # synchronises
    return X


def training_set(ctx: Context, graphs: list[EdgeList], k: int, passes: int):
    """Features and targets log1p(r / passes) of zero-start Seq runs on `graphs`."""
    torch = _torch()
    xs, ys = [], []
    for el in graphs:
        g = build_graph(ctx, el)
        if g.n == 0:
            continue
        xs.append(features(g))
        r = seq_passes(g, k, passes)
        ys.append(torch.from_numpy(np.log1p(r.astype(np.float64) / passes).astype(np.float32)).cuda())
        g.close()
    return torch.cat(xs), torch.cat(ys)


class WarmModel:
    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        h = C.c_void_p()
        _check(_lib.kclpp_warm_create(ctx.handle, seed, C.byref(h)))
        self._h = h

    def params(self) -> np.ndarray:
        p = np.empty(NPARAMS, dtype=np.float32)
        _check(_lib.kclpp_warm_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(_lib.kclpp_warm_set_params(self.ctx.handle, self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def predict(self, X):
        torch = _torch()
        _after_torch()
        Y = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
        _check(_lib.kclpp_warm_predict_dev(self.ctx.handle, self._h, C.c_void_p(X.data_ptr()), X.shape[0],
                                           C.c_void_p(Y.data_ptr())))
        self.ctx.synchronize()
        return Y

    def grad(self, X, Y) -> tuple[np.ndarray, float]:
        _after_torch()
        g = np.empty(NPARAMS, dtype=np.float32)
        loss = C.c_float()
        _check(_lib.kclpp_warm_grad_dev(self.ctx.handle, self._h, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                        X.shape[0], g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return g, loss.value

    def train(self, X, Y, steps: int = 400, lr: float = 1e-2) -> float:
        _after_torch()
        loss = C.c_float()
        _check(_lib.kclpp_warm_train(self.ctx.handle, self._h, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                     X.shape[0], steps, lr, C.byref(loss)))
        return loss.value

    def start_r(self, g: Graph, t0: float):
        """r0 (uint64 device tensor viewed as int64) for g."""
        torch = _torch()
        r0 = torch.empty(g.n, dtype=torch.int64, device="cuda")
        _check(_lib.kclpp_warm_start_r(self.ctx.handle, g._h, self._h, t0, C.c_void_p(r0.data_ptr())))
        return r0

    def close(self):
        if getattr(self, "_h", None):
            _lib.kclpp_warm_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


# Passes' worth of predicted load a warm start begins with.  The upper bound
# uses only the loads the run's own passes add, which first have to correct
# the prediction's error, so a start worth many passes delays the certificate
# (t0 = 16: 1.6x slower than the zero start on held-out RMAT-16 graphs); one
# or two passes' worth breaks the first passes' ties by the prediction and
# costs little (t0 = 2: 1.4-1.9x fewer passes there, measured over t0 = 1..16).
DEFAULT_T0 = 2.0


def time_to_gap(g: Graph, k: int, gap: float = 0.01, max_passes: int = 512, model: WarmModel | None = None,
                t0: float = DEFAULT_T0, trace: bool = False, det_mode: int = SEQ_EDGE_STREAMS) -> dict:
    """Run Seq passes (per-root-edge streams; waves with det_mode=SEQ_WAVES;
    shared loads with det_mode=SEQ_SHARED) until (ub - density) / ub <= gap.

    Zero start when model is None; otherwise start at r0 = model.start_r(g, t0)
    (the features, the inference and r0 are inside the timed region).  With
    trace=True the result also holds every pass's (seconds, density, ub)."""
    torch = _torch()
    torch.cuda.synchronize()
    t_start = time.perf_counter()
    if model is None:
        r_dev = torch.zeros(g.n, dtype=torch.int64, device="cuda")
        _after_torch()
        r0 = None
    else:
        r_dev = model.start_r(g, t0)
        r0 = r_dev.cpu().numpy().view(np.uint64).copy()
    info = DensestInfo()
    reached = False
    p = 0
    hist = []
    while p < max_passes:
        seq_passes_dev(g, k, 1, r_dev.data_ptr(), det_mode)
        g.ctx.synchronize()
        p += 1
        r = r_dev.cpu().numpy().view(np.uint64)
        info = extract_densest_seq(g, k, p, r)[0] if r0 is None else extract_densest_seq_warm(g, k, p, r, r0)
        if trace:
            hist.append((time.perf_counter() - t_start, info.density, info.ub))
        if info.ub > 0 and (info.ub - info.density) / info.ub <= gap:
            reached = True
            break
    torch.cuda.synchronize()
    out = {"passes": p, "seconds": time.perf_counter() - t_start, "reached": reached,
           "density": info.density, "ub": info.ub, "n": info.n, "cliques": info.cliques}
    if trace:
        out["trace"] = hist
    return out


def passes_to_density(trace: list, target: float) -> tuple[int, float]:
    """First pass (and its elapsed seconds) whose prefix density reaches target."""
    for i, (sec, dens, _) in enumerate(trace):
        if dens >= target:
            return i + 1, sec
    return len(trace) + 1, float("inf")
