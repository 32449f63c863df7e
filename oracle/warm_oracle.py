"""FP64 restatement of the warm-start MLP (TEST INFRASTRUCTURE ONLY).

The checker for the library's forward and backward kernels: the same
4 -> 64 (ReLU) -> 1 network and mean-squared-error gradient, computed in
float64 with the weights rounded to bfloat16 exactly as the device stores
them.  Parameter layout: W1 (64 x 4 row-major), b1 (64), W2 (64), b2 (1).
"""
import numpy as np

F, H = 4, 64
NP = H * F + 2 * H + 1


def to_bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p: np.ndarray):
    p = to_bf16(p)
    W1 = p[: H * F].reshape(H, F)
    b1 = p[H * F: H * F + H]
    W2 = p[H * F + H: H * F + 2 * H]
    b2 = p[-1]
    return W1, b1, W2, b2


def forward(p: np.ndarray, X: np.ndarray) -> np.ndarray:
    W1, b1, W2, b2 = unpack(p)
    Hd = np.maximum(X.astype(np.float64) @ W1.T + b1, 0.0)
    return Hd @ W2 + b2


def grad(p: np.ndarray, X: np.ndarray, Y: np.ndarray):
    """(gradient of mean squared error w.r.t. the parameters, loss), float64."""
    W1, b1, W2, b2 = unpack(p)
    X = X.astype(np.float64)
    A = X @ W1.T + b1
    Hd = np.maximum(A, 0.0)
    e = Hd @ W2 + b2 - Y.astype(np.float64)
    n = len(Y)
    dy = 2.0 * e / n
    gW2 = Hd.T @ dy
    gb2 = dy.sum()
    dH = np.outer(dy, W2) * (A > 0)
    gW1 = dH.T @ X
    gb1 = dH.sum(axis=0)
    return np.concatenate([gW1.ravel(), gb1, gW2, [gb2]]), float(np.mean(e * e))
