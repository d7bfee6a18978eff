"""Learned work predictor for the distance scheduler (host side).

profile(w)      -> per-bin-pair features and measured log2 device cycles of one
                   clustering of workload w (idb_profile_binpairs)
train(X, T)     -> 2x64 MLP parameters fitted on the device (idb_mlp_train)
install(ctx, p) -> BF16 copy used by idb_params.schedule = 1 (idb_mlp_load)
save / load     -> parameters as a .npy file

The network only orders the work; the clustering result is the same under every
schedule.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Tuple

import numpy as np

from . import _lib
from .interlink import Context, make_params
from .tuning import _input

F = _lib.MLP_FEATURES
NPARAM = _lib.MLP_PARAMS
H = 64


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised parameters in the library's layout:
    W1[16][64] b1[64] W2[64][64] b2[64] w3[64] b3."""
    rng = np.random.default_rng(seed)
    w1 = rng.normal(0, np.sqrt(2.0 / F), size=(F, H))
    w2 = rng.normal(0, np.sqrt(2.0 / H), size=(H, H))
    w3 = rng.normal(0, np.sqrt(1.0 / H), size=H)
    p = np.concatenate([w1.ravel(), np.zeros(H), w2.ravel(), np.zeros(H), w3, [0.0]])
    return p.astype(np.float32)


def unpack(p: np.ndarray):
    p = np.asarray(p, np.float64)
    o = 0
    w1 = p[o:o + F * H].reshape(F, H); o += F * H
    b1 = p[o:o + H]; o += H
    w2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return w1, b1, w2, b2, w3, b3


def forward(p: np.ndarray, X: np.ndarray) -> np.ndarray:
    """CPU forward pass (float64) -- predicted log2 cycles."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    h1 = np.maximum(X @ w1 + b1, 0)
    h2 = np.maximum(h1 @ w2 + b2, 0)
    return h2 @ w3 + b3


def profile(w, ctx: Optional[Context] = None, tune=None) -> Tuple[np.ndarray, np.ndarray]:
    inp, keep = _input(w)
    prm = make_params(w.threshold, w.abs_eps, w.min_pts, w.use_hamming, tune=tune,
                      candidates=w.candidates)
    cap = 1 << 22
    X = np.zeros((cap, F), np.float32)
    T = np.zeros(cap, np.float32)
    n = C.c_uint64()
    _lib.check(_lib.lib().idb_profile_binpairs(ctx.handle if ctx else None, C.byref(inp), C.byref(prm),
                                               X.ctypes.data, T.ctypes.data, cap, C.byref(n)))
    return X[: n.value].copy(), T[: n.value].copy()


def train(X: np.ndarray, T: np.ndarray, ctx: Optional[Context] = None, epochs: int = 200,
          lr: float = 3e-3, seed: int = 0, params: Optional[np.ndarray] = None):
    """Fit on the device; returns (params, final mean squared error)."""
    X = np.ascontiguousarray(X, np.float32)
    T = np.ascontiguousarray(T, np.float32)
    perm = np.random.default_rng(seed).permutation(len(T))
    X, T = np.ascontiguousarray(X[perm]), np.ascontiguousarray(T[perm])
    p = init_params(seed) if params is None else np.array(params, np.float32)
    loss = C.c_float()
    _lib.check(_lib.lib().idb_mlp_train(ctx.handle if ctx else None, X.ctypes.data, T.ctypes.data,
                                        len(T), epochs, lr, p.ctypes.data, C.byref(loss)))
    return p, float(loss.value)


def install(ctx: Context, params: Optional[np.ndarray]) -> None:
    if params is None:
        _lib.check(_lib.lib().idb_mlp_load(ctx.handle, None))
        return
    p = np.ascontiguousarray(params, np.float32)
    assert p.size == NPARAM
    _lib.check(_lib.lib().idb_mlp_load(ctx.handle, p.ctypes.data))


def save(path: str, params: np.ndarray) -> None:
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    np.save(path, np.asarray(params, np.float32))


def load(path: str) -> np.ndarray:
    p = np.load(path).astype(np.float32)
    if p.size != NPARAM:
        raise ValueError(f"{path}: expected {NPARAM} parameters, found {p.size}")
    return p


def device_grad(params: np.ndarray, X: np.ndarray, T: np.ndarray, ctx: Optional[Context] = None):
    """Gradient and loss from the training kernel (for the CPU check)."""
    X = np.ascontiguousarray(X, np.float32)
    T = np.ascontiguousarray(T, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    g = np.zeros(NPARAM, np.float32)
    loss = C.c_float()
    _lib.check(_lib.lib().idb_diag_mlp_grad(ctx.handle if ctx else None, p.ctypes.data, X.ctypes.data,
                                            T.ctypes.data, len(T), g.ctypes.data, C.byref(loss)))
    return g, float(loss.value)


def device_forward(params: np.ndarray, X: np.ndarray, ctx: Optional[Context] = None) -> np.ndarray:
    """The scheduler's BF16 inference (log2 cycles) on feature rows X."""
    X = np.ascontiguousarray(X, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    y = np.zeros(len(X), np.float32)
    _lib.check(_lib.lib().idb_diag_mlp_predict(ctx.handle if ctx else None, p.ctypes.data,
                                               X.ctypes.data, len(X), y.ctypes.data))
    return y


def _bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 (nearest, ties to even), kept as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward_bf16(p: np.ndarray, X: np.ndarray) -> np.ndarray:
    """CPU model of the BF16 inference: parameters, inputs and hidden
    activations rounded to BF16 as the device rounds them, float64 sums."""
    w1, b1, w2, b2, w3, b3 = [np.asarray(_bf16(np.asarray(t, np.float32)), np.float64)
                              for t in unpack(p)]
    x = np.asarray(_bf16(np.asarray(X, np.float32)), np.float64)
    h1 = np.asarray(_bf16(np.maximum(x @ w1 + b1, 0).astype(np.float32)), np.float64)
    h2 = np.asarray(_bf16(np.maximum(h1 @ w2 + b2, 0).astype(np.float32)), np.float64)
    return h2 @ w3 + b3


def cpu_grad(params: np.ndarray, X: np.ndarray, T: np.ndarray):
    """Reference gradient of the mean squared error (float64, NumPy)."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    X = np.asarray(X, np.float64)
    n = len(T)
    z1 = X @ w1 + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ w2 + b2
    h2 = np.maximum(z2, 0)
    y = h2 @ w3 + b3
    err = y - np.asarray(T, np.float64)
    loss = float(np.mean(err ** 2))
    dy = 2 * err / n
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    d2 = np.outer(dy, w3) * (z2 > 0)
    gw2 = h1.T @ d2
    gb2 = d2.sum(0)
    d1 = (d2 @ w2.T) * (z1 > 0)
    gw1 = X.T @ d1
    gb1 = d1.sum(0)
    g = np.concatenate([gw1.ravel(), gb1, gw2.ravel(), gb2, gw3, [gb3]])
    return g, loss
