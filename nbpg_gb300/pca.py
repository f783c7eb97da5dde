"""PCA compression (the step before the 4-bit search) on the GPU, plus the FP64 fitter.

`encode` replaces PCACompress's projection + quantisation (data_tools/ANNs/data_proc/
base/matrix.h:86-125) and `u8_to_u4` / `f32_to_u8` FmtConv's conversions
(data_tools/ANNs/data_proc/FmtConv.cpp:63-131); all three run through the C ABI.

The reference ships no PCA fitter (PCACompress only reads a `.mat`), so `fit` is this
repository's own: FP64 mean and covariance, the top `d_out` eigenvectors, each output
scaled so that +-`clip_sigma` standard deviations map to +-1 (the range PCACompress's
quantiser spreads over its codes), bias = -mat . mean.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import check

_IN = {np.dtype(np.float32): _lib.DTYPES["f32"], np.dtype(np.uint8): _lib.DTYPES["u8"],
       np.dtype(np.int8): _lib.DTYPES["i8"]}


def fit(x: np.ndarray, d_out: int, clip_sigma: float = 3.0) -> tuple[np.ndarray, np.ndarray]:
    """(mat d_out x d_in float32, bias float32) from rows x (float, u8 or i8), in FP64."""
    x64 = np.asarray(x, dtype=np.float64)
    mean = x64.mean(axis=0)
    xc = x64 - mean
    cov = xc.T @ xc / max(1, x64.shape[0] - 1)
    w, v = np.linalg.eigh(cov)
    order = np.argsort(w)[::-1][:d_out]
    w, v = np.maximum(w[order], 1e-30), v[:, order]
    # a fixed sign per component (largest-magnitude coefficient positive) makes fits reproducible
    v = v * np.sign(v[np.abs(v).argmax(axis=0), np.arange(v.shape[1])])
    mat = (v / (clip_sigma * np.sqrt(w))).T
    bias = -mat @ mean
    return mat.astype(np.float32), bias.astype(np.float32)


def encode(x: np.ndarray, mat: np.ndarray, bias: np.ndarray | None, out: str, device: int = 0) -> np.ndarray:
    """PCACompress on the GPU: out in {"f32", "u8", "i8", "u4", "i4"}; returns the rows as written."""
    x = np.ascontiguousarray(x)
    mat = np.ascontiguousarray(mat, dtype=np.float32)
    b = None if bias is None else np.ascontiguousarray(bias, dtype=np.float32)
    n, d_in = x.shape
    d_out = mat.shape[0]
    width = d_out // 2 if out in ("u4", "i4") else d_out
    res = np.empty((n, width), np.float32 if out == "f32" else np.uint8)
    f32p = _lib.C.POINTER(_lib.C.c_float)
    check(_lib.lib().nbpg_pca_encode(_IN[x.dtype], x.ctypes.data, n, d_in, mat.ctypes.data_as(f32p),
                                     None if b is None else b.ctypes.data_as(f32p), d_out, _lib.DTYPES[out],
                                     res.ctypes.data, device))
    return res


def u8_to_u4(rows: np.ndarray, device: int = 0) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.uint8)
    out = np.empty((rows.shape[0], rows.shape[1] // 2), np.uint8)
    check(_lib.lib().nbpg_u8_to_u4(rows.ctypes.data, rows.shape[0], rows.shape[1], out.ctypes.data, device))
    return out


def f32_to_u8(rows: np.ndarray, device: int = 0) -> np.ndarray:
    rows = np.ascontiguousarray(rows, dtype=np.float32)
    out = np.empty(rows.shape, np.uint8)
    check(_lib.lib().nbpg_f32_to_u8(rows.ctypes.data_as(_lib.C.POINTER(_lib.C.c_float)), rows.shape[0],
                                    rows.shape[1], out.ctypes.data, device))
    return out
