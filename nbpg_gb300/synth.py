"""Seeded synthetic datasets standing in for SIFT-style public sets.

The NBPG README evaluates on SIFT1M, which is not available offline.  These
generators reproduce the shapes and value distributions the workloads are quoted
on: Gaussian mixtures quantised to u8 (1M x 128), unit-normalised mixtures scaled
to i8 (inner product), and float mixtures for the PCA/4-bit path.  Seeds are
fixed per role (centres 0, base 1, queries 2) so every run sees the same data.
"""
from __future__ import annotations

import numpy as np


def _mixture(rng_c, rng_x, n: int, dim: int, n_centres: int, centre_lo: float, centre_hi: float, sigma: float,
             chunk: int = 1 << 18) -> np.ndarray:
    centres = rng_c.uniform(centre_lo, centre_hi, size=(n_centres, dim)).astype(np.float32)
    out = np.empty((n, dim), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        lab = rng_x.integers(0, n_centres, size=e - s)
        out[s:e] = centres[lab] + rng_x.standard_normal(size=(e - s, dim), dtype=np.float32) * sigma
    return out


def u8_mixture(n_base: int, n_query: int, dim: int = 128, n_centres: int = 256, sigma: float = 20.0,
               seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Base and query u8 vectors: centres ~ U[0,120]^dim, per-dim sigma, rounded, clipped."""
    def q(x):
        return np.clip(np.rint(x), 0, 255).astype(np.uint8)
    base = q(_mixture(np.random.default_rng(seed), np.random.default_rng(seed + 1), n_base, dim, n_centres, 0.0,
                      120.0, sigma))
    query = q(_mixture(np.random.default_rng(seed), np.random.default_rng(seed + 2), n_query, dim, n_centres, 0.0,
                       120.0, sigma))
    return base, query


def i8_unit_mixture(n_base: int, n_query: int, dim: int = 96, n_centres: int = 1000, seed: int = 0):
    """Unit-normalised Gaussian-mixture vectors scaled by 127 and rounded to i8."""
    def q(x):
        x = x / np.maximum(np.linalg.norm(x, axis=1, keepdims=True), 1e-12)
        return np.clip(np.rint(x * 127.0), -127, 127).astype(np.int8)
    base = q(_mixture(np.random.default_rng(seed), np.random.default_rng(seed + 1), n_base, dim, n_centres, -1.0,
                      1.0, 0.35))
    query = q(_mixture(np.random.default_rng(seed), np.random.default_rng(seed + 2), n_query, dim, n_centres, -1.0,
                       1.0, 0.35))
    return base, query


def f32_mixture(n_base: int, n_query: int, dim: int = 128, n_centres: int = 1000, seed: int = 0):
    """Float vectors: centres ~ N(0, 4I), unit-variance noise."""
    def gen(rx, n):
        rc = np.random.default_rng(seed)
        centres = (rc.standard_normal(size=(n_centres, dim)) * 2.0).astype(np.float32)
        out = np.empty((n, dim), np.float32)
        for s in range(0, n, 1 << 18):
            e = min(n, s + (1 << 18))
            lab = rx.integers(0, n_centres, size=e - s)
            out[s:e] = centres[lab] + rx.standard_normal(size=(e - s, dim), dtype=np.float32)
        return out
    return gen(np.random.default_rng(seed + 1), n_base), gen(np.random.default_rng(seed + 2), n_query)


def pack_u4(codes: np.ndarray) -> np.ndarray:
    """Pack 4-bit codes (values 0..15, even count per row) two per byte, high nibble first."""
    codes = np.asarray(codes, dtype=np.uint8)
    return ((codes[:, 0::2] & 0xF) << 4 | (codes[:, 1::2] & 0xF)).astype(np.uint8)
