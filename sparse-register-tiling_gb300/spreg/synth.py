"""Seeded synthetic sparse weights and dense operands for the benchmark workloads.

The reference measures on DLMC / SuiteSparse matrices that are not shipped with it; these
generators stand in with the shapes, sparsities and value distributions of the workloads:
  * ``bernoulli``: i.i.d. Bernoulli(1 - sparsity) mask (uniform unstructured sparsity);
  * ``row_skew``: magnitude-pruning-like rows -- per-row keep probability p_i proportional to
    exp(sigma * z_i), z_i ~ N(0, 1), rescaled so the mean is 1 - sparsity and clipped to [0, 1],
    then Bernoulli(p_i) per element.
All randomness comes from numpy's PCG64 with an explicit seed.
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def bernoulli(m: int, k: int, sparsity: float, seed: int = 0, std: float = 1.0, dist: str = "normal") -> np.ndarray:
    g = rng(seed)
    mask = g.random((m, k)) < (1.0 - sparsity)
    vals = _values(g, (m, k), std, dist)
    return np.where(mask, vals, 0.0).astype(np.float32)


def row_keep_probs(m: int, sparsity: float, sigma: float, g: np.random.Generator) -> np.ndarray:
    z = g.standard_normal(m)
    w = np.exp(sigma * z)
    p = w / w.mean() * (1.0 - sparsity)
    return np.clip(p, 0.0, 1.0)


def row_skew(m: int, k: int, sparsity: float, seed: int = 0, sigma: float = 0.5, std: float = 0.02,
             dist: str = "normal") -> np.ndarray:
    g = rng(seed)
    p = row_keep_probs(m, sparsity, sigma, g)
    mask = g.random((m, k)) < p[:, None]
    vals = _values(g, (m, k), std, dist)
    return np.where(mask, vals, 0.0).astype(np.float32)


def _values(g, shape, std, dist):
    if dist == "normal":
        v = g.standard_normal(shape) * std
    elif dist == "uniform":  # U[0, 1) as SPMM_demo.cpp:448-450
        v = g.random(shape)
    elif dist == "ones":
        v = np.ones(shape)
    else:
        raise ValueError(dist)
    v = v.astype(np.float32)
    v[v == 0] = np.float32(std if dist == "normal" else 1.0)  # a drawn exact zero would change the mask
    return v


def dense(k: int, n: int, seed: int = 1, std: float = 1.0) -> np.ndarray:
    return (rng(seed).standard_normal((k, n)) * std).astype(np.float32)


def to_csr(a: np.ndarray):
    """(row_ptrs int32, col_inds int32, values float32) of a dense array (nonzeros only)."""
    rows, cols = np.nonzero(a)
    row_ptrs = np.zeros(a.shape[0] + 1, dtype=np.int32)
    np.add.at(row_ptrs, rows + 1, 1)
    row_ptrs = np.cumsum(row_ptrs).astype(np.int32)
    return row_ptrs, cols.astype(np.int32), a[rows, cols].astype(np.float32)


def sparsity_of(a: np.ndarray) -> float:
    return 1.0 - np.count_nonzero(a) / max(a.size, 1)


def round_bf16(a: np.ndarray) -> np.ndarray:
    """FP32 values rounded to the nearest BF16 value (ties to even), returned as FP32 (finite input)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def token_counts(count: int, median: float = 64.0, sigma: float = 1.0, lo: int = 1, hi: int = 2048,
                 seed: int = 0) -> np.ndarray:
    """Per-request token counts ~ log-normal(median, sigma), rounded and clipped to [lo, hi]."""
    g = rng(seed)
    n = np.rint(median * np.exp(sigma * g.standard_normal(count)))
    return np.clip(n, lo, hi).astype(np.int64)


def poisson_arrivals(count: int, rate: float, seed: int = 0) -> np.ndarray:
    """Arrival times (s) of a Poisson process of the given rate (req/s); rate = inf puts all at 0."""
    if not np.isfinite(rate):
        return np.zeros(count)
    g = rng(seed)
    return np.cumsum(g.exponential(1.0 / rate, count))
