"""Seeded synthetic sparse matrices with the shapes of the AccSpMM workloads.

The reference's only example matrix (an ogbl-ddi-derived graph) is not
available, so these generators stand in for it.  Every generator is
deterministic for a given seed and returns CSR arrays with sorted, unique
column indices per row.  That is the only input form on which the reference's
METCF layout is self-consistent: include/format.hpp:241-261 appends values in
CSR order, while the kernels index them in bitmap order.

Degrees follow a discrete power law: d = floor(x_min * U**(-1/(alpha-1)))
clipped to [1, d_max], with x_min found by bisection so that the clipped mean
matches the requested mean.
"""
from __future__ import annotations

import numpy as np


def powerlaw_degrees(n: int, alpha: float, mean: float, d_max: int,
                     rng: np.random.Generator) -> np.ndarray:
    """n degrees from a clipped Pareto(alpha - 1) with the given mean."""
    u = rng.random(n)
    # clip away from 0 so the power stays finite
    u = np.maximum(u, 1e-300)
    tail = u ** (-1.0 / (alpha - 1.0))

    def realised(xmin: float) -> float:
        return float(np.clip(np.floor(xmin * tail), 1, d_max).mean())

    lo, hi = 0.01, float(mean)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if realised(mid) < mean:
            lo = mid
        else:
            hi = mid
    return np.clip(np.floor(hi * tail), 1, d_max).astype(np.int64)


def _dedupe_sorted(rows: np.ndarray, cols: np.ndarray, n_cols: int):
    key = rows.astype(np.int64) * np.int64(n_cols) + cols.astype(np.int64)
    key.sort()
    keep = np.empty(key.size, dtype=bool)
    if key.size:
        keep[0] = True
        np.not_equal(key[1:], key[:-1], out=keep[1:])
    key = key[keep]
    return (key // n_cols).astype(np.uint32), (key % n_cols).astype(np.uint32)


def coo_to_csr(n_rows: int, rows: np.ndarray, cols: np.ndarray,
               vals: np.ndarray):
    """rows must already be sorted (ties in input order)."""
    counts = np.bincount(rows.astype(np.int64), minlength=n_rows)
    row_ptr = np.zeros(n_rows + 1, dtype=np.uint32)
    np.cumsum(counts, out=row_ptr[1:])
    return row_ptr, cols.astype(np.uint32), vals.astype(np.float32)


def powerlaw_symmetric(n: int = 16384, alpha: float = 2.1, mean: float = 16.0,
                       d_max: int = 512, seed: int = 0):
    """Symmetric power-law adjacency (the small CPU-runnable workload).

    Out-degrees ~ clipped Zipf(alpha) with the given mean, neighbours uniform
    without duplicates, values uniform[0, 1).  The graph is symmetrised
    (union with its transpose) and returned as its lower triangle (row >= col)
    sorted by (row, col), one value per unordered pair, ready to be written as
    a `symmetric` Matrix Market file.  Returns (rows, cols, vals) of the lower
    triangle.
    """
    rng = np.random.default_rng(seed)
    deg = powerlaw_degrees(n, alpha, mean, d_max, rng)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    dst = rng.integers(0, n, size=src.size, dtype=np.int64)
    lo = np.minimum(src, dst)
    hi = np.maximum(src, dst)
    r, c = _dedupe_sorted(hi, lo, n)
    vals = rng.random(r.size, dtype=np.float32)
    return r, c, vals


def expand_symmetric(rows, cols, vals):
    """Full symmetric COO from a lower triangle (diagonal kept once)."""
    off = rows != cols
    r = np.concatenate([rows, cols[off]])
    c = np.concatenate([cols, rows[off]])
    v = np.concatenate([vals, vals[off]])
    return r, c, v


def powerlaw_local(n: int = 1 << 20, alpha: float = 2.1, mean: float = 32.0,
                   d_max: int = 4096, local_frac: float = 0.5,
                   local_radius: int = 1024, seed: int = 0):
    """Power-law graph with locality (the 1M-row scale workload).

    Each neighbour is, with probability local_frac, drawn uniformly within
    +-local_radius of its row (clipped to the matrix), otherwise uniformly
    over all columns; duplicates within a row are dropped, so the realised
    mean degree is slightly below `mean`.  Values uniform[0, 1).
    Returns CSR (row_ptr, col_idx, vals).
    """
    rng = np.random.default_rng(seed)
    deg = powerlaw_degrees(n, alpha, mean, d_max, rng)
    rows = np.repeat(np.arange(n, dtype=np.int64), deg)
    m = rows.size
    local = rng.random(m) < local_frac
    off = rng.integers(-local_radius, local_radius + 1, size=m, dtype=np.int64)
    cols = np.where(local, np.clip(rows + off, 0, n - 1),
                    rng.integers(0, n, size=m, dtype=np.int64))
    r, c = _dedupe_sorted(rows, cols, n)
    del rows, cols, local, off
    vals = rng.random(r.size, dtype=np.float32)
    return coo_to_csr(n, r, c, vals)


def gcn_normalised(n: int = 1 << 21, alpha: float = 2.1, mean: float = 24.0,
                   d_max: int = 4096, seed: int = 0):
    """D^-1/2 (A + I) D^-1/2 of a symmetric power-law graph (precision workload).

    Edge weights are log-uniform in [1e-3, 1e3] before normalisation; D is the
    weighted degree of A + I (unit self loops).  Returns CSR (row_ptr,
    col_idx, vals) with vals in float32.
    """
    rng = np.random.default_rng(seed)
    deg = powerlaw_degrees(n, alpha, mean / 2.0, d_max, rng)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    dst = rng.integers(0, n, size=src.size, dtype=np.int64)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    lo, hi = np.minimum(src, dst), np.maximum(src, dst)
    r, c = _dedupe_sorted(hi, lo, n)
    w = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), size=r.size))
    # symmetric A plus unit diagonal
    diag = np.arange(n, dtype=np.uint32)
    rows = np.concatenate([r, c, diag]).astype(np.int64)
    cols = np.concatenate([c, r, diag]).astype(np.int64)
    wts = np.concatenate([w, w, np.ones(n)])
    order = np.lexsort((cols, rows))
    rows, cols, wts = rows[order], cols[order], wts[order]
    d = np.bincount(rows, weights=wts, minlength=n)
    dinv = 1.0 / np.sqrt(d)
    vals = (dinv[rows] * wts * dinv[cols]).astype(np.float32)
    return coo_to_csr(n, rows.astype(np.uint32), cols.astype(np.uint32), vals)


def dense_uniform(rows: int, k: int, seed: int = 0) -> np.ndarray:
    """B with entries uniform[-1, 1), float32, row-major."""
    rng = np.random.default_rng(seed + 1_000_003)
    return rng.uniform(-1.0, 1.0, size=(rows, k)).astype(np.float32)


def dense_scaled_normal(rows: int, k: int, seed: int = 0) -> np.ndarray:
    """B = N(0, 1) times a per-column scale log-uniform in [1e-2, 1e2]."""
    rng = np.random.default_rng(seed + 2_000_003)
    scale = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), size=k))
    return (rng.standard_normal((rows, k)) * scale).astype(np.float32)


def write_mtx(path: str, n_rows: int, n_cols: int, rows, cols, vals,
              symmetric: bool = False, field: str = "real") -> None:
    """Write a coordinate Matrix Market file (1-based indices)."""
    kind = "symmetric" if symmetric else "general"
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {kind}\n")
        f.write(f"{n_rows} {n_cols} {len(rows)}\n")
        r = np.asarray(rows, dtype=np.int64) + 1
        c = np.asarray(cols, dtype=np.int64) + 1
        if field == "pattern":
            body = np.column_stack([r, c])
            np.savetxt(f, body, fmt="%d %d")
        else:
            v = np.asarray(vals, dtype=np.float64)
            for chunk in range(0, len(r), 1 << 20):
                sl = slice(chunk, chunk + (1 << 20))
                lines = [f"{a} {b} {x:.9g}\n" for a, b, x in zip(r[sl], c[sl], v[sl])]
                f.writelines(lines)
