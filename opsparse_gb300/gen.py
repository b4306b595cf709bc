"""Seeded synthetic CSR generators for the benchmark and test workloads.

Every generator returns ``(rpt, col, val)`` as numpy arrays (int32, int32, float64) with
ascending, unique column indices per row.  The default seed is 20261203.

Workloads (the SuiteSparse inputs that OpSparse benchmarks on are not available offline,
so these stand in for them):
  * ``laplacian2d(128)``   2-D 5-point stencil, 16,384 rows, 81,408 nnz, diag 4, off -1.
  * ``web_powerlaw()``     1,000,000-row web-like graph: row lengths power-law (exponent 2.1,
                           min 1, drawn up to 4,700 before de-duplication); half of each
                           row's columns uniform within +-512 of the row, half Zipf(s=1)
                           over a random ranking of all columns; U(0,1) values.
  * ``stencil27(80)``      3-D 27-point stencil on an 80^3 grid, N(0,1) values.
  * ``erdos_renyi``        uniform random pattern with a given mean degree, N(0,1) values.
  * ``powerlaw_square``    power-law row degrees (given mean and exponent), uniform columns.
"""
from __future__ import annotations

import numpy as np

SEED = 20261203


def _csr_from_keys(keys: np.ndarray, rows: int, cols: int, vals: np.ndarray | None = None):
    """keys = row * cols + col, already unique and sorted."""
    r = (keys // cols).astype(np.int64)
    c = (keys % cols).astype(np.int32)
    rpt = np.zeros(rows + 1, dtype=np.int64)
    np.add.at(rpt, r + 1, 1)
    rpt = np.cumsum(rpt).astype(np.int32)
    return rpt, c, vals


def laplacian2d(n: int = 128):
    """5-point Laplacian on an n x n grid (row-major), diagonal 4.0, neighbours -1.0."""
    idx = np.arange(n * n, dtype=np.int64)
    i, j = idx // n, idx % n
    parts_r, parts_c, parts_v = [], [], []
    for di, dj, v in ((-1, 0, -1.0), (0, -1, -1.0), (0, 0, 4.0), (0, 1, -1.0), (1, 0, -1.0)):
        ok = (i + di >= 0) & (i + di < n) & (j + dj >= 0) & (j + dj < n)
        parts_r.append(idx[ok])
        parts_c.append(((i + di) * n + (j + dj))[ok])
        parts_v.append(np.full(ok.sum(), v))
    r = np.concatenate(parts_r)
    c = np.concatenate(parts_c)
    v = np.concatenate(parts_v)
    order = np.argsort(r * (n * n) + c, kind="stable")
    rpt, col, _ = _csr_from_keys((r * (n * n) + c)[order], n * n, n * n)
    return rpt, col, v[order].astype(np.float64)


def stencil27(n: int = 80, seed: int = SEED):
    """27-point stencil on an n^3 grid, values N(0,1)."""
    rng = np.random.default_rng(seed)
    N = n ** 3
    idx = np.arange(N, dtype=np.int64)
    x, y, z = idx // (n * n), (idx // n) % n, idx % n
    keys = []
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                ok = (x + dx >= 0) & (x + dx < n) & (y + dy >= 0) & (y + dy < n) & (z + dz >= 0) & (z + dz < n)
                keys.append(idx[ok] * N + ((x + dx) * n * n + (y + dy) * n + (z + dz))[ok])
    k = np.sort(np.concatenate(keys))
    rpt, col, _ = _csr_from_keys(k, N, N)
    val = rng.standard_normal(k.size)
    return rpt, col, val


def web_powerlaw(M: int = 1_000_000, alpha: float = 2.1, lmax: int = 4700, window: int = 512,
                 zipf_s: float = 1.0, seed: int = SEED):
    """Web-like graph: power-law row lengths, half local (+-window) and half Zipf-global columns."""
    rng = np.random.default_rng(seed)
    lmax = max(1, min(lmax, M))
    ls = np.arange(1, lmax + 1, dtype=np.float64)
    p = ls ** -alpha
    p /= p.sum()
    lens = rng.choice(np.arange(1, lmax + 1), size=M, p=p)
    rows = np.repeat(np.arange(M, dtype=np.int64), lens)
    n = rows.size
    local = rng.random(n) < 0.5
    cols = np.empty(n, dtype=np.int64)
    nl = int(local.sum())
    cols[local] = np.clip(rows[local] + rng.integers(-window, window + 1, size=nl), 0, M - 1)
    cdf = np.cumsum(np.arange(1, M + 1, dtype=np.float64) ** -zipf_s)
    cdf /= cdf[-1]
    ranks = np.minimum(np.searchsorted(cdf, rng.random(n - nl)), M - 1)
    cols[~local] = rng.permutation(M)[ranks]
    keys = np.unique(rows * M + cols)
    rpt, col, _ = _csr_from_keys(keys, M, M)
    val = rng.random(keys.size)
    return rpt, col, val


def erdos_renyi(n: int, mean_degree: float, seed: int = SEED, ncols: int | None = None):
    """Each row draws Poisson(mean_degree) columns uniformly (deduplicated), values N(0,1)."""
    rng = np.random.default_rng(seed)
    ncols = n if ncols is None else ncols
    deg = np.minimum(rng.poisson(mean_degree, size=n), ncols)
    rows = np.repeat(np.arange(n, dtype=np.int64), deg)
    cols = rng.integers(0, ncols, size=rows.size)
    keys = np.unique(rows * ncols + cols)
    rpt, col, _ = _csr_from_keys(keys, n, ncols)
    return rpt, col, rng.standard_normal(keys.size)


def powerlaw_square(n: int, mean_degree: float = 16.0, alpha: float = 2.2, seed: int = SEED):
    """n x n, row degrees ~ discrete power law (exponent alpha) rescaled to the mean degree,
    columns uniform, values N(0,1)."""
    rng = np.random.default_rng(seed)
    u = rng.random(n)
    raw = (1.0 - u) ** (-1.0 / (alpha - 1.0))  # Pareto(alpha - 1), min 1
    deg = np.maximum(1, np.round(raw * mean_degree / raw.mean())).astype(np.int64)
    deg = np.minimum(deg, n)
    rows = np.repeat(np.arange(n, dtype=np.int64), deg)
    cols = rng.integers(0, n, size=rows.size)
    keys = np.unique(rows * n + cols)
    rpt, col, _ = _csr_from_keys(keys, n, n)
    return rpt, col, rng.standard_normal(keys.size)


def transpose_pattern(rpt: np.ndarray, col: np.ndarray, ncols: int, seed: int = SEED):
    """Pattern of A^T (ncols x rows) with fresh N(0,1) values."""
    rng = np.random.default_rng(seed + 1)
    rows = np.repeat(np.arange(rpt.size - 1, dtype=np.int64), np.diff(rpt))
    nrows_t = ncols
    keys = np.sort(col.astype(np.int64) * (rpt.size - 1) + rows)
    trpt, tcol, _ = _csr_from_keys(keys, nrows_t, rpt.size - 1)
    return trpt, tcol, rng.standard_normal(keys.size)


def row_flop(arpt: np.ndarray, acol: np.ndarray, brpt: np.ndarray) -> np.ndarray:
    """Intermediate products per row (int64)."""
    blen = np.diff(brpt).astype(np.int64)
    per = blen[acol]
    cs = np.concatenate([[0], np.cumsum(per)])
    return cs[arpt[1:]] - cs[arpt[:-1]]
