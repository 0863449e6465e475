"""Seeded synthetic matrices with the shapes and value distributions of the benchmark
configurations (host numpy arrays, 1-based, CSR unless stated).

* ``random_poisson``  -- n x n, nnz per row ~ Poisson(mean), columns uniform without
  replacement, values U(0, 1) (the plain n = 100,000 CSR/CSC/COO SpMV case)
* ``laplacian_2d``    -- 5-point Laplacian on a g x g grid, 4 / -1 (g = 2048: n = 4,194,304,
  nnz = 20,963,328)
* ``power_law``       -- n x n, row lengths min(cap, ceil(x_m U^(-1/a))) with x_m chosen so the
  uncapped mean is ``mean``; columns uniform without replacement; complex N(0,1) parts
* ``permuted_coo``    -- the triplets of a CSR matrix in a seeded random order
"""
from __future__ import annotations

import numpy as np


def _rows_from_lengths(rng, n_cols, lengths):
    """Sorted, duplicate-free column indices (0-based) per row with the given lengths."""
    lengths = np.minimum(lengths, n_cols).astype(np.int64)
    rowptr = np.zeros(lengths.size + 1, np.int64)
    np.cumsum(lengths, out=rowptr[1:])
    nnz = int(rowptr[-1])
    rows = np.repeat(np.arange(lengths.size, dtype=np.int64), lengths)
    cols = rng.integers(0, n_cols, size=nnz, dtype=np.int64)
    # resample duplicates inside a row until none is left
    while True:
        key = rows * n_cols + cols
        order = np.argsort(key, kind="stable")
        ks = key[order]
        dup = np.zeros(nnz, bool)
        dup[order[1:][ks[1:] == ks[:-1]]] = True
        if not dup.any():
            break
        cols[dup] = rng.integers(0, n_cols, size=int(dup.sum()), dtype=np.int64)
    order = np.lexsort((cols, rows))
    return rowptr, cols[order]


def random_poisson(n=100_000, mean=10.0, seed=0, itype=np.int64, dtype=np.float64):
    rng = np.random.default_rng(seed)
    lengths = rng.poisson(mean, size=n)
    rowptr, cols = _rows_from_lengths(rng, n, lengths)
    vals = rng.uniform(0.0, 1.0, size=cols.size).astype(dtype)
    return n, n, (rowptr + 1).astype(itype), (cols + 1).astype(itype), vals


def laplacian_2d(g=2048, itype=np.int32, dtype=np.float64):
    n = g * g
    i = np.arange(n, dtype=np.int64)
    r, c = i // g, i % g
    # neighbours in column order: up (i-g), left (i-1), self, right (i+1), down (i+g)
    cand = np.stack([i - g, i - 1, i, i + 1, i + g], axis=1)
    ok = np.stack([r > 0, c > 0, np.ones(n, bool), c < g - 1, r < g - 1], axis=1)
    lengths = ok.sum(axis=1)
    rowptr = np.zeros(n + 1, np.int64)
    np.cumsum(lengths, out=rowptr[1:])
    cols = cand[ok]
    vals = np.where(cols == np.repeat(i, lengths), 4.0, -1.0).astype(dtype)
    return n, n, (rowptr + 1).astype(itype), (cols + 1).astype(itype), vals


def power_law(n=1_000_000, a=1.5, mean=16.0, cap=50_000, seed=0, itype=np.int64,
              dtype=np.complex128):
    rng = np.random.default_rng(seed)
    xm = mean * (a - 1.0) / a
    u = 1.0 - rng.uniform(0.0, 1.0, size=n)  # (0, 1]
    lengths = np.minimum(cap, np.ceil(xm * u ** (-1.0 / a))).astype(np.int64)
    rowptr, cols = _rows_from_lengths(rng, n, lengths)
    nnz = cols.size
    if np.issubdtype(np.dtype(dtype), np.complexfloating):
        vals = (rng.standard_normal(nnz) + 1j * rng.standard_normal(nnz)).astype(dtype)
    else:
        vals = rng.standard_normal(nnz).astype(dtype)
    return n, n, (rowptr + 1).astype(itype), (cols + 1).astype(itype), vals


def csr_to_csc(m, n, rowptr, colval, nzval):
    """The same matrix in CSC (host, 1-based)."""
    import scipy.sparse as sp
    S = sp.csr_matrix((nzval, colval.astype(np.int64) - 1, rowptr.astype(np.int64) - 1), shape=(m, n))
    X = S.tocsc()
    X.sort_indices()
    it = rowptr.dtype
    return m, n, (X.indptr + 1).astype(it), (X.indices + 1).astype(it), X.data


def csr_rows(rowptr):
    """Row index (1-based) of every stored entry."""
    lengths = np.diff(rowptr.astype(np.int64))
    return (np.repeat(np.arange(lengths.size, dtype=np.int64), lengths) + 1).astype(rowptr.dtype)


def permuted_coo(m, n, rowptr, colval, nzval, seed=0):
    rng = np.random.default_rng(seed)
    rows = csr_rows(rowptr)
    p = rng.permutation(colval.size)
    return m, n, rows[p], colval[p], nzval[p]
