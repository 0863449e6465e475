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


def banded_batch(count=4096, lo=64, hi=8192, half_band=3, extra_mean=8.0, seed=0,
                 itype=np.int64, dtype=np.complex128, device="cpu"):
    """``count`` square CSR matrices, n log-uniform in [lo, hi]; row i holds the band
    [i - half_band, i + half_band] (clipped) plus Poisson(extra_mean) off-band columns drawn
    uniformly without replacement; values complex N(0,1) (or N(0,1) for real types).

    Built with torch on ``device`` (the 4096-matrix batch has ~1e8 entries).  Returns
    (sizes, rowptr, colval, nzval, row_offset, entry_offset): all matrices stored back to back
    in one rowptr (1-based within each matrix) / colval / nzval; matrix i owns rows
    [row_offset[i], row_offset[i+1]) and entries [entry_offset[i], entry_offset[i+1])."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    ls = torch.empty(count).uniform_(np.log(lo), np.log(hi), generator=g)
    sizes = torch.exp(ls).round().to(torch.int64).clamp(lo, hi)
    m_tot = int(sizes.sum())
    dev = torch.device(device)
    sizes_d = sizes.to(dev)
    mat = torch.repeat_interleave(torch.arange(count, device=dev), sizes_d)           # matrix of row
    row_off = torch.zeros(count + 1, dtype=torch.int64, device=dev)
    row_off[1:] = torch.cumsum(sizes_d, 0)
    local = torch.arange(m_tot, device=dev) - row_off[mat]                            # row within matrix
    n_of = sizes_d[mat]
    gd = torch.Generator(device=dev).manual_seed(seed + 1)
    extra = torch.poisson(torch.full((m_tot,), float(extra_mean), device=dev), generator=gd).to(torch.int64)
    # band candidates
    offs = torch.arange(-half_band, half_band + 1, device=dev)
    band = local[:, None] + offs[None, :]
    ok = (band >= 0) & (band < n_of[:, None])
    brow = torch.arange(m_tot, device=dev)[:, None].expand_as(band)[ok]
    bcol = band[ok]
    # off-band candidates: uniform in [0, n), in-band picks drawn again (a few rounds, the
    # rest dropped); duplicates collapse in the unique() below
    erow = torch.repeat_interleave(torch.arange(m_tot, device=dev), extra)
    ecol = (torch.rand(erow.numel(), generator=gd, device=dev) * n_of[erow]).to(torch.int64)
    ecol = torch.minimum(ecol, n_of[erow] - 1)
    for _ in range(8):
        bad = (ecol - local[erow]).abs() <= half_band
        if not bool(bad.any()):
            break
        fresh = (torch.rand(int(bad.sum()), generator=gd, device=dev) * n_of[erow[bad]]).to(torch.int64)
        ecol[bad] = torch.minimum(fresh, n_of[erow[bad]] - 1)
    keep = (ecol - local[erow]).abs() > half_band
    erow, ecol = erow[keep], ecol[keep]
    rows = torch.cat([brow, erow])
    cols = torch.cat([bcol, ecol])
    key = rows * (int(hi) + 1) + cols
    key = torch.unique(key)                                                            # sorted, distinct
    rows = key // (int(hi) + 1)
    cols = key % (int(hi) + 1)
    counts = torch.bincount(rows, minlength=m_tot)
    rowptr_g = torch.zeros(m_tot + 1, dtype=torch.int64, device=dev)
    rowptr_g[1:] = torch.cumsum(counts, 0)
    entry_off = rowptr_g[row_off]
    # per-matrix 1-based pointers: subtract each matrix's first entry offset
    rowptr_local = torch.empty(m_tot + count, dtype=torch.int64, device=dev)
    # matrix i's rowptr occupies [row_off[i] + i, row_off[i+1] + i + 1)
    idx_rows = torch.arange(m_tot, device=dev) + mat
    rowptr_local[idx_rows] = rowptr_g[:-1] - entry_off[mat] + 1
    ends = row_off[1:] + torch.arange(count, device=dev)
    rowptr_local[ends] = entry_off[1:] - entry_off[:-1] + 1
    nnz = cols.numel()
    tdt = {np.dtype(np.complex128): torch.complex128, np.dtype(np.complex64): torch.complex64,
           np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32}[np.dtype(dtype)]
    if tdt.is_complex:
        vals = torch.complex(torch.randn(nnz, generator=gd, device=dev, dtype=torch.float64),
                             torch.randn(nnz, generator=gd, device=dev, dtype=torch.float64)).to(tdt)
    else:
        vals = torch.randn(nnz, generator=gd, device=dev, dtype=torch.float64).to(tdt)
    ti = torch.int64 if np.dtype(itype) == np.dtype(np.int64) else torch.int32
    colval = (cols + 1).to(ti)
    return (sizes.tolist(), rowptr_local.to(ti), colval, vals, row_off.cpu(), entry_off.cpu())
