"""Sparse + dense (`A + B`, src/core.jl:66-88) on the GPU: C = copy(B) plus every stored
entry of A, duplicates adding up; against numpy (integers bit-exact, floats within 1e-12 of
|B| + sum|a| per element)."""
import numpy as np
import pytest
import torch

from helpers import INDEX_TYPES, VALUE_TYPES, is_int, parts, rand_values, sprand

pytestmark = pytest.mark.gpu

CLS = {"csr": "GenericSparseMatrixCSR", "csc": "GenericSparseMatrixCSC", "coo": "GenericSparseMatrixCOO"}


def dense_of(m, n, fmt, p0, p1, v):
    D = np.zeros((m, n), dtype=v.dtype)
    S = np.zeros((m, n))
    if fmt == "coo":
        rows, cols = p0 - 1, p1 - 1
    elif fmt == "csr":
        rows = np.repeat(np.arange(m), np.diff(p0.astype(np.int64)))
        cols = p1 - 1
    else:
        cols = np.repeat(np.arange(n), np.diff(p0.astype(np.int64)))
        rows = p1 - 1
    np.add.at(D, (rows, cols), v)
    np.add.at(S, (rows, cols), np.abs(v).astype(np.float64))
    return D, S


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_sparse_plus_dense(gsa, cuda, fmt, it, dt):
    rng = np.random.default_rng(3)
    m, n = 300, 200
    S = sprand(rng, m, n, 0.05, dt)
    p0, p1, v = parts(S, fmt, it)
    if fmt == "coo":  # duplicates, in any order
        p0, p1, v = np.concatenate([p0, p0[:40]]), np.concatenate([p1, p1[:40]]), np.concatenate([v, v[:40]])
        perm = rng.permutation(v.size)
        p0, p1, v = p0[perm], p1[perm], v[perm]
    A = gsa.adapt(cuda, getattr(gsa, CLS[fmt])(m, n, p0, p1, v))
    B = rand_values(rng, (m, n), dt)
    C = gsa.add(A, torch.from_numpy(B).to(cuda)).cpu().numpy()
    D, Sabs = dense_of(m, n, fmt, p0, p1, v)
    if is_int(dt):
        assert np.array_equal(C, B + D)
    else:
        scale = np.abs(B).astype(np.float64) + Sabs
        tol = 1e-5 if dt in (np.float32, np.complex64) else 1e-12
        assert np.max(np.abs(C - (B + D)) / np.maximum(scale, 1e-300)) <= tol


def test_sparse_plus_dense_long_rows(gsa, cuda):
    """Rows of 0 to 20 000 entries (G lanes per row from the warp's average)."""
    rng = np.random.default_rng(5)
    m, n = 2000, 30_000
    lengths = rng.poisson(3, m)
    lengths[[3, 1500]] = [20_000, 5_000]
    rp = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64) + 1
    cv = np.concatenate([rng.choice(n, size=l, replace=False) for l in lengths]).astype(np.int64) + 1
    v = rng.standard_normal(cv.size)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, v))
    B = rng.standard_normal((m, n))
    C = gsa.add(A, torch.from_numpy(B).to(cuda)).cpu().numpy()
    D, _ = dense_of(m, n, "csr", rp, cv, v)
    assert np.array_equal(C, B + D)  # one add per element: exact


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("dt", [np.float64, np.complex64, np.int32])
@pytest.mark.parametrize("it", INDEX_TYPES)
def test_dropzeros(gsa, oracle, cuda, fmt, dt, it):
    """dropzeros keeps the nonzero entries in storage order: bit-exact against a numpy mask,
    pointers recomputed; an all-zero matrix and an empty one."""
    rng = np.random.default_rng(11)
    m, n = 400, 300
    S = sprand(rng, m, n, 0.05, dt)
    p0, p1, v = parts(S, fmt, it)
    v = v.copy()
    v[rng.random(v.size) < 0.3] = 0  # stored zeros
    A = gsa.adapt(cuda, getattr(gsa, CLS[fmt])(m, n, p0, p1, v))
    D = gsa.dropzeros(A)
    keep = v != 0
    if fmt == "coo":
        assert np.array_equal(D.rowind.cpu().numpy(), p0[keep])
        assert np.array_equal(D.colind.cpu().numpy(), p1[keep])
    else:
        ptr, idx = (D.rowptr, D.colval) if fmt == "csr" else (D.colptr, D.rowval)
        per_outer = np.array([keep[b - 1:e - 1].sum() for b, e in zip(p0[:-1], p0[1:])])
        assert np.array_equal(ptr.cpu().numpy(), np.concatenate([[1], 1 + np.cumsum(per_outer)]).astype(it))
        assert np.array_equal(idx.cpu().numpy(), p1[keep])
    assert np.array_equal(D.nzval.cpu().numpy(), v[keep])
    Z = gsa.dropzeros(gsa.adapt(cuda, getattr(gsa, CLS[fmt])(m, n, p0, p1, np.zeros_like(v))))
    assert gsa.nnz(Z) == 0
