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


# ---------------------------------------------------------------------------
# Sparse + sparse for COO (src/matrix_coo/matrix_coo.jl:300-575): the GPU result equals the
# oracle's restatement entry for entry -- same column-major order, same sums (summed in the
# same order, so the same bits), zero sums dropped.

def _coo_tuple(X):
    return (X.rowind.cpu().numpy(), X.colind.cpu().numpy(), X.nzval.cpu().numpy())


def _assert_same(got, want):
    for g, w in zip(got, want):
        assert g.dtype == w.dtype and g.shape == w.shape
        assert np.array_equal(g, w)


def _shuffled_with_duplicates(rng, S, it, extra):
    r, c, v = parts(S, "coo", it)
    pick = rng.integers(0, v.size, extra)
    r, c = np.concatenate([r, r[pick]]), np.concatenate([c, c[pick]])
    v = np.concatenate([v, rand_values(rng, extra, v.dtype)])
    p = rng.permutation(v.size)
    return r[p], c[p], v[p]


@pytest.mark.parametrize("op_a", ["N", "T", "C"])
@pytest.mark.parametrize("op_b", ["N", "T", "C"])
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_coo_plus_coo(gsa, cuda, oracle, op_a, op_b, it, dt):
    rng = np.random.default_rng(21)
    m = n = 70
    a = _shuffled_with_duplicates(rng, sprand(rng, m, n, 0.1, dt), it, 60)
    b = _shuffled_with_duplicates(rng, sprand(rng, m, n, 0.15, dt), it, 60)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, *a))
    B = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, *b))
    wrap = {"N": lambda X: X, "T": gsa.transpose, "C": gsa.adjoint}
    C = wrap[op_a](A) + wrap[op_b](B)
    assert isinstance(C, gsa.GenericSparseMatrixCOO) and C.shape == (m, n)
    _assert_same(_coo_tuple(C), oracle.coo_sum(m, n, a, op_a=op_a, b=b, op_b=op_b))
    D = wrap[op_a](A) - wrap[op_b](B)
    _assert_same(_coo_tuple(D), oracle.coo_sum(m, n, a, op_a=op_a, b=b, op_b=op_b, neg_b=True))
    # test/shared/matrix_coo.jl:383-386: op(A) - op(A) stores nothing (A without duplicates:
    # with them, a1 + a2 - a1 - a2 need not round to zero)
    U = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, *parts(sprand(rng, m, n, 0.1, dt), "coo", it)))
    assert gsa.nnz(wrap[op_a](U) - wrap[op_a](U)) == 0


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_coo_plus_coo_rectangular_known_answer(gsa, cuda, it):
    """test/shared/matrix_coo.jl:388-395 on the GPU."""
    import json, os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))["coo_add_overlap"]
    mk = lambda d: gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(g["m"], g["n"], np.array(d["rowind"], it),
                                                             np.array(d["colind"], it), np.array(d["nzval"])))
    C = mk(g["a"]) + mk(g["b"])
    r, c, v = _coo_tuple(C)
    assert (r.tolist(), c.tolist(), v.tolist()) == (g["expected"]["rowind"], g["expected"]["colind"],
                                                    g["expected"]["nzval"])


@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_coo_plus_uniform_scaling(gsa, cuda, oracle, dt):
    rng = np.random.default_rng(22)
    n = 50
    a = _shuffled_with_duplicates(rng, sprand(rng, n, n, 0.2, dt), np.int64, 20)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(n, n, *a))
    lam = {np.dtype(np.complex64): 2 + 1j, np.dtype(np.complex128): 2 + 1j}.get(np.dtype(dt), 3)
    _assert_same(_coo_tuple(A + gsa.I), oracle.coo_sum(n, n, a, n_diag=n, lam=1))
    _assert_same(_coo_tuple(gsa.I + A), oracle.coo_sum(n, n, a, n_diag=n, lam=1))
    _assert_same(_coo_tuple(A + lam * gsa.I), oracle.coo_sum(n, n, a, n_diag=n, lam=lam))
    _assert_same(_coo_tuple(A - lam * gsa.I), oracle.coo_sum(n, n, a, n_diag=n, lam=-lam))
    # J - A = J + (-A) = (-A) + J (src/core.jl:89,94): A's negated entries first, then the diagonal
    _assert_same(_coo_tuple(lam * gsa.I - A), oracle.coo_sum(n, n, a, neg_a=True, n_diag=n, lam=lam))
    Z = A + 0 * gsa.I  # iszero(λ): copy(A), duplicates kept
    _assert_same(_coo_tuple(Z), a)


def test_coo_plus_identity_known_answer(gsa, cuda):
    """test/shared/matrix_coo.jl:276-281: A_nodiag + I."""
    import json, os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))
    g = g["coo_add_identity_nodiag"]
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(3, 3, np.array(g["a"]["rowind"]), np.array(g["a"]["colind"]),
                                                   np.array(g["a"]["nzval"])))
    r, c, v = _coo_tuple(A + gsa.I)
    assert (r.tolist(), c.tolist(), v.tolist()) == (g["expected"]["rowind"], g["expected"]["colind"],
                                                    g["expected"]["nzval"])


def test_coo_sum_large_with_long_runs(gsa, cuda, oracle):
    """200k entries over few positions (runs of up to a few thousand) plus a power-law spread."""
    rng = np.random.default_rng(23)
    m, n = 3000, 5000
    k = 200_000
    r = np.where(rng.random(k) < 0.3, rng.integers(1, 4, k), rng.integers(1, m + 1, k)).astype(np.int32)
    c = np.where(rng.random(k) < 0.3, rng.integers(1, 3, k), rng.integers(1, n + 1, k)).astype(np.int32)
    v = rng.standard_normal(k)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, r, c, v))
    B = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, c[:1000] % m + 1, r[:1000], v[:1000]))
    _assert_same(_coo_tuple(A + B), oracle.coo_sum(m, n, (r, c, v), b=(c[:1000] % m + 1, r[:1000], v[:1000])))


def test_coo_sum_empty(gsa, cuda):
    e = np.zeros(0, np.int64)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(4, 4, e, e, np.zeros(0)))
    C = A + A
    assert gsa.nnz(C) == 0 and C.shape == (4, 4)
    D = A + gsa.I
    r, c, v = _coo_tuple(D)
    assert r.tolist() == [1, 2, 3, 4] and c.tolist() == [1, 2, 3, 4] and v.tolist() == [1.0] * 4


# ---------------------------------------------------------------------------
# CSR + CSR, CSC + CSC (src/matrix_csr/matrix_csr.jl:290-356 and the CSC method) and
# A + λI (:358-402): the reference's per-row walks, bit-exact against the oracle.

def _cmp(C, want, csr):
    ptr, idx = (C.rowptr, C.colval) if csr else (C.colptr, C.rowval)
    _assert_same((ptr.cpu().numpy(), idx.cpu().numpy(), C.nzval.cpu().numpy()), want)


@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_compressed_plus_compressed(gsa, cuda, oracle, fmt, it, dt):
    rng = np.random.default_rng(31)
    m, n = 60, 45
    SA, SB = sprand(rng, m, n, 0.1, dt), sprand(rng, m, n, 0.15, dt)
    a, b = parts(SA, fmt, it), parts(SB, fmt, it)
    cls = gsa.GenericSparseMatrixCSR if fmt == "csr" else gsa.GenericSparseMatrixCSC
    A, B = gsa.adapt(cuda, cls(m, n, *a)), gsa.adapt(cuda, cls(m, n, *b))
    outer = m if fmt == "csr" else n
    C = A + B
    assert isinstance(C, cls) and C.shape == (m, n)
    _cmp(C, oracle.compressed_add(outer, a, b), fmt == "csr")
    _cmp(A - B, oracle.compressed_add(outer, a, b, neg_b=True), fmt == "csr")
    assert gsa.nnz(A - A) == 0


@pytest.mark.parametrize("fmt", ["csr", "csc"])
def test_compressed_sum_unsorted_duplicates(gsa, cuda, oracle, fmt):
    """Rows in shuffled order with repeated indices: the two-pointer walk's own result."""
    rng = np.random.default_rng(32)
    m = n = 40
    def messy(S):
        p, i, v = parts(S, fmt, np.int64)
        pi, vi, pp = [], [], [1]
        for r in range(p.size - 1):
            ii, vv = i[p[r] - 1:p[r + 1] - 1].copy(), v[p[r] - 1:p[r + 1] - 1].copy()
            if r % 4 == 0 and ii.size:
                ii, vv = np.append(ii, ii[-1]), np.append(vv, 1.5)
            q = rng.permutation(ii.size)
            pi.append(ii[q]); vi.append(vv[q]); pp.append(pp[-1] + ii.size)
        return np.array(pp, np.int64), np.concatenate(pi), np.concatenate(vi)
    a, b = messy(sprand(rng, m, n, 0.15, np.float64)), messy(sprand(rng, m, n, 0.15, np.float64))
    cls = gsa.GenericSparseMatrixCSR if fmt == "csr" else gsa.GenericSparseMatrixCSC
    C = gsa.adapt(cuda, cls(m, n, *a)) + gsa.adapt(cuda, cls(m, n, *b))
    _cmp(C, oracle.compressed_add(m, a, b), fmt == "csr")


@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("op_a", ["N", "T", "C"])
@pytest.mark.parametrize("op_b", ["N", "T", "C"])
def test_compressed_sum_transposes(gsa, cuda, fmt, op_a, op_b):
    rng = np.random.default_rng(33)
    n = 35
    dt = np.complex128
    SA, SB = sprand(rng, n, n, 0.15, dt), sprand(rng, n, n, 0.15, dt)
    cls = gsa.GenericSparseMatrixCSR if fmt == "csr" else gsa.GenericSparseMatrixCSC
    A = gsa.adapt(cuda, cls(n, n, *parts(SA, fmt, np.int64)))
    B = gsa.adapt(cuda, cls(n, n, *parts(SB, fmt, np.int64)))
    wrap = {"N": lambda X: X, "T": gsa.transpose, "C": gsa.adjoint}
    op = {"N": lambda S: S, "T": lambda S: S.T, "C": lambda S: S.conj().T}
    C = wrap[op_a](A) + wrap[op_b](B)
    assert isinstance(C, cls)
    want = (op[op_a](SA) + op[op_b](SB)).toarray()
    assert np.allclose(gsa.collect(C), want, rtol=0, atol=1e-14)
    D = wrap[op_a](A) - wrap[op_b](B)
    assert np.allclose(gsa.collect(D), (op[op_a](SA) - op[op_b](SB)).toarray(), rtol=0, atol=1e-14)


@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_compressed_plus_uniform_scaling(gsa, cuda, oracle, fmt, dt):
    rng = np.random.default_rng(34)
    n = 50
    S = sprand(rng, n, n, 0.1, dt).tolil()
    for r in (3, 7, 8, 9):  # rows without a stored diagonal get one more entry
        S[r, r] = 0
    S = S.tocsr()
    a = parts(S, fmt, np.int64)
    cls = gsa.GenericSparseMatrixCSR if fmt == "csr" else gsa.GenericSparseMatrixCSC
    A = gsa.adapt(cuda, cls(n, n, *a))
    lam = {np.dtype(np.complex64): 2 + 1j, np.dtype(np.complex128): 2 + 1j}.get(np.dtype(dt), 3)
    _cmp(A + lam * gsa.I, oracle.compressed_add_diag(n, a, lam), fmt == "csr")
    _cmp(gsa.I + A, oracle.compressed_add_diag(n, a, 1), fmt == "csr")
    _cmp(A - lam * gsa.I, oracle.compressed_add_diag(n, a, -lam), fmt == "csr")
    neg = (a[0], a[1], -a[2])
    _cmp(lam * gsa.I - A, oracle.compressed_add_diag(n, neg, lam), fmt == "csr")
    Z = A + 0 * gsa.I
    _cmp(Z, a, fmt == "csr")
