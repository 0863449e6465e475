"""Sparse x sparse products (src/matrix_csr/matrix_csr.jl:498-609, the CSC and COO methods)
on the GPU: structure and values equal the oracle's restatement of the reference's kernels
bit for bit -- the same positions (zero sums kept), the same in-order sums of Julia-rounded
products."""
import numpy as np
import pytest
import torch

from helpers import INDEX_TYPES, VALUE_TYPES, parts, rand_values, sprand

pytestmark = pytest.mark.gpu


def np_(t):
    return t.cpu().numpy()


def _same(got, want):
    for g, w in zip(got, want):
        assert g.dtype == w.dtype and g.shape == w.shape, (g.dtype, w.dtype, g.shape, w.shape)
        assert np.array_equal(g, w)


def _csr(gsa, cuda, S, it):
    p, i, v = parts(S, "csr", it)
    return gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(S.shape[0], S.shape[1], p, i, v)), (p, i, v)


def _csc(gsa, cuda, S, it):
    p, i, v = parts(S, "csc", it)
    return gsa.adapt(cuda, gsa.GenericSparseMatrixCSC(S.shape[0], S.shape[1], p, i, v)), (p, i, v)


@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_csr_times_csr(gsa, cuda, oracle, it, dt):
    rng = np.random.default_rng(61)
    SA, SB = sprand(rng, 60, 50, 0.1, dt), sprand(rng, 50, 70, 0.15, dt)
    A, a = _csr(gsa, cuda, SA, it)
    B, b = _csr(gsa, cuda, SB, it)
    C = A @ B
    assert isinstance(C, gsa.GenericSparseMatrixCSR) and C.shape == (60, 70)
    _same((np_(C.rowptr), np_(C.colval), np_(C.nzval)), oracle.spgemm("csr", 60, 50, 70, a, b))


@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_csc_times_csc(gsa, cuda, oracle, it, dt):
    rng = np.random.default_rng(62)
    SA, SB = sprand(rng, 40, 55, 0.12, dt), sprand(rng, 55, 45, 0.1, dt)
    A, a = _csc(gsa, cuda, SA, it)
    B, b = _csc(gsa, cuda, SB, it)
    C = A @ B
    assert isinstance(C, gsa.GenericSparseMatrixCSC) and C.shape == (40, 45)
    _same((np_(C.colptr), np_(C.rowval), np_(C.nzval)), oracle.spgemm("csc", 40, 55, 45, a, b))


@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
def test_long_rows_and_cancellation(gsa, cuda, oracle, fmt, dt):
    """Rows of thousands of products (the global expansion and sort), rows of exactly 256
    and 257 products, products that cancel to exact zeros (kept, as the reference keeps
    every reached position), empty rows and empty selected rows."""
    rng = np.random.default_rng(63)
    m, k, n = 300, 400, 500
    SA = sprand(rng, m, k, 0.02, dt).tolil()
    SA[5, :] = rand_values(rng, k, dt)          # a dense row: ~k * 10 products
    SA[6, :] = 0
    SA[6, :16] = rand_values(rng, 16, dt)
    SB = sprand(rng, k, n, 0.02, dt).tolil()
    SB[:16, :] = 0
    for r in range(16):                          # row 6 of A selects 16 B rows of 16 entries
        SB[r, rng.choice(n, 16, replace=False)] = rand_values(rng, 16, dt)
    SB[20, :] = 0                                 # an empty B row
    SA, SB = SA.tocsr(), SB.tocsr()
    # cancellation: B rows 30 and 31 equal, A row 7 = x at 30 and -x at 31 -> exact zeros
    SB = SB.tolil()
    SB[31, :] = SB[30, :]
    SB = SB.tocsr()
    SA = SA.tolil()
    SA[7, :] = 0
    SA[7, 30], SA[7, 31] = 3, -3
    SA = SA.tocsr()
    SA.eliminate_zeros(); SB.eliminate_zeros()
    mk = _csr if fmt == "csr" else _csc
    A, a = mk(gsa, cuda, SA, np.int64)
    B, b = mk(gsa, cuda, SB, np.int64)
    C = A @ B
    ptr, idx = (C.rowptr, C.colval) if fmt == "csr" else (C.colptr, C.rowval)
    want = oracle.spgemm(fmt, m, k, n, a, b)
    _same((np_(ptr), np_(idx), np_(C.nzval)), want)
    if fmt == "csr" and SB[30].nnz:
        assert np.any(want[2][want[0][7] - 1:want[0][8] - 1] == 0)


def test_empty_and_zero_sized(gsa, cuda, oracle):
    e = np.zeros(0, np.int64)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(4, 3, np.ones(5, np.int64), e, np.zeros(0)))
    B = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(3, 6, np.ones(4, np.int64), e, np.zeros(0)))
    C = A @ B
    assert C.shape == (4, 6) and gsa.nnz(C) == 0 and np_(C.rowptr).tolist() == [1] * 5
    Z = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(0, 3, np.ones(1, np.int64), e, np.zeros(0)))
    assert (Z @ B).shape == (0, 6)


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("op_a", ["N", "T", "C"])
@pytest.mark.parametrize("op_b", ["N", "T", "C"])
def test_transposes_and_coo(gsa, cuda, oracle, fmt, op_a, op_b):
    """op(A) * op(B) for every format: the reference's route (CSR operands to CSC and back,
    CSC to CSR and back, COO through CSC), so the result equals the oracle's product of the
    same converted operands."""
    rng = np.random.default_rng(64)
    dt = np.complex128
    m, k, n = 30, 25, 35
    SA = sprand(rng, *((m, k) if op_a == "N" else (k, m)), 0.15, dt)
    SB = sprand(rng, *((k, n) if op_b == "N" else (n, k)), 0.15, dt)
    cls = {"csr": gsa.GenericSparseMatrixCSR, "csc": gsa.GenericSparseMatrixCSC, "coo": gsa.GenericSparseMatrixCOO}[fmt]
    A = gsa.adapt(cuda, cls(SA.shape[0], SA.shape[1], *parts(SA, fmt, np.int64)))
    B = gsa.adapt(cuda, cls(SB.shape[0], SB.shape[1], *parts(SB, fmt, np.int64)))
    wrap = {"N": lambda X: X, "T": gsa.transpose, "C": gsa.adjoint}
    C = wrap[op_a](A) @ wrap[op_b](B)
    assert isinstance(C, cls) and C.shape == (m, n)
    op = {"N": lambda S: S, "T": lambda S: S.T, "C": lambda S: S.conj().T}
    want = (op[op_a](SA) @ op[op_b](SB)).toarray()
    got = gsa.collect(C)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12)
    # exact: the oracle's product of the operands converted as the reference converts them
    route = "csr" if fmt == "csc" and (op_a != "N" or op_b != "N") else "csc"
    if fmt == "csr" and op_a == "N" and op_b == "N":
        route = "csr"
    conv = lambda S: parts(op[S[1]](S[0]).tocsr() if route == "csr" else op[S[1]](S[0]).tocsc(), route, np.int64)
    ptr, idx, val = oracle.spgemm(route, m, k, n, conv((SA, op_a)), conv((SB, op_b)))
    import scipy.sparse as sp
    Mat = (sp.csr_matrix if route == "csr" else sp.csc_matrix)((val, idx - 1, ptr - 1), shape=(m, n))
    exact = Mat.toarray()
    assert np.array_equal(got, exact)
    assert gsa.nnz(C) == val.size


def test_laplacian_squared(gsa, cuda, oracle):
    """The 2D Laplacian on a 256 x 256 grid, squared: every row a small row (at most 25
    products), bit-exact against the oracle."""
    from genericsparsearrays_gb300 import workloads
    m, n, rp, cv, nz = workloads.laplacian_2d(256, itype=np.int32, dtype=np.float64)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    C = A @ A
    _same((np_(C.rowptr), np_(C.colval), np_(C.nzval)), oracle.spgemm("csr", m, n, n, (rp, cv, nz), (rp, cv, nz)))


def test_checks(gsa, cuda):
    rng = np.random.default_rng(65)
    A, _ = _csr(gsa, cuda, sprand(rng, 10, 8, 0.3, np.float64), np.int64)
    B, _ = _csr(gsa, cuda, sprand(rng, 9, 8, 0.3, np.float64), np.int64)
    with pytest.raises(gsa.DimensionMismatch, match="second dimension of A, 8, does not match first dimension of B, 9"):
        A @ B
    K, _ = _csc(gsa, cuda, sprand(rng, 8, 8, 0.3, np.float64), np.int64)
    with pytest.raises(gsa.ArgumentError):
        A @ K


@pytest.mark.parametrize("dt", [np.float64, np.complex64])
def test_unsorted_and_duplicate_rows(gsa, cuda, oracle, dt):
    """B rows in shuffled order and with repeated columns (what a COO-built matrix can hold):
    the same reached positions and in-order sums as the reference's dense accumulator, for
    rows of every size class (the sorted-run merge must not be used on such rows)."""
    rng = np.random.default_rng(67)
    m, k, n = 200, 150, 120
    SA, SB = sprand(rng, m, k, 0.03, dt), sprand(rng, k, n, 0.05, dt)
    a = parts(SA, "csr", np.int64)
    bp, bi, bv = parts(SB, "csr", np.int64)
    rows_i, rows_v, ptr = [], [], [1]
    for r in range(k):  # shuffle each row and repeat a column in every third row
        lo, hi = bp[r] - 1, bp[r + 1] - 1
        i, v = bi[lo:hi].copy(), bv[lo:hi].copy()
        if r % 3 == 0 and i.size:
            i, v = np.append(i, i[0]), np.append(v, rand_values(rng, 1, dt))
        p = rng.permutation(i.size)
        rows_i.append(i[p]); rows_v.append(v[p]); ptr.append(ptr[-1] + i.size)
    b = (np.array(ptr, np.int64), np.concatenate(rows_i), np.concatenate(rows_v).astype(dt))
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, k, *a))
    B = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(k, n, *b))
    C = A @ B
    _same((np_(C.rowptr), np_(C.colval), np_(C.nzval)), oracle.spgemm("csr", m, k, n, a, b))
