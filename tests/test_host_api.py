"""Host-side behaviour of the Python mirror (CPU only): constructors, error order, wrappers,
dense layouts, and the absence of any CPU fallback."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import torch

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def small_csr(gsa, dt=np.float64, it=np.int64):
    S = sp.random(6, 5, density=0.4, random_state=1, format="csr")
    S.sort_indices()
    return gsa.GenericSparseMatrixCSR(6, 5, (S.indptr + 1).astype(it), (S.indices + 1).astype(it),
                                      S.data.astype(dt)), S


def test_constructor_error_fixture(gsa):
    """test/shared/matrix_csr.jl:61-67: rowptr of length 2 for m = 2 -> ArgumentError."""
    g = GOLDEN["csr_ctor_error"]
    with pytest.raises(gsa.ArgumentError):
        gsa.GenericSparseMatrixCSR(g["m"], g["n"], np.array(g["rowptr"]), np.array(g["colval"]),
                                   np.array(g["nzval"]))


def test_constructor_checks(gsa):
    with pytest.raises(gsa.ArgumentError, match="m must be non-negative"):
        gsa.GenericSparseMatrixCSR(-1, 2, np.array([1]), np.array([], np.int64), np.array([]))
    with pytest.raises(gsa.ArgumentError, match="same length"):
        gsa.GenericSparseMatrixCSR(1, 2, np.array([1, 2]), np.array([1]), np.array([1.0, 2.0]))
    with pytest.raises(gsa.ArgumentError, match="does not fit in Ti"):
        gsa.GenericSparseMatrixCSR(2**31, 2, np.ones(3, np.int32), np.array([], np.int32), np.array([]))
    with pytest.raises(gsa.ArgumentError, match="same length"):
        gsa.GenericSparseMatrixCOO(2, 2, np.array([1, 2]), np.array([1]), np.array([1.0, 2.0]))
    with pytest.raises(gsa.ArgumentError, match="colptr length"):
        gsa.GenericSparseMatrixCSC(2, 2, np.array([1, 1]), np.array([], np.int64), np.array([]))


def test_constructor_copies_buffers(gsa):
    rowptr = np.array([1, 2, 3], np.int64)
    A = gsa.GenericSparseMatrixCSR(2, 2, rowptr, np.array([1, 2]), np.array([1.0, 2.0]))
    rowptr[1] = 99
    assert A.rowptr.tolist() == [1, 2, 3]
    assert A.shape == (2, 2) and gsa.nnz(A) == 2 and len(A) == 4


def test_scipy_round_trips_on_host(gsa):
    """SparseMatrixCSC <-> Generic* host constructors (src/conversions/conversions.jl:7-79)."""
    S = sp.random(30, 20, density=0.2, random_state=4, format="csc")
    for cls in (gsa.GenericSparseMatrixCSR, gsa.GenericSparseMatrixCSC, gsa.GenericSparseMatrixCOO):
        A = cls(S)
        assert np.allclose(gsa.collect(A), S.toarray())
        assert (gsa.SparseMatrixCSC(A) != S).nnz == 0
    coo = gsa.GenericSparseMatrixCOO(S)
    # column-major entry order, as GenericSparseMatrixCOO(::SparseMatrixCSC) builds it
    assert np.all(np.diff(coo.colind.numpy()) >= 0)
    g = GOLDEN["csr_2x2_structure"]
    B = sp.csc_matrix(np.array(g["dense"]))
    C = gsa.GenericSparseMatrixCSR(B)
    assert C.rowptr.tolist() == g["expected_csr"]["rowptr"]
    assert C.colval.tolist() == g["expected_csr"]["colval"]
    assert C.nzval.tolist() == g["expected_csr"]["nzval"]


def test_transpose_adjoint_wrappers(gsa):
    A, S = small_csr(gsa)
    assert gsa.transpose(gsa.transpose(A)) is A
    assert gsa.adjoint(gsa.adjoint(A)) is A
    assert gsa.transpose(A).shape == (5, 6)
    assert np.allclose(gsa.collect(gsa.transpose(A)), S.toarray().T)
    Z = gsa.GenericSparseMatrixCSR(2, 2, np.array([1, 2, 3]), np.array([1, 2]),
                                   np.array([1 + 2j, 3 - 1j]))
    assert np.allclose(gsa.collect(gsa.adjoint(Z)), np.array([[1 + 2j, 0], [0, 3 - 1j]]).conj().T)
    # transpose(CSR) -> CSC reuses the structure (src/conversions/conversions.jl:88-95)
    T = gsa.GenericSparseMatrixCSC(gsa.transpose(A))
    assert T.shape == (5, 6) and np.allclose(gsa.collect(T), S.toarray().T)


def test_mul_errors_in_reference_order(gsa):
    A, _ = small_csr(gsa)
    x = torch.zeros(5, dtype=torch.float64)
    with pytest.raises(gsa.DimensionMismatch, match="second dimension of A, 5, does not match the first dimension of B, 4"):
        gsa.mul_(torch.zeros(6, dtype=torch.float64), A, torch.zeros(4, dtype=torch.float64))
    with pytest.raises(gsa.DimensionMismatch, match="first dimension of A, 6, does not match the first dimension of C, 7"):
        gsa.mul_(torch.zeros(7, dtype=torch.float64), A, x)
    with pytest.raises(gsa.DimensionMismatch, match="second dimension of B, 1, does not match the second dimension of C, 2"):
        gsa.mul_(torch.zeros(6, 2, dtype=torch.float64), A, x)
    with pytest.raises(gsa.ArgumentError, match="promotable"):
        gsa.mul_(torch.zeros(6, dtype=torch.float64), A, x, 1j, 0)
    with pytest.raises(gsa.ArgumentError, match="promotable"):
        gsa.mul_(torch.zeros(6, dtype=torch.float64), A, x.to(torch.complex128))


def test_no_cpu_fallback(gsa):
    """Host-resident operands are rejected: the product runs only in libgsa on the GPU."""
    A, _ = small_csr(gsa)
    with pytest.raises(gsa.ArgumentError, match="GPU only"):
        gsa.mul_(torch.zeros(6, dtype=torch.float64), A, torch.zeros(5, dtype=torch.float64))
    coo = gsa.GenericSparseMatrixCOO(6, 5, np.array([1, 2]), np.array([1, 2]), np.array([1.0, 2.0]))
    with pytest.raises(gsa.ArgumentError, match="GPU only"):
        gsa.GenericSparseMatrixCSR(coo)


def _materialise(buf, ld, op, rows, cols):
    """op(B) from the (buffer, ld, op) triple the C ABI receives."""
    n = buf.untyped_storage().nbytes() // buf.element_size() - buf.storage_offset()
    flat = torch.as_strided(buf, (n,), (1,))
    out = torch.empty(rows, cols, dtype=buf.dtype)
    for i in range(rows):
        for c in range(cols):
            v = flat[i + c * ld] if op == 0 else flat[c + i * ld]
            out[i, c] = v.conj() if op == 2 else v
    return out


@pytest.mark.parametrize("layout", ["colmajor", "rowmajor", "strided"])
@pytest.mark.parametrize("wrap", ["none", "transpose", "adjoint"])
def test_dense_operand_layouts(gsa, layout, wrap):
    from genericsparsearrays_gb300.sparse import _dense_operand
    g = torch.Generator().manual_seed(0)
    base = torch.randn(4, 3, dtype=torch.complex128, generator=g)
    if layout == "colmajor":
        P = base.t().contiguous().t()
    elif layout == "rowmajor":
        P = base.contiguous()
    else:
        P = torch.randn(8, 6, dtype=torch.complex128, generator=g)[::2, ::2]
    ref = {"none": P, "transpose": P.t(), "adjoint": P.conj().t()}[wrap]
    B = {"none": P, "transpose": gsa.transpose(P), "adjoint": gsa.adjoint(P)}[wrap]
    buf, ld, op, rows, cols = _dense_operand(B)
    assert (rows, cols) == tuple(ref.shape)
    assert torch.equal(_materialise(buf, ld, op, rows, cols), ref.resolve_conj())


def test_vector_operands(gsa):
    from genericsparsearrays_gb300.sparse import _dense_operand
    v = torch.arange(5, dtype=torch.float64)
    buf, ld, op, rows, cols = _dense_operand(v)
    assert (rows, cols, op, ld) == (5, 1, 0, 5)
    buf, ld, op, rows, cols = _dense_operand(gsa.transpose(v))
    assert (rows, cols) == (1, 5)
    assert torch.equal(_materialise(buf, ld, op, rows, cols), v.unsqueeze(0))


def test_dot_checks_match_reference_order(gsa):
    """dot(x, A, y): first-dimension, then second-dimension DimensionMismatch, then the
    backend ArgumentError (src/matrix_csr/matrix_csr.jl:223-240); the GPU-only check last."""
    A, S = small_csr(gsa)  # 6 x 5, host tensors
    x, y = torch.zeros(6, dtype=torch.float64), torch.zeros(5, dtype=torch.float64)
    with pytest.raises(gsa.DimensionMismatch, match="first dimension of A, 6, does not match the length of x, 5"):
        gsa.dot(torch.zeros(5, dtype=torch.float64), A, y)
    with pytest.raises(gsa.DimensionMismatch, match="second dimension of A, 5, does not match the length of y, 6"):
        gsa.dot(x, A, torch.zeros(6, dtype=torch.float64))
    with pytest.raises(gsa.DimensionMismatch, match="first dimension of A, 5"):
        gsa.dot(x, gsa.transpose(A), y)  # op(A) is 5 x 6
    with pytest.raises(gsa.ArgumentError, match="GPU only"):
        gsa.dot(x, A, y)


def test_add_checks_match_reference_order(gsa):
    """A + B with a dense B (src/core.jl:66-88): DimensionMismatch on sizes, then the backend
    ArgumentError; the GPU-only check last."""
    A, S = small_csr(gsa)  # 6 x 5 on the host
    with pytest.raises(gsa.DimensionMismatch, match=r"dimensions must match: A has dims \(6, 5\), B has dims \(5, 5\)"):
        gsa.add(A, torch.zeros(5, 5, dtype=torch.float64))
    with pytest.raises(gsa.ArgumentError, match="GPU only"):
        gsa.add(A, torch.zeros(6, 5, dtype=torch.float64))


def test_sparse_add_checks_match_reference_order(gsa):
    """COO + COO (src/matrix_coo/matrix_coo.jl:300-311): DimensionMismatch on sizes, then the
    backend ArgumentError; A + J needs a square A (:389); operators map to add / subtract."""
    e = np.zeros(0, np.int64)
    A = gsa.GenericSparseMatrixCOO(6, 5, np.array([1, 2]), np.array([1, 5]), np.array([1.0, 2.0]))
    B = gsa.GenericSparseMatrixCOO(5, 5, e, e, np.zeros(0))
    with pytest.raises(gsa.DimensionMismatch, match=r"dimensions must match: A has dims \(6, 5\), B has dims \(5, 5\)"):
        A + B
    with pytest.raises(gsa.DimensionMismatch, match=r"A has dims \(5, 6\), B has dims \(5, 5\)"):
        gsa.transpose(A) - B
    with pytest.raises(gsa.DimensionMismatch, match="Matrix must be square to add UniformScaling."):
        A + gsa.I
    with pytest.raises(gsa.DimensionMismatch, match="square"):
        2 * gsa.I - A
    with pytest.raises(gsa.ArgumentError, match="GPU only"):
        A + gsa.GenericSparseMatrixCOO(6, 5, e, e, np.zeros(0))
    C = gsa.GenericSparseMatrixCSR(6, 5, np.ones(7, np.int64), e, np.zeros(0))
    K = gsa.GenericSparseMatrixCSC(6, 5, np.ones(6, np.int64), e, np.zeros(0))
    with pytest.raises(gsa.ArgumentError, match="GPU only"):
        C + C
    with pytest.raises(gsa.ArgumentError, match="no method"):
        C + K
    with pytest.raises(gsa.DimensionMismatch, match="square"):
        C + gsa.I
    # iszero(λ) returns a copy without touching the device: op(A) with the promoted type
    Sq = gsa.GenericSparseMatrixCOO(3, 3, np.array([1, 1]), np.array([2, 2]), np.array([1.0, 0.0]))
    Z = Sq + 0 * gsa.I
    assert gsa.nnz(Z) == 2 and Z.nzval.tolist() == [1.0, 0.0]
    Zn = 0 * gsa.I - Sq
    assert Zn.nzval.tolist() == [-1.0, -0.0]
