"""Host mirror of GenericSparseArrays.jl's sparse x dense API over libgsa.

The reference's user-facing surface for this path is kept, with Python spelling:

=========================================  ===============================================
Julia (reference)                          here
=========================================  ===============================================
``GenericSparseMatrixCSR(m,n,rowptr,...)``  ``GenericSparseMatrixCSR(m, n, rowptr, colval, nzval)``
``GenericSparseMatrixCSC(...)`` / ``COO``   same names
``adapt(CuArray, A)``                       ``adapt("cuda", A)`` (``adapt("cpu", A)`` back)
``mul!(C, A, B, α, β)``, ``mul!(C, A, B)``  ``mul_(C, A, B, alpha, beta)``, ``mul_(C, A, B)``
``A * x``                                   ``A @ x`` or ``mul(A, x)``
``transpose(A)``, ``adjoint(A)`` / ``A'``    ``transpose(A)``, ``adjoint(A)`` (also on dense tensors)
``GenericSparseMatrixCSR(A_coo)`` etc.      same constructors, one argument
``SparseMatrixCSC(A)``, ``collect(A)``      ``SparseMatrixCSC(A)`` (scipy), ``collect(A)`` (numpy)
``nnz(A)``, ``size(A)``                     ``nnz(A)``, ``A.shape`` / ``size(A)``
=========================================  ===============================================

Buffers are torch tensors (device memory on CUDA; host tensors before ``adapt``);
indices are 1-based, as in the reference (``rowptr[0] == 1``).  Dense operands are torch
tensors; any 2-D tensor with one unit stride is used in place (column-major as given, a
row-major tensor as the transpose of its column-major parent).

Products and COO -> CSR/CSC conversions run only in libgsa on the GPU.  A call on host
buffers raises ``ArgumentError``: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Tuple

import numpy as np
import torch

from . import _lib
from .errors import ArgumentError, DimensionMismatch

_DTYPE = {torch.float32: _lib.F32, torch.float64: _lib.F64, torch.complex64: _lib.C32,
          torch.complex128: _lib.C64, torch.int32: _lib.I32, torch.int64: _lib.I64}
_ITYPE = {torch.int32: _lib.IDX32, torch.int64: _lib.IDX64}
_NP_OF = {torch.float32: np.float32, torch.float64: np.float64, torch.complex64: np.complex64,
          torch.complex128: np.complex128, torch.int32: np.int32, torch.int64: np.int64}
_IMAX = {torch.int32: 2**31 - 1, torch.int64: 2**63 - 1}

# Index base of every buffer this layer creates or accepts (Julia's).
BASE = 1


def _tensor(x, dtype=None) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x if dtype is None else x.to(dtype)
    if isinstance(x, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(x))
        return t if dtype is None else t.to(dtype)
    return torch.as_tensor(x, dtype=dtype)


def _stream_ptr(device: torch.device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _ptr(t: Optional[torch.Tensor]) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None and t.numel() else 0)


def _check_Ti(m: int, n: int, itype: torch.dtype) -> None:
    """SparseArrays.sparse_check_Ti as called by the reference constructors."""
    if not (0 <= m <= _IMAX[itype]):
        raise ArgumentError(f"number of rows (m = {m}) does not fit in Ti = {itype}")
    if not (0 <= n <= _IMAX[itype]):
        raise ArgumentError(f"number of columns (n = {n}) does not fit in Ti = {itype}")


class AbstractGenericSparseMatrix:
    """Common part of the three storage formats (src/core.jl:11-22)."""

    m: int
    n: int
    nzval: torch.Tensor

    @property
    def shape(self) -> Tuple[int, int]:
        return (self.m, self.n)

    @property
    def dtype(self) -> torch.dtype:
        return self.nzval.dtype

    @property
    def device(self) -> torch.device:
        return self.nzval.device

    def __len__(self):
        return self.m * self.n

    def __matmul__(self, B):
        return mul(self, B)

    def __add__(self, B):
        return add(self, B)

    def __radd__(self, B):
        return add(self, B)

    def __sub__(self, B):
        return subtract(self, B)

    def __rsub__(self, B):
        return subtract(B, self)

    @property
    def T(self):
        return transpose(self)

    @property
    def H(self):
        return adjoint(self)


def _check_same_device(*ts):
    devs = {t.device for t in ts}
    if len(devs) != 1:
        raise ArgumentError("All storage vectors must be on the same device/backend.")


class GenericSparseMatrixCSR(AbstractGenericSparseMatrix):
    """CSR matrix with generic storage (src/matrix_csr/matrix_csr.jl:17-63).

    ``GenericSparseMatrixCSR(m, n, rowptr, colval, nzval)`` copies the three buffers, as the
    reference constructor does.  One argument converts: a COO or CSC matrix (on the GPU), a
    ``Transpose``/``Adjoint`` of a CSC matrix, or a scipy sparse matrix (host).
    """

    def __init__(self, *args):
        if len(args) == 1:
            src = _convert_to(GenericSparseMatrixCSR, args[0])
            self.m, self.n = src.m, src.n
            self.rowptr, self.colval, self.nzval = src.rowptr, src.colval, src.nzval
            return
        if len(args) != 5:
            raise TypeError("GenericSparseMatrixCSR(m, n, rowptr, colval, nzval) or (A)")
        m, n, rowptr, colval, nzval = args
        rowptr, colval, nzval = _tensor(rowptr), _tensor(colval), _tensor(nzval)
        _check_same_device(rowptr, colval, nzval)
        if rowptr.dtype not in _ITYPE or colval.dtype != rowptr.dtype:
            raise ArgumentError("rowptr and colval must share an index type (int32 or int64)")
        if m < 0:
            raise ArgumentError("m must be non-negative")
        if n < 0:
            raise ArgumentError("n must be non-negative")
        _check_Ti(m, n, rowptr.dtype)
        if rowptr.numel() != m + 1:
            raise ArgumentError("rowptr length must be m+1")
        if colval.numel() != nzval.numel():
            raise ArgumentError("colval and nzval must have same length")
        self.m, self.n = int(m), int(n)
        self.rowptr = rowptr.clone().contiguous()
        self.colval = colval.clone().contiguous()
        self.nzval = nzval.clone().contiguous()

    @property
    def itype(self) -> torch.dtype:
        return self.rowptr.dtype

    def __repr__(self):
        return f"GenericSparseMatrixCSR({self.m}x{self.n}, nnz={nnz(self)}, {self.dtype}, {self.device})"


class GenericSparseMatrixCSC(AbstractGenericSparseMatrix):
    """CSC matrix with generic storage (src/matrix_csc/matrix_csc.jl:17-63)."""

    def __init__(self, *args):
        if len(args) == 1:
            src = _convert_to(GenericSparseMatrixCSC, args[0])
            self.m, self.n = src.m, src.n
            self.colptr, self.rowval, self.nzval = src.colptr, src.rowval, src.nzval
            return
        if len(args) != 5:
            raise TypeError("GenericSparseMatrixCSC(m, n, colptr, rowval, nzval) or (A)")
        m, n, colptr, rowval, nzval = args
        colptr, rowval, nzval = _tensor(colptr), _tensor(rowval), _tensor(nzval)
        _check_same_device(colptr, rowval, nzval)
        if colptr.dtype not in _ITYPE or rowval.dtype != colptr.dtype:
            raise ArgumentError("colptr and rowval must share an index type (int32 or int64)")
        if m < 0:
            raise ArgumentError("m must be non-negative")
        if n < 0:
            raise ArgumentError("n must be non-negative")
        _check_Ti(m, n, colptr.dtype)
        if colptr.numel() != n + 1:
            raise ArgumentError("colptr length must be n+1")
        if rowval.numel() != nzval.numel():
            raise ArgumentError("rowval and nzval must have same length")
        self.m, self.n = int(m), int(n)
        self.colptr = colptr.clone().contiguous()
        self.rowval = rowval.clone().contiguous()
        self.nzval = nzval.clone().contiguous()

    @property
    def itype(self) -> torch.dtype:
        return self.colptr.dtype

    def __repr__(self):
        return f"GenericSparseMatrixCSC({self.m}x{self.n}, nnz={nnz(self)}, {self.dtype}, {self.device})"


class GenericSparseMatrixCOO(AbstractGenericSparseMatrix):
    """COO matrix with generic storage, any entry order (src/matrix_coo/matrix_coo.jl:17-61)."""

    def __init__(self, *args):
        if len(args) == 1:
            src = _convert_to(GenericSparseMatrixCOO, args[0])
            self.m, self.n = src.m, src.n
            self.rowind, self.colind, self.nzval = src.rowind, src.colind, src.nzval
            return
        if len(args) != 5:
            raise TypeError("GenericSparseMatrixCOO(m, n, rowind, colind, nzval) or (A)")
        m, n, rowind, colind, nzval = args
        rowind, colind, nzval = _tensor(rowind), _tensor(colind), _tensor(nzval)
        _check_same_device(rowind, colind, nzval)
        if rowind.dtype not in _ITYPE or colind.dtype != rowind.dtype:
            raise ArgumentError("rowind and colind must share an index type (int32 or int64)")
        if m < 0:
            raise ArgumentError("m must be non-negative")
        if n < 0:
            raise ArgumentError("n must be non-negative")
        _check_Ti(m, n, rowind.dtype)
        if not (rowind.numel() == colind.numel() == nzval.numel()):
            raise ArgumentError("rowind, colind, and nzval must have same length")
        self.m, self.n = int(m), int(n)
        self.rowind = rowind.clone().contiguous()
        self.colind = colind.clone().contiguous()
        self.nzval = nzval.clone().contiguous()

    @property
    def itype(self) -> torch.dtype:
        return self.rowind.dtype

    def __repr__(self):
        return f"GenericSparseMatrixCOO({self.m}x{self.n}, nnz={nnz(self)}, {self.dtype}, {self.device})"


# the three array fields of each format
_FIELDS = {GenericSparseMatrixCSR: ("rowptr", "colval", "nzval"),
           GenericSparseMatrixCSC: ("colptr", "rowval", "nzval"),
           GenericSparseMatrixCOO: ("rowind", "colind", "nzval")}


# ---------------------------------------------------------------------------
# Lazy Transpose / Adjoint wrappers (LinearAlgebra.Transpose / Adjoint)

class Transpose:
    def __init__(self, parent):
        self.parent = parent

    @property
    def shape(self):
        s = tuple(self.parent.shape)
        return (s[1], s[0]) if len(s) == 2 else (1, s[0])

    def __matmul__(self, B):
        return mul(self, B)

    def __add__(self, B):
        return add(self, B)

    def __radd__(self, B):
        return add(self, B)

    def __sub__(self, B):
        return subtract(self, B)

    def __rsub__(self, B):
        return subtract(B, self)


class Adjoint(Transpose):
    pass


def _is_real(dtype) -> bool:
    return not dtype.is_complex


def transpose(A):
    """``transpose(A)``: lazy for sparse matrices and dense tensors; ``transpose(transpose(A)) === A``."""
    if isinstance(A, Adjoint):
        p = A.parent
        return p if _is_real(p.dtype) else _conj_copy(p)
    if isinstance(A, Transpose):
        return A.parent
    return Transpose(A)


def adjoint(A):
    """``adjoint(A)`` (``A'``): conjugate transpose, lazy; for real element types it is ``transpose``."""
    if isinstance(A, Adjoint):
        return A.parent
    if isinstance(A, Transpose):
        p = A.parent
        return p if _is_real(p.dtype) else _conj_copy(p)
    return Adjoint(A)


def _conj_copy(p):
    if isinstance(p, torch.Tensor):
        return p.conj().resolve_conj()
    q = _same_structure(p, p.nzval.conj().resolve_conj())
    return q


def _owned(cls, m, n, p0, p1, val):
    """A matrix that takes ownership of arrays the library has just allocated (no copy; the
    public constructors copy, as the reference's do)."""
    X = cls.__new__(cls)
    X.m, X.n = int(m), int(n)
    f0, f1, f2 = _FIELDS[cls]
    setattr(X, f0, p0.contiguous())
    setattr(X, f1, p1.contiguous())
    setattr(X, f2, val.contiguous())
    return X


def _same_structure(A, nzval):
    if isinstance(A, GenericSparseMatrixCSR):
        return GenericSparseMatrixCSR(A.m, A.n, A.rowptr, A.colval, nzval)
    if isinstance(A, GenericSparseMatrixCSC):
        return GenericSparseMatrixCSC(A.m, A.n, A.colptr, A.rowval, nzval)
    return GenericSparseMatrixCOO(A.m, A.n, A.rowind, A.colind, nzval)


# ---------------------------------------------------------------------------

def nnz(A) -> int:
    if isinstance(A, Transpose):
        return nnz(A.parent)
    return int(A.nzval.numel())


def size(A, dim: Optional[int] = None):
    s = tuple(A.shape)
    if len(s) == 1:
        s = (s[0], 1)
    return s if dim is None else s[dim - 1]


def _to_device(t: torch.Tensor, to) -> torch.Tensor:
    return t.to(to).contiguous() if t.device != torch.device(to) else t


def adapt(to, A):
    """``Adapt.adapt_structure(to, A)`` (src/matrix_csr/matrix_csr.jl:65-71 and the CSC/COO
    equivalents): the same matrix with every buffer moved to ``to`` ("cuda", "cuda:1", "cpu",
    or a torch.device).  The constructor copies the buffers, as the reference's does."""
    dev = torch.device(to)
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    if isinstance(A, Transpose):
        return type(A)(adapt(to, A.parent))
    if isinstance(A, torch.Tensor):
        return A.to(dev)
    if isinstance(A, GenericSparseMatrixCSR):
        return GenericSparseMatrixCSR(A.m, A.n, A.rowptr.to(dev), A.colval.to(dev), A.nzval.to(dev))
    if isinstance(A, GenericSparseMatrixCSC):
        return GenericSparseMatrixCSC(A.m, A.n, A.colptr.to(dev), A.rowval.to(dev), A.nzval.to(dev))
    if isinstance(A, GenericSparseMatrixCOO):
        return GenericSparseMatrixCOO(A.m, A.n, A.rowind.to(dev), A.colind.to(dev), A.nzval.to(dev))
    raise ArgumentError(f"cannot adapt {type(A).__name__}")


# ---------------------------------------------------------------------------
# mul!

def _unwrap_sparse(A):
    """(parent, opA) following trans_adj_wrappers (src/core.jl:102-113)."""
    if isinstance(A, Adjoint):
        return A.parent, (_lib.OP_T if _is_real(A.parent.dtype) else _lib.OP_C)
    if isinstance(A, Transpose):
        return A.parent, _lib.OP_T
    return A, _lib.OP_N


def _dense_operand(B) -> Tuple[torch.Tensor, int, int, int, int]:
    """op(B) as (buffer, ldb, opB, rows, cols) for the C ABI.

    The C ABI reads op(B)(i, c) = buf[i + c*ld] for opB == N and buf[c + i*ld] (conjugated for
    opB == C) otherwise.  A column-major parent P is used as is; a row-major P is the
    transpose of a column-major buffer, so the op flips.  Only a conjugated row-major parent
    (op(P) = conj of a column-major buffer) and layouts without a unit stride are copied.
    """
    op = _lib.OP_N
    if isinstance(B, Adjoint):
        t, op = B.parent, (_lib.OP_T if _is_real(B.parent.dtype) else _lib.OP_C)
    elif isinstance(B, Transpose):
        t, op = B.parent, _lib.OP_T
    else:
        t = B
    if not isinstance(t, torch.Tensor):
        raise ArgumentError(f"dense operand must be a torch tensor, got {type(t).__name__}")
    if t.is_conj():
        t = t.resolve_conj()
    if t.dim() == 1:
        t = t.unsqueeze(1)  # an L-vector is the L x 1 parent
    if t.dim() != 2:
        raise ArgumentError("dense operands must be vectors or matrices")
    r, c = t.shape
    rows, cols = (r, c) if op == _lib.OP_N else (c, r)
    if r <= 1 or t.stride(0) == 1:  # column-major parent
        ld = t.stride(1) if c > 1 else max(r, 1)
        return t, max(ld, r, 1), op, rows, cols
    if c <= 1 or t.stride(1) == 1:  # row-major parent = transpose of a column-major buffer
        ld = t.stride(0) if r > 1 else max(c, 1)
        if op == _lib.OP_N:
            return t, max(ld, c, 1), _lib.OP_T, rows, cols
        if op == _lib.OP_T:
            return t, max(ld, c, 1), _lib.OP_N, rows, cols
    # copy op(B) into a column-major buffer
    opb = t if op == _lib.OP_N else (t.t() if op == _lib.OP_T else t.conj().t())
    buf = opb.resolve_conj().t().contiguous().t()
    return buf, max(buf.shape[0], 1), _lib.OP_N, rows, cols


def _scalar_buf(v, dtype: torch.dtype):
    """alpha/beta as a host buffer of the element type; complex into a real C -> ArgumentError."""
    npdt = _NP_OF[dtype]
    if isinstance(v, bool):
        v = int(v)
    if isinstance(v, complex) and not np.issubdtype(npdt, np.complexfloating):
        if v.imag != 0:
            raise ArgumentError(
                "element types of A, B, α, and β must be promotable to the element type of C")
        v = v.real
    if isinstance(v, float) and np.issubdtype(npdt, np.integer):
        if v != int(v):
            raise ArgumentError(
                "element types of A, B, α, and β must be promotable to the element type of C")
        v = int(v)
    return np.array([v], dtype=npdt)


class _PlanHandle:
    """Owns a gsa_plan (the outer entries of one structure longer than 32, cut into chunks)."""

    def __init__(self, handle: int, nlong: int, nchunks: int, max_len: int):
        self.handle, self.nlong, self.nchunks, self.max_len = handle, nlong, nchunks, max_len

    def __del__(self):
        try:
            _lib.load().gsa_plan_destroy(ctypes.c_void_p(self.handle))
        except Exception:  # interpreter shutdown
            pass


def _gather_plan(A) -> Optional[_PlanHandle]:
    """The plan of A's compressed structure, made on first use and kept on the matrix
    (None when no outer entry is longer than 32, so plain calls are as good).  Making it
    synchronizes the stream once; the structure must not be changed in place afterwards."""
    cached = A.__dict__.get("_plan", False)
    if cached is not False:
        return cached
    csr = isinstance(A, GenericSparseMatrixCSR)
    ptr = A.rowptr if csr else A.colptr
    outer = A.m if csr else A.n
    lib = _lib.load()
    h = ctypes.c_void_p(0)
    with torch.cuda.device(A.device):
        st = lib.gsa_plan_create(_stream_ptr(A.device), _ITYPE[A.itype], outer, nnz(A), _ptr(ptr),
                                 BASE, ctypes.byref(h))
    _lib.check(st)
    ml, nl, nc = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    lib.gsa_plan_info(h, ctypes.byref(ml), ctypes.byref(nl), ctypes.byref(nc))
    if nl.value == 0:
        lib.gsa_plan_destroy(h)
        A._plan = None
    else:
        A._plan = _PlanHandle(h.value, nl.value, nc.value, ml.value)
    return A._plan


def _coo_plan(A) -> Optional[_PlanHandle]:
    """The plan of a COO matrix whose row indices are non-decreasing (row pointers built on
    the GPU once and kept on the matrix, so the CSR kernels serve it); None otherwise.  Made
    on first use (one stream synchronisation); the indices must not change in place after."""
    cached = A.__dict__.get("_plan", False)
    if cached is not False:
        return cached
    lib = _lib.load()
    h = ctypes.c_void_p(0)
    with torch.cuda.device(A.device):
        st = lib.gsa_coo_plan_create(_stream_ptr(A.device), _ITYPE[A.itype], A.m, A.n, nnz(A),
                                     _ptr(A.rowind), BASE, ctypes.byref(h))
    _lib.check(st)
    srt = ctypes.c_int(0)
    lib.gsa_coo_plan_info(h, ctypes.byref(srt))
    if not srt.value:
        lib.gsa_plan_destroy(h)
        A._plan = None
    else:
        ml, nl, nc = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        lib.gsa_plan_info(h, ctypes.byref(ml), ctypes.byref(nl), ctypes.byref(nc))
        A._plan = _PlanHandle(h.value, nl.value, nc.value, ml.value)
    return A._plan


def mul_(C: torch.Tensor, A, B, alpha=1, beta=0, algo: int = _lib.ALGO_AUTO,
         workspace: Optional[torch.Tensor] = None) -> torch.Tensor:
    """``mul!(C, A, B, α, β)``: ``C = β C + α op(A) op(B)`` on the GPU; returns ``C``.

    Checks follow the reference's generated methods (src/matrix_csr/matrix_csr.jl:160-190):
    three ``DimensionMismatch`` checks, the element-type check and the backend check, in that
    order.  ``beta == 0`` never reads ``C``.  Asynchronous on the current torch stream.
    """
    Ap, opA = _unwrap_sparse(A)
    if not isinstance(Ap, AbstractGenericSparseMatrix):
        raise ArgumentError("A must be a GenericSparseMatrixCSR/CSC/COO or its transpose/adjoint")
    Am, An = (Ap.m, Ap.n) if opA == _lib.OP_N else (Ap.n, Ap.m)
    Bbuf, ldb, opB, Br, Bc = _dense_operand(B)
    if not isinstance(C, torch.Tensor):
        raise ArgumentError("C must be a torch tensor")
    Cr, Cc = (C.shape[0], 1) if C.dim() == 1 else tuple(C.shape)
    if An != Br:
        raise DimensionMismatch(
            f"second dimension of A, {An}, does not match the first dimension of B, {Br}")
    if Am != Cr:
        raise DimensionMismatch(
            f"first dimension of A, {Am}, does not match the first dimension of C, {Cr}")
    if Bc != Cc:
        raise DimensionMismatch(
            f"second dimension of B, {Bc}, does not match the second dimension of C, {Cc}")
    dt = C.dtype
    if dt not in _DTYPE:
        raise ArgumentError(f"unsupported element type {dt}")
    if Ap.dtype != dt or Bbuf.dtype != dt:
        if (Ap.dtype.is_complex or Bbuf.dtype.is_complex) and not dt.is_complex:
            raise ArgumentError(
                "element types of A, B, α, and β must be promotable to the element type of C")
        raise ArgumentError(
            f"mixed element types (A {Ap.dtype}, B {Bbuf.dtype}, C {dt}) are not provided by the "
            "GPU path; convert the operands to one type")
    al, be = _scalar_buf(alpha, dt), _scalar_buf(beta, dt)
    devs = {Ap.device, Bbuf.device, C.device}
    if len(devs) != 1:
        raise ArgumentError("All arrays must have the same backend")
    dev = C.device
    if dev.type != "cuda":
        raise ArgumentError("mul! runs on the GPU only; adapt the operands to CUDA first")
    # C must be column-major (unit row stride); otherwise compute into a column-major
    # buffer and copy back.
    C2 = C.unsqueeze(1) if C.dim() == 1 else C
    direct = C2.shape[0] <= 1 or C2.stride(0) == 1
    Cw = C2 if direct else C2.t().contiguous().t()
    ldc = Cw.stride(1) if Cw.shape[1] > 1 else Cw.shape[0]
    ldc = max(ldc, Cw.shape[0], 1)
    lib = _lib.load()
    k = Cc
    stream = _stream_ptr(dev)
    with torch.cuda.device(dev):
        if isinstance(Ap, (GenericSparseMatrixCSR, GenericSparseMatrixCSC)):
            csr = isinstance(Ap, GenericSparseMatrixCSR)
            ptr, idx = (Ap.rowptr, Ap.colval) if csr else (Ap.colptr, Ap.rowval)
            gather = (opA == _lib.OP_N) == csr
            plan = _gather_plan(Ap) if algo == _lib.ALGO_AUTO else None
        if isinstance(Ap, (GenericSparseMatrixCSR, GenericSparseMatrixCSC)) and plan is not None:
            ws_bytes = lib.gsa_plan_workspace_size(ctypes.c_void_p(plan.handle), _DTYPE[dt], k)
            if ws_bytes and (workspace is None or workspace.numel() < ws_bytes):
                workspace = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
            fn = lib.gsa_csr_mul_planned if csr else lib.gsa_csc_mul_planned
            st = fn(stream, _DTYPE[dt], _ITYPE[Ap.itype], Ap.m, Ap.n, nnz(Ap), _ptr(ptr), _ptr(idx),
                    _ptr(Ap.nzval), BASE, opA, k, _ptr(Bbuf), ldb, opB, _ptr(Cw), ldc,
                    al.ctypes.data_as(ctypes.c_void_p), be.ctypes.data_as(ctypes.c_void_p),
                    ctypes.c_void_p(plan.handle),
                    _ptr(workspace) if ws_bytes else ctypes.c_void_p(0),
                    workspace.numel() if ws_bytes else 0)
        elif isinstance(Ap, (GenericSparseMatrixCSR, GenericSparseMatrixCSC)):
            ws_bytes = lib.gsa_mul_workspace_size(0 if csr else 1, _DTYPE[dt], _ITYPE[Ap.itype],
                                                  Ap.m, Ap.n, nnz(Ap), opA, k, algo)
            if ws_bytes and (workspace is None or workspace.numel() < ws_bytes):
                workspace = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
            fn = lib.gsa_csr_mul if csr else lib.gsa_csc_mul
            st = fn(stream, _DTYPE[dt], _ITYPE[Ap.itype], Ap.m, Ap.n, nnz(Ap), _ptr(ptr), _ptr(idx),
                    _ptr(Ap.nzval), BASE, opA, k, _ptr(Bbuf), ldb, opB, _ptr(Cw), ldc,
                    al.ctypes.data_as(ctypes.c_void_p), be.ctypes.data_as(ctypes.c_void_p), algo,
                    _ptr(workspace) if ws_bytes else ctypes.c_void_p(0),
                    workspace.numel() if ws_bytes else 0)
        else:
            cplan = _coo_plan(Ap) if algo == _lib.ALGO_AUTO else None
            if cplan is not None:  # row-sorted: the CSR kernels on the plan's row pointers
                ws_bytes = lib.gsa_plan_workspace_size(ctypes.c_void_p(cplan.handle), _DTYPE[dt], k)
                if ws_bytes and (workspace is None or workspace.numel() < ws_bytes):
                    workspace = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
                st = lib.gsa_coo_mul_planned(stream, _DTYPE[dt], _ITYPE[Ap.itype], Ap.m, Ap.n, nnz(Ap),
                                             _ptr(Ap.rowind), _ptr(Ap.colind), _ptr(Ap.nzval), BASE, opA,
                                             k, _ptr(Bbuf), ldb, opB, _ptr(Cw), ldc,
                                             al.ctypes.data_as(ctypes.c_void_p),
                                             be.ctypes.data_as(ctypes.c_void_p),
                                             ctypes.c_void_p(cplan.handle),
                                             _ptr(workspace) if ws_bytes else ctypes.c_void_p(0),
                                             workspace.numel() if ws_bytes else 0)
            else:
                st = lib.gsa_coo_mul(stream, _DTYPE[dt], _ITYPE[Ap.itype], Ap.m, Ap.n, nnz(Ap),
                                     _ptr(Ap.rowind), _ptr(Ap.colind), _ptr(Ap.nzval), BASE, opA, k,
                                     _ptr(Bbuf), ldb, opB, _ptr(Cw), ldc,
                                     al.ctypes.data_as(ctypes.c_void_p),
                                     be.ctypes.data_as(ctypes.c_void_p))
    _lib.check(st)
    if not direct:
        C2.copy_(Cw)
    return C


def _is_sparse_operand(X) -> bool:
    return isinstance(X, AbstractGenericSparseMatrix) or (
        isinstance(X, Transpose) and isinstance(X.parent, AbstractGenericSparseMatrix))


def _spgemm(A, B):
    """C = A * B for two unwrapped matrices of the same compressed format (gsa_spgemm_*)."""
    csr = isinstance(A, GenericSparseMatrixCSR)
    cls = type(A)
    dtype = torch.promote_types(A.dtype, B.dtype)
    it, dev = A.itype, A.device
    pa, ia = (A.rowptr, A.colval) if csr else (A.colptr, A.rowval)
    pb, ib = (B.rowptr, B.colval) if csr else (B.colptr, B.rowval)
    pb, ib = pb.to(it), ib.to(it)
    va, vb = A.nzval.to(dtype), B.nzval.to(dtype)
    outer = A.m if csr else B.n
    ptr = torch.empty(outer + 1, dtype=it, device=dev)
    lib = _lib.load()
    nnz_c = ctypes.c_int64(0)
    handle = ctypes.c_void_p(0)
    stream = _stream_ptr(dev)
    with torch.cuda.device(dev):
        _lib.check(lib.gsa_spgemm_create(stream, 0 if csr else 1, _DTYPE[dtype], _ITYPE[it], A.m, A.n, B.n, _ptr(pa),
                                         _ptr(ia), _ptr(va), va.numel(), _ptr(pb), _ptr(ib), _ptr(vb), vb.numel(),
                                         BASE, _ptr(ptr), ctypes.byref(nnz_c), ctypes.byref(handle)))
        try:
            idx = torch.empty(nnz_c.value, dtype=it, device=dev)
            val = torch.empty(nnz_c.value, dtype=dtype, device=dev)
            _lib.check(lib.gsa_spgemm_compute(stream, handle, _ptr(idx), _ptr(val)))
        finally:
            lib.gsa_spgemm_destroy(handle)
    return _owned(cls, A.m, B.n, ptr, idx, val)


def _sparse_mul(A, B):
    """``A * B`` of two sparse matrices (src/matrix_csr/matrix_csr.jl:498-609 and the CSC and
    COO methods): CSR * CSR and CSC * CSC directly; COO through CSC and back; with a
    transpose or adjoint on either side, CSR operands are converted to CSC (CSC operands to
    CSR) and the result converted back, as the reference does."""
    if A.shape[1] != B.shape[0]:
        raise DimensionMismatch(f"second dimension of A, {A.shape[1]}, does not match first dimension of B, "
                                f"{B.shape[0]}")
    PA = A.parent if isinstance(A, Transpose) else A
    PB = B.parent if isinstance(B, Transpose) else B
    if PA.device != PB.device:
        raise ArgumentError("Both matrices must have the same backend")
    if type(PA) is not type(PB):
        raise ArgumentError(f"no method for {type(PA).__name__} * {type(PB).__name__}")
    if PA.device.type != "cuda":
        raise ArgumentError("sparse * sparse runs on the GPU only; adapt the matrices to CUDA first")
    wrapped = isinstance(A, Transpose) or isinstance(B, Transpose)
    if isinstance(PA, GenericSparseMatrixCOO):
        return GenericSparseMatrixCOO(_spgemm(GenericSparseMatrixCSC(A), GenericSparseMatrixCSC(B)))
    if not wrapped:
        return _spgemm(A, B)
    if isinstance(PA, GenericSparseMatrixCSR):
        return GenericSparseMatrixCSR(_spgemm(GenericSparseMatrixCSC(A), GenericSparseMatrixCSC(B)))
    return GenericSparseMatrixCSC(_spgemm(GenericSparseMatrixCSR(A), GenericSparseMatrixCSR(B)))


def mul(A, B):
    """``A * B`` for a sparse ``A``.  With a dense ``B`` (LinearAlgebra's generic ``*`` ->
    ``mul!``): a new column-major result with ``β = 0``.  With a sparse ``B``: the sparse
    product (SpGEMM)."""
    if _is_sparse_operand(B):
        return _sparse_mul(A, B)
    Ap, opA = _unwrap_sparse(A)
    Am = Ap.m if opA == _lib.OP_N else Ap.n
    _, _, _, Br, Bc = _dense_operand(B)
    Bt = B.parent if isinstance(B, Transpose) else B
    vec = isinstance(Bt, torch.Tensor) and Bt.dim() == 1 and not isinstance(B, Transpose)
    if vec:
        C = torch.empty(Am, dtype=Ap.dtype, device=Ap.device)
    else:
        C = torch.empty((Bc, Am), dtype=Ap.dtype, device=Ap.device).t()
    return mul_(C, A, B)


def dot(x: torch.Tensor, A, y: torch.Tensor):
    """Three-argument ``dot(x, A, y) = x' A y`` (LinearAlgebra.dot; the reference's methods at
    src/matrix_csr/matrix_csr.jl:213-277, src/matrix_csc/matrix_csc.jl:219,
    src/matrix_coo/matrix_coo.jl:227): the sum over stored entries of conj(x_l) a y_r.

    Same checks and messages as the reference (two ``DimensionMismatch``, then the backend
    ``ArgumentError``); the element type is the promotion of the three, as there.  Returns a
    numpy scalar; synchronizes the current stream (the reference returns the scalar to the
    host as well).
    """
    Ap, opA = _unwrap_sparse(A)
    if not isinstance(Ap, AbstractGenericSparseMatrix):
        raise ArgumentError("A must be a GenericSparseMatrixCSR/CSC/COO or its transpose/adjoint")
    if not isinstance(x, torch.Tensor) or not isinstance(y, torch.Tensor) or x.dim() != 1 or y.dim() != 1:
        raise ArgumentError("x and y must be torch vectors")
    Am, An = (Ap.m, Ap.n) if opA == _lib.OP_N else (Ap.n, Ap.m)
    if Am != x.shape[0]:
        raise DimensionMismatch(f"first dimension of A, {Am}, does not match the length of x, {x.shape[0]}")
    if An != y.shape[0]:
        raise DimensionMismatch(f"second dimension of A, {An}, does not match the length of y, {y.shape[0]}")
    if not (x.device == Ap.device == y.device):
        raise ArgumentError("All arrays must have the same backend")
    if Ap.device.type != "cuda":
        raise ArgumentError("dot runs on the GPU only; adapt the arrays to CUDA first")
    dt = torch.promote_types(torch.promote_types(Ap.dtype, x.dtype), y.dtype)
    if dt not in _DTYPE:
        raise ArgumentError(f"unsupported element type {dt}")
    val = Ap.nzval if Ap.dtype == dt else Ap.nzval.to(dt)
    xv = x.to(dt).contiguous()
    yv = y.to(dt).contiguous()
    lib = _lib.load()
    out = np.zeros(1, dtype=_NP_OF[dt])
    stream = _stream_ptr(Ap.device)
    with torch.cuda.device(Ap.device):
        if isinstance(Ap, GenericSparseMatrixCOO):
            cplan = _coo_plan(Ap)
            st = lib.gsa_coo_dot(stream, _DTYPE[dt], _ITYPE[Ap.itype], Ap.m, Ap.n, nnz(Ap), _ptr(Ap.rowind),
                                 _ptr(Ap.colind), _ptr(val), BASE, opA, _ptr(xv), _ptr(yv),
                                 out.ctypes.data_as(ctypes.c_void_p),
                                 ctypes.c_void_p(cplan.handle) if cplan is not None else None, None, 0)
        else:
            csr = isinstance(Ap, GenericSparseMatrixCSR)
            ptr, idx = (Ap.rowptr, Ap.colval) if csr else (Ap.colptr, Ap.rowval)
            plan = _gather_plan(Ap)
            fn = lib.gsa_csr_dot if csr else lib.gsa_csc_dot
            st = fn(stream, _DTYPE[dt], _ITYPE[Ap.itype], Ap.m, Ap.n, nnz(Ap), _ptr(ptr), _ptr(idx), _ptr(val),
                    BASE, opA, _ptr(xv), _ptr(yv), out.ctypes.data_as(ctypes.c_void_p),
                    ctypes.c_void_p(plan.handle) if plan is not None else None, None, 0)
    _lib.check(st)
    return out[0]


def dropzeros(A):
    """``dropzeros(A)``: a new matrix of A's format without the stored entries that are zero,
    in storage order (src/matrix_csr/matrix_csr.jl:723-745 and the CSC/COO methods)."""
    if not isinstance(A, AbstractGenericSparseMatrix):
        raise ArgumentError("A must be a GenericSparseMatrixCSR/CSC/COO")
    if A.device.type != "cuda":
        raise ArgumentError("dropzeros runs on the GPU only; adapt the matrix to CUDA first")
    lib = _lib.load()
    nz = nnz(A)
    ws = torch.empty(max(lib.gsa_dropzeros_workspace_size(nz), 1), dtype=torch.uint8, device=A.device)
    kept = ctypes.c_int64(0)
    stream = _stream_ptr(A.device)
    with torch.cuda.device(A.device):
        _lib.check(lib.gsa_dropzeros_count(stream, _DTYPE[A.dtype], nz, _ptr(A.nzval), _ptr(ws), ws.numel(),
                                           ctypes.byref(kept)))
        k = kept.value
        it, dev = A.itype, A.device
        if isinstance(A, GenericSparseMatrixCOO):
            fmt, outer, p0, p1 = 2, 0, A.rowind, A.colind
            o0 = torch.empty(k, dtype=it, device=dev)
        elif isinstance(A, GenericSparseMatrixCSR):
            fmt, outer, p0, p1 = 0, A.m, A.rowptr, A.colval
            o0 = torch.empty(A.m + 1, dtype=it, device=dev)
        else:
            fmt, outer, p0, p1 = 1, A.n, A.colptr, A.rowval
            o0 = torch.empty(A.n + 1, dtype=it, device=dev)
        o1 = torch.empty(k, dtype=it, device=dev)
        ov = torch.empty(k, dtype=A.dtype, device=dev)
        _lib.check(lib.gsa_dropzeros_copy(stream, fmt, _DTYPE[A.dtype], _ITYPE[it], outer, nz, _ptr(p0), _ptr(p1),
                                          _ptr(A.nzval), BASE, _ptr(ws), _ptr(o0), _ptr(o1), _ptr(ov)))
    return _owned(type(A), A.m, A.n, o0, o1, ov)


class UniformScaling:
    """``LinearAlgebra.UniformScaling``: ``λ * I`` of any square size."""

    def __init__(self, lam=1):
        self.lam = lam

    def __mul__(self, c):
        return UniformScaling(self.lam * c)

    __rmul__ = __mul__

    def __neg__(self):
        return UniformScaling(-self.lam)

    def __repr__(self):
        return f"UniformScaling({self.lam})"


I = UniformScaling(1)


def _coo_operand(X):
    """(parent COO, op code) of a COO matrix or its lazy Transpose / Adjoint, else None."""
    if isinstance(X, GenericSparseMatrixCOO):
        return X, _lib.OP_N
    if isinstance(X, Transpose) and isinstance(X.parent, GenericSparseMatrixCOO):
        conj = isinstance(X, Adjoint) and not _is_real(X.parent.dtype)
        return X.parent, _lib.OP_C if conj else _lib.OP_T
    return None


def _coo_sum(m: int, n: int, a, op_a: int, b=None, op_b: int = _lib.OP_N, n_diag: int = 0, lam=0,
             dtype=None):
    """The COO sum of (up to) two COO parents and n_diag diagonal entries of lam, zero sums
    dropped (gsa_coo_sum_count / _copy)."""
    lib = _lib.load()
    dev, it = a.device, a.itype
    dtype = dtype or a.dtype
    parts = []
    for X in (a, b):
        if X is None:
            parts.append((None, None, None, 0))
            continue
        val = X.nzval if X.dtype == dtype else X.nzval.to(dtype)
        r = X.rowind if X.itype == it else X.rowind.to(it)
        c = X.colind if X.itype == it else X.colind.to(it)
        parts.append((r, c, val, nnz(X)))
    total = parts[0][3] + parts[1][3] + n_diag
    ws = torch.empty(max(lib.gsa_coo_sum_workspace_size(_DTYPE[dtype], m, n, total), 1), dtype=torch.uint8, device=dev)
    lam_buf = _scalar_buf(lam, dtype)
    kept = ctypes.c_int64(0)
    stream = _stream_ptr(dev)
    (ra, ca, va, na), (rb, cb, vb, nb) = parts
    with torch.cuda.device(dev):
        _lib.check(lib.gsa_coo_sum_count(stream, _DTYPE[dtype], _ITYPE[it], m, n, na, _ptr(ra), _ptr(ca), _ptr(va),
                                         op_a, nb, _ptr(rb), _ptr(cb), _ptr(vb), op_b, n_diag,
                                         lam_buf.ctypes.data_as(ctypes.c_void_p), BASE,
                                         _ptr(ws), ws.numel(), ctypes.byref(kept)))
        k = kept.value
        ro = torch.empty(k, dtype=it, device=dev)
        co = torch.empty(k, dtype=it, device=dev)
        vo = torch.empty(k, dtype=dtype, device=dev)
        _lib.check(lib.gsa_coo_sum_copy(stream, _DTYPE[dtype], _ITYPE[it], m, n, total, k, BASE, _ptr(ws), _ptr(ro),
                                        _ptr(co), _ptr(vo)))
    return _owned(GenericSparseMatrixCOO, m, n, ro, co, vo)


def _compressed_sum(A, B=None, negate_b=False, lam=None):
    """A + B (two unwrapped CSR or two CSC matrices; dropzeros after, as the reference) or
    A + lam*I (B None; no dropzeros), through gsa_compressed_add_count / _copy."""
    csr = isinstance(A, GenericSparseMatrixCSR)
    cls = type(A)
    it, dev = A.itype, A.device
    outer = A.m if csr else A.n
    pa, ia = (A.rowptr, A.colval) if csr else (A.colptr, A.rowval)
    if B is not None:
        dtype = torch.promote_types(A.dtype, B.dtype)
        pb, ib = (B.rowptr, B.colval) if csr else (B.colptr, B.rowval)
        pb, ib, vb = pb.to(it), ib.to(it), B.nzval.to(dtype)
        lam_buf = None
    else:
        dtype = torch.result_type(A.nzval, lam)
        pb = ib = vb = None
        lam_buf = _scalar_buf(lam, dtype)
    va = A.nzval.to(dtype)
    lib = _lib.load()
    ws = torch.empty(max(lib.gsa_compressed_add_workspace_size(outer), 1), dtype=torch.uint8, device=dev)
    ptr = torch.empty(outer + 1, dtype=it, device=dev)
    cnt = ctypes.c_int64(0)
    stream = _stream_ptr(dev)
    with torch.cuda.device(dev):
        _lib.check(lib.gsa_compressed_add_count(stream, _ITYPE[it], outer, _ptr(pa), _ptr(ia), _ptr(pb), _ptr(ib),
                                                BASE, _ptr(ws), ws.numel(), _ptr(ptr), ctypes.byref(cnt)))
        idx = torch.empty(cnt.value, dtype=it, device=dev)
        val = torch.empty(cnt.value, dtype=dtype, device=dev)
        _lib.check(lib.gsa_compressed_add_copy(
            stream, _DTYPE[dtype], _ITYPE[it], outer, _ptr(pa), _ptr(ia), _ptr(va), _ptr(pb), _ptr(ib), _ptr(vb),
            1 if negate_b else 0, lam_buf.ctypes.data_as(ctypes.c_void_p) if lam_buf is not None else None, BASE,
            _ptr(ws), _ptr(idx), _ptr(val)))
    C = _owned(cls, A.m, A.n, ptr, idx, val)
    return dropzeros(C) if B is not None else C


def _neg_copy(X):
    """-X for an unwrapped sparse matrix (Base.:-, src/matrix_csr/matrix_csr.jl:88-90)."""
    return _same_structure(X, -X.nzval)


def _sparse_add(A, B, negate_b: bool):
    """Sparse + sparse and sparse + λI (src/matrix_coo/matrix_coo.jl:300-575,
    src/matrix_csr/matrix_csr.jl:290-458, src/matrix_csc/matrix_csc.jl:292-460)."""
    if isinstance(B, UniformScaling) or isinstance(A, UniformScaling):
        if isinstance(A, UniformScaling):  # J + A, J - A
            J, X, neg_x, neg_j = A, B, negate_b, False
        else:
            J, X, neg_x, neg_j = B, A, False, negate_b
        if isinstance(X, (GenericSparseMatrixCSR, GenericSparseMatrixCSC)):
            if X.m != X.n:
                raise DimensionMismatch("Matrix must be square to add UniformScaling.")
            lam = -J.lam if neg_j else J.lam
            Y = _neg_copy(X) if neg_x else X  # J - X = (-X) + J (src/core.jl:89,94)
            if lam == 0:  # iszero(λ) && return copy(A)
                return _same_structure(Y, Y.nzval.to(torch.result_type(Y.nzval, lam)).clone())
            if Y.device.type != "cuda":
                raise ArgumentError("sparse addition runs on the GPU only; adapt the matrix to CUDA first")
            return _compressed_sum(Y, lam=lam)
        op = _coo_operand(X)
        if op is None:
            raise ArgumentError("sparse + UniformScaling is provided for unwrapped CSR / CSC and COO matrices")
        P, code = op
        m, n = X.shape
        if m != n:
            raise DimensionMismatch("Matrix must be square to add UniformScaling.")
        lam = -J.lam if neg_j else J.lam
        dtype = torch.result_type(P.nzval, lam)  # a Python scalar keeps A's precision
        if lam == 0:  # iszero(λ) && return copy(A), A being -X for J - X
            m_, n_, r, c, v = _coo_parts(P, code, dtype)
            return GenericSparseMatrixCOO(m_, n_, r, c, -v if neg_x else v)
        if P.device.type != "cuda":
            raise ArgumentError("sparse addition runs on the GPU only; adapt the matrix to CUDA first")
        return _coo_sum(m, n, P, code | (_lib.SUM_NEGATE if neg_x else 0), n_diag=n, lam=lam, dtype=dtype)
    if not _is_sparse_operand(A) or not _is_sparse_operand(B):
        raise ArgumentError("A and B must be sparse matrices (or their transposes)")
    PA = A.parent if isinstance(A, Transpose) else A
    PB = B.parent if isinstance(B, Transpose) else B
    if isinstance(PA, (GenericSparseMatrixCSR, GenericSparseMatrixCSC)):
        if tuple(A.shape) != tuple(B.shape):
            raise DimensionMismatch(f"dimensions must match: A has dims ({A.shape[0]}, {A.shape[1]}), B has dims "
                                    f"({B.shape[0]}, {B.shape[1]})")
        if PA.device != PB.device:
            raise ArgumentError("Both matrices must have the same backend")
        if type(PA) is not type(PB):
            raise ArgumentError(f"no method for {type(PA).__name__} + {type(PB).__name__}")
        if PA.device.type != "cuda":
            raise ArgumentError("sparse addition runs on the GPU only; adapt the matrices to CUDA first")
        if not isinstance(A, Transpose) and not isinstance(B, Transpose):
            return _compressed_sum(A, B, negate_b)
        # transposed / adjoint pairs: to the other compressed format, add, convert back
        # (src/matrix_csr/matrix_csr.jl:405-436, src/matrix_csc/matrix_csc.jl:410-442)
        cls, other = type(PA), (GenericSparseMatrixCSC if isinstance(PA, GenericSparseMatrixCSR)
                                else GenericSparseMatrixCSR)
        return cls(_compressed_sum(other(A), other(B), negate_b))
    oa, ob = _coo_operand(A), _coo_operand(B)
    if oa is None or ob is None:
        raise ArgumentError("sparse + sparse needs two matrices of one format")
    if tuple(A.shape) != tuple(B.shape):
        raise DimensionMismatch(f"dimensions must match: A has dims ({A.shape[0]}, {A.shape[1]}), B has dims "
                                f"({B.shape[0]}, {B.shape[1]})")
    (PA, ca), (PB, cb) = oa, ob
    if PA.device != PB.device:
        raise ArgumentError("Both matrices must have the same backend")
    if PA.device.type != "cuda":
        raise ArgumentError("sparse addition runs on the GPU only; adapt the matrices to CUDA first")
    dtype = torch.promote_types(PA.dtype, PB.dtype)
    m, n = A.shape
    return _coo_sum(m, n, PA, ca, PB, cb | (_lib.SUM_NEGATE if negate_b else 0), dtype=dtype)


def _coo_parts(P, code, dtype):
    """copy(op(P)) as COO arrays (the reference's `iszero(λ) && return copy(A)`)."""
    r, c = (P.colind, P.rowind) if code != _lib.OP_N else (P.rowind, P.colind)
    v = P.nzval.to(dtype)
    if code == _lib.OP_C:
        v = v.conj().resolve_conj()
    m, n = (P.n, P.m) if code != _lib.OP_N else (P.m, P.n)
    return m, n, r, c, v


def subtract(A, B):
    """``A - B``: for COO matrices (and their transposes, and ``λ * I``) the sparse sum
    ``A + (-B)`` with zeros dropped (src/matrix_coo/matrix_coo.jl:572-574); for a dense ``B``
    the dense result ``A + (-B)``."""
    if isinstance(B, torch.Tensor):
        return add(A, -B)
    return _sparse_add(A, B, True)


def add(A, B):
    """``A + B``.  With a dense matrix ``B`` (src/core.jl:66-88): a new dense column-major
    ``C = copy(B)`` with every stored entry of ``A`` added (duplicates add up).  With COO
    matrices (or their lazy transposes / adjoints) on both sides, or a ``UniformScaling`` on
    one side (src/matrix_coo/matrix_coo.jl:300-575): a new COO holding the sum, column-major,
    entries at equal positions summed in order, zero sums dropped.  Same checks and messages
    as the reference: ``DimensionMismatch`` on sizes, then ``ArgumentError`` on backends."""
    if not isinstance(B, torch.Tensor):
        return _sparse_add(A, B, False)
    if not isinstance(A, AbstractGenericSparseMatrix):
        raise ArgumentError("A must be a GenericSparseMatrixCSR/CSC/COO")
    if not isinstance(B, torch.Tensor) or B.dim() != 2:
        raise ArgumentError("B must be a dense torch matrix")
    if (A.m, A.n) != tuple(B.shape):
        raise DimensionMismatch(f"dimensions must match: A has dims ({A.m}, {A.n}), B has dims "
                                f"({B.shape[0]}, {B.shape[1]})")
    if A.device != B.device:
        raise ArgumentError("Both arrays must have the same backend")
    if A.device.type != "cuda":
        raise ArgumentError("sparse + dense runs on the GPU only; adapt the arrays to CUDA first")
    if A.dtype != B.dtype:
        raise ArgumentError(f"element types of A ({A.dtype}) and B ({B.dtype}) must match")
    C = torch.empty((B.shape[1], B.shape[0]), dtype=B.dtype, device=B.device).t()  # column-major
    C.copy_(B)
    if isinstance(A, GenericSparseMatrixCOO):
        fmt, p0, p1 = 2, A.rowind, A.colind
    elif isinstance(A, GenericSparseMatrixCSR):
        fmt, p0, p1 = 0, A.rowptr, A.colval
    else:
        fmt, p0, p1 = 1, A.colptr, A.rowval
    with torch.cuda.device(A.device):
        st = _lib.load().gsa_add_to_dense(_stream_ptr(A.device), fmt, _DTYPE[A.dtype], _ITYPE[A.itype], A.m,
                                          A.n, nnz(A), _ptr(p0), _ptr(p1), _ptr(A.nzval), BASE, _ptr(C),
                                          max(C.stride(1), A.m, 1))
    _lib.check(st)
    return C


# ---------------------------------------------------------------------------
# Conversions (src/conversions/conversions.jl)

def _require_cuda(A):
    if A.device.type != "cuda":
        raise ArgumentError("format conversion runs on the GPU only; adapt the matrix to CUDA first")


def _coo_to_compressed(A: GenericSparseMatrixCOO, colmajor: bool):
    _require_cuda(A)
    lib = _lib.load()
    dev = A.device
    nz = nnz(A)
    major_n = A.n if colmajor else A.m
    ptr = torch.empty(major_n + 1, dtype=A.itype, device=dev)
    idx = torch.empty(nz, dtype=A.itype, device=dev)
    val = torch.empty(nz, dtype=A.dtype, device=dev)
    with torch.cuda.device(dev):
        ws_bytes = lib.gsa_coo_to_compressed_workspace_size(int(colmajor), _DTYPE[A.dtype],
                                                            _ITYPE[A.itype], A.m, A.n, nz)
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
        fn = lib.gsa_coo_to_csc if colmajor else lib.gsa_coo_to_csr
        st = fn(_stream_ptr(dev), _DTYPE[A.dtype], _ITYPE[A.itype], A.m, A.n, nz, _ptr(A.rowind),
                _ptr(A.colind), _ptr(A.nzval), BASE, _ptr(ptr), _ptr(idx), _ptr(val), _ptr(ws),
                ws.numel())
    _lib.check(st)
    return ptr, idx, val


def _compressed_to_coo(A, colmajor: bool):
    _require_cuda(A)
    lib = _lib.load()
    dev = A.device
    nz = nnz(A)
    ptr, idx = (A.colptr, A.rowval) if colmajor else (A.rowptr, A.colval)
    r = torch.empty(nz, dtype=A.itype, device=dev)
    c = torch.empty(nz, dtype=A.itype, device=dev)
    v = torch.empty(nz, dtype=A.dtype, device=dev)
    with torch.cuda.device(dev):
        fn = lib.gsa_csc_to_coo if colmajor else lib.gsa_csr_to_coo
        st = fn(_stream_ptr(dev), _DTYPE[A.dtype], _ITYPE[A.itype], A.m, A.n, nz, _ptr(ptr),
                _ptr(idx), _ptr(A.nzval), BASE, _ptr(r), _ptr(c), _ptr(v))
    _lib.check(st)
    return r, c, v


def _from_scipy(cls, S):
    import scipy.sparse as sp
    m, n = S.shape
    if cls is GenericSparseMatrixCSR:
        X = sp.csr_matrix(S)
        X.sort_indices()
        it = np.int64 if X.indptr.dtype == np.int64 else np.int32
        return GenericSparseMatrixCSR(m, n, X.indptr.astype(it) + 1, X.indices.astype(it) + 1, X.data)
    if cls is GenericSparseMatrixCSC:
        X = sp.csc_matrix(S)
        X.sort_indices()
        it = np.int64 if X.indptr.dtype == np.int64 else np.int32
        return GenericSparseMatrixCSC(m, n, X.indptr.astype(it) + 1, X.indices.astype(it) + 1, X.data)
    # COO from SparseMatrixCSC walks columns in order (src/matrix_coo/matrix_coo.jl:64-83)
    X = sp.csc_matrix(S)
    X.sort_indices()
    it = np.int64 if X.indptr.dtype == np.int64 else np.int32
    cols = np.repeat(np.arange(n, dtype=it), np.diff(X.indptr))
    return GenericSparseMatrixCOO(m, n, X.indices.astype(it) + 1, cols + 1, X.data)


def _convert_to(cls, A):
    """One-argument constructors of src/conversions/conversions.jl."""
    if isinstance(A, cls):
        return _same_structure(A, A.nzval) if cls is not GenericSparseMatrixCOO else A
    try:
        import scipy.sparse as sp
        if sp.issparse(A):
            return _from_scipy(cls, A)
    except ImportError:  # pragma: no cover
        pass
    if isinstance(A, Transpose):
        P = A.parent
        conj = isinstance(A, Adjoint) and P.dtype.is_complex
        val = (lambda v: v.conj().resolve_conj()) if conj else (lambda v: v)
        # conversions.jl:88-103,106-123: transpose(CSR) <-> CSC reuse the buffers
        if cls is GenericSparseMatrixCSC and isinstance(P, GenericSparseMatrixCSR):
            return GenericSparseMatrixCSC(P.n, P.m, P.rowptr, P.colval, val(P.nzval))
        if cls is GenericSparseMatrixCSR and isinstance(P, GenericSparseMatrixCSC):
            return GenericSparseMatrixCSR(P.n, P.m, P.colptr, P.rowval, val(P.nzval))
        # conversions.jl:125-147,214-258,325-346: COO of a transpose swaps the index arrays
        coo = P if isinstance(P, GenericSparseMatrixCOO) else GenericSparseMatrixCOO(P)
        T = GenericSparseMatrixCOO(coo.n, coo.m, coo.colind, coo.rowind, val(coo.nzval))
        return T if cls is GenericSparseMatrixCOO else cls(T)
    if cls is GenericSparseMatrixCOO:
        if isinstance(A, GenericSparseMatrixCSR):  # conversions.jl:264-280
            r, c, v = _compressed_to_coo(A, colmajor=False)
        elif isinstance(A, GenericSparseMatrixCSC):  # conversions.jl:153-169
            r, c, v = _compressed_to_coo(A, colmajor=True)
        else:
            raise ArgumentError(f"cannot convert {type(A).__name__} to COO")
        return _owned(GenericSparseMatrixCOO, A.m, A.n, r, c, v)
    if isinstance(A, (GenericSparseMatrixCSR, GenericSparseMatrixCSC)):
        # CSC <-> CSR through COO (conversions.jl:85-86,104-105)
        return cls(GenericSparseMatrixCOO(A))
    if isinstance(A, GenericSparseMatrixCOO):
        colmajor = cls is GenericSparseMatrixCSC
        ptr, idx, val = _coo_to_compressed(A, colmajor)  # conversions.jl:171-212 / 282-323
        return _owned(cls, A.m, A.n, ptr, idx, val)
    raise ArgumentError(f"cannot convert {type(A).__name__} to {cls.__name__}")


# ---------------------------------------------------------------------------
# Host views

def SparseMatrixCSC(A):
    """``SparseMatrixCSC(A)``: a scipy.sparse CSC matrix on the host (sums duplicates, as
    ``sparse(I, J, V)`` does for COO in the reference)."""
    import scipy.sparse as sp
    if isinstance(A, Transpose):
        S = SparseMatrixCSC(A.parent).T
        if isinstance(A, Adjoint):
            S = S.conj()
        return sp.csc_matrix(S)
    if isinstance(A, GenericSparseMatrixCSR):
        p, i, v = (t.cpu().numpy() for t in (A.rowptr, A.colval, A.nzval))
        return sp.csr_matrix((v, i - 1, p - 1), shape=A.shape).tocsc()
    if isinstance(A, GenericSparseMatrixCSC):
        p, i, v = (t.cpu().numpy() for t in (A.colptr, A.rowval, A.nzval))
        return sp.csc_matrix((v, i - 1, p - 1), shape=A.shape)
    if isinstance(A, GenericSparseMatrixCOO):
        r, c, v = (t.cpu().numpy() for t in (A.rowind, A.colind, A.nzval))
        return sp.coo_matrix((v, (r - 1, c - 1)), shape=A.shape).tocsc()
    raise ArgumentError(f"cannot convert {type(A).__name__}")


def collect(A) -> np.ndarray:
    """Dense host copy (``collect(A)``)."""
    if isinstance(A, torch.Tensor):
        return A.cpu().numpy()
    return SparseMatrixCSC(A).toarray()


def validate(A) -> None:
    """Device-side structure check (pointers monotone from 1 to nnz+1, indices in range);
    raises ``ArgumentError`` on a malformed matrix.  Synchronizes the stream."""
    if isinstance(A, GenericSparseMatrixCOO):
        r, c = A.rowind.cpu(), A.colind.cpu()
        if r.numel() and (int(r.min()) < 1 or int(r.max()) > A.m or int(c.min()) < 1 or
                          int(c.max()) > A.n):
            raise ArgumentError("COO index out of range")
        return
    _require_cuda(A)
    csr = isinstance(A, GenericSparseMatrixCSR)
    ptr, idx = (A.rowptr, A.colval) if csr else (A.colptr, A.rowval)
    outer, inner = (A.m, A.n) if csr else (A.n, A.m)
    lib = _lib.load()
    with torch.cuda.device(A.device):
        st = lib.gsa_validate_compressed(_stream_ptr(A.device), _ITYPE[A.itype], outer, inner,
                                         nnz(A), _ptr(ptr), _ptr(idx), BASE)
    _lib.check(st)
