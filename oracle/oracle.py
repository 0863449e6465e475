"""CPU oracle for the sparse x dense mul! path and the COO <-> CSR/CSC conversions.

TEST INFRASTRUCTURE, NOT PRODUCT.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, and only to check results (or, for
the baseline, as the timed CPU restatement of the reference).  The CUDA library and
the ``genericsparsearrays_gb300`` package never import it.

The arithmetic lives in ``gsa_oracle.c`` / ``gsa_oracle_impl.h`` (plain C, built by
``build()`` below with ``-ffp-contract=off`` so that it rounds like Julia).  Each C
function cites the reference file:line it restates:

* ``mul``            -- ``LinearAlgebra.mul!`` for CSR/CSC/COO with identity, transpose
  and adjoint on A and B (src/matrix_csr/matrix_csr.jl:145-211,
  src/matrix_csc/matrix_csc.jl:144-213, src/matrix_coo/matrix_coo.jl:155-221 and the
  kernels in src/matrix_*/matrix_*_kernels.jl:1-45).
* ``mul_exact``      -- the same product in double-double plus the per-output scale
  ``|alpha| sum|a||b| + |beta||C0|`` that the tolerance is relative to.
* ``coo_to_csr`` / ``coo_to_csc`` -- src/conversions/conversions.jl:171-212,282-323.
* ``csr_to_coo`` / ``csc_to_coo`` -- src/conversions/conversion_kernels.jl:2-35.

Parity pin: Julia is not available to run the reference, so the restatement is
pinned against the reference's known-answer fixtures (tests/golden/) and checked
against scipy.sparse, which stands in for SparseArrays.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libgsa_oracle.so")
_SRC = [os.path.join(_HERE, "gsa_oracle.c"), os.path.join(_HERE, "gsa_oracle_impl.h")]
_lock = threading.Lock()
_lib = None

FMT = {"csr": 0, "csc": 1, "coo": 2}
OP = {"N": 0, "T": 1, "C": 2}
DTYPE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.complex64): 2,
         np.dtype(np.complex128): 3, np.dtype(np.int32): 4, np.dtype(np.int64): 5}
ITYPE = {np.dtype(np.int32): 0, np.dtype(np.int64): 1}


def build(force: bool = False) -> str:
    """Compile the C restatement into oracle/_build/libgsa_oracle.so (gcc, OpenMP)."""
    os.makedirs(_BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _SRC)
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < newest:
        tmp = _SO + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
               "-o", tmp, _SRC[0], "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_SO)
            i64, i32, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
            L.oracle_mul.argtypes = [i32, i32, i32, i32, i64, i64, i64, vp, vp, vp, i32,
                                     i64, vp, i64, i32, vp, i64, vp, vp, i32]
            L.oracle_mul_exact.argtypes = [i32, i32, i32, i32, i64, i64, i64, vp, vp, vp, i32,
                                           i64, vp, i64, i32, vp, i64, vp, vp, vp, vp, vp]
            L.oracle_coo_to_compressed.argtypes = [i32, i32, i32, i64, i64, i64, vp, vp, vp,
                                                   i32, vp, vp, vp]
            L.oracle_compressed_to_coo.argtypes = [i32, i32, i32, i64, i64, i64, vp, vp, vp,
                                                   i32, vp, vp, vp]
            L.oracle_dot.argtypes = [i32, i32, i32, i32, i64, i64, i64, vp, vp, vp, i32,
                                     vp, vp, vp, vp, vp, vp]
            L.oracle_coo_sum.argtypes = [i32, i32, i64, i64, i64, vp, vp, vp, i32, i64, vp, vp, vp, i32,
                                         i64, vp, i32, vp, vp, vp, ctypes.POINTER(i64)]
            L.oracle_spgemm.argtypes = [i32, i32, i32, i64, i64, i64, vp, vp, vp, vp, vp, vp, i32, vp, vp, vp, i64,
                                        ctypes.POINTER(i64)]
            L.oracle_compressed_add.argtypes = [i32, i32, i64, vp, vp, vp, vp, vp, vp, i32, i32, vp, vp, vp,
                                                ctypes.POINTER(i64)]
            L.oracle_compressed_add_diag.argtypes = [i32, i32, i64, vp, vp, vp, vp, i32, vp, vp, vp,
                                                     ctypes.POINTER(i64)]
            for f in ("oracle_mul", "oracle_mul_exact", "oracle_coo_to_compressed", "oracle_compressed_to_coo",
                      "oracle_max_threads", "oracle_dot", "oracle_coo_sum", "oracle_spgemm", "oracle_compressed_add",
                      "oracle_compressed_add_diag"):
                getattr(L, f).restype = ctypes.c_int
            _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else ctypes.c_void_p(0)


def _scalar(v, dtype):
    return np.array([v], dtype=dtype)


def _dense_parts(B, opB):
    """(array as Fortran-ordered 2-D view, ldb, rows_of_op(B), cols_of_op(B))."""
    B2 = B.reshape(-1, 1) if B.ndim == 1 else B
    B2 = np.asfortranarray(B2)
    ld = max(B2.shape[0], 1)
    if opB == "N":
        return B2, ld, B2.shape[0], B2.shape[1]
    return B2, ld, B2.shape[1], B2.shape[0]


def mul(fmt, opA, m, n, p0, p1, val, base, B, C, alpha=1, beta=0, opB="N", nthreads=1):
    """mul!(C, op(A), op(B), alpha, beta) on the CPU; C (1-D or Fortran 2-D) is updated in place.

    ``p0, p1`` are (rowptr, colval) for CSR, (colptr, rowval) for CSC and (rowind, colind)
    for COO, in index base ``base``.  Returns C.
    """
    val = np.ascontiguousarray(val)
    dt = val.dtype
    p0 = np.ascontiguousarray(p0)
    p1 = np.ascontiguousarray(p1, dtype=p0.dtype)
    B2, ldb, rb, k = _dense_parts(np.asarray(B, dtype=dt), opB)
    C2 = C.reshape(-1, 1) if C.ndim == 1 else C
    assert C2.flags.f_contiguous and C2.dtype == dt
    rows_out = m if opA == "N" else n
    assert C2.shape == (rows_out, k), (C2.shape, rows_out, k)
    assert rb == (n if opA == "N" else m)
    nnz = val.size
    al, be = _scalar(alpha, dt), _scalar(beta, dt)  # kept alive across the call
    rc = lib().oracle_mul(FMT[fmt], OP[opA], DTYPE[dt], ITYPE[p0.dtype], m, n, nnz,
                          _p(p0), _p(p1), _p(val), base, k, _p(B2), ldb, OP[opB],
                          _p(C2), max(C2.shape[0], 1), _p(al), _p(be), nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_mul failed: {rc}")
    return C


def mul_exact(fmt, opA, m, n, p0, p1, val, base, B, C0, alpha=1, beta=0, opB="N"):
    """Double-double product; returns (y, scale) with y complex128 or float64 and scale
    = |alpha| * sum|a||b| + |beta| * |C0| per output element (same shape as C0)."""
    val = np.ascontiguousarray(val)
    dt = val.dtype
    p0 = np.ascontiguousarray(p0)
    p1 = np.ascontiguousarray(p1, dtype=p0.dtype)
    B2, ldb, rb, k = _dense_parts(np.asarray(B, dtype=dt), opB)
    rows_out = m if opA == "N" else n
    C02 = np.asfortranarray((C0.reshape(-1, 1) if C0.ndim == 1 else C0).astype(dt))
    assert C02.shape == (rows_out, k)
    yre = np.zeros((rows_out, k), dtype=np.float64, order="F")
    yim = np.zeros((rows_out, k), dtype=np.float64, order="F")
    sc = np.zeros((rows_out, k), dtype=np.float64, order="F")
    al, be = _scalar(alpha, dt), _scalar(beta, dt)  # kept alive across the call
    rc = lib().oracle_mul_exact(FMT[fmt], OP[opA], DTYPE[dt], ITYPE[p0.dtype], m, n, val.size,
                                _p(p0), _p(p1), _p(val), base, k, _p(B2), ldb, OP[opB],
                                _p(C02), max(rows_out, 1), _p(al), _p(be), _p(yre), _p(yim),
                                _p(sc))
    if rc != 0:
        raise RuntimeError(f"oracle_mul_exact failed: {rc}")
    y = yre + 1j * yim if np.iscomplexobj(val) else yre
    if C0.ndim == 1:
        return y[:, 0], sc[:, 0]
    return y, sc


def dot(fmt, opA, m, n, p0, p1, val, base, x, y):
    """dot(x, op(A), y): returns (value in the reference's arithmetic with terms in storage
    order, double-double value as complex128/float64, scale sum|x||a||y|)."""
    val = np.ascontiguousarray(val)
    dt = val.dtype
    p0 = np.ascontiguousarray(p0)
    p1 = np.ascontiguousarray(p1, dtype=p0.dtype)
    x = np.ascontiguousarray(x, dtype=dt)
    y = np.ascontiguousarray(y, dtype=dt)
    out = np.zeros(1, dtype=dt)
    re, im, sc = (ctypes.c_double(0.0) for _ in range(3))
    rc = lib().oracle_dot(FMT[fmt], OP[opA], DTYPE[dt], ITYPE[p0.dtype], m, n, val.size, _p(p0),
                          _p(p1), _p(val), base, _p(x), _p(y), _p(out), ctypes.byref(re),
                          ctypes.byref(im), ctypes.byref(sc))
    if rc != 0:
        raise RuntimeError(f"oracle_dot failed: {rc}")
    exact = complex(re.value, im.value) if np.iscomplexobj(val) else re.value
    return out[0], exact, sc.value


def _coo_to(colmajor, m, n, rowind, colind, val, base):
    rowind = np.ascontiguousarray(rowind)
    colind = np.ascontiguousarray(colind, dtype=rowind.dtype)
    val = np.ascontiguousarray(val)
    nnz = val.size
    major_n = n if colmajor else m
    ptr = np.empty(major_n + 1, dtype=rowind.dtype)
    idx = np.empty(nnz, dtype=rowind.dtype)
    out = np.empty(nnz, dtype=val.dtype)
    rc = lib().oracle_coo_to_compressed(colmajor, DTYPE[val.dtype], ITYPE[rowind.dtype], m, n,
                                        nnz, _p(rowind), _p(colind), _p(val), base, _p(ptr),
                                        _p(idx), _p(out))
    if rc != 0:
        raise RuntimeError(f"oracle_coo_to_compressed failed: {rc}")
    return ptr, idx, out


def coo_to_csr(m, n, rowind, colind, val, base=1):
    """GenericSparseMatrixCSR(::GenericSparseMatrixCOO) -> (rowptr, colval, nzval)."""
    return _coo_to(0, m, n, rowind, colind, val, base)


def coo_to_csc(m, n, rowind, colind, val, base=1):
    """GenericSparseMatrixCSC(::GenericSparseMatrixCOO) -> (colptr, rowval, nzval)."""
    return _coo_to(1, m, n, rowind, colind, val, base)


def _to_coo(colmajor, m, n, ptr, idx, val, base):
    ptr = np.ascontiguousarray(ptr)
    idx = np.ascontiguousarray(idx, dtype=ptr.dtype)
    val = np.ascontiguousarray(val)
    nnz = val.size
    r = np.empty(nnz, dtype=ptr.dtype)
    c = np.empty(nnz, dtype=ptr.dtype)
    v = np.empty(nnz, dtype=val.dtype)
    rc = lib().oracle_compressed_to_coo(colmajor, DTYPE[val.dtype], ITYPE[ptr.dtype], m, n, nnz,
                                        _p(ptr), _p(idx), _p(val), base, _p(r), _p(c), _p(v))
    if rc != 0:
        raise RuntimeError(f"oracle_compressed_to_coo failed: {rc}")
    return r, c, v


def csr_to_coo(m, n, rowptr, colval, nzval, base=1):
    """GenericSparseMatrixCOO(::GenericSparseMatrixCSR) -> (rowind, colind, nzval)."""
    return _to_coo(0, m, n, rowptr, colval, nzval, base)


def csc_to_coo(m, n, colptr, rowval, nzval, base=1):
    """GenericSparseMatrixCOO(::GenericSparseMatrixCSC) -> (rowind, colind, nzval)."""
    return _to_coo(1, m, n, colptr, rowval, nzval, base)


_OPS = {"N": 0, "T": 1, "C": 2}


def coo_sum(m, n, a, op_a="N", b=None, op_b="N", neg_b=False, n_diag=0, lam=0, base=1, neg_a=False):
    """Base.:+ of COO matrices (A + B, A - B with neg_b, -A + lam*I with neg_a, A + lam*I with n_diag = n), dropzeros
    included: a and b are (rowind, colind, nzval) triplets of the stored (parent) matrices,
    op_a / op_b "N", "T" or "C".  Returns the result's (rowind, colind, nzval), column-major."""
    ra, ca, va = (np.ascontiguousarray(x) for x in a)
    ca = ca.astype(ra.dtype, copy=False)
    if b is None:
        rb = cb = np.empty(0, dtype=ra.dtype)
        vb = np.empty(0, dtype=va.dtype)
    else:
        rb, cb, vb = (np.ascontiguousarray(x) for x in b)
        rb, cb = rb.astype(ra.dtype, copy=False), cb.astype(ra.dtype, copy=False)
    vb = vb.astype(va.dtype, copy=False)
    total = va.size + vb.size + n_diag
    r = np.empty(max(total, 1), dtype=ra.dtype)
    c = np.empty(max(total, 1), dtype=ra.dtype)
    v = np.empty(max(total, 1), dtype=va.dtype)
    lamv = np.array([lam], dtype=va.dtype)
    kept = ctypes.c_int64(0)
    rc = lib().oracle_coo_sum(DTYPE[va.dtype], ITYPE[ra.dtype], m, n, va.size, _p(ra), _p(ca), _p(va),
                              _OPS[op_a] | (4 if neg_a else 0), vb.size, _p(rb), _p(cb), _p(vb), _OPS[op_b] | (4 if neg_b else 0),
                              n_diag, _p(lamv), base, _p(r), _p(c), _p(v), ctypes.byref(kept))
    if rc != 0:
        raise RuntimeError(f"oracle_coo_sum failed: {rc}")
    k = kept.value
    return r[:k].copy(), c[:k].copy(), v[:k].copy()


def spgemm(fmt, m, kk, n, a, b, base=1):
    """A * B for CSR (fmt "csr": a, b = (rowptr, colval, nzval)) or CSC (fmt "csc": (colptr,
    rowval, nzval)) operands of sizes m x kk and kk x n, restating the reference's kernels.
    Returns the product's (ptr, idx, val); zero sums stay stored."""
    pa, ia, va = (np.ascontiguousarray(x) for x in a)
    pb, ib, vb = (np.ascontiguousarray(x) for x in b)
    ia, pb, ib = ia.astype(pa.dtype, copy=False), pb.astype(pa.dtype, copy=False), ib.astype(pa.dtype, copy=False)
    vb = vb.astype(va.dtype, copy=False)
    f = 0 if fmt == "csr" else 1
    outer = m if f == 0 else n
    ptr = np.empty(outer + 1, dtype=pa.dtype)
    cnt = ctypes.c_int64(0)
    args = (f, DTYPE[va.dtype], ITYPE[pa.dtype], m, kk, n, _p(pa), _p(ia), _p(va), _p(pb), _p(ib), _p(vb), base)
    rc = lib().oracle_spgemm(*args, _p(ptr), ctypes.c_void_p(0), ctypes.c_void_p(0), 0, ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"oracle_spgemm failed: {rc}")
    idx = np.empty(max(cnt.value, 1), dtype=pa.dtype)
    val = np.empty(max(cnt.value, 1), dtype=va.dtype)
    rc = lib().oracle_spgemm(*args, _p(ptr), _p(idx), _p(val), idx.size, ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"oracle_spgemm failed: {rc}")
    return ptr, idx[:cnt.value].copy(), val[:cnt.value].copy()


def compressed_add(outer_n, a, b, neg_b=False, base=1):
    """CSR + CSR (or CSC + CSC) as the reference computes it: a, b = (ptr, idx, val); the
    result's (ptr, idx, val) after dropzeros."""
    pa, ia, va = (np.ascontiguousarray(x) for x in a)
    pb, ib, vb = (np.ascontiguousarray(x) for x in b)
    ia, pb, ib = ia.astype(pa.dtype, copy=False), pb.astype(pa.dtype, copy=False), ib.astype(pa.dtype, copy=False)
    vb = vb.astype(va.dtype, copy=False)
    ptr = np.empty(outer_n + 1, dtype=pa.dtype)
    idx = np.empty(max(va.size + vb.size, 1), dtype=pa.dtype)
    val = np.empty(max(va.size + vb.size, 1), dtype=va.dtype)
    cnt = ctypes.c_int64(0)
    rc = lib().oracle_compressed_add(DTYPE[va.dtype], ITYPE[pa.dtype], outer_n, _p(pa), _p(ia), _p(va), _p(pb),
                                     _p(ib), _p(vb), 1 if neg_b else 0, base, _p(ptr), _p(idx), _p(val),
                                     ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"oracle_compressed_add failed: {rc}")
    return ptr, idx[:cnt.value].copy(), val[:cnt.value].copy()


def compressed_add_diag(n, a, lam, base=1):
    """CSR + lam*I (or CSC + lam*I) as the reference computes it; no dropzeros."""
    pa, ia, va = (np.ascontiguousarray(x) for x in a)
    ia = ia.astype(pa.dtype, copy=False)
    ptr = np.empty(n + 1, dtype=pa.dtype)
    idx = np.empty(va.size + n + 1, dtype=pa.dtype)
    val = np.empty(va.size + n + 1, dtype=va.dtype)
    lv = np.array([lam], dtype=va.dtype)
    cnt = ctypes.c_int64(0)
    rc = lib().oracle_compressed_add_diag(DTYPE[va.dtype], ITYPE[pa.dtype], n, _p(pa), _p(ia), _p(va), _p(lv), base,
                                          _p(ptr), _p(idx), _p(val), ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"oracle_compressed_add_diag failed: {rc}")
    return ptr, idx[:cnt.value].copy(), val[:cnt.value].copy()


def max_rel_error(y, y_exact, scale):
    """max_i |y_i - y_exact_i| / scale_i (scale 0 -> absolute error)."""
    y = np.asarray(y).astype(np.complex128 if np.iscomplexobj(y) else np.float64)
    err = np.abs(y - y_exact)
    s = np.where(scale > 0, scale, 1.0)
    return float(np.max(err / s)) if err.size else 0.0
