"""gsa_csr_spmv_noalloc: the CSR SpMV entry point that allocates nothing.

It exists for callers that cannot allocate device memory when they need the product (a
process whose device memory is owned by another pool, or code that must not let an
allocation synchronize the device or run Julia's garbage collector); its scratch is a static
device array in the library.  This file is collected last so that a run stopping at the first
failure has run every other test already; it passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _regular(lib, L, stream, A, x, y, alpha, beta, dtype_code):
    ws_bytes = lib.gsa_mul_workspace_size(0, dtype_code, L.IDX64, A["m"], A["n"], A["nnz"], 0, 1, 0)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=y.device)
    st = lib.gsa_csr_mul(stream, dtype_code, L.IDX64, A["m"], A["n"], A["nnz"], _ptr(A["rowptr"]),
                         _ptr(A["colval"]), _ptr(A["nzval"]), 1, L.OP_N, 1, _ptr(x), A["n"], L.OP_N,
                         _ptr(y), A["m"], alpha.ctypes.data_as(ctypes.c_void_p),
                         beta.ctypes.data_as(ctypes.c_void_p), L.ALGO_AUTO, _ptr(ws), ws.numel())
    L.check(st)


def _noalloc(lib, L, stream, A, x, y, alpha, beta, dtype_code):
    st = lib.gsa_csr_spmv_noalloc(stream, dtype_code, L.IDX64, A["m"], A["n"], A["nnz"],
                                  _ptr(A["rowptr"]), _ptr(A["colval"]), _ptr(A["nzval"]), 1,
                                  _ptr(x), _ptr(y), alpha.ctypes.data_as(ctypes.c_void_p),
                                  beta.ctypes.data_as(ctypes.c_void_p))
    L.check(st)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_noalloc_matches_regular_entry_point(gsa, cuda, dt):
    """Two calls in a row through the C ABI; each equals gsa_csr_mul's result within the
    tests' FP64 tolerance (1e-12 of |alpha| sum|a||x| + |beta||y| per row)."""
    from genericsparsearrays_gb300 import workloads
    L = gsa._lib
    lib = L.load()
    code = L.F64 if dt == np.float64 else L.C64
    m, n, rp, cv, nz = workloads.power_law(200_000, seed=9, itype=np.int64, dtype=dt)
    dev = cuda
    A = {"m": m, "n": n, "nnz": int(cv.size), "rowptr": torch.from_numpy(rp).to(dev),
         "colval": torch.from_numpy(cv).to(dev), "nzval": torch.from_numpy(nz).to(dev)}
    rng = np.random.default_rng(10)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    import scipy.sparse as sp
    absA = sp.csr_matrix((np.abs(nz), cv - 1, rp - 1), shape=(m, n))
    for call in range(2):
        xh = rng.standard_normal(n).astype(dt)
        y0 = rng.standard_normal(m).astype(dt)
        alpha = np.array([1.5 if call == 0 else -0.25], dtype=dt)
        beta = np.array([0.5 if call == 0 else 0.0], dtype=dt)
        x = torch.from_numpy(xh).to(dev)
        y_ref = torch.from_numpy(y0.copy()).to(dev)
        y_new = torch.from_numpy(y0.copy()).to(dev)
        _regular(lib, L, stream, A, x, y_ref, alpha, beta, code)
        _noalloc(lib, L, stream, A, x, y_new, alpha, beta, code)
        torch.cuda.synchronize()
        # per-row scale |alpha| sum|a||x| + |beta||y0|
        scale = abs(alpha[0]) * (absA @ np.abs(xh)) + abs(beta[0]) * np.abs(y0)
        diff = np.abs(y_new.cpu().numpy() - y_ref.cpu().numpy())
        err = float(np.max(diff / np.where(scale > 0, scale, 1.0)))
        assert err <= 1e-12, f"call {call}: noalloc differs from gsa_csr_mul by {err:.3e}"
    st = lib.gsa_check_device_status(stream)
    assert st == 0, L.last_error()
