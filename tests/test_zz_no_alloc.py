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
    ws_bytes = lib.gsa_mul_workspace_size(0, dtype_code, A["itype"], A["m"], A["n"], A["nnz"], 0, 1, 0)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=y.device)
    st = lib.gsa_csr_mul(stream, dtype_code, A["itype"], A["m"], A["n"], A["nnz"], _ptr(A["rowptr"]),
                         _ptr(A["colval"]), _ptr(A["nzval"]), A["base"], L.OP_N, 1, _ptr(x), A["n"], L.OP_N,
                         _ptr(y), A["m"], alpha.ctypes.data_as(ctypes.c_void_p),
                         beta.ctypes.data_as(ctypes.c_void_p), L.ALGO_AUTO, _ptr(ws), ws.numel())
    L.check(st)


def _noalloc(lib, L, stream, A, x, y, alpha, beta, dtype_code):
    return lib.gsa_csr_spmv_noalloc(stream, dtype_code, A["itype"], A["m"], A["n"], A["nnz"],
                                    _ptr(A["rowptr"]), _ptr(A["colval"]), _ptr(A["nzval"]), A["base"],
                                    _ptr(x), _ptr(y), alpha.ctypes.data_as(ctypes.c_void_p),
                                    beta.ctypes.data_as(ctypes.c_void_p))


CASES = [(np.float64, np.int64, 1, 512), (np.complex128, np.int64, 1, 512), (np.float64, np.int32, 0, 512),
         (np.complex128, np.int32, 1, 256), (np.float64, np.int64, 0, 256)]


@pytest.mark.parametrize("dt,it,base,threads", CASES)
def test_noalloc_matches_regular_entry_point_and_oracle(gsa, oracle, cuda, dt, it, base, threads):
    """Two calls in a row through the C ABI; each equals gsa_csr_mul's result and the
    double-double oracle's within the tests' FP64 tolerance (1e-12 of |alpha| sum|a||x| +
    |beta||y| per row), for Int32 and Int64 indices, 0- and 1-based buffers and both CTA sizes
    of the pipelined kernel.  The second call leaves the device's free memory unchanged."""
    from genericsparsearrays_gb300 import workloads
    L = gsa._lib
    lib = L.load()
    code = L.F64 if dt == np.float64 else L.C64
    m, n, rp, cv, nz = workloads.power_law(200_000, seed=9, itype=it, dtype=dt)
    rp, cv = rp - (1 - base), cv - (1 - base)
    dev = cuda
    A = {"m": m, "n": n, "nnz": int(cv.size), "rowptr": torch.from_numpy(rp).to(dev), "base": base,
         "colval": torch.from_numpy(cv).to(dev), "nzval": torch.from_numpy(nz).to(dev),
         "itype": L.IDX32 if it == np.int32 else L.IDX64}
    rng = np.random.default_rng(10)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    saved = lib.gsa_get_tuning(L.TUNE_PIPE_THREADS)
    assert lib.gsa_set_tuning(L.TUNE_PIPE_THREADS, threads) == L.OK
    try:
        calls = []
        for call in range(2):
            xh = rng.standard_normal(n).astype(dt)
            y0 = rng.standard_normal(m).astype(dt)
            alpha = np.array([1.5 if call == 0 else -0.25], dtype=dt)
            beta = np.array([0.5 if call == 0 else 0.0], dtype=dt)
            calls.append((xh, y0, alpha, beta, torch.from_numpy(xh).to(dev), torch.from_numpy(y0.copy()).to(dev),
                          torch.from_numpy(y0.copy()).to(dev)))
        torch.cuda.synchronize()
        for call, (xh, y0, alpha, beta, x, y_ref, y_new) in enumerate(calls):
            _regular(lib, L, stream, A, x, y_ref, alpha, beta, code)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info(dev)[0]
            L.check(_noalloc(lib, L, stream, A, x, y_new, alpha, beta, code))
            torch.cuda.synchronize()
            free_after = torch.cuda.mem_get_info(dev)[0]
            if call == 1:
                assert free_after == free_before, "the second noalloc call changed the device's free memory"
            ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, base, xh, y0, alpha[0], beta[0])
            got = y_new.cpu().numpy()
            err_oracle = oracle.max_rel_error(got, ye, sc)
            diff = np.abs(got - y_ref.cpu().numpy())
            err_regular = float(np.max(diff / np.where(sc > 0, sc, 1.0)))
            assert err_oracle <= 1e-12, f"call {call}: noalloc vs oracle {err_oracle:.3e}"
            assert err_regular <= 1e-12, f"call {call}: noalloc differs from gsa_csr_mul by {err_regular:.3e}"
    finally:
        lib.gsa_set_tuning(L.TUNE_PIPE_THREADS, saved)
    st = lib.gsa_check_device_status(stream)
    assert st == 0, L.last_error()


def test_noalloc_empty_and_invalid(gsa, cuda):
    """m == 0 returns at once; a NULL pointer and an unknown dtype are rejected before any launch."""
    L = gsa._lib
    lib = L.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    rp = torch.ones(4, dtype=torch.int64, device=cuda)  # a valid empty 3-row structure
    one, zero = np.array([1.0]), np.array([0.0])
    a, b = one.ctypes.data_as(ctypes.c_void_p), zero.ctypes.data_as(ctypes.c_void_p)
    x = torch.zeros(4, dtype=torch.float64, device=cuda)
    assert lib.gsa_csr_spmv_noalloc(stream, L.F64, L.IDX64, 0, 4, 0, _ptr(rp), None, None, 1, _ptr(x), None,
                                    a, b) == L.OK
    assert lib.gsa_csr_spmv_noalloc(stream, L.F64, L.IDX64, 3, 4, 0, None, None, None, 1, _ptr(x), _ptr(x),
                                    a, b) == L.ERR_INVALID_ARG
    assert lib.gsa_csr_spmv_noalloc(stream, 17, L.IDX64, 3, 4, 0, _ptr(rp), None, None, 1, _ptr(x), _ptr(x),
                                    a, b) != L.OK
    torch.cuda.synchronize()
