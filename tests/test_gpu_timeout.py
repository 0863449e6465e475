"""Failure detection on the GPU without a fault: a bounded device-side wait that runs out.

The pipelined SpMV (GSA_ALGO_PIPE, and the no-allocation entry point built on it) waits on
mbarriers for the bulk copies of each tile.  Every such wait is bounded; with the bound set to
zero polls (GSA_TUNE_WAIT_LIMIT = 0) the first wait of every CTA gives up at once, the CTA lets
its copies in flight land, sets the device error word and returns.  The host then reads
GSA_ERR_TIMEOUT from gsa_check_device_status, the word is cleared, and the context stays
usable: the next call with the default bound gives the right product.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("entry", ["pipe", "noalloc"])
def test_wait_that_runs_out_reports_timeout_and_context_survives(gsa, oracle, cuda, entry):
    from genericsparsearrays_gb300 import workloads
    L = gsa._lib
    lib = L.load()
    m, n, rp, cv, nz = workloads.random_poisson(100_000, seed=5)
    nnz = int(cv.size)
    A = [torch.from_numpy(a).to(cuda) for a in (rp, cv, nz)]
    xh = np.random.default_rng(6).uniform(-1, 1, n)
    x = torch.from_numpy(xh).to(cuda)
    y = torch.zeros(m, dtype=torch.float64, device=cuda)
    one, zero = np.array([1.0]), np.array([0.0])
    ws_bytes = lib.gsa_mul_workspace_size(0, L.F64, L.IDX64, m, n, nnz, L.OP_N, 1, L.ALGO_PIPE)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=cuda)
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)

    def call():
        if entry == "pipe":
            return lib.gsa_csr_mul(stream, L.F64, L.IDX64, m, n, nnz, *(_ptr(a) for a in A), 1, L.OP_N, 1,
                                   _ptr(x), n, L.OP_N, _ptr(y), m, one.ctypes.data_as(ctypes.c_void_p),
                                   zero.ctypes.data_as(ctypes.c_void_p), L.ALGO_PIPE, _ptr(ws), ws.numel())
        return lib.gsa_csr_spmv_noalloc(stream, L.F64, L.IDX64, m, n, nnz, *(_ptr(a) for a in A), 1, _ptr(x),
                                        _ptr(y), one.ctypes.data_as(ctypes.c_void_p),
                                        zero.ctypes.data_as(ctypes.c_void_p))

    default = lib.gsa_get_tuning(L.TUNE_WAIT_LIMIT)
    assert default == 1 << 24
    assert lib.gsa_check_device_status(stream) == L.OK  # nothing pending from earlier tests
    try:
        assert lib.gsa_set_tuning(L.TUNE_WAIT_LIMIT, 0) == L.OK
        assert call() == L.OK  # the launch itself succeeds; the waits give up on the device
        assert lib.gsa_check_device_status(stream) == L.ERR_TIMEOUT
        assert "gave up" in L.last_error()
        assert lib.gsa_check_device_status(stream) == L.OK  # read once, then cleared
    finally:
        lib.gsa_set_tuning(L.TUNE_WAIT_LIMIT, default)
    # the context is usable and the same call now gives the right product
    assert call() == L.OK
    torch.cuda.synchronize()
    assert lib.gsa_check_device_status(stream) == L.OK
    ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, 1, xh, np.zeros(m))
    assert oracle.max_rel_error(y.cpu().numpy(), ye, sc) <= 1e-12
