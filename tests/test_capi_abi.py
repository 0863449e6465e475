"""libgsa.so loads, exports every symbol include/gsa.h declares, and rejects bad arguments
before touching the GPU (CPU only: no compute call is made here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gsa.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gsa_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib(gsa):
    return gsa._lib.load()


def test_every_declared_symbol_is_exported(lib, gsa):
    names = declared_functions()
    assert len(names) >= 12
    for name in names:
        assert hasattr(lib, name), f"{name} declared in gsa.h but not exported"
        assert name in gsa._lib.SIGNATURES, f"{name} has no ctypes signature"


def test_version_and_error_string(lib):
    assert lib.gsa_version() == 100
    assert isinstance(lib.gsa_last_error_string(), bytes)


def _mul_call(lib, **kw):
    a = dict(stream=None, dtype=1, itype=0, m=4, n=3, nnz=0, p0=None, p1=None, v=None, base=1,
             opA=0, k=1, B=None, ldb=3, opB=0, C=None, ldc=4)
    a.update(kw)
    one = np.array([1.0])
    zero = np.array([0.0])
    return lib.gsa_csr_mul(a["stream"], a["dtype"], a["itype"], a["m"], a["n"], a["nnz"], a["p0"],
                           a["p1"], a["v"], a["base"], a["opA"], a["k"], a["B"], a["ldb"], a["opB"],
                           a["C"], a["ldc"], one.ctypes.data_as(ctypes.c_void_p),
                           zero.ctypes.data_as(ctypes.c_void_p), 0, None, 0)


def test_argument_checks_precede_gpu_work(lib, gsa):
    L = gsa._lib
    assert _mul_call(lib, dtype=99) == L.ERR_UNSUPPORTED
    assert b"unsupported dtype" in lib.gsa_last_error_string()
    assert _mul_call(lib, itype=7) == L.ERR_UNSUPPORTED
    assert _mul_call(lib, opA=5) == L.ERR_INVALID_ARG
    assert _mul_call(lib, m=-1) == L.ERR_INVALID_ARG
    assert _mul_call(lib, ldb=2) == L.ERR_DIM  # op(A) is 4x3 -> B needs ldb >= 3
    assert _mul_call(lib, ldc=3) == L.ERR_DIM  # C needs ldc >= 4
    assert _mul_call(lib, opA=1, ldb=3) == L.ERR_DIM  # op(A) 3x4 -> B needs ldb >= 4
    # misaligned dense operand (an odd address)
    assert _mul_call(lib, B=ctypes.c_void_p(8 * 1000 + 4), C=ctypes.c_void_p(8 * 2000)) == L.ERR_INVALID_ARG
    assert b"aligned" in lib.gsa_last_error_string()


def test_workspace_size_queries(lib):
    # gather (CSR, opA = N): the default row-block kernel and the vector kernel need none,
    # merge-path tiles need coordinates + carries, the pipelined kernel carries per CTA run;
    # scatter (CSR, opA = T): none for the default outer blocks, tile coordinates for merge
    auto = lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 0, 1, 0)
    g = lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 0, 1, 1)
    p = lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 0, 1, 3)
    s = lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 1, 1, 0)
    sm = lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 1, 1, 1)
    v = lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 0, 1, 2)
    assert auto == 0 and v == 0 and g > 0 and p > 0 and s == 0 and sm > 0
    assert lib.gsa_mul_workspace_size(0, 1, 0, 1000, 1000, 5000, 0, 16, 1) > g
    assert lib.gsa_mul_workspace_size(0, 99, 0, 10, 10, 5, 0, 1, 0) == 0
    # bucket sort: two 8-byte keys per entry, counters per row
    w = lib.gsa_coo_to_compressed_workspace_size(0, 1, 0, 1000, 1000, 5000)
    assert w >= 5000 * 16 + 1000 * 8
    assert lib.gsa_coo_to_compressed_workspace_size(0, 1, 0, 10, 10, 0) == 0


def test_dot_argument_checks(lib, gsa):
    L = gsa._lib
    out = np.zeros(1)
    res = out.ctypes.data_as(ctypes.c_void_p)
    fake = ctypes.c_void_p(8 * 4096)  # never dereferenced: the checks fail first
    # NULL result
    assert lib.gsa_csr_dot(None, 1, 0, 4, 3, 0, fake, None, None, 1, 0, fake, fake, None, None, None, 0) \
        == L.ERR_INVALID_ARG
    # bad op, bad dtype, negative size, NULL vectors
    assert lib.gsa_csr_dot(None, 1, 0, 4, 3, 0, fake, None, None, 1, 7, fake, fake, res, None, None, 0) \
        == L.ERR_INVALID_ARG
    assert lib.gsa_coo_dot(None, 99, 0, 4, 3, 0, None, None, None, 1, 0, fake, fake, res, None, None, 0) \
        == L.ERR_UNSUPPORTED
    assert lib.gsa_csc_dot(None, 1, 0, -1, 3, 0, fake, None, None, 1, 0, fake, fake, res, None, None, 0) \
        == L.ERR_INVALID_ARG
    assert lib.gsa_csr_dot(None, 1, 0, 4, 3, 0, fake, None, None, 1, 0, None, fake, res, None, None, 0) \
        == L.ERR_INVALID_ARG
    # Int32 structures hold at most 2^31 - 1 entries
    assert lib.gsa_csr_dot(None, 1, 0, 4, 3, 2**31, fake, fake, fake, 1, 0, fake, fake, res, None, None, 0) \
        == L.ERR_INVALID_ARG
    assert lib.gsa_dot_workspace_size(2, 1, 0, 10, 10, None) > 0
    assert lib.gsa_dot_workspace_size(0, 3, 1, 1000, 10, None) >= (1000 // 128 + 1) * 4 * 16
    assert lib.gsa_dot_workspace_size(5, 1, 0, 10, 10, None) == 0


def test_sum_and_spgemm_argument_checks(lib, gsa):
    """The COO sum, compressed sum and SpGEMM entry points refuse bad arguments before any
    device work (no GPU needed)."""
    L = gsa._lib
    fake = ctypes.c_void_p(8 * 4096)  # never dereferenced: the checks fail first
    kept = ctypes.c_int64(0)
    lam = np.ones(1).ctypes.data_as(ctypes.c_void_p)
    # COO sum: bad op code, n_diag beyond min(m, n), lambda missing, unsupported dtype
    assert lib.gsa_coo_sum_count(None, 1, 1, 4, 4, 1, fake, fake, fake, 7, 0, None, None, None, 0, 0, None, 1,
                                 fake, 1 << 20, ctypes.byref(kept)) == L.ERR_INVALID_ARG
    assert lib.gsa_coo_sum_count(None, 1, 1, 4, 3, 0, None, None, None, 0, 0, None, None, None, 0, 4, lam, 1,
                                 fake, 1 << 20, ctypes.byref(kept)) == L.ERR_DIM
    assert lib.gsa_coo_sum_count(None, 1, 1, 4, 4, 0, None, None, None, 0, 0, None, None, None, 0, 4, None, 1,
                                 fake, 1 << 20, ctypes.byref(kept)) == L.ERR_INVALID_ARG
    assert lib.gsa_coo_sum_count(None, 9, 1, 4, 4, 0, None, None, None, 0, 0, None, None, None, 0, 0, None, 1,
                                 fake, 1 << 20, ctypes.byref(kept)) == L.ERR_UNSUPPORTED
    assert lib.gsa_coo_sum_copy(None, 1, 1, 4, 4, 3, 5, 1, fake, None, None, None) == L.ERR_INVALID_ARG  # kept > total
    assert lib.gsa_coo_sum_workspace_size(1, 4, 4, 10) > 0 and lib.gsa_coo_sum_workspace_size(9, 4, 4, 10) == 0
    # compressed sum: NULL pointers, a workspace too small, no B and no lambda
    nnz = ctypes.c_int64(0)
    assert lib.gsa_compressed_add_count(None, 1, 4, None, None, None, None, 1, fake, 1 << 20, fake,
                                        ctypes.byref(nnz)) == L.ERR_INVALID_ARG
    assert lib.gsa_compressed_add_count(None, 1, 1000, fake, fake, fake, fake, 1, fake, 16, fake,
                                        ctypes.byref(nnz)) == L.ERR_INVALID_ARG
    assert lib.gsa_compressed_add_copy(None, 1, 1, 4, fake, fake, fake, None, None, None, 0, None, 1, fake, fake,
                                       fake) == L.ERR_INVALID_ARG
    assert lib.gsa_compressed_add_workspace_size(1000) >= 2 * 1001 * 4
    # SpGEMM: bad format, NULL handle, negative size; destroy(NULL) is a no-op
    h = ctypes.c_void_p(0)
    args = (fake, fake, fake, 4, fake, fake, fake, 4, 1, fake, ctypes.byref(nnz), ctypes.byref(h))
    assert lib.gsa_spgemm_create(None, 2, 1, 1, 4, 4, 4, *args) == L.ERR_INVALID_ARG
    assert lib.gsa_spgemm_create(None, 0, 1, 1, -4, 4, 4, *args) == L.ERR_INVALID_ARG
    assert lib.gsa_spgemm_create(None, 0, 9, 1, 4, 4, 4, *args) == L.ERR_UNSUPPORTED
    assert h.value is None
    assert lib.gsa_spgemm_compute(None, None, fake, fake) == L.ERR_INVALID_ARG
    assert lib.gsa_spgemm_destroy(None) == 0


def test_tuning_knobs(lib, gsa):
    """gsa_set_tuning / gsa_get_tuning round trip, reject bad values and keys, and stay
    consistent when several host threads set them at once (the knobs are process-wide)."""
    import threading
    L = gsa._lib
    keys = (L.TUNE_PIPE_THREADS, L.TUNE_SPMM_COLUMNS, L.TUNE_PLAN_ORDER, L.TUNE_WAIT_LIMIT, L.TUNE_STAGE_ROWS,
            L.TUNE_X_PAIRS, L.TUNE_SORT_STAGED)
    saved = {key: lib.gsa_get_tuning(key) for key in keys}
    try:
        assert lib.gsa_set_tuning(L.TUNE_SPMM_COLUMNS, 4) == 0
        assert lib.gsa_get_tuning(L.TUNE_SPMM_COLUMNS) == 4
        assert lib.gsa_set_tuning(L.TUNE_SPMM_COLUMNS, 3) == L.ERR_INVALID_ARG
        assert lib.gsa_get_tuning(L.TUNE_SPMM_COLUMNS) == 4
        assert lib.gsa_set_tuning(L.TUNE_PLAN_ORDER, 1) == 0
        assert lib.gsa_get_tuning(L.TUNE_PLAN_ORDER) == 1
        assert lib.gsa_set_tuning(L.TUNE_PLAN_ORDER, 2) == 0 and lib.gsa_get_tuning(L.TUNE_PLAN_ORDER) == 2
        assert lib.gsa_set_tuning(L.TUNE_PLAN_ORDER, 3) == L.ERR_INVALID_ARG
        assert lib.gsa_get_tuning(L.TUNE_WAIT_LIMIT) == saved[L.TUNE_WAIT_LIMIT] == 1 << 24
        assert lib.gsa_get_tuning(L.TUNE_STAGE_ROWS) == saved[L.TUNE_STAGE_ROWS] == 0
        assert lib.gsa_set_tuning(L.TUNE_STAGE_ROWS, 1) == 0
        assert lib.gsa_get_tuning(L.TUNE_STAGE_ROWS) == 1
        assert lib.gsa_set_tuning(L.TUNE_STAGE_ROWS, 3) == L.ERR_INVALID_ARG
        assert lib.gsa_get_tuning(L.TUNE_X_PAIRS) == saved[L.TUNE_X_PAIRS] == 1
        assert lib.gsa_set_tuning(L.TUNE_X_PAIRS, 0) == 0 and lib.gsa_get_tuning(L.TUNE_X_PAIRS) == 0
        assert lib.gsa_set_tuning(L.TUNE_X_PAIRS, 3) == L.ERR_INVALID_ARG
        assert lib.gsa_get_tuning(L.TUNE_SORT_STAGED) == saved[L.TUNE_SORT_STAGED] == 1
        assert lib.gsa_set_tuning(L.TUNE_SORT_STAGED, 0) == 0 and lib.gsa_get_tuning(L.TUNE_SORT_STAGED) == 0
        assert lib.gsa_set_tuning(L.TUNE_SORT_STAGED, 2) == L.ERR_INVALID_ARG
        assert lib.gsa_set_tuning(L.TUNE_WAIT_LIMIT, 0) == 0
        assert lib.gsa_get_tuning(L.TUNE_WAIT_LIMIT) == 0
        assert lib.gsa_set_tuning(L.TUNE_WAIT_LIMIT, -1) == L.ERR_INVALID_ARG
        assert lib.gsa_get_tuning(L.TUNE_WAIT_LIMIT) == 0
        assert lib.gsa_set_tuning(999, 0) == L.ERR_INVALID_ARG
        assert lib.gsa_get_tuning(999) == -1

        values = (1, 2, 4, 8)
        errors = []

        def setter(t):
            for i in range(2000):
                if lib.gsa_set_tuning(L.TUNE_SPMM_COLUMNS, values[(t + i) % 4]) != 0:
                    errors.append(t)
                if lib.gsa_get_tuning(L.TUNE_SPMM_COLUMNS) not in values:
                    errors.append(-t)

        threads = [threading.Thread(target=setter, args=(t,)) for t in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        assert not errors
        assert lib.gsa_get_tuning(L.TUNE_SPMM_COLUMNS) in values
    finally:
        for key, v in saved.items():
            lib.gsa_set_tuning(key, v)


def test_group_item_layout_matches_header(gsa):
    """batch.ITEM_DTYPE (the bytes Python hands to gsa_grouped_tiles / gsa_grouped_mul) has the
    field order, offsets and size of gsa_group_item in include/gsa.h."""
    from helpers import c_struct_layout
    import importlib
    batch = importlib.import_module(gsa.__name__ + ".batch")
    layout, total = c_struct_layout(open(HEADER).read(), "gsa_group_item")
    assert total == 144 == batch.ITEM_DTYPE.itemsize
    assert [f for f, _, _ in layout] == list(batch.ITEM_DTYPE.names)
    for fname, off, size in layout:
        dt, py_off = batch.ITEM_DTYPE.fields[fname][:2]
        assert (py_off, dt.itemsize) == (off, size), fname
