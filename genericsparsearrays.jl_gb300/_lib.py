"""ctypes binding of libgsa.so (the C ABI declared in include/gsa.h).

The library is the only compute path: if it cannot be loaded, every product and
conversion raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgsa.so")

# Status codes (gsa_status)
OK, ERR_INVALID_ARG, ERR_DIM, ERR_UNSUPPORTED, ERR_CUDA, ERR_ALLOC, ERR_STRUCTURE, ERR_TIMEOUT = range(8)
# Element and index type codes (gsa_dtype / gsa_itype)
F32, F64, C32, C64, I32, I64 = range(6)
IDX32, IDX64 = 0, 1
# op codes (gsa_op) and algorithms (gsa_algo)
OP_N, OP_T, OP_C = 0, 1, 2
SUM_NEGATE = 4
ALGO_AUTO, ALGO_MERGE, ALGO_VECTOR, ALGO_PIPE = 0, 1, 2, 3
(TUNE_PIPE_THREADS, TUNE_SPMM_COLUMNS, TUNE_PLAN_ORDER, TUNE_WAIT_LIMIT, TUNE_STAGE_ROWS,
 TUNE_X_PAIRS, TUNE_SORT_STAGED) = 1, 2, 3, 4, 5, 6, 7
BATCH_GROUPED, BATCH_GRAPH, BATCH_PER_CALL = 0, 1, 2

# Every exported symbol of include/gsa.h with its ctypes signature.
_i32, _i64, _vp, _sz = ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_size_t
_MUL = [_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _i32, _i64, _vp, _i64, _i32, _vp,
        _i64, _vp, _vp]
SIGNATURES = {
    "gsa_version": ([], _i32),
    "gsa_last_error_string": ([], ctypes.c_char_p),
    "gsa_set_kernel_timer": ([_vp, _vp], None),
    "gsa_set_tuning": ([_i32, _i32], _i32),
    "gsa_get_tuning": ([_i32], _i32),
    "gsa_csr_mul": (_MUL + [_i32, _vp, _sz], _i32),
    "gsa_csc_mul": (_MUL + [_i32, _vp, _sz], _i32),
    "gsa_coo_mul": (_MUL, _i32),
    "gsa_plan_create": ([_vp, _i32, _i64, _i64, _vp, _i32, ctypes.POINTER(_vp)], _i32),
    "gsa_plan_destroy": ([_vp], _i32),
    "gsa_plan_info": ([_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64)], _i32),
    "gsa_plan_workspace_size": ([_vp, _i32, _i64], _sz),
    "gsa_csr_mul_planned": (_MUL + [_vp, _vp, _sz], _i32),
    "gsa_csc_mul_planned": (_MUL + [_vp, _vp, _sz], _i32),
    "gsa_plan_bin_order": ([_vp, ctypes.POINTER(_vp), ctypes.POINTER(_i64)], _i32),
    "gsa_coo_plan_create": ([_vp, _i32, _i64, _i64, _i64, _vp, _i32, ctypes.POINTER(_vp)], _i32),
    "gsa_coo_plan_info": ([_vp, ctypes.POINTER(_i32)], _i32),
    "gsa_coo_mul_planned": (_MUL + [_vp, _vp, _sz], _i32),
    "gsa_csr_dot": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp,
                     _vp, _sz], _i32),
    "gsa_csc_dot": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp,
                     _vp, _sz], _i32),
    "gsa_coo_dot": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp,
                     _vp, _sz], _i32),
    "gsa_dot_workspace_size": ([_i32, _i32, _i32, _i64, _i64, _vp], _sz),
    "gsa_dropzeros_workspace_size": ([_i64], _sz),
    "gsa_dropzeros_count": ([_vp, _i32, _i64, _vp, _vp, _sz, ctypes.POINTER(_i64)], _i32),
    "gsa_dropzeros_copy": ([_vp, _i32, _i32, _i32, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp], _i32),
    "gsa_coo_sum_workspace_size": ([_i32, _i64, _i64, _i64], _sz),
    "gsa_coo_sum_count": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _i64, _vp, _vp, _vp, _i32,
                           _i64, _vp, _i32, _vp, _sz, ctypes.POINTER(_i64)], _i32),
    "gsa_coo_sum_copy": ([_vp, _i32, _i32, _i64, _i64, _i64, _i64, _i32, _vp, _vp, _vp, _vp], _i32),
    "gsa_compressed_add_workspace_size": ([_i64], _sz),
    "gsa_compressed_add_count": ([_vp, _i32, _i64, _vp, _vp, _vp, _vp, _i32, _vp, _sz, _vp, ctypes.POINTER(_i64)], _i32),
    "gsa_compressed_add_copy": ([_vp, _i32, _i32, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp, _vp],
                                _i32),
    "gsa_spgemm_create": ([_vp, _i32, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _i32,
                           _vp, ctypes.POINTER(_i64), ctypes.POINTER(_vp)], _i32),
    "gsa_spgemm_compute": ([_vp, _vp, _vp, _vp], _i32),
    "gsa_spgemm_destroy": ([_vp], _i32),
    "gsa_add_to_dense": ([_vp, _i32, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _i64], _i32),
    "gsa_csr_spmv_noalloc": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp,
                              _vp, _vp], _i32),
    "gsa_mul_workspace_size": ([_i32, _i32, _i32, _i64, _i64, _i64, _i32, _i64, _i32], _sz),
    "gsa_grouped_tiles": ([_i32, _vp, _i64, _i32, ctypes.POINTER(_i64)], _i32),
    "gsa_grouped_mul": ([_vp, _i32, _i32, _i32, _vp, _i64, _i64, _i32, _i32], _i32),
    "gsa_batch_create": ([_vp, _i32, _i32, _i32, _vp, _i64, _i32, _i32, ctypes.POINTER(_vp)], _i32),
    "gsa_batch_run": ([_vp, _vp, _i32], _i32),
    "gsa_batch_destroy": ([_vp], _i32),
    "gsa_coo_to_csr": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp,
                        _sz], _i32),
    "gsa_coo_to_csc": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp,
                        _sz], _i32),
    "gsa_coo_to_compressed_workspace_size": ([_i32, _i32, _i32, _i64, _i64, _i64], _sz),
    "gsa_csr_to_coo": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _vp],
                       _i32),
    "gsa_csc_to_coo": ([_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp, _vp, _vp],
                       _i32),
    "gsa_validate_compressed": ([_vp, _i32, _i64, _i64, _i64, _vp, _vp, _i32], _i32),
    "gsa_check_device_status": ([_vp], _i32),
}

_lock = threading.Lock()
_lib = None


class GSAError(RuntimeError):
    """A libgsa call returned a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"libgsa status {status}: {message}")
        self.status = status


def load() -> ctypes.CDLL:
    """Load libgsa.so (built by ``build.py``); raises if it is missing."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"libgsa.so not found at {LIB_PATH}; build it with "
                    "`python -c \"import __graft_entry__ as g; g.build()\"`")
            lib = ctypes.CDLL(LIB_PATH)
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = res
            _lib = lib
    return _lib


def last_error() -> str:
    msg = load().gsa_last_error_string()
    return msg.decode() if msg else ""


def check(status: int) -> None:
    """Map a status to the exception the reference raises for the same condition."""
    if status == OK:
        return
    msg = last_error()
    from .errors import ArgumentError, DimensionMismatch
    if status == ERR_DIM:
        raise DimensionMismatch(msg)
    if status in (ERR_INVALID_ARG, ERR_UNSUPPORTED, ERR_STRUCTURE):
        raise ArgumentError(msg)
    raise GSAError(status, msg)
