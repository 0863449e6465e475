"""GB300-native sparse x dense ``mul!`` and COO -> CSR/CSC conversion for GenericSparseArrays.jl.

The compute lives in ``libgsa.so`` (hand-written sm_103a CUDA behind the C ABI of
``include/gsa.h``); this package is the host-side mirror of the reference's Julia API for
that path.  Import it as ``genericsparsearrays_gb300`` (``__graft_entry__.load_package()``
registers the directory under that name, since its folder name is not an identifier).
"""
from . import _lib, workloads
from .errors import ArgumentError, DimensionMismatch
from .sparse import (
    AbstractGenericSparseMatrix,
    Adjoint,
    GenericSparseMatrixCOO,
    GenericSparseMatrixCSC,
    GenericSparseMatrixCSR,
    I,
    SparseMatrixCSC,
    Transpose,
    UniformScaling,
    adapt,
    add,
    adjoint,
    collect,
    dot,
    dropzeros,
    mul,
    mul_,
    nnz,
    size,
    subtract,
    transpose,
    validate,
)

ALGO_AUTO, ALGO_MERGE, ALGO_VECTOR, ALGO_PIPE = (_lib.ALGO_AUTO, _lib.ALGO_MERGE, _lib.ALGO_VECTOR,
                                                 _lib.ALGO_PIPE)

__all__ = [
    "AbstractGenericSparseMatrix", "Adjoint", "ArgumentError", "DimensionMismatch",
    "GenericSparseMatrixCOO", "GenericSparseMatrixCSC", "GenericSparseMatrixCSR",
    "SparseMatrixCSC", "Transpose", "adapt", "adjoint", "collect", "mul", "mul_", "nnz", "size",
    "transpose", "validate", "dot", "add", "subtract", "dropzeros", "I", "UniformScaling", "ALGO_AUTO", "ALGO_MERGE", "ALGO_VECTOR", "ALGO_PIPE",
]
