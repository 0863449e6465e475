"""Grouped products: many CSR ``mul!`` in one launch (and CUDA-graph replay).

``BatchedMul([(A_1, x_1, y_1, alpha_1, beta_1), ...])`` packs one item per product into the
C ABI's ``gsa_group_item`` array, keeps it on the device and runs all products with one
persistent grouped launch (``mode="grouped"``), the same launch replayed from a captured CUDA
graph (``mode="graph"``), or one plain ``gsa_csr_mul`` per product (``mode="per_call"``, the
baseline).  The operand buffers are fixed when the batch is made; refill their contents and
call ``run`` again.  ``GroupedLauncher`` does the same for a product list that changes at every
launch (the serving loop), with pinned staging and no allocation per launch.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .errors import ArgumentError, DimensionMismatch
from .sparse import (BASE, GenericSparseMatrixCSR, _DTYPE, _ITYPE, _gather_plan, _scalar_buf, _stream_ptr,
                     nnz)

ITEM_DTYPE = np.dtype([("rowptr", "<u8"), ("colval", "<u8"), ("nzval", "<u8"), ("B", "<u8"),
                       ("C", "<u8"), ("m", "<i8"), ("n", "<i8"), ("nnz", "<i8"), ("ldb", "<i8"),
                       ("ldc", "<i8"), ("k", "<i4"), ("b_rowmajor", "<i4"), ("first_tile", "<i8"),
                       ("bin_order", "<u8"), ("bin_warps", "<i8"),
                       ("alpha", "u1", 16), ("beta", "u1", 16)])
assert ITEM_DTYPE.itemsize == 144


def bin_order_of(A, k: int = 1) -> Tuple[int, int]:
    """(device view, warps) of the bin order of A's plan when a product of A with k
    right-hand sides is FP64-bound (ComplexF64, or Float64 with k > 1: every idle lane is lost
    FP64 time); (0, 0) otherwise.  Makes the plan on first use (one synchronisation) and keeps
    it on the matrix."""
    if not (A.dtype == torch.complex128 or (A.dtype == torch.float64 and k > 1)):
        return 0, 0
    plan = _gather_plan(A)
    if plan is None:
        return 0, 0
    view, warps = ctypes.c_void_p(0), ctypes.c_int64(0)
    _lib.check(_lib.load().gsa_plan_bin_order(ctypes.c_void_p(plan.handle), ctypes.byref(view),
                                              ctypes.byref(warps)))
    return (view.value or 0), warps.value

Product = Tuple[GenericSparseMatrixCSR, torch.Tensor, torch.Tensor, object, object]

_MODES = {"grouped": _lib.BATCH_GROUPED, "graph": _lib.BATCH_GRAPH, "per_call": _lib.BATCH_PER_CALL}


def _column_major(t: torch.Tensor, what: str) -> Tuple[int, int]:
    """(k, ld) of a vector or column-major matrix operand."""
    if t.dim() == 1:
        return 1, max(t.shape[0], 1)
    if t.dim() == 2 and (t.shape[0] <= 1 or t.stride(0) == 1):
        ld = t.stride(1) if t.shape[1] > 1 else t.shape[0]
        return t.shape[1], max(ld, t.shape[0], 1)
    raise ArgumentError(f"{what} of a grouped product must be a vector or column-major matrix")


def _dense_in(t: torch.Tensor) -> Tuple[int, int, int]:
    """(k, ld, rowmajor) of a right-hand side: a vector, a column-major matrix, or a
    row-major one (row i's k values contiguous, rows ld apart)."""
    if t.dim() == 2 and t.shape[1] > 1 and t.stride(1) == 1 and t.shape[0] > 1:
        return t.shape[1], max(t.stride(0), t.shape[1]), 1
    if t.dim() == 1 and t.shape[0] > 1 and t.stride(0) != 1:  # a column of a row-major block
        return 1, t.stride(0), 1
    if t.dim() == 2 and t.shape[1] == 1 and t.shape[0] > 1 and t.stride(0) != 1:
        return 1, t.stride(0), 1
    k, ld = _column_major(t, "B")
    return k, ld, 0


def pack_items(products: Sequence[Product], out: Optional[np.ndarray] = None,
               use_plans: bool = True) -> Tuple[np.ndarray, torch.dtype, torch.dtype]:
    """The ``gsa_group_item`` array of a product list (checks as ``mul!`` does).  With
    use_plans, FP64-bound items (ComplexF64, Float64 with k > 1) carry their plan's bin order
    (see bin_order_of)."""
    if not products:
        raise ArgumentError("no products")
    dt, it = products[0][0].dtype, products[0][0].itype
    arr = out[: len(products)] if out is not None else np.zeros(len(products), ITEM_DTYPE)
    for i, (A, B, C, alpha, beta) in enumerate(products):
        if not isinstance(A, GenericSparseMatrixCSR):
            raise ArgumentError("grouped products take GenericSparseMatrixCSR matrices")
        if A.dtype != dt or A.itype != it or B.dtype != dt or C.dtype != dt:
            raise ArgumentError("all operands of a grouped launch share one element and index type")
        kb, ldb, brow = _dense_in(B)
        if kb > 0x7fffffff:
            raise ArgumentError("a grouped product takes fewer than 2^31 right-hand sides")
        kc, ldc = _column_major(C, "C")
        if A.n != B.shape[0]:
            raise DimensionMismatch(
                f"second dimension of A, {A.n}, does not match the first dimension of B, {B.shape[0]}")
        if A.m != C.shape[0]:
            raise DimensionMismatch(
                f"first dimension of A, {A.m}, does not match the first dimension of C, {C.shape[0]}")
        if kb != kc:
            raise DimensionMismatch(
                f"second dimension of B, {kb}, does not match the second dimension of C, {kc}")
        row = arr[i]
        row["rowptr"], row["colval"], row["nzval"] = A.rowptr.data_ptr(), A.colval.data_ptr(), A.nzval.data_ptr()
        row["B"], row["C"] = B.data_ptr(), C.data_ptr()
        row["m"], row["n"], row["nnz"], row["ldb"], row["ldc"], row["k"] = A.m, A.n, nnz(A), ldb, ldc, kb
        row["b_rowmajor"] = brow
        row["bin_order"], row["bin_warps"] = bin_order_of(A, kb) if use_plans else (0, 0)
        a = _scalar_buf(alpha, dt).view(np.uint8)
        b = _scalar_buf(beta, dt).view(np.uint8)
        row["alpha"][:] = 0
        row["beta"][:] = 0
        row["alpha"][: a.size] = a
        row["beta"][: b.size] = b
    return arr, dt, it


def tiles(items: np.ndarray, dtype: torch.dtype, columns: int) -> int:
    """Fill first_tile (gsa_grouped_tiles) and return the tile count."""
    n = ctypes.c_int64(0)
    _lib.check(_lib.load().gsa_grouped_tiles(_DTYPE[dtype], items.ctypes.data_as(ctypes.c_void_p),
                                             items.size, columns, ctypes.byref(n)))
    return n.value


class BatchedMul:
    """All products of a fixed list in one grouped launch; see the module docstring."""

    def __init__(self, products: Sequence[Product], columns: int = 0, g1_avg: int = 0,
                 use_plans: bool = True):
        self.products = list(products)  # keeps the operand buffers alive
        items, self.dtype, self.itype = pack_items(self.products, use_plans=use_plans)
        self.columns, self.g1_avg = columns, g1_avg
        self.device = self.products[0][0].device
        lib = _lib.load()
        h = ctypes.c_void_p(0)
        with torch.cuda.device(self.device):
            _lib.check(lib.gsa_batch_create(_stream_ptr(self.device), _DTYPE[self.dtype],
                                            _ITYPE[self.itype], BASE,
                                            items.ctypes.data_as(ctypes.c_void_p), items.size,
                                            columns, g1_avg, ctypes.byref(h)))
        self._h = h

    def run(self, mode: str = "graph") -> None:
        """Enqueue all products on the current stream (asynchronous)."""
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().gsa_batch_run(self._h, _stream_ptr(self.device), _MODES[mode]))

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.load().gsa_batch_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GroupedLauncher:
    """Grouped launches of changing product lists on one device: items are packed into a
    pinned host buffer, copied to a device buffer on the launch stream and consumed there;
    buffers grow as needed and are reused (two slots, so a launch can be packed while the
    previous one's copy may still be in flight)."""

    def __init__(self, device, capacity: int = 1024, columns: int = 0, g1_avg: int = 0):
        self.device = torch.device(device)
        self.columns, self.g1_avg = columns, g1_avg
        self._slots = [self._alloc(capacity), self._alloc(capacity)]
        self._next = 0

    def _alloc(self, cap):
        host = torch.empty(cap * ITEM_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        dev = torch.empty(cap * ITEM_DTYPE.itemsize, dtype=torch.uint8, device=self.device)
        return {"cap": cap, "host": host, "dev": dev, "event": None}

    def launch(self, products: Sequence[Product], stream: Optional[torch.cuda.Stream] = None,
               columns: Optional[int] = None) -> None:
        stream = stream or torch.cuda.current_stream(self.device)
        columns = self.columns if columns is None else columns
        slot = self._slots[self._next]
        self._next ^= 1
        if slot["event"] is not None:
            slot["event"].synchronize()  # the host buffer's previous copy has left
        if len(products) > slot["cap"]:
            slot.update(self._alloc(max(len(products), 2 * slot["cap"])))
        view = slot["host"].numpy().view(ITEM_DTYPE)
        items, dt, it = pack_items(products, out=view)
        ntiles = tiles(items, dt, columns)
        nbytes = len(products) * ITEM_DTYPE.itemsize
        with torch.cuda.stream(stream), torch.cuda.device(self.device):
            slot["dev"].record_stream(stream)  # a regrown slot frees the old buffer stream-safely
            slot["dev"][:nbytes].copy_(slot["host"][:nbytes], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
            slot["event"] = ev
            _lib.check(_lib.load().gsa_grouped_mul(ctypes.c_void_p(stream.cuda_stream), _DTYPE[dt],
                                                   _ITYPE[it], BASE,
                                                   ctypes.c_void_p(slot["dev"].data_ptr()),
                                                   len(products), ntiles, columns,
                                                   self.g1_avg))
