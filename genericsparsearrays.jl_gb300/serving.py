"""Serving loop: ``mul!`` requests against a device-resident registry of CSR matrices,
admitted under an HBM budget and coalesced into grouped launches (continuous batching).

* ``Registry``  the resident matrices and the HBM budget.  Registering a matrix charges
  its bytes; admitting a request charges its output; both fail (or wait) when the budget
  is spent.
* ``Server``    the scheduler.  ``submit`` queues a request; every ``step`` retires the
  launches that have finished, expires requests past their deadline, and -- for each free
  launch slot (one CUDA stream each) -- admits queued requests in arrival order while the
  budget allows and their work (FP64 multiply-adds) stays under the launch's work cap, and
  launches them together.  The cap keeps a launch to about a millisecond of GPU time, so a
  slot frees often; requests that arrive while others are on the GPU are admitted into
  whichever slot frees first, and their work overlaps the running launches on the other
  streams.
* ``GroupedExecutor``  runs one admitted set on the slot's stream: one grouped launch
  (gsa_grouped_mul) per element type for the small products, a plain planned call for each
  large one, timed by CUDA events mapped to the host clock.
* ``serve_per_call``   the baseline: one public-API ``mul_`` per request as it arrives.

The reference has no serving layer: its ``mul!`` (src/matrix_csr/matrix_csr.jl:153-209)
launches one kernel per call.  Each request here computes exactly that product
(y = alpha A x + beta y, k right-hand sides), with the same row code as a plain call.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Any, Callable, Dict, List, Optional, Sequence

import numpy as np

from .errors import ArgumentError, DimensionMismatch


class BudgetExceeded(MemoryError):
    """A matrix or request does not fit the registry's HBM budget."""


def _elem_size(dtype) -> int:
    import torch
    return torch.empty(0, dtype=dtype).element_size()


def matrix_bytes(A) -> int:
    """Device bytes of a CSR matrix's three arrays."""
    return sum(t.numel() * t.element_size() for t in (A.rowptr, A.colval, A.nzval))


class Registry:
    """Resident CSR matrices under an HBM budget (bytes); also the budget's ledger for
    request outputs."""

    def __init__(self, budget_bytes: int):
        if budget_bytes <= 0:
            raise ArgumentError("budget must be positive")
        self.budget = int(budget_bytes)
        self.used = 0       # matrices + admitted outputs
        self.resident = 0   # matrices alone
        self._mats: Dict[int, Any] = {}
        self._bytes: Dict[int, int] = {}
        self._next = 0

    def add(self, A) -> int:
        """Register a resident matrix (its bytes are charged).  A ComplexF64 matrix gets its
        plan now (bin order for the grouped kernel), not at its first request."""
        b = matrix_bytes(A)
        if self.used + b > self.budget:
            raise BudgetExceeded(f"matrix of {b} bytes does not fit: {self.used} of {self.budget} in use")
        mid = self._next
        self._next += 1
        if getattr(A, "device", None) is not None and A.device.type == "cuda":
            from .batch import bin_order_of
            bin_order_of(A)
        self._mats[mid] = A
        self._bytes[mid] = b
        self.used += b
        self.resident += b
        return mid

    def remove(self, mid: int) -> None:
        b = self._bytes.pop(mid)
        self.used -= b
        self.resident -= b
        del self._mats[mid]

    def __getitem__(self, mid: int):
        return self._mats[mid]

    def __len__(self):
        return len(self._mats)

    def ids(self) -> List[int]:
        return list(self._mats)

    def reserve(self, nbytes: int) -> bool:
        if self.used + nbytes > self.budget:
            return False
        self.used += nbytes
        return True

    def release(self, nbytes: int) -> None:
        self.used -= nbytes


@dataclasses.dataclass
class Request:
    """y = alpha * A x + beta * y for registry matrix ``matrix``; X a device vector (n,) or
    column-major (n, k) matrix.  Y is allocated at admission unless given (it must be given
    when beta is not zero).  Times are host-clock seconds."""
    matrix: int
    X: Any
    alpha: Any = 1
    beta: Any = 0
    Y: Any = None
    arrival: float = 0.0
    deadline: Optional[float] = None
    id: int = -1
    state: str = "new"        # queued, running, done, rejected, cancelled, expired
    admitted: float = math.nan
    finished: float = math.nan
    error: Optional[str] = None
    out_bytes: int = 0
    owns_y: bool = False
    fma: int = 0              # FP64 multiply-adds of the product (set at submission)

    @property
    def k(self) -> int:
        return 1 if self.X.dim() == 1 else int(self.X.shape[1])

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def product_fma(A, k: int) -> int:
    """FP64 multiply-adds of y = A x with k right-hand sides: one per stored entry and column,
    four for a complex one (real types other than Float64 count one as well)."""
    from .sparse import nnz
    return nnz(A) * k * (4 if A.dtype.is_complex else 1)


class Server:
    """Continuous batching over ``slots`` launch slots; see the module docstring.

    ``work_cap``: FP64 multiply-adds one launch may take (a request larger than that is
    launched alone); ``max_batch``: requests one launch may take."""

    def __init__(self, registry: Registry, executor, max_batch: int = 1024, slots: int = 4,
                 clock: Callable[[], float] = time.perf_counter, keep_outputs: bool = True,
                 work_cap: int = 1 << 28):
        self.registry = registry
        self.keep_outputs = keep_outputs  # False: drop server-allocated outputs when done
        self.executor = executor
        self.max_batch = int(max_batch)
        self.work_cap = int(work_cap)
        self.slots = int(slots)
        self.clock = clock
        self.queue: collections.deque = collections.deque()
        self.running: Dict[int, tuple] = {}     # slot -> (handle, [requests])
        self.finished: List[Request] = []
        self.launches = 0
        self._next_id = 0
        self._deadlines = 0  # queued requests with a deadline (the expiry sweep runs only then)

    # -- client side -------------------------------------------------------------
    def submit(self, req: Request) -> int:
        A = self.registry[req.matrix]
        if req.X.dim() not in (1, 2) or req.X.shape[0] != A.n:
            raise DimensionMismatch(
                f"second dimension of A, {A.n}, does not match the first dimension of B, {req.X.shape[0]}")
        if req.X.dtype != A.dtype or req.X.device != A.device:
            raise ArgumentError("X must share A's element type and device")
        beta_zero = req.beta == 0
        if req.Y is None and not beta_zero:
            raise ArgumentError("a request with beta != 0 must supply Y")
        if req.Y is not None and (req.Y.shape[0] != A.m or (req.Y.dim() == 2 and req.Y.shape[1] != req.k)):
            raise DimensionMismatch(f"first dimension of A, {A.m}, does not match the first dimension of C")
        req.id = self._next_id
        self._next_id += 1
        req.fma = product_fma(A, req.k)
        req.out_bytes = 0 if req.Y is not None else A.m * req.k * _elem_size(A.dtype)
        if req.out_bytes > self.registry.budget - self.registry.resident:
            # even with every running launch retired it would not fit
            self._end(req, "rejected", "output does not fit the HBM budget")
            return req.id
        req.state = "queued"
        if not req.arrival:
            req.arrival = self.clock()
        if req.deadline is not None:
            self._deadlines += 1
        self.queue.append(req)
        return req.id

    def cancel(self, rid: int) -> bool:
        for r in self.queue:
            if r.id == rid:
                self.queue.remove(r)
                if r.deadline is not None:
                    self._deadlines -= 1
                self._end(r, "cancelled", "cancelled")
                return True
        return False  # running or finished: a launch is never interrupted

    # -- scheduler -----------------------------------------------------------------
    def busy(self) -> bool:
        return bool(self.queue or self.running)

    def step(self) -> bool:
        """One scheduling pass; returns whether work is queued or running."""
        self._retire()
        self._expire()
        for slot in range(self.slots):
            if slot in self.running or not self.queue:
                continue
            batch = self._admit()
            if not batch:
                break  # budget: wait for a launch to retire
            now = self.clock()
            for r in batch:
                r.state, r.admitted = "running", now
            try:
                handle = self.executor.launch(slot, [(self.registry[r.matrix], r) for r in batch])
            except Exception as e:  # the whole set fails; its memory is returned
                for r in batch:
                    self._release(r)
                    self._end(r, "rejected", f"launch failed: {e}")
                continue
            self.running[slot] = (handle, batch)
            self.launches += 1
        return self.busy()

    def run(self, requests: Sequence[Request] = (), realtime: bool = True) -> None:
        """Submit ``requests`` at their arrival times (host clock) and serve until idle."""
        pending = sorted(requests, key=lambda r: r.arrival)
        i = 0
        while i < len(pending) or self.busy():
            now = self.clock()
            while i < len(pending) and (not realtime or pending[i].arrival <= now):
                self.submit(pending[i])
                i += 1
            self.step()

    def _admit(self) -> List[Request]:
        batch, work = [], 0
        while self.queue and len(batch) < self.max_batch:
            r = self.queue[0]
            if batch and work + r.fma > self.work_cap:
                break  # the launch is full; the next free slot takes it
            if r.out_bytes and not self.registry.reserve(r.out_bytes):
                if r.out_bytes > self.registry.budget - self.registry.resident:
                    self.queue.popleft()  # matrices registered since it was queued
                    self._dequeued(r)
                    self._end(r, "rejected", "output does not fit the HBM budget")
                    continue
                break
            self.queue.popleft()
            self._dequeued(r)
            if r.Y is None:
                r.owns_y = True
            batch.append(r)
            work += r.fma
        return batch

    def _dequeued(self, r: Request) -> None:
        if r.deadline is not None:
            self._deadlines -= 1

    def _retire(self) -> None:
        for slot in list(self.running):
            handle, batch = self.running[slot]
            if not self.executor.done(handle):
                continue
            t = self.executor.finish_time(handle)
            err = self.executor.error(handle)
            del self.running[slot]
            for r in batch:
                r.finished = t
                self._release(r)
                if r.owns_y and not self.keep_outputs:
                    r.Y = None
                self._end(r, "done" if err is None else "rejected", err)

    def _expire(self) -> None:
        if not self._deadlines:
            return
        now = self.clock()
        keep = collections.deque()
        for r in self.queue:
            if r.deadline is not None and now > r.deadline:
                self._deadlines -= 1
                self._end(r, "expired", "deadline passed while queued")
            else:
                keep.append(r)
        self.queue = keep

    def _release(self, r: Request) -> None:
        if r.out_bytes and r.state in ("running", "queued") and r.owns_y:
            self.registry.release(r.out_bytes)

    def _end(self, r: Request, state: str, error: Optional[str]) -> None:
        r.state, r.error = state, error
        self.finished.append(r)

    # -- metrics -------------------------------------------------------------------
    def stats(self) -> dict:
        return summarize(self.finished, launches=self.launches)


def summarize(reqs: Sequence[Request], launches: Optional[int] = None) -> dict:
    done = [r for r in reqs if r.state == "done"]
    out = {"done": len(done), "rejected": sum(r.state == "rejected" for r in reqs),
           "expired": sum(r.state == "expired" for r in reqs),
           "cancelled": sum(r.state == "cancelled" for r in reqs)}
    if launches is not None:
        out["launches"] = launches
    if done:
        lat = np.array([r.latency for r in done]) * 1e3
        t0 = min(r.arrival for r in done)
        t1 = max(r.finished for r in done)
        span = max(t1 - t0, 1e-9)
        out.update({"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                    "mean_ms": float(lat.mean()), "mul_per_s": len(done) / span,
                    "fma_per_s": float(sum(r.fma for r in done)) / span, "span_s": t1 - t0})
    return out


class GroupedExecutor:
    """Runs an admitted set on slot ``slot``'s CUDA stream: output allocation, then one
    grouped launch per element type for the small products (pinned item staging, no
    allocation per launch in the library), a plain planned call for each product of at least
    ``solo_fma`` multiply-adds (there a launch is cheap against the work, and the plain call
    has the plan's chunk warps) and for a set of one, then a timing event.  Finish times are CUDA-event times
    mapped onto the host clock through a reference event taken at construction."""

    def __init__(self, device, slots: int = 4, columns: int = 0, g1_avg: int = 0,
                 clock: Callable[[], float] = time.perf_counter, solo_fma: int = 1 << 24):
        import torch
        from .batch import GroupedLauncher
        self.torch = torch
        self.device = torch.device(device)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self.solo_fma = solo_fma
        self.columns = columns
        self.launchers = [GroupedLauncher(self.device, 256, columns, g1_avg) for _ in range(slots)]
        self.ref = torch.cuda.Event(enable_timing=True)
        self.ref.record(torch.cuda.current_stream(self.device))
        self.ref.synchronize()
        self.t_ref = clock()

    def launch(self, slot: int, work):
        torch = self.torch
        s = self.streams[slot]
        groups: Dict[Any, list] = collections.defaultdict(list)
        with torch.cuda.stream(s):
            torch.cuda.nvtx.range_push(f"gsa.serve.launch[{len(work)}]")
            from .sparse import mul_, nnz
            for A, r in work:
                if r.Y is None:
                    shape = (A.m,) if r.X.dim() == 1 else (r.k, A.m)
                    Y = torch.empty(shape, dtype=A.dtype, device=self.device)
                    r.Y = Y if r.X.dim() == 1 else Y.t()
                if len(work) == 1 or nnz(A) * r.k >= self.solo_fma:
                    mul_(r.Y, A, r.X, r.alpha, r.beta)
                else:
                    groups[(A.dtype, A.itype)].append((A, r.X, r.Y, r.alpha, r.beta))
            for (dt, _), prods in groups.items():
                # rows of a row-major X: a thread takes 8 columns of a row (its values share
                # cache lines; Float64 ones are read two per 16-byte load)
                cols = self.columns or 8
                self.launchers[slot].launch(prods, s, columns=cols)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(s)
            torch.cuda.nvtx.range_pop()
        return ev

    def done(self, ev) -> bool:
        return ev.query()

    def finish_time(self, ev) -> float:
        return self.t_ref + self.ref.elapsed_time(ev) / 1e3

    def error(self, ev) -> Optional[str]:
        return None


def serve_per_call(registry: Registry, requests: Sequence[Request], device,
                   clock: Callable[[], float] = time.perf_counter, keep_outputs: bool = True) -> dict:
    """Baseline: each request as one ``mul_`` on one stream as soon as it arrives (the
    kernel queue overlaps host and device); latency from arrival to the request's event.
    Without keep_outputs an output is dropped once its product is enqueued (the caching
    allocator reuses it in stream order)."""
    import torch
    from .sparse import mul_
    dev = torch.device(device)
    ref = torch.cuda.Event(enable_timing=True)
    ref.record(torch.cuda.current_stream(dev))
    ref.synchronize()
    t_ref = clock()
    pending = sorted(requests, key=lambda r: r.arrival)
    evs = []
    for r in pending:
        while clock() < r.arrival:
            pass
        A = registry[r.matrix]
        r.fma = product_fma(A, r.k)
        if r.Y is None:
            r.Y = torch.empty((A.m,) if r.X.dim() == 1 else (r.k, A.m), dtype=A.dtype, device=dev)
            if r.X.dim() == 2:
                r.Y = r.Y.t()
        mul_(r.Y, A, r.X, r.alpha, r.beta)
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        evs.append(ev)
        if not keep_outputs:
            r.Y = None
    torch.cuda.synchronize(dev)
    for r, ev in zip(pending, evs):
        r.finished = t_ref + ref.elapsed_time(ev) / 1e3
        r.state = "done"
    return summarize(pending)


# ---------------------------------------------------------------------------
# The served-stream workload.

def registry_matrices(count=512, n_lo=1_000, n_hi=2_000_000, len_lo=5, len_hi=40, seed=0,
                      device="cuda", itype=None):
    """``count`` square CSR matrices, n log-uniform in [n_lo, n_hi]; row lengths in
    [len_lo, len_hi], uniform for even-numbered matrices and Pareto(1.5) truncated to the
    range for odd ones; columns uniform (sorted within a row, repeats possible); Float64
    for matrices with i % 4 < 2, else ComplexF64; values U(-1, 1) parts.  Built on the GPU."""
    import torch
    from .sparse import GenericSparseMatrixCSR
    itype = itype or torch.int32
    g = torch.Generator(device="cpu").manual_seed(seed)
    ns = torch.exp(torch.empty(count).uniform_(math.log(n_lo), math.log(n_hi), generator=g)).round().long()
    dev = torch.device(device)
    gd = torch.Generator(device=dev).manual_seed(seed + 1)
    mats = []
    for i in range(count):
        n = int(ns[i])
        if i % 2 == 0:
            lens = torch.randint(len_lo, len_hi + 1, (n,), generator=gd, device=dev)
        else:
            u = torch.rand(n, generator=gd, device=dev, dtype=torch.float64).clamp_min(1e-12)
            lens = (len_lo * u.pow(-1.0 / 1.5)).floor().clamp(len_lo, len_hi).long()
        rowptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        torch.cumsum(lens, 0, out=rowptr[1:])
        nnz = int(rowptr[-1])
        rows = torch.repeat_interleave(torch.arange(n, device=dev), lens, output_size=nnz)
        cols = torch.randint(0, n, (nnz,), generator=gd, device=dev)
        key, _ = torch.sort(rows * n + cols)
        cols = key - rows * n
        del key
        cplx = i % 4 >= 2
        if cplx:
            vals = torch.complex(torch.rand(nnz, generator=gd, device=dev, dtype=torch.float64) * 2 - 1,
                                 torch.rand(nnz, generator=gd, device=dev, dtype=torch.float64) * 2 - 1)
        else:
            vals = torch.rand(nnz, generator=gd, device=dev, dtype=torch.float64) * 2 - 1
        mats.append(GenericSparseMatrixCSR(n, n, (rowptr + 1).to(itype), (cols + 1).to(itype), vals))
        del rows, cols, vals, rowptr, lens
    return mats


def poisson_requests(registry: Registry, xs: Dict[int, Any], rate: float, duration: float,
                     k_lo=1, k_hi=32, seed=0, t0: float = 0.0) -> List[Request]:
    """Arrivals of a Poisson process of ``rate`` per second over ``duration`` seconds from
    ``t0``; each picks a matrix uniformly and k uniformly in [k_lo, k_hi], X the first k
    columns of that matrix's resident (n, k_hi) block ``xs[id]`` (row-major blocks keep one
    entry's k values in one cache line); alpha 1, beta 0."""
    rng = np.random.default_rng(seed)
    n = rng.poisson(rate * duration)
    times = np.sort(rng.uniform(0, duration, n)) + t0
    ids = registry.ids()
    picks = rng.integers(0, len(ids), n)
    ks = rng.integers(k_lo, k_hi + 1, n)
    out = []
    for t, p, k in zip(times, picks, ks):
        mid = ids[int(p)]
        X = xs[mid][:, 0] if k == 1 else xs[mid][:, : int(k)]
        out.append(Request(matrix=mid, X=X, arrival=float(t)))
    return out
