"""Serving loop scheduler on the host: admission under the HBM budget, continuous batching
over launch slots, cancellation, deadlines and launch failures, with a fake executor and a
manual clock (no GPU)."""
import pytest
import torch

import __graft_entry__

__graft_entry__.load_package()
from genericsparsearrays_gb300 import serving  # noqa: E402
from genericsparsearrays_gb300.errors import ArgumentError, DimensionMismatch  # noqa: E402


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeMatrix:
    def __init__(self, m, n, nnz, dtype=torch.float64):
        self.m, self.n = m, n
        self.rowptr = torch.zeros(m + 1, dtype=torch.int32)
        self.colval = torch.zeros(nnz, dtype=torch.int32)
        self.nzval = torch.zeros(nnz, dtype=dtype)
        self.dtype, self.itype, self.device = dtype, torch.int32, self.nzval.device


class FakeExecutor:
    """Each launch takes ``per_launch`` seconds of the manual clock; launches may fail."""

    def __init__(self, clock, per_launch=1.0, fail_on=()):
        self.clock, self.per_launch, self.fail_on = clock, per_launch, set(fail_on)
        self.launched = []

    def launch(self, slot, work):
        n = len(self.launched)
        self.launched.append((slot, [r.id for _, r in work], self.clock()))
        if n in self.fail_on:
            raise RuntimeError("injected launch failure")
        return self.clock() + self.per_launch

    def done(self, h):
        return self.clock() >= h

    def finish_time(self, h):
        return h

    def error(self, h):
        return None


def setup(budget=10_000, per_launch=1.0, fail_on=(), slots=2, max_batch=64, work_cap=1 << 28):
    clk = Clock()
    reg = serving.Registry(budget)
    mid = reg.add(FakeMatrix(100, 100, 50))  # 101*4 + 50*4 + 50*8 = 1004 bytes
    ex = FakeExecutor(clk, per_launch, fail_on)
    srv = serving.Server(reg, ex, max_batch=max_batch, slots=slots, clock=clk, work_cap=work_cap)
    return clk, reg, mid, ex, srv


def req(mid, k=1, arrival=0.0, **kw):
    X = torch.zeros(100, dtype=torch.float64) if k == 1 else torch.zeros(100, k, dtype=torch.float64)
    return serving.Request(matrix=mid, X=X, arrival=arrival, **kw)


def test_registry_budget():
    reg = serving.Registry(2000)
    reg.add(FakeMatrix(100, 100, 50))
    with pytest.raises(serving.BudgetExceeded):
        reg.add(FakeMatrix(100, 100, 100))
    assert reg.resident == reg.used == 1004
    with pytest.raises(ArgumentError):
        serving.Registry(0)


def test_continuous_batching_overlaps_slots():
    clk, reg, mid, ex, srv = setup()
    srv.submit(req(mid, arrival=0.0))
    srv.step()                       # launch 0 on slot 0 with request 0
    clk.t = 0.2
    srv.submit(req(mid, arrival=0.2))
    srv.submit(req(mid, arrival=0.2))
    srv.step()                       # arrivals while slot 0 runs go to slot 1 at once
    assert [(s, ids) for s, ids, _ in ex.launched] == [(0, [0]), (1, [1, 2])]
    clk.t = 0.5
    srv.submit(req(mid, arrival=0.5))
    srv.step()                       # both slots busy: it waits
    assert len(ex.launched) == 2 and len(srv.queue) == 1
    clk.t = 1.0
    srv.step()                       # slot 0 retires, the waiting request takes it
    assert ex.launched[-1][:2] == (0, [3])
    clk.t = 3.0
    assert not srv.step()
    st = srv.stats()
    assert st["done"] == 4 and st["launches"] == 3
    lat = sorted(r.latency for r in srv.finished)
    assert lat == pytest.approx([1.0, 1.0, 1.0, 1.5])
    assert reg.used == reg.resident   # every output reservation returned


def test_budget_holds_requests_back_and_rejects_oversize():
    # 1004 bytes resident; an output of 100 x k float64 is 800 k bytes
    clk, reg, mid, ex, srv = setup(budget=1004 + 2000)
    srv.submit(req(mid))
    srv.submit(req(mid))
    srv.submit(req(mid, k=4))        # 3200 bytes > budget - resident: can never fit
    assert srv.finished[-1].state == "rejected"
    srv.step()                       # both 800-byte outputs admitted together
    assert ex.launched[0][1] == [0, 1]
    srv.submit(req(mid))             # 800 more does not fit while the first set runs
    srv.step()
    assert len(ex.launched) == 1 and len(srv.queue) == 1
    clk.t = 1.0
    srv.step()
    assert ex.launched[1][1] == [3]
    clk.t = 2.0
    srv.step()
    assert reg.used == reg.resident
    assert [r.state for r in sorted(srv.finished, key=lambda r: r.id)] == ["done", "done", "rejected", "done"]


def test_cancel_and_deadline():
    clk, reg, mid, ex, srv = setup(slots=1)
    srv.submit(req(mid))
    srv.step()
    a = srv.submit(req(mid))
    srv.submit(req(mid, deadline=0.5))
    assert srv.cancel(a)
    assert not srv.cancel(0)          # running: not interruptible
    clk.t = 0.6
    srv.step()
    states = {r.id: r.state for r in srv.finished}
    assert states == {1: "cancelled", 2: "expired"}
    clk.t = 1.0
    srv.step()
    assert {r.id: r.state for r in srv.finished}[0] == "done"


def test_launch_failure_releases_budget():
    clk, reg, mid, ex, srv = setup(fail_on={0})
    srv.submit(req(mid, k=2))
    srv.step()
    r = srv.finished[0]
    assert r.state == "rejected" and "injected" in r.error
    assert reg.used == reg.resident
    srv.submit(req(mid, k=2))
    srv.step()
    clk.t = 1.0
    srv.step()
    assert srv.finished[-1].state == "done"


def test_submit_checks():
    clk, reg, mid, ex, srv = setup()
    with pytest.raises(DimensionMismatch):
        srv.submit(serving.Request(matrix=mid, X=torch.zeros(99, dtype=torch.float64)))
    with pytest.raises(ArgumentError):
        srv.submit(serving.Request(matrix=mid, X=torch.zeros(100, dtype=torch.float32)))
    with pytest.raises(ArgumentError):
        srv.submit(serving.Request(matrix=mid, X=torch.zeros(100, dtype=torch.float64), beta=0.5))


def test_run_realtime_with_manual_clock():
    clk, reg, mid, ex, srv = setup(per_launch=0.01)
    reqs = [req(mid, arrival=0.001 * i) for i in range(50)]

    def tick():
        clk.t += 0.0005
        return clk.t
    srv.clock = tick
    ex.clock = lambda: clk.t
    srv.run(reqs)
    st = srv.stats()
    assert st["done"] == 50
    assert st["launches"] < 50       # coalesced
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_work_cap_splits_launches():
    """A launch takes queued requests while their multiply-adds stay under the work cap (50
    per SpMV of the 50-entry matrix, 150 with k = 3); a request over the cap goes alone, and
    the next free slot takes the rest in arrival order."""
    clk, reg, mid, ex, srv = setup(slots=3, work_cap=120)
    ids = [srv.submit(req(mid)) for _ in range(3)] + [srv.submit(req(mid, k=3))] + [srv.submit(req(mid))]
    assert [r.fma for r in srv.queue] == [50, 50, 50, 150, 50]
    srv.step()
    assert [w for _, w, _ in ex.launched] == [[ids[0], ids[1]], [ids[2]], [ids[3]]]
    assert [s for s, _, _ in ex.launched] == [0, 1, 2]
    clk.t = 1.0
    srv.step()
    assert ex.launched[-1][1] == [ids[4]]
    clk.t = 2.0
    srv.step()
    assert not srv.busy()
    assert sum(r.state == "done" for r in srv.finished) == 5
    st = srv.stats()
    assert st["fma_per_s"] == pytest.approx(350 / 2.0)
