"""Served mul! stream on the GPU: every request's result is the same alone and in the mix
(continuous batching into grouped launches on two streams), within 1e-12 of the request's
per-row scale sum |a||x|; a sample also against the double-double oracle."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_results_alone_equal_results_in_the_mix(gsa, oracle, cuda):
    from genericsparsearrays_gb300 import serving
    mats = serving.registry_matrices(count=16, n_lo=500, n_hi=20_000, seed=4, device=cuda)
    reg = serving.Registry(8 << 30)
    ids = [reg.add(A) for A in mats]
    g = torch.Generator(device=cuda).manual_seed(9)
    xs = {}
    for mid in ids:
        A = reg[mid]
        re = torch.rand((8, A.n), generator=g, device=cuda, dtype=torch.float64) * 2 - 1
        if A.dtype == torch.complex128:
            im = torch.rand((8, A.n), generator=g, device=cuda, dtype=torch.float64) * 2 - 1
            xs[mid] = torch.complex(re, im).t()
        else:
            xs[mid] = re.t()
    torch.cuda.synchronize()
    reqs = serving.poisson_requests(reg, xs, rate=20_000, duration=0.02, k_lo=1, k_hi=8, seed=2)
    assert len(reqs) > 200
    ex = serving.GroupedExecutor(cuda, slots=2)
    srv = serving.Server(reg, ex, max_batch=64, slots=2)
    t0 = srv.clock()
    for r in reqs:
        r.arrival += t0
    srv.run(reqs)
    torch.cuda.synchronize()
    st = srv.stats()
    assert st["done"] == len(reqs) and st["launches"] < len(reqs)
    assert reg.used == reg.resident
    for i, r in enumerate(reqs):
        A = reg[r.matrix]
        alone = torch.empty_like(r.Y)
        gsa.mul_(alone, A, r.X)
        absA = gsa.GenericSparseMatrixCSR(A.m, A.n, A.rowptr, A.colval, A.nzval.abs().to(torch.float64))
        scale = torch.empty(r.Y.shape, dtype=torch.float64, device=cuda)
        gsa.mul_(scale, absA, r.X.abs().to(torch.float64).contiguous() if r.X.dim() == 1 else
                 r.X.abs().to(torch.float64).t().contiguous().t())
        err = ((r.Y - alone).abs() / scale.clamp_min(1e-300)).max().item() if r.Y.numel() else 0.0
        assert err <= 1e-12, (i, err)
        if i % 40 == 0:  # against the double-double oracle too
            Xh = r.X.cpu().numpy()
            ye, sc = oracle.mul_exact("csr", "N", A.m, A.n, A.rowptr.cpu().numpy(), A.colval.cpu().numpy(),
                                      A.nzval.cpu().numpy(), 1, Xh, np.zeros(Xh.shape, Xh.dtype))
            assert oracle.max_rel_error(r.Y.cpu().numpy(), ye, sc) <= 1e-12


def test_per_call_baseline_runs(gsa, cuda):
    from genericsparsearrays_gb300 import serving
    mats = serving.registry_matrices(count=4, n_lo=500, n_hi=5_000, seed=5, device=cuda)
    reg = serving.Registry(1 << 30)
    ids = [reg.add(A) for A in mats]
    xs = {mid: torch.ones((4, reg[mid].n), dtype=reg[mid].dtype, device=cuda).t() for mid in ids}
    reqs = serving.poisson_requests(reg, xs, rate=5_000, duration=0.01, k_lo=1, k_hi=4, seed=1)
    t0 = serving.time.perf_counter()
    for r in reqs:
        r.arrival += t0
    st = serving.serve_per_call(reg, reqs, cuda)
    assert st["done"] == len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0
