"""Grouped products (one launch for many CSR mul!): against the per-call path (bit for bit:
same row code and order) and the oracle; CUDA-graph replay after refilling the operands."""
import numpy as np
import pytest
import torch

from helpers import rand_values

pytestmark = pytest.mark.gpu


def make_products(gsa, wl, cuda, count, dt, ks, seed):
    sizes, rp, cv, nz, ro, eo = wl.banded_batch(count=count, lo=16, hi=3000, seed=seed,
                                                itype=np.int64, dtype=dt, device=cuda)
    rng = np.random.default_rng(seed)
    prods, host = [], []
    for i, m in enumerate(sizes):
        p = rp[int(ro[i]) + i: int(ro[i + 1]) + i + 1]
        c = cv[int(eo[i]): int(eo[i + 1])]
        v = nz[int(eo[i]): int(eo[i + 1])]
        A = gsa.GenericSparseMatrixCSR(m, m, p, c, v)
        k = ks[i % len(ks)]
        X = rand_values(rng, (m,) if k == 1 else (m, k), dt)
        Y0 = rand_values(rng, (m,) if k == 1 else (m, k), dt)
        Xd = torch.from_numpy(np.asfortranarray(X)).to(cuda)
        Yd = torch.from_numpy(np.asfortranarray(Y0)).to(cuda)
        alpha, beta = (1.5, 0.5) if i % 3 else (1, 0)
        prods.append((A, Xd, Yd, alpha, beta))
        host.append((p.cpu().numpy(), c.cpu().numpy(), v.cpu().numpy(), X, Y0, alpha, beta, m))
    return prods, host


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_grouped_matches_per_call_and_oracle(gsa, oracle, cuda, dt):
    from genericsparsearrays_gb300 import batch, workloads as wl
    prods, host = make_products(gsa, wl, cuda, 96, dt, ks=(1, 4, 3, 8), seed=3)
    Y0s = [p[2].clone() for p in prods]
    b = batch.BatchedMul(prods, use_plans=False)  # natural row blocks: the per-call code exactly
    b.run("grouped")
    grouped = [p[2].clone() for p in prods]
    for p, y0 in zip(prods, Y0s):
        p[2].copy_(y0)
    b.run("per_call")
    per_call = [p[2].clone() for p in prods]
    torch.cuda.synchronize()
    for g, q in zip(grouped, per_call):
        assert torch.equal(g, q), "grouped and per-call results differ"
    for (p, c, v, X, Y0, alpha, beta, m), g in zip(host, grouped):
        ye, sc = oracle.mul_exact("csr", "N", m, m, p, c, v, 1, X, Y0, alpha=alpha, beta=beta)
        assert oracle.max_rel_error(g.cpu().numpy(), ye, sc) <= 1e-12
    b.close()
    # with plans: ComplexF64 items and Float64 items with k > 1 walk their plans' bin order
    for p, y0 in zip(prods, Y0s):
        p[2].copy_(y0)
    items, _, _ = batch.pack_items(prods)
    if dt == np.complex128:
        assert (items["bin_warps"] > 0).sum() > len(prods) // 2
    else:  # Float64: the FP64-bound products (k > 1) walk the bin order, SpMVs do not
        assert (items["bin_warps"][items["k"] == 1] == 0).all()
        assert (items["bin_warps"][items["k"] > 1] > 0).sum() > (items["k"] > 1).sum() // 2
    b2 = batch.BatchedMul(prods)
    b2.run("graph")
    torch.cuda.synchronize()
    for (p, c, v, X, Y0, alpha, beta, m), q in zip(host, prods):
        ye, sc = oracle.mul_exact("csr", "N", m, m, p, c, v, 1, X, Y0, alpha=alpha, beta=beta)
        assert oracle.max_rel_error(q[2].cpu().numpy(), ye, sc) <= 1e-12
    b2.close()


def test_graph_replay_after_refill(gsa, oracle, cuda):
    from genericsparsearrays_gb300 import batch, workloads as wl
    prods, host = make_products(gsa, wl, cuda, 40, np.complex128, ks=(1,), seed=5)
    b = batch.BatchedMul(prods)
    rng = np.random.default_rng(6)
    for rep in range(3):
        xs = []
        for (A, X, Y, alpha, beta), h in zip(prods, host):
            xn = rand_values(rng, X.shape[0], np.complex128)
            X.copy_(torch.from_numpy(xn))
            Y.zero_()
            xs.append(xn)
        b.run("graph")
        torch.cuda.synchronize()
        for (A, X, Y, alpha, beta), (p, c, v, _, _, _, _, m), xn in zip(prods, host, xs):
            ye, sc = oracle.mul_exact("csr", "N", m, m, p, c, v, 1, xn, np.zeros(m, np.complex128),
                                      alpha=alpha, beta=beta)
            assert oracle.max_rel_error(Y.cpu().numpy(), ye, sc) <= 1e-12
    b.close()


def test_grouped_launcher_and_autotune(gsa, cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("GSA_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    from genericsparsearrays_gb300 import autotune, batch, workloads as wl
    prods, host = make_products(gsa, wl, cuda, 30, np.float64, ks=(1,), seed=8)
    cols, g1 = autotune.tune(prods, reps=1)
    assert cols in autotune.CANDIDATE_COLUMNS and g1 in autotune.CANDIDATE_G1
    assert autotune.tune(prods) == (cols, g1)  # cached
    Y0s = [p[2].clone() for p in prods]
    b = batch.BatchedMul(prods, columns=cols, g1_avg=g1)
    b.run("grouped")
    ref = [p[2].clone() for p in prods]
    for p, y0 in zip(prods, Y0s):
        p[2].copy_(y0)
    launcher = batch.GroupedLauncher(cuda, capacity=4, columns=cols, g1_avg=g1)
    launcher.launch(prods[:10])
    launcher.launch(prods[10:])
    torch.cuda.synchronize()
    for p, r in zip(prods, ref):
        assert torch.equal(p[2], r)
    b.close()


def test_row_major_right_hand_sides(gsa, oracle, cuda):
    """Row-major X blocks (and a strided column of one) in a grouped launch: the same bits
    as the per-call path (which reads them as op(B) = T of the parent), and the oracle."""
    from genericsparsearrays_gb300 import batch, workloads as wl
    sizes, rp, cv, nz, ro, eo = wl.banded_batch(count=24, lo=16, hi=2000, seed=7, itype=np.int32,
                                                dtype=np.complex128, device=cuda)
    rng = np.random.default_rng(7)
    prods, host = [], []
    for i, m in enumerate(sizes):
        p = rp[int(ro[i]) + i: int(ro[i + 1]) + i + 1]
        c = cv[int(eo[i]): int(eo[i + 1])]
        v = nz[int(eo[i]): int(eo[i + 1])]
        A = gsa.GenericSparseMatrixCSR(m, m, p, c, v)
        block = torch.from_numpy(rand_values(rng, (m, 8), np.complex128)).to(cuda)  # row-major
        k = (1, 3, 8)[i % 3]
        X = block[:, 0] if k == 1 else block[:, :k]
        Y = torch.zeros((m,) if k == 1 else (k, m), dtype=torch.complex128, device=cuda)
        Y = Y if k == 1 else Y.t()
        prods.append((A, X, Y, 2.0, 0))
        host.append((p.cpu().numpy(), c.cpu().numpy(), v.cpu().numpy(), X.cpu().numpy(), m, k))
    b = batch.BatchedMul(prods, use_plans=False)
    b.run("graph")
    got = [q[2].clone() for q in prods]
    b.run("per_call")
    torch.cuda.synchronize()
    for q, g in zip(prods, got):
        assert torch.equal(q[2], g)
    for (p, c, v, X, m, k), g in zip(host, got):
        ye, sc = oracle.mul_exact("csr", "N", m, m, p, c, v, 1, X, np.zeros((m,) if k == 1 else (m, k), np.complex128),
                                  alpha=2.0)
        assert oracle.max_rel_error(g.cpu().numpy(), ye, sc) <= 1e-12
    b.close()


def test_full_uneven_mix_every_product(gsa, oracle, cuda):
    """The benchmark's batched workload at full size: 4096 banded ComplexF64 CSR matrices (n
    log-uniform in [64, 8192], half-band 3 plus Poisson(8) off-band entries per row, Int64
    indices), k cycled 1/4/8, one grouped launch replayed from a CUDA graph with the bin
    orders of their plans; every product against the double-double oracle (1e-12)."""
    from concurrent.futures import ThreadPoolExecutor
    from genericsparsearrays_gb300 import batch, workloads as wl
    count, ks = 4096, (1, 4, 8)
    sizes, rp, cv, nz, ro, eo = wl.banded_batch(count=count, lo=64, hi=8192, seed=11, itype=np.int64,
                                                dtype=np.complex128, device=cuda)
    g = torch.Generator(device=cuda).manual_seed(13)
    prods = []
    for i, m in enumerate(sizes):
        A = gsa.GenericSparseMatrixCSR(m, m, rp[int(ro[i]) + i: int(ro[i + 1]) + i + 1],
                                       cv[int(eo[i]): int(eo[i + 1])], nz[int(eo[i]): int(eo[i + 1])])
        k = ks[i % len(ks)]
        shape = (m,) if k == 1 else (k, m)
        X = torch.complex(torch.rand(shape, generator=g, device=cuda, dtype=torch.float64) * 2 - 1,
                          torch.rand(shape, generator=g, device=cuda, dtype=torch.float64) * 2 - 1)
        Y = torch.full(shape, float("nan"), dtype=torch.complex128, device=cuda)  # beta = 0 never reads Y
        if k > 1:
            X, Y = X.t(), Y.t()
        prods.append((A, X, Y, 1, 0))
    del rp, cv, nz
    b = batch.BatchedMul(prods)
    b.run("graph")
    b.run("graph")  # a replay of the captured graph
    torch.cuda.synchronize()
    host = [(A.m, A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy(),
             np.asfortranarray(X.cpu().numpy()), Y.cpu().numpy()) for A, X, Y, _, _ in prods]
    b.close()

    def err(h):
        m, p, c, v, X, Y = h
        ye, sc = oracle.mul_exact("csr", "N", m, m, p, c, v, 1, X, np.zeros(Y.shape, np.complex128))
        return oracle.max_rel_error(Y, ye, sc)

    with ThreadPoolExecutor(max_workers=oracle.max_threads()) as ex:
        errs = list(ex.map(err, host))
    assert len(errs) == count
    worst = int(np.argmax(errs))
    assert errs[worst] <= 1e-12, f"product {worst}: {errs[worst]:.3e}"
