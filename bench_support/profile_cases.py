"""Run one benchmark workload a few times, for a profiler to capture its kernels.

    python bench_support/profile_cases.py CASE [--reps N]

Cases (the bench workloads, same seeds):
  laplacian_csr_f64_i32   CSR SpMV of the 2048^2 5-point Laplacian, Float64 / Int32
  laplacian_csr_f64_i64   the same with Int64 indices
  laplacian_spmm16        the same matrix times a 16-column column-major X
  laplacian_csc_f64_i32   CSC SpMV of the Laplacian (outer-block scatter)
  laplacian_coo_to_csr    COO -> CSR of the Laplacian's randomly permuted triplets
  laplacian_coo_plus_t    the same triplets as a COO, A + transpose(A) (COO sum)
  laplacian_spgemm        A * A of the Laplacian (Float64 / Int32 CSR)
  powerlaw_csr_c64        n = 1e6 power-law ComplexF64 CSR SpMV (planned row blocks)
  powerlaw_coo_c64        the same matrix as row-sorted COO
  powerlaw_coo_to_csr     COO -> CSR of the power-law matrix's randomly permuted triplets
  powerlaw_spgemm_1e5     A * A of an n = 1e5 power-law ComplexF64 CSR matrix
  batched_mix             4096 banded ComplexF64 products in one grouped launch

Each case makes its inputs, runs the product ``--reps`` times (default 3) and synchronizes;
nothing is timed here.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--columns", type=int, default=1,
                    help="batched_mix: right-hand-side columns per thread (the autotuner's pick on GB300: 1)")
    args = ap.parse_args(argv)
    sys.path.insert(0, ROOT)
    import torch
    import __graft_entry__
    gsa = __graft_entry__.load_package()
    from genericsparsearrays_gb300 import workloads as wl
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(0)
    c = args.case
    if c.startswith("laplacian"):
        it = np.int64 if c.endswith("i64") or c in ("laplacian_coo_to_csr", "laplacian_coo_plus_t") else np.int32
        m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=it, dtype=np.float64)
        x = torch.from_numpy(rng.uniform(-1, 1, n)).to(dev)
        y = torch.empty(m, dtype=torch.float64, device=dev)
        if c in ("laplacian_csr_f64_i32", "laplacian_csr_f64_i64"):
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
            run = lambda: gsa.mul_(y, A, x)
        elif c == "laplacian_spmm16":
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
            X = torch.from_numpy(rng.uniform(-1, 1, (16, n))).to(dev).t()
            Y = torch.empty((16, m), dtype=torch.float64, device=dev).t()
            run = lambda: gsa.mul_(Y, A, X)
        elif c == "laplacian_csc_f64_i32":
            K = gsa.adapt(dev, gsa.GenericSparseMatrixCSC(*wl.csr_to_csc(m, n, rp, cv, nz)))
            run = lambda: gsa.mul_(y, K, x)
        elif c in ("laplacian_coo_to_csr", "laplacian_coo_plus_t"):
            _, _, r, cc, v = wl.permuted_coo(m, n, rp, cv, nz, seed=7)
            C = gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, r, cc, v))
            if c == "laplacian_coo_to_csr":
                run = lambda: gsa.GenericSparseMatrixCSR(C)
            else:
                run = lambda: C + gsa.transpose(C)
        elif c == "laplacian_spgemm":
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
            run = lambda: A @ A
        else:
            raise SystemExit(f"unknown case {c}")
    elif c.startswith("powerlaw"):
        m, n, rp, cv, nz = wl.power_law(1_000_000, seed=0, itype=np.int64, dtype=np.complex128)
        x = torch.from_numpy(rng.standard_normal(n) + 1j * rng.standard_normal(n)).to(dev)
        y = torch.empty(m, dtype=torch.complex128, device=dev)
        if c == "powerlaw_csr_c64":
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
        elif c == "powerlaw_coo_c64":
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, wl.csr_rows(rp), cv, nz))
        elif c == "powerlaw_coo_to_csr":
            _, _, r, cc, v = wl.permuted_coo(m, n, rp, cv, nz, seed=2)
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, r, cc, v))
        elif c == "powerlaw_spgemm_1e5":
            m, n, rp, cv, nz = wl.power_law(100_000, seed=0, itype=np.int64, dtype=np.complex128)
            A = gsa.adapt(dev, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
        else:
            raise SystemExit(f"unknown case {c}")
        if c == "powerlaw_coo_to_csr":
            run = lambda: gsa.GenericSparseMatrixCSR(A)
        elif c == "powerlaw_spgemm_1e5":
            run = lambda: A @ A
        else:
            run = lambda: gsa.mul_(y, A, x)
    elif c == "batched_mix":
        from genericsparsearrays_gb300 import batch
        sys.path.insert(0, ROOT)
        import bench
        prods, _ = bench.batched_products(gsa, wl, torch, dev)
        b = batch.BatchedMul(prods, columns=args.columns)
        run = lambda: b.run("grouped")
    else:
        raise SystemExit(f"unknown case {c}")
    for _ in range(args.reps):
        run()
    torch.cuda.synchronize()
    print(f"{c}: {args.reps} runs done")


if __name__ == "__main__":
    main()
