"""mul! on the GPU through the C ABI against the oracle (parity tests proper).

Floating point: per-row error against the double-double oracle within 1e-12 (F64/C64) or 1e-5
(F32/C32) of |alpha| sum|a||b| + |beta||C|.  Integers: bit-exact against the oracle's
restatement of the reference kernels.
"""
import zlib

import numpy as np
import pytest
import torch

from helpers import (INDEX_TYPES, OPS, VALUE_TYPES, dense_parent, is_complex, is_int, op_apply,
                     parts, rand_values, sprand, tol)

pytestmark = pytest.mark.gpu

CLS = {"csr": "GenericSparseMatrixCSR", "csc": "GenericSparseMatrixCSC", "coo": "GenericSparseMatrixCOO"}


def make(gsa, fmt, m, n, p0, p1, v, dev):
    return gsa.adapt(dev, getattr(gsa, CLS[fmt])(m, n, p0, p1, v))


def wrap(gsa, X, op):
    return X if op == "N" else (gsa.transpose(X) if op == "T" else gsa.adjoint(X))


def check(oracle, fmt, opA, m, n, p0, p1, v, P, opB, C0, C_gpu, alpha, beta, dt):
    C_gpu = C_gpu.cpu().numpy()
    if is_int(dt):
        C = np.asfortranarray(C0.copy())
        oracle.mul(fmt, opA, m, n, p0, p1, v, 1, P, C, alpha=alpha, beta=beta, opB=opB)
        assert np.array_equal(C_gpu, C), "integer product differs from the oracle"
        return 0.0
    ye, sc = oracle.mul_exact(fmt, opA, m, n, p0, p1, v, 1, P, C0, alpha=alpha, beta=beta, opB=opB)
    err = oracle.max_rel_error(C_gpu, ye, sc)
    assert err <= tol(dt), f"{fmt} op(A)={opA} op(B)={opB}: max rel error {err:.3e} > {tol(dt)}"
    return err


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_shared_suite_parity(gsa, oracle, cuda, fmt, it, dt):
    """test/shared/matrix_{csr,csc,coo}.jl mul! sections: 100x80 at density 0.1, b of 80, B of
    80x50, all op(A) x op(B); plus alpha/beta (the reference never tests 5-arg mul!).  Complex
    CSR-T, CSC-N and COO, skipped by the reference (KA @atomic), are covered here."""
    rng = np.random.default_rng(zlib.crc32(f"{fmt}-{np.dtype(it)}-{np.dtype(dt)}".encode()))
    scalars = [(1, 0), (2, 1), (3, 2)]
    if is_complex(dt):
        scalars.append((0.5 - 1j, 2 + 0.25j))
    for opA in OPS:
        m, n = (100, 80) if opA == "N" else (80, 100)
        S = sprand(rng, m, n, 0.1, dt)
        p0, p1, v = parts(S, fmt, it)
        A = wrap(gsa, make(gsa, fmt, m, n, p0, p1, v, cuda), opA)
        for opB in OPS:
            for k in (1, 50):
                P = dense_parent(rng, 80, k, opB, dt)
                Pd = torch.from_numpy(P).to(cuda)
                if k == 1 and opB == "N":
                    P, Pd = P[:, 0].copy(), Pd[:, 0].contiguous()
                B = wrap(gsa, Pd, opB)
                for alpha, beta in scalars:
                    C0 = rand_values(rng, (100,) if (k == 1 and opB == "N") else (100, k), dt)
                    C0 = np.asfortranarray(C0)
                    C = torch.from_numpy(C0).to(cuda)
                    gsa.mul_(C, A, B, alpha, beta)
                    check(oracle, fmt, opA, m, n, p0, p1, v, P, opB, C0, C, alpha, beta, dt)


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
def test_star_matches_mul(gsa, oracle, cuda, fmt):
    """``A * b`` and 3-arg ``mul!`` (what the reference tests call) give the same answer."""
    rng = np.random.default_rng(2)
    S = sprand(rng, 100, 80, 0.1, np.float64)
    p0, p1, v = parts(S, fmt, np.int64)
    A = make(gsa, fmt, 100, 80, p0, p1, v, cuda)
    b = torch.from_numpy(rng.uniform(-1, 1, 80)).to(cuda)
    c1 = (A @ b).cpu().numpy()
    c2 = torch.full((100,), float("nan"), dtype=torch.float64, device=cuda)
    gsa.mul_(c2, A, b)
    if fmt == "csr":  # the gather has no atomics: identical results
        assert np.array_equal(c1, c2.cpu().numpy())
    ye, sc = oracle.mul_exact(fmt, "N", 100, 80, p0, p1, v, 1, b.cpu().numpy(), np.zeros(100))
    assert oracle.max_rel_error(c1, ye, sc) <= 1e-12
    assert oracle.max_rel_error(c2.cpu().numpy(), ye, sc) <= 1e-12


def test_docs_example(gsa, cuda):
    """docs/src/index.md:47-58 on the GPU: CSC times [1,2,3] == [10, 3, 15] exactly."""
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))["docs_spmv_3x3"]
    for fmt, keys in (("csc", ("colptr", "rowval")), ("csr", ("rowptr", "colval")), ("coo", ("rowind", "colind"))):
        a = g[fmt]
        A = make(gsa, fmt, 3, 3, np.array(a[keys[0]]), np.array(a[keys[1]]), np.array(a["nzval"]), cuda)
        c = A @ torch.tensor(g["b"], dtype=torch.float64, device=cuda)
        assert c.cpu().tolist() == g["c"]


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
def test_beta_zero_overwrites_nan(gsa, cuda, fmt):
    rng = np.random.default_rng(9)
    S = sprand(rng, 64, 48, 0.2, np.float64)
    p0, p1, v = parts(S, fmt, np.int32)
    A = make(gsa, fmt, 64, 48, p0, p1, v, cuda)
    x = torch.from_numpy(rng.uniform(-1, 1, 48)).to(cuda)
    C = torch.full((64,), float("nan"), dtype=torch.float64, device=cuda)
    gsa.mul_(C, A, x, 1.0, 0.0)
    assert torch.isfinite(C).all()


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("algo", [0, 2])
def test_edge_shapes(gsa, oracle, cuda, fmt, algo):
    """Empty matrix, empty rows, k = 0, m = 0 and n = 0: beta still applies (or not)."""
    rng = np.random.default_rng(4)
    cases = [(0, 5), (5, 0), (7, 6), (1, 1)]
    for m, n in cases:
        for density in (0.0, 0.5):
            S = sprand(rng, m, n, density, np.float64) if m and n else None
            if S is None:
                import scipy.sparse as sp
                S = sp.csr_matrix((m, n))
            p0, p1, v = parts(S, fmt, np.int64)
            A = make(gsa, fmt, m, n, p0, p1, v, cuda)
            for k in (0, 1, 3):
                X = np.asfortranarray(rng.uniform(-1, 1, (n, k)))
                C0 = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
                C = torch.from_numpy(C0).to(cuda)
                if fmt == "coo":
                    gsa.mul_(C, A, torch.from_numpy(X).to(cuda), 2.0, 0.5)
                else:
                    gsa.mul_(C, A, torch.from_numpy(X).to(cuda), 2.0, 0.5, algo=algo)
                if m and k:
                    ye, sc = oracle.mul_exact(fmt, "N", m, n, p0, p1, v, 1, X, C0, alpha=2.0, beta=0.5)
                    assert oracle.max_rel_error(C.cpu().numpy(), ye, sc) <= 1e-12


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
@pytest.mark.parametrize("k", [1, 3])
def test_long_rows_cross_tiles(gsa, oracle, cuda, dt, k):
    """Rows of 0, 1, 5 000 and 60 000 entries mixed: merge-path tiles split long rows over
    many CTAs; the open-row partials must come back in full (integers: bit-exact)."""
    rng = np.random.default_rng(12)
    n = 70_000
    lengths = np.array([0, 60_000, 1, 0, 5_000, 3, 0, 0, 2, 60_000] + [4] * 500 + [0] * 40)
    m = lengths.size
    rowptr = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64) + 1
    cols = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lengths]).astype(np.int64) + 1
    vals = rand_values(rng, cols.size, dt)
    for algo in (0, 1, 2, 3):
        if algo == 3 and k > 1:
            continue
        for fmt in ("csr", "csc_t"):
            if fmt == "csr":
                A = make(gsa, "csr", m, n, rowptr, cols, vals, cuda)
                opA, f, mm, nn = "N", "csr", m, n
            else:  # the same arrays as a CSC of the transpose; op(A) = T gathers
                A = gsa.transpose(make(gsa, "csc", n, m, rowptr, cols, vals, cuda))
                opA, f, mm, nn = "T", "csc", n, m
            X = np.asfortranarray(rand_values(rng, (n, k), dt))
            C0 = np.asfortranarray(rand_values(rng, (m, k), dt))
            C = torch.from_numpy(C0).to(cuda)
            gsa.mul_(C, A, torch.from_numpy(X).to(cuda), 3, 2, algo=algo)
            check(oracle, f, opA, mm, nn, rowptr, cols, vals, X, "N", C0, C, 3, 2, dt)


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
@pytest.mark.parametrize("k", [1, 3])
def test_long_columns_scatter(gsa, oracle, cuda, dt, k):
    """The scatter directions (CSC N, CSR T) over outer entries of 0 to 60 000 entries: the
    default outer blocks with and without a plan (long entries chunked over warps) and the
    merge-path tiles; integers bit-exact."""
    rng = np.random.default_rng(13)
    m = 70_000
    lengths = np.array([0, 60_000, 1, 0, 5_000, 3, 0, 0, 2, 60_000, 40] + [4] * 500 + [0] * 40)
    n = lengths.size
    colptr = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64) + 1
    rows = np.concatenate([np.sort(rng.choice(m, size=l, replace=False)) for l in lengths]).astype(np.int64) + 1
    vals = rand_values(rng, rows.size, dt)
    for algo in (0, 1, 2):
        for fmt in ("csc", "csr_t"):
            if fmt == "csc":
                A = make(gsa, "csc", m, n, colptr, rows, vals, cuda)
                opA, f, mm, nn = "N", "csc", m, n
            else:  # the same arrays as a CSR of the transpose; op(A) = T scatters
                A = gsa.transpose(make(gsa, "csr", n, m, colptr, rows, vals, cuda))
                opA, f, mm, nn = "T", "csr", n, m
            X = np.asfortranarray(rand_values(rng, (n, k), dt))
            C0 = np.asfortranarray(rand_values(rng, (m, k), dt))
            C = torch.from_numpy(C0).to(cuda)
            gsa.mul_(C, A, torch.from_numpy(X).to(cuda), 3, 2, algo=algo)
            check(oracle, f, opA, mm, nn, colptr, rows, vals, X, "N", C0, C, 3, 2, dt)


def test_gather_is_deterministic(gsa, cuda):
    """The CSR gather uses no atomics: two runs are bit-identical."""
    from genericsparsearrays_gb300 import workloads
    m, n, rp, cv, nz = workloads.power_law(n=200_000, seed=3, itype=np.int64, dtype=np.float64)
    A = make(gsa, "csr", m, n, rp, cv, nz, cuda)
    x = torch.randn(n, dtype=torch.float64, device=cuda)
    for algo in (gsa.ALGO_AUTO, gsa.ALGO_MERGE, gsa.ALGO_PIPE):
        y1 = torch.empty(m, dtype=torch.float64, device=cuda)
        y2 = torch.empty(m, dtype=torch.float64, device=cuda)
        gsa.mul_(y1, A, x, algo=algo)
        gsa.mul_(y2, A, x, algo=algo)
        assert torch.equal(y1, y2)


@pytest.mark.parametrize("order", ["rows", "storage", "shuffle"])
def test_coo_orders_and_duplicates(gsa, oracle, cuda, order):
    """COO in row order, column order (as built from SparseMatrixCSC) and random order, with
    duplicated entries: every stored entry contributes (no merging), as in the reference."""
    rng = np.random.default_rng(21)
    S = sprand(rng, 300, 200, 0.05, np.complex128)
    r, c, v = parts(S, "coo", np.int32, order=order, rng=rng)
    r = np.concatenate([r, r[:50]])
    c = np.concatenate([c, c[:50]])
    v = np.concatenate([v, v[:50] * 2])
    A = make(gsa, "coo", 300, 200, r, c, v, cuda)
    for opA in OPS:
        rows_out, inner = (300, 200) if opA == "N" else (200, 300)
        X = np.asfortranarray(rand_values(rng, (inner, 4), np.complex128))
        C0 = np.asfortranarray(rand_values(rng, (rows_out, 4), np.complex128))
        C = torch.from_numpy(C0).to(cuda)
        gsa.mul_(C, wrap(gsa, A, opA), torch.from_numpy(X).to(cuda), 1 + 1j, 0.5)
        check(oracle, "coo", opA, 300, 200, r, c, v, X, "N", C0, C, 1 + 1j, 0.5, np.complex128)


def test_row_major_dense_operands(gsa, oracle, cuda):
    """Row-major torch tensors for B and C work in place of column-major ones."""
    rng = np.random.default_rng(5)
    S = sprand(rng, 120, 90, 0.1, np.float64)
    p0, p1, v = parts(S, "csr", np.int32)
    A = make(gsa, "csr", 120, 90, p0, p1, v, cuda)
    X = rng.uniform(-1, 1, (90, 7))
    Xd = torch.from_numpy(np.ascontiguousarray(X)).to(cuda)  # row-major
    C = torch.zeros(120, 7, dtype=torch.float64, device=cuda)  # row-major
    gsa.mul_(C, A, Xd)
    ye, sc = oracle.mul_exact("csr", "N", 120, 90, p0, p1, v, 1, np.asfortranarray(X), np.zeros((120, 7)))
    assert oracle.max_rel_error(C.cpu().numpy(), ye, sc) <= 1e-12


def test_validate(gsa, cuda):
    rowptr = np.array([1, 3, 2, 4], np.int64)  # decreasing
    A = make(gsa, "csr", 3, 3, rowptr, np.array([1, 2, 3]), np.array([1.0, 2.0, 3.0]), cuda)
    with pytest.raises(gsa.ArgumentError, match="decreasing"):
        gsa.validate(A)
    B = make(gsa, "csr", 3, 3, np.array([1, 2, 3, 4]), np.array([1, 2, 3]), np.array([1.0, 2.0, 3.0]), cuda)
    gsa.validate(B)


@pytest.mark.parametrize("dt", [np.float64, np.complex64, np.int32])
def test_sparse_rows_span_many_tiles(gsa, oracle, cuda, dt):
    """Mostly empty rows: one merge-path tile spans thousands of rows, beyond the 512-row
    probe, so tile ends come from the pointer search; beta keeps the empty rows' scaling."""
    rng = np.random.default_rng(44)
    m, n = 200_000, 3_000
    lengths = np.zeros(m, np.int64)
    hot = rng.choice(m, 700, replace=False)
    lengths[hot] = rng.integers(1, 40, 700)
    lengths[m // 2] = 2_500  # one long row among them
    rowptr = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int32) + 1
    cols = np.concatenate([np.sort(rng.choice(n, size=int(l), replace=False)) for l in lengths]).astype(np.int32) + 1
    vals = rand_values(rng, cols.size, dt)
    A = make(gsa, "csr", m, n, rowptr, cols, vals, cuda)
    x = rand_values(rng, n, dt)
    C0 = rand_values(rng, m, dt)
    for algo in (0, 1, 2, 3):
        C = torch.from_numpy(C0.copy()).to(cuda)
        gsa.mul_(C, A, torch.from_numpy(x).to(cuda), 2, 3, algo=algo)
        check(oracle, "csr", "N", m, n, rowptr, cols, vals, x, "N", C0, C, 2, 3, dt)


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
@pytest.mark.parametrize("k", [1, 3])
def test_plan_orders(gsa, oracle, cuda, dt, k):
    """Power-law rows: the plan puts them in bin order (rows grouped by length) and chunks
    rows over 512; the natural order (GSA_TUNE_PLAN_ORDER = 1) and the bin order for every FP64
    product (= 2) with the same plan, each for CSR N and the same arrays as a transposed CSC,
    match the oracle."""
    from genericsparsearrays_gb300 import _lib, workloads
    lib = _lib.load()
    m, n, rp, cv, nz = workloads.power_law(n=60_000, cap=5_000, seed=5, itype=np.int64, dtype=np.float64)
    rng = np.random.default_rng(3)
    vals = rand_values(rng, cv.size, dt)
    X = np.asfortranarray(rand_values(rng, (n, k), dt))
    C0 = np.asfortranarray(rand_values(rng, (m, k), dt))
    try:
        for natural in (0, 1, 2):
            assert lib.gsa_set_tuning(_lib.TUNE_PLAN_ORDER, natural) == 0
            for fmt in ("csr", "csc_t"):
                if fmt == "csr":
                    A = make(gsa, "csr", m, n, rp, cv, vals, cuda)
                    opA, f = "N", "csr"
                else:
                    A = gsa.transpose(make(gsa, "csc", n, m, rp, cv, vals, cuda))
                    opA, f = "T", "csc"
                C = torch.from_numpy(C0).to(cuda)
                beta = 3 if is_int(dt) else 0.5
                gsa.mul_(C, A, torch.from_numpy(X).to(cuda), 2, beta)
                plan = (A.parent if fmt == "csc_t" else A)._plan
                assert plan is not None and plan.nlong == m  # bin order takes every row
                mm, nn = (m, n) if fmt == "csr" else (n, m)
                check(oracle, f, opA, mm, nn, rp, cv, vals, X, "N", C0, C, 2, beta, dt)
    finally:
        lib.gsa_set_tuning(_lib.TUNE_PLAN_ORDER, 0)


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
@pytest.mark.parametrize("it", INDEX_TYPES)
def test_row_sorted_coo_uses_row_pointers(gsa, oracle, cuda, dt, it):
    """A COO whose rows are non-decreasing (columns in any order, duplicates adjacent or not
    within a row) gets a plan with row pointers and runs the CSR kernels: every op, k = 1 and
    3, against the oracle; an unsorted COO keeps the COO kernel and gives the same answers."""
    rng = np.random.default_rng(8)
    m, n = 5000, 700
    lengths = rng.poisson(6, m)
    lengths[[7, 4000]] = [2000, 900]  # long rows: chunks
    lengths[100:140] = 0
    rows = np.repeat(np.arange(m), lengths)
    cols = rng.integers(0, n, rows.size)  # repeats allowed, unsorted inside rows
    vals = rand_values(rng, rows.size, dt)
    r1, c1 = (rows + 1).astype(it), (cols + 1).astype(it)
    for order in ("sorted", "shuffled"):
        if order == "shuffled":
            p = rng.permutation(rows.size)
            r, c, v = r1[p], c1[p], vals[p]
        else:
            r, c, v = r1, c1, vals
        A = make(gsa, "coo", m, n, r, c, v, cuda)
        for opA in OPS:
            rows_out, inner = (m, n) if opA == "N" else (n, m)
            for k in (1, 3):
                X = np.asfortranarray(rand_values(rng, (inner, k), dt))
                C0 = np.asfortranarray(rand_values(rng, (rows_out, k), dt))
                C = torch.from_numpy(C0).to(cuda)
                gsa.mul_(C, wrap(gsa, A, opA), torch.from_numpy(X).to(cuda), 2, 3)
                check(oracle, "coo", opA, m, n, r, c, v, X, "N", C0, C, 2, 3, dt)
        assert (A._plan is not None) == (order == "sorted")


@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_window_scatter(gsa, oracle, cuda, dt, it):
    """GSA_ALGO_VECTOR on the scatter directions (CSC N, CSR T/C) with one right-hand side:
    products near the CTA's outer range summed in a shared-memory window first.  A banded
    matrix (half-band 70, wider than the window's halo) plus random far entries and empty
    columns, alpha and beta general, against the oracle (integers bit-exact)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(zlib.crc32(f"win-{np.dtype(it)}-{np.dtype(dt)}".encode()))
    m = n = 3000
    offs = list(range(-70, 71, 7))
    S = sp.diags([np.ones(n - abs(o)) for o in offs], offs, shape=(m, n), format="csr")
    S = (S + sprand(rng, m, n, 0.002, np.float64)).tocsr()
    S = S.tolil()
    S[:, 1500:1510] = 0  # empty columns
    S = S.tocsr()
    S.eliminate_zeros()
    S.sort_indices()
    S = sp.csr_matrix((rand_values(rng, S.nnz, dt), S.indices, S.indptr), shape=(m, n))
    for fmt, opA in (("csc", "N"), ("csr", "T"), ("csr", "C")):
        p0, p1, v = parts(S, fmt, it)
        A = wrap(gsa, make(gsa, fmt, m, n, p0, p1, v, cuda), opA)
        x = rand_values(rng, n, dt)
        C0 = rand_values(rng, m, dt)
        C = torch.from_numpy(C0).to(cuda)
        alpha, beta = (3, 2) if not is_complex(dt) else (0.5 - 1j, 2 + 0.25j)
        gsa.mul_(C, A, torch.from_numpy(x).to(cuda), alpha, beta, algo=gsa.ALGO_VECTOR)
        check(oracle, fmt, opA, m, n, p0, p1, v, x, "N", C0, C, alpha, beta, dt)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_staged_rows_match_direct(gsa, oracle, cuda, dt):
    """GSA_TUNE_STAGE_ROWS = 1 (warps of thread-per-row rows copy their entry span with 16-byte
    loads) and 2 (each lane reads its row in 16-byte pieces into registers): bit-identical to the
    direct loads (same summation order), within the oracle's
    tolerance; with long rows taken by a plan, empty rows, a last CTA with a warp past the last
    row, the last warp's span at the end of the arrays, and misaligned arrays (a view one entry
    in), which take the direct path."""
    from genericsparsearrays_gb300 import workloads
    L = gsa._lib
    lib = L.load()
    m, n, rp, cv, nz = workloads.random_poisson(50_001, mean=4.0, seed=12, itype=np.int32, dtype=dt)
    lens = np.diff(rp.astype(np.int64))
    lens[::997] = 0          # empty rows
    lens[5:4000:401] = 700   # long rows (plan chunks)
    rng = np.random.default_rng(13)
    rp = np.concatenate([[1], 1 + np.cumsum(lens)]).astype(np.int32)
    cv = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lens]).astype(np.int32) + 1
    nz = rng.uniform(-1, 1, cv.size).astype(dt)
    x = rng.uniform(-1, 1, n).astype(dt)
    ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, 1, x, np.zeros(m, dt))
    tol = 1e-12 if dt == np.float64 else 1e-5
    xd = torch.from_numpy(x).to(cuda)
    cv_pad = torch.from_numpy(np.concatenate([[1], cv]).astype(np.int32)).to(cuda)
    nz_pad = torch.from_numpy(np.concatenate([[0], nz]).astype(dt)).to(cuda)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    Am = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    Am.colval, Am.nzval = cv_pad[1:], nz_pad[1:]  # the constructor copies: point at the views
    assert Am.colval.data_ptr() % 16 == 4
    saved = lib.gsa_get_tuning(L.TUNE_STAGE_ROWS)
    try:
        for M in (A, Am):
            ys = []
            for stage in (0, 1, 2):
                assert lib.gsa_set_tuning(L.TUNE_STAGE_ROWS, stage) == L.OK
                y = torch.full((m,), float("nan"), dtype=xd.dtype, device=cuda)
                gsa.mul_(y, M, xd)
                ys.append(y.cpu().numpy())
            assert np.array_equal(ys[0], ys[1]) and np.array_equal(ys[0], ys[2])
            assert oracle.max_rel_error(ys[1], ye, sc) <= tol
    finally:
        lib.gsa_set_tuning(L.TUNE_STAGE_ROWS, saved)


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_row_major_pairs_match_single_loads(gsa, oracle, cuda, it):
    """Float64 SpMM with a row-major X (the served layout: the first k columns of an n x 32
    block): two columns per 16-byte load (GSA_TUNE_X_PAIRS = 1, the default) gives the bits of
    one load per column, for odd and even k, planned and plain, and is within the oracle's
    tolerance; an odd row stride falls back to single loads."""
    L = gsa._lib
    lib = L.load()
    rng = np.random.default_rng(31)
    S = sprand(rng, 3000, 2500, 0.006, np.float64)
    p0, p1, v = parts(S, "csr", it)
    A = make(gsa, "csr", 3000, 2500, p0, p1, v, cuda)
    for ld in (32, 33):
        block = rand_values(rng, (2500, ld), np.float64)
        Bd = torch.from_numpy(block).to(cuda)
        for k in (2, 5, 8, 16, 32 if ld == 32 else 31):
            X = Bd[:, :k]
            ye, sc = oracle.mul_exact("csr", "N", 3000, 2500, p0, p1, v, 1, np.asfortranarray(block[:, :k]),
                                      np.zeros((3000, k), order="F"))
            got = []
            for pairs in (1, 0):
                assert lib.gsa_set_tuning(L.TUNE_X_PAIRS, pairs) == L.OK
                Y = torch.empty((k, 3000), dtype=torch.float64, device=cuda).t()
                gsa.mul_(Y, A, X)
                got.append(Y.cpu().numpy())
            lib.gsa_set_tuning(L.TUNE_X_PAIRS, 1)
            assert np.array_equal(got[0], got[1]), (ld, k)
            assert oracle.max_rel_error(got[0], ye, sc) <= 1e-12
