"""Three-argument dot(x, op(A), y) on the GPU through the C ABI against the oracle.

The reference's shared suites (test/shared/matrix_{csr,csc,coo}.jl "Three-argument dot")
take 100x80 sprand at density 0.1 for every element type and op(A); here also both index
types, long rows (planned), and integers bit-exact."""
import numpy as np
import pytest
import torch

from helpers import INDEX_TYPES, OPS, VALUE_TYPES, is_int, parts, rand_values, sprand, tol

pytestmark = pytest.mark.gpu

CLS = {"csr": "GenericSparseMatrixCSR", "csc": "GenericSparseMatrixCSC", "coo": "GenericSparseMatrixCOO"}


def wrap(gsa, A, op):
    return A if op == "N" else (gsa.transpose(A) if op == "T" else gsa.adjoint(A))


def check(oracle, fmt, op, m, n, p0, p1, v, x, y, got):
    ref, exact, scale = oracle.dot(fmt, op, m, n, p0, p1, v, 1, x, y)
    if is_int(v.dtype):
        assert got == ref, f"{fmt} {op}: {got} != {ref}"
    else:
        err = abs(complex(got) - complex(exact)) / (scale if scale > 0 else 1.0)
        assert err <= tol(v.dtype), f"{fmt} {op}: rel error {err:.3e}"


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_shared_suite_dot(gsa, oracle, cuda, fmt, it, dt):
    rng = np.random.default_rng(17)
    for op in OPS:
        m, n = (100, 80) if op == "N" else (80, 100)
        S = sprand(rng, m, n, 0.1, dt)
        p0, p1, v = parts(S, fmt, it)
        A = getattr(gsa, CLS[fmt])(m, n, p0, p1, v)
        A = gsa.adapt(cuda, A)
        rows, cols = (m, n) if op == "N" else (n, m)
        x = rand_values(rng, rows, dt)
        y = rand_values(rng, cols, dt)
        got = gsa.dot(torch.from_numpy(x).to(cuda), wrap(gsa, A, op), torch.from_numpy(y).to(cuda))
        check(oracle, fmt, op, m, n, p0, p1, v, x, y, got)


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
def test_dot_long_rows_and_empty(gsa, oracle, cuda, dt):
    """Rows of 0 to 60 000 entries (plan chunks), an empty matrix, and a deterministic sum."""
    rng = np.random.default_rng(31)
    n = 70_000
    lengths = np.array([0, 60_000, 1, 0, 5_000, 3, 0, 2, 60_000, 40] + [4] * 5000 + [0] * 40)
    m = lengths.size
    rowptr = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64) + 1
    cols = np.concatenate([np.sort(rng.choice(n, size=l, replace=False)) for l in lengths]).astype(np.int64) + 1
    vals = rand_values(rng, cols.size, dt)
    for fmt, op in (("csr", "N"), ("csr", "C"), ("csc", "N"), ("csc", "T")):
        mm, nn = (m, n) if fmt == "csr" else (n, m)
        A = gsa.adapt(cuda, getattr(gsa, CLS[fmt])(mm, nn, rowptr, cols, vals))
        rows, cnt = (mm, nn) if op == "N" else (nn, mm)
        x = rand_values(rng, rows, dt)
        y = rand_values(rng, cnt, dt)
        xd, yd = torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)
        got = gsa.dot(xd, wrap(gsa, A, op), yd)
        assert gsa.dot(xd, wrap(gsa, A, op), yd) == got  # fixed summation order
        check(oracle, fmt, op, mm, nn, rowptr, cols, vals, x, y, got)
    E = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(5, 4, np.ones(6, np.int64), np.zeros(0, np.int64),
                                                   np.zeros(0, dt)))
    z = gsa.dot(torch.ones(5, dtype=E.dtype, device=cuda), E, torch.ones(4, dtype=E.dtype, device=cuda))
    assert z == 0


def test_dot_power_law_full_size(gsa, oracle, cuda):
    """The n = 1e6 power-law ComplexF64 matrix (rows up to 50 000 entries)."""
    from genericsparsearrays_gb300 import workloads
    m, n, rp, cv, nz = workloads.power_law(1_000_000, seed=0, itype=np.int64, dtype=np.complex128)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    got = gsa.dot(torch.from_numpy(x).to(cuda), A, torch.from_numpy(y).to(cuda))
    check(oracle, "csr", "N", m, n, rp, cv, nz, x, y, got)
