"""Full-size benchmark workloads on the GPU against the oracle: the 2048x2048 Laplacian (SpMV
and SpMM, CSR and CSC, F64 and F32, Int32 and Int64 indices, permuted-COO conversion), the
n = 1e6 power-law ComplexF64 matrix (CSR and COO) and the n = 1e5 Poisson(10) matrix."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wl(gsa):
    from genericsparsearrays_gb300 import workloads
    return workloads


def rel_err_vs(y, ref, scale):
    y = np.asarray(y)
    return float(np.max(np.abs(y - ref) / np.where(scale > 0, scale, 1)))


@pytest.mark.parametrize("it", [np.int32, np.int64])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_laplacian_spmv_csr_csc(gsa, oracle, cuda, wl, it, dt):
    m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=it, dtype=dt)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, n).astype(dt)
    S = sp.csr_matrix((nz.astype(np.float64), cv.astype(np.int64) - 1, rp.astype(np.int64) - 1), shape=(m, n))
    ref = S @ x.astype(np.float64)
    scale = abs(S) @ np.abs(x.astype(np.float64))
    tol = 1e-12 if dt == np.float64 else 1e-5
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    xd = torch.from_numpy(x).to(cuda)
    for algo in (gsa.ALGO_AUTO, gsa.ALGO_MERGE, gsa.ALGO_VECTOR, gsa.ALGO_PIPE):
        y = torch.empty(m, dtype=xd.dtype, device=cuda)
        gsa.mul_(y, A, xd, algo=algo)
        assert rel_err_vs(y.cpu().numpy(), ref, scale) <= tol
    _, _, cp, rv, cz = wl.csr_to_csc(m, n, rp, cv, nz)
    K = gsa.adapt(cuda, gsa.GenericSparseMatrixCSC(m, n, cp, rv, cz))
    y = K @ xd
    assert rel_err_vs(y.cpu().numpy(), ref, scale) <= tol


@pytest.mark.parametrize("it", [np.int32, np.int64])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_laplacian_spmm_k16(gsa, oracle, cuda, wl, it, dt):
    """SpMM with a 16-column column-major X, CSR and CSC, every value/index type pair of the
    benchmark, against the double-double oracle (1e-12 for Float64, 1e-5 for Float32)."""
    m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=it, dtype=dt)
    rng = np.random.default_rng(1)
    X = np.asfortranarray(rng.uniform(-1, 1, (n, 16)).astype(dt))
    ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, 1, X, np.zeros((m, 16), dtype=dt, order="F"))
    tol = 1e-12 if dt == np.float64 else 1e-5
    Xd = torch.from_numpy(X).to(cuda)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    assert oracle.max_rel_error((A @ Xd).cpu().numpy(), ye, sc) <= tol
    del A
    _, _, cp, rv, cz = wl.csr_to_csc(m, n, rp, cv, nz)
    K = gsa.adapt(cuda, gsa.GenericSparseMatrixCSC(m, n, cp, rv, cz))
    assert oracle.max_rel_error((K @ Xd).cpu().numpy(), ye, sc) <= tol


@pytest.mark.parametrize("staged", [1, 0])
@pytest.mark.parametrize("it", [np.int32, np.int64])
def test_laplacian_permuted_coo_conversion(gsa, cuda, wl, it, staged):
    """COO -> CSR and COO -> CSC of the randomly permuted Laplacian triplets are bit-exact
    (keys need 44 bits: the reference's Int32 keys would wrap here), with the bucket sort's
    staged and unstaged passes."""
    lib = gsa._lib.load()
    saved = lib.gsa_get_tuning(gsa._lib.TUNE_SORT_STAGED)
    assert lib.gsa_set_tuning(gsa._lib.TUNE_SORT_STAGED, staged) == 0
    try:
        _laplacian_conversion(gsa, cuda, wl, it)
    finally:
        lib.gsa_set_tuning(gsa._lib.TUNE_SORT_STAGED, saved)


def _laplacian_conversion(gsa, cuda, wl, it):
    m, n, rp, cv, nz = wl.laplacian_2d(2048, itype=it, dtype=np.float64)
    _, _, r, c, v = wl.permuted_coo(m, n, rp, cv, nz, seed=7)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, r, c, v))
    B = gsa.GenericSparseMatrixCSR(A)
    assert np.array_equal(B.rowptr.cpu().numpy(), rp)
    assert np.array_equal(B.colval.cpu().numpy(), cv)
    assert np.array_equal(B.nzval.cpu().numpy(), nz)
    _, _, cp, rv, cz = wl.csr_to_csc(m, n, rp, cv, nz)
    K = gsa.GenericSparseMatrixCSC(A)
    assert np.array_equal(K.colptr.cpu().numpy(), cp)
    assert np.array_equal(K.rowval.cpu().numpy(), rv)
    assert np.array_equal(K.nzval.cpu().numpy(), cz)


def test_power_law_complex_csr_coo(gsa, oracle, cuda, wl):
    m, n, rp, cv, nz = wl.power_law(1_000_000, seed=0, itype=np.int64, dtype=np.complex128)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, 1, x, np.zeros(m, np.complex128))
    xd = torch.from_numpy(x).to(cuda)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    for algo in (gsa.ALGO_AUTO, gsa.ALGO_MERGE, gsa.ALGO_PIPE):
        y = torch.empty(m, dtype=torch.complex128, device=cuda)
        gsa.mul_(y, A, xd, algo=algo)
        assert oracle.max_rel_error(y.cpu().numpy(), ye, sc) <= 1e-12
    rows = wl.csr_rows(rp)
    C = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(m, n, rows, cv, nz))
    assert oracle.max_rel_error((C @ xd).cpu().numpy(), ye, sc) <= 1e-12


def test_power_law_complex_coo_random_order_atomics(gsa, oracle, cuda, wl):
    """The power-law ComplexF64 COO with its triplets in a seeded random order, through the
    atomic COO kernel (gsa_coo_mul: segmented shuffle over adjacent equal rows, then one
    atomic per run), against the double-double oracle; alpha and beta general."""
    import ctypes
    L = gsa._lib
    lib = L.load()
    m, n, rp, cv, nz = wl.power_law(1_000_000, seed=0, itype=np.int64, dtype=np.complex128)
    _, _, r, c, v = wl.permuted_coo(m, n, rp, cv, nz, seed=13)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y0 = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    alpha, beta = np.array([0.75 - 0.5j]), np.array([-1.25 + 0.25j])
    ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, 1, x, y0, alpha=alpha[0], beta=beta[0])
    d = [torch.from_numpy(a).to(cuda) for a in (r, c, v, x, y0)]
    stream = ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream)
    st = lib.gsa_coo_mul(stream, L.C64, L.IDX64, m, n, int(v.size), *(ctypes.c_void_p(t.data_ptr()) for t in d[:3]),
                         1, L.OP_N, 1, ctypes.c_void_p(d[3].data_ptr()), n, L.OP_N, ctypes.c_void_p(d[4].data_ptr()),
                         m, alpha.ctypes.data_as(ctypes.c_void_p), beta.ctypes.data_as(ctypes.c_void_p))
    L.check(st)
    assert oracle.max_rel_error(d[4].cpu().numpy(), ye, sc) <= 1e-12


def test_random_poisson_three_formats(gsa, oracle, cuda, wl):
    m, n, rp, cv, nz = wl.random_poisson(100_000, seed=0)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, n)
    ye, sc = oracle.mul_exact("csr", "N", m, n, rp, cv, nz, 1, x, np.zeros(m))
    xd = torch.from_numpy(x).to(cuda)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(m, n, rp, cv, nz))
    assert oracle.max_rel_error((A @ xd).cpu().numpy(), ye, sc) <= 1e-12
    _, _, cp, rv, cz = wl.csr_to_csc(m, n, rp, cv, nz)
    K = gsa.adapt(cuda, gsa.GenericSparseMatrixCSC(m, n, cp, rv, cz))
    assert oracle.max_rel_error((K @ xd).cpu().numpy(), ye, sc) <= 1e-12
    C = gsa.adapt(cuda, gsa.GenericSparseMatrixCOO(K))  # column-major triplets
    assert oracle.max_rel_error((C @ xd).cpu().numpy(), ye, sc) <= 1e-12
