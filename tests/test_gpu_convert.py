"""COO -> CSR/CSC and CSR/CSC -> COO on the GPU: bit-exact against the oracle and the
reference's known answers."""
import json
import os

import numpy as np
import pytest
import torch

from helpers import INDEX_TYPES, VALUE_TYPES, parts, rand_values, sprand

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


@pytest.fixture(params=[1, 0], ids=["staged", "unstaged"])
def sort_staged(request, gsa):
    """Both forms of the bucket sort's passes (GSA_TUNE_SORT_STAGED), restored afterwards."""
    lib = gsa._lib.load()
    key = gsa._lib.TUNE_SORT_STAGED
    saved = lib.gsa_get_tuning(key)
    assert lib.gsa_set_tuning(key, request.param) == 0
    yield request.param
    lib.gsa_set_tuning(key, saved)


def coo(gsa, dev, m, n, r, c, v):
    return gsa.adapt(dev, gsa.GenericSparseMatrixCOO(m, n, r, c, v))


def np_(t):
    return t.cpu().numpy()


def test_structure_pin_2x2(gsa, cuda):
    """test/shared/matrix_csr.jl:34-58 through the GPU COO -> CSR path."""
    g = GOLDEN["csr_2x2_structure"]
    A = coo(gsa, cuda, 2, 2, np.array(g["coo"]["rowind"]), np.array(g["coo"]["colind"]),
            np.array(g["coo"]["nzval"]))
    C = gsa.GenericSparseMatrixCSR(A)
    assert C.rowptr.tolist() == g["expected_csr"]["rowptr"]
    assert C.colval.tolist() == g["expected_csr"]["colval"]
    assert C.nzval.tolist() == g["expected_csr"]["nzval"]
    K = gsa.GenericSparseMatrixCSC(A)
    assert K.colptr.tolist() == g["csc"]["colptr"] and K.rowval.tolist() == g["csc"]["rowval"]


@pytest.mark.parametrize("name", ["single", "full_row", "full_col"])
def test_edge_cases(gsa, cuda, name):
    """test/shared/conversions.jl:128-152: CSC -> COO (nnz kept) and CSC -> CSR via COO."""
    g = GOLDEN[f"conversion_edge_{name}"]
    csc = gsa.adapt(cuda, gsa.GenericSparseMatrixCSC(3, 4, np.array(g["csc"]["colptr"]),
                                                     np.array(g["csc"]["rowval"]),
                                                     np.array(g["csc"]["nzval"])))
    c = gsa.GenericSparseMatrixCOO(csc)
    assert gsa.nnz(c) == len(g["coo"]["nzval"])
    assert c.rowind.tolist() == g["coo"]["rowind"] and c.colind.tolist() == g["coo"]["colind"]
    r = gsa.GenericSparseMatrixCSR(csc)
    assert r.rowptr.tolist() == g["expected_csr"]["rowptr"]
    assert r.colval.tolist() == g["expected_csr"]["colval"]
    assert r.nzval.tolist() == g["expected_csr"]["nzval"]
    assert np.array_equal(gsa.collect(r), np.array(g["dense"]))


@pytest.mark.parametrize("m,n", [(0, 0), (5, 3), (0, 4)])
def test_empty(gsa, cuda, m, n):
    e = np.zeros(0, np.int64)
    A = coo(gsa, cuda, m, n, e, e, np.zeros(0))
    C = gsa.GenericSparseMatrixCSR(A)
    assert C.rowptr.tolist() == [1] * (m + 1) and gsa.nnz(C) == 0
    K = gsa.GenericSparseMatrixCSC(A)
    assert K.colptr.tolist() == [1] * (n + 1)


@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_permuted_coo_bit_exact(gsa, oracle, cuda, sort_staged, it, dt):
    """test/shared/conversions.jl shapes (100x200 at 0.05), triplets shuffled, with duplicate
    (row, col) pairs: CSR and CSC structure and values equal the oracle's bit for bit."""
    rng = np.random.default_rng(31)
    S = sprand(rng, 100, 200, 0.05, dt)
    r, c, v = parts(S, "coo", it, order="shuffle", rng=rng)
    dup = rng.choice(v.size, 40, replace=False)
    r = np.concatenate([r, r[dup]])
    c = np.concatenate([c, c[dup]])
    v = np.concatenate([v, rand_values(rng, 40, dt)])
    p = rng.permutation(v.size)
    r, c, v = r[p], c[p], v[p]
    A = coo(gsa, cuda, 100, 200, r, c, v)
    for cls, f in ((gsa.GenericSparseMatrixCSR, oracle.coo_to_csr), (gsa.GenericSparseMatrixCSC, oracle.coo_to_csc)):
        B = cls(A)
        ptr, idx = (B.rowptr, B.colval) if cls is gsa.GenericSparseMatrixCSR else (B.colptr, B.rowval)
        e_ptr, e_idx, e_val = f(100, 200, r, c, v)
        assert np.array_equal(np_(ptr), e_ptr)
        assert np.array_equal(np_(idx), e_idx)
        assert np.array_equal(np_(B.nzval), e_val)


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_compressed_to_coo_and_round_trips(gsa, oracle, cuda, it):
    rng = np.random.default_rng(8)
    S = sprand(rng, 150, 90, 0.07, np.complex128)
    p0, p1, v = parts(S, "csr", it)
    A = gsa.adapt(cuda, gsa.GenericSparseMatrixCSR(150, 90, p0, p1, v))
    C = gsa.GenericSparseMatrixCOO(A)
    er, ec, ev = oracle.csr_to_coo(150, 90, p0, p1, v)
    assert np.array_equal(np_(C.rowind), er) and np.array_equal(np_(C.colind), ec)
    assert np.array_equal(np_(C.nzval), ev)
    q0, q1, w = parts(S, "csc", it)
    K = gsa.adapt(cuda, gsa.GenericSparseMatrixCSC(150, 90, q0, q1, w))
    Ck = gsa.GenericSparseMatrixCOO(K)
    er, ec, ev = oracle.csc_to_coo(150, 90, q0, q1, w)
    assert np.array_equal(np_(Ck.rowind), er) and np.array_equal(np_(Ck.colind), ec)
    # round trips CSR -> COO -> CSR, CSC -> CSR -> CSC, and transposes
    R = gsa.GenericSparseMatrixCSR(gsa.GenericSparseMatrixCOO(A))
    assert torch.equal(R.rowptr, A.rowptr) and torch.equal(R.colval, A.colval)
    assert torch.equal(R.nzval, A.nzval)
    K2 = gsa.GenericSparseMatrixCSC(gsa.GenericSparseMatrixCSR(K))
    assert torch.equal(K2.colptr, K.colptr) and torch.equal(K2.rowval, K.rowval)
    assert torch.equal(K2.nzval, K.nzval)
    At = gsa.GenericSparseMatrixCSR(gsa.adjoint(K))
    assert np.allclose(gsa.collect(At), S.toarray().conj().T)
    Tc = gsa.GenericSparseMatrixCSC(gsa.transpose(C))
    assert np.allclose(gsa.collect(Tc), S.toarray().T)


def test_power_law_rows_conversion(gsa, oracle, cuda, sort_staged):
    """Rows of up to 50,000 entries, shuffled triplets: bit-exact against the oracle."""
    from genericsparsearrays_gb300 import workloads
    m, n, rp, cv, nz = workloads.power_law(n=100_000, seed=4, itype=np.int64, dtype=np.float64)
    _, _, r, c, v = workloads.permuted_coo(m, n, rp, cv, nz, seed=5)
    A = coo(gsa, cuda, m, n, r, c, v)
    B = gsa.GenericSparseMatrixCSR(A)
    assert np.array_equal(np_(B.rowptr), rp) and np.array_equal(np_(B.colval), cv)
    assert np.array_equal(np_(B.nzval), nz)


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_bucket_sizes_with_duplicates(gsa, oracle, cuda, sort_staged, it):
    """Rows and columns of 0..16 (sorted by a thread), 17..256 (a warp), 257..16384 (a CTA in
    shared memory) and beyond 16384 entries (CTA chunks merged pairwise), each with repeated
    (row, col) pairs carrying different values, shuffled: CSR and CSC equal the oracle's bit
    for bit, so ties keep their input order in every bucket size."""
    rng = np.random.default_rng(41)
    m, n = 600, 20_000
    lengths = {3: 17, 10: 256, 11: 257, 40: 4096, 41: 4097, 77: 9000, 90: 16384, 91: 40000, 500: 16, 501: 1}
    rows, cols = [], []
    for r, L in lengths.items():
        c = rng.integers(1, n + 1, L)
        c[: L // 3] = c[0]  # a run of equal columns
        rows.append(np.full(L, r + 1))
        cols.append(c)
    base_r = rng.integers(1, m + 1, 3000)
    base_c = rng.integers(1, 50, 3000)  # few columns: long columns for CSC
    r = np.concatenate(rows + [base_r]).astype(it)
    c = np.concatenate(cols + [base_c]).astype(it)
    v = rng.standard_normal(r.size)
    p = rng.permutation(r.size)
    r, c, v = r[p], c[p], v[p]
    A = coo(gsa, cuda, m, n, r, c, v)
    for cls, f in ((gsa.GenericSparseMatrixCSR, oracle.coo_to_csr), (gsa.GenericSparseMatrixCSC, oracle.coo_to_csc)):
        B = cls(A)
        ptr, idx = (B.rowptr, B.colval) if cls is gsa.GenericSparseMatrixCSR else (B.colptr, B.rowval)
        e_ptr, e_idx, e_val = f(m, n, r, c, v)
        assert np.array_equal(np_(ptr), e_ptr)
        assert np.array_equal(np_(idx), e_idx)
        assert np.array_equal(np_(B.nzval), e_val)


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_short_rows_with_long_ones(gsa, oracle, cuda, sort_staged, it):
    """Rows averaging about two entries (the staged row pass runs) with a few rows and columns
    of 17, 200, 256, 257, 3000, 4096, 4097 and 40,000 entries among them: rows sorted by a
    thread, by a warp, by rank counting, by the bitonic sort and in chunks, buckets staged in
    shared memory and one too large for its buffer; repeated (row, col) pairs; shuffled.  CSR
    and CSC equal the oracle's bit for bit."""
    rng = np.random.default_rng(61)
    m, n = 200_000, 150_000
    rows = [rng.integers(1, m + 1, 2 * m)]
    cols = [rng.integers(1, n + 1, 2 * m)]
    for L in (17, 200, 256, 257, 3000, 4096, 4097, 40_000):
        r0, c0 = rng.integers(1, m + 1), rng.integers(1, n + 1)
        c = rng.integers(1, n + 1, L)
        c[: L // 4] = c[0]  # repeated (row, col) pairs
        rows += [np.full(L, r0), rng.integers(1, m + 1, L)]
        cols += [c, np.full(L, c0)]  # the same lengths as columns
    r = np.concatenate(rows).astype(it)
    c = np.concatenate(cols).astype(it)
    v = rng.standard_normal(r.size)
    p = rng.permutation(r.size)
    r, c, v = r[p], c[p], v[p]
    assert r.size <= 8 * min(m, n)
    A = coo(gsa, cuda, m, n, r, c, v)
    for cls, f in ((gsa.GenericSparseMatrixCSR, oracle.coo_to_csr), (gsa.GenericSparseMatrixCSC, oracle.coo_to_csc)):
        B = cls(A)
        ptr, idx = (B.rowptr, B.colval) if cls is gsa.GenericSparseMatrixCSR else (B.colptr, B.rowval)
        e_ptr, e_idx, e_val = f(m, n, r, c, v)
        assert np.array_equal(np_(ptr), e_ptr)
        assert np.array_equal(np_(idx), e_idx)
        assert np.array_equal(np_(B.nzval), e_val)


@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("offset", [0, 1, 3])
def test_unaligned_and_ragged_inputs(gsa, oracle, cuda, sort_staged, it, offset):
    """Index and value arrays that start `offset` elements into their allocations (not 16-byte
    aligned for offsets 1 and 3: the staged placement then falls back to plain loads), with
    entry counts that end inside a 16-byte piece, through the C ABI: bit-exact CSR and CSC."""
    import ctypes
    lib = gsa._lib.load()
    rng = np.random.default_rng(57 + offset)
    m, n = 3000, 1700
    for nz in (1, 7, 4099, 50_001):
        r = rng.integers(1, m + 1, nz).astype(it)
        c = rng.integers(1, n + 1, nz).astype(it)
        v = rng.standard_normal(nz)
        pad = lambda a: torch.from_numpy(np.concatenate([np.zeros(offset, a.dtype), a])).to(cuda)
        rd, cd, vd = pad(r), pad(c), pad(v)
        ptr_at = lambda t: ctypes.c_void_p(t.data_ptr() + offset * t.element_size())
        itype = gsa._lib.IDX32 if it == np.int32 else gsa._lib.IDX64
        for colmajor, f in ((0, oracle.coo_to_csr), (1, oracle.coo_to_csc)):
            major_n = n if colmajor else m
            ws_bytes = lib.gsa_coo_to_compressed_workspace_size(colmajor, gsa._lib.F64, itype, m, n, nz)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=cuda)
            tt = torch.int32 if it == np.int32 else torch.int64
            ptr = torch.empty(major_n + 1, dtype=tt, device=cuda)
            idx = torch.empty(nz, dtype=tt, device=cuda)
            val = torch.empty(nz, dtype=torch.float64, device=cuda)
            fn = lib.gsa_coo_to_csc if colmajor else lib.gsa_coo_to_csr
            st = fn(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), gsa._lib.F64, itype, m, n, nz,
                    ptr_at(rd), ptr_at(cd), ptr_at(vd), 1, ctypes.c_void_p(ptr.data_ptr()),
                    ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(val.data_ptr()),
                    ctypes.c_void_p(ws.data_ptr()), ws.numel())
            assert st == 0, gsa._lib.last_error()
            e_ptr, e_idx, e_val = f(m, n, r, c, v)
            assert np.array_equal(np_(ptr), e_ptr)
            assert np.array_equal(np_(idx), e_idx)
            assert np.array_equal(np_(val), e_val)
