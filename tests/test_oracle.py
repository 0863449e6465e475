"""The CPU oracle against the reference's known answers and against scipy.sparse (CPU only)."""
import json
import os

import numpy as np
import pytest

from helpers import INDEX_TYPES, OPS, VALUE_TYPES, dense_parent, is_int, op_apply, parts, sprand, tol

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
def test_docs_example_spmv(oracle, fmt):
    """docs/src/index.md:47-58: c = A * [1,2,3] == [10, 3, 15] (exact)."""
    g = GOLDEN["docs_spmv_3x3"]
    key = {"csr": ("rowptr", "colval"), "csc": ("colptr", "rowval"), "coo": ("rowind", "colind")}[fmt]
    a = g[fmt]
    p0, p1 = np.array(a[key[0]], np.int64), np.array(a[key[1]], np.int64)
    c = np.full(3, np.nan)
    oracle.mul(fmt, "N", 3, 3, p0, p1, np.array(a["nzval"]), 1, np.array(g["b"]), c)
    assert c.tolist() == g["c"]


def test_csr_structure_pin(oracle):
    """test/shared/matrix_csr.jl:34-58: CSR arrays of the 2x2 fixture, bit for bit."""
    g = GOLDEN["csr_2x2_structure"]
    coo = g["coo"]
    ptr, idx, val = oracle.coo_to_csr(2, 2, np.array(coo["rowind"], np.int64),
                                      np.array(coo["colind"], np.int64), np.array(coo["nzval"]))
    assert ptr.tolist() == g["expected_csr"]["rowptr"]
    assert idx.tolist() == g["expected_csr"]["colval"]
    assert val.tolist() == g["expected_csr"]["nzval"]
    csc = g["csc"]
    r, c, v = oracle.csc_to_coo(2, 2, np.array(csc["colptr"], np.int64),
                                np.array(csc["rowval"], np.int64), np.array(csc["nzval"]))
    assert r.tolist() == coo["rowind"] and c.tolist() == coo["colind"] and v.tolist() == coo["nzval"]


@pytest.mark.parametrize("name", ["single", "full_row", "full_col"])
@pytest.mark.parametrize("it", INDEX_TYPES)
def test_conversion_edge_cases(oracle, name, it):
    """test/shared/conversions.jl:128-152: CSC -> COO -> CSR for the three edge matrices."""
    g = GOLDEN[f"conversion_edge_{name}"]
    csc = g["csc"]
    r, c, v = oracle.csc_to_coo(3, 4, np.array(csc["colptr"], it), np.array(csc["rowval"], it),
                                np.array(csc["nzval"]))
    assert r.tolist() == g["coo"]["rowind"] and c.tolist() == g["coo"]["colind"]
    ptr, idx, val = oracle.coo_to_csr(3, 4, r, c, v)
    assert ptr.tolist() == g["expected_csr"]["rowptr"]
    assert idx.tolist() == g["expected_csr"]["colval"]
    assert val.tolist() == g["expected_csr"]["nzval"]
    ptr2, idx2, val2 = oracle.coo_to_csc(3, 4, r, c, v)
    assert ptr2.tolist() == csc["colptr"] and idx2.tolist() == csc["rowval"]


def test_empty_conversion(oracle):
    g = GOLDEN["empty_0x0"]
    e = np.zeros(0, np.int64)
    ptr, idx, val = oracle.coo_to_csr(0, 0, e, e, np.zeros(0))
    assert ptr.tolist() == g["expected_csr"]["rowptr"] and idx.size == 0 and val.size == 0
    ptr, _, _ = oracle.coo_to_csr(5, 3, e, e, np.zeros(0))
    assert ptr.tolist() == [1] * 6


@pytest.mark.parametrize("dt", VALUE_TYPES)
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
def test_mul_matches_scipy(oracle, dt, it, fmt):
    """Shared-suite shapes (test/shared/matrix_csr.jl:281-327): 100x80 at 0.1, b of 80,
    B of 80x50, every (op(A), op(B)) pair, alpha = 2, beta = 0 and beta = 0.5."""
    rng = np.random.default_rng(7)
    for opA in OPS:
        dims = (100, 80) if opA == "N" else (80, 100)
        S = sprand(rng, *dims, 0.1, dt)
        p0, p1, v = parts(S, fmt, it)
        Sop = op_apply(S, opA)
        for opB in OPS:
            for k in (1, 50):
                P = dense_parent(rng, 80, k, opB, dt)
                Bop = op_apply(P, opB) if opB != "N" else P
                C0 = dense_parent(rng, 100, k, "N", dt)
                for alpha, beta in ((2, 0), (1, 1), (3, 2)):
                    C = C0.copy(order="F")
                    oracle.mul(fmt, opA, *dims, p0, p1, v, 1, P, C, alpha=alpha, beta=beta, opB=opB)
                    ref = alpha * (Sop @ Bop) + beta * C0
                    if is_int(dt):
                        assert np.array_equal(C, ref.astype(dt)), (fmt, opA, opB, k)
                    else:
                        scale = abs(alpha) * (abs(Sop) @ abs(Bop)) + abs(beta) * abs(C0)
                        err = np.max(np.abs(C - ref) / np.where(scale > 0, scale, 1))
                        assert err <= 4 * tol(dt), (fmt, opA, opB, k, err)


def test_beta_zero_ignores_nan(oracle):
    """_rmul_or_fill!: beta == 0 overwrites C without reading it (NaN does not propagate)."""
    rng = np.random.default_rng(3)
    S = sprand(rng, 30, 20, 0.2, np.float64)
    p0, p1, v = parts(S, "csr", np.int64)
    x = rng.uniform(-1, 1, 20)
    for fmt in ("csr", "csc", "coo"):
        q0, q1, w = parts(S, fmt, np.int64)
        C = np.full(30, np.nan)
        oracle.mul(fmt, "N", 30, 20, q0, q1, w, 1, x, C, alpha=1, beta=0)
        assert np.all(np.isfinite(C))
        assert np.allclose(C, S @ x, rtol=0, atol=1e-13)


def test_error_oracle_is_tighter_than_plain(oracle):
    """The double-double oracle agrees with the plain restatement within 1e-14 relative."""
    rng = np.random.default_rng(11)
    S = sprand(rng, 200, 150, 0.3, np.complex128)
    p0, p1, v = parts(S, "csr", np.int32)
    x = rng.standard_normal(150) + 1j * rng.standard_normal(150)
    y = np.zeros(200, np.complex128)
    oracle.mul("csr", "N", 200, 150, p0, p1, v, 1, x, y, alpha=1 - 2j, beta=0)
    ye, sc = oracle.mul_exact("csr", "N", 200, 150, p0, p1, v, 1, x, np.zeros(200, np.complex128),
                              alpha=1 - 2j, beta=0)
    assert oracle.max_rel_error(y, ye, sc) < 1e-14


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_conversion_matches_scipy_and_keeps_duplicates(oracle, it):
    """COO -> CSR/CSC equals scipy's sorted structure; duplicates stay, in input order."""
    rng = np.random.default_rng(5)
    S = sprand(rng, 100, 200, 0.05, np.float64)
    r, c, v = parts(S, "coo", it, order="shuffle", rng=rng)
    for colmajor, fmt in ((False, "csr"), (True, "csc")):
        f = oracle.coo_to_csc if colmajor else oracle.coo_to_csr
        ptr, idx, val = f(100, 200, r, c, v)
        e0, e1, ev = parts(S, fmt, it)
        assert np.array_equal(ptr, e0) and np.array_equal(idx, e1) and np.array_equal(val, ev)
    # duplicates: (2,3) twice with different values, in input order
    r = np.array([2, 1, 2, 2], it)
    c = np.array([3, 1, 3, 1], it)
    v = np.array([10.0, 20.0, 30.0, 40.0])
    ptr, idx, val = oracle.coo_to_csr(3, 3, r, c, v)
    assert ptr.tolist() == [1, 2, 5, 5] and idx.tolist() == [1, 1, 3, 3]
    assert val.tolist() == [20.0, 40.0, 10.0, 30.0]


def _coo(g, it=np.int64):
    return (np.array(g["rowind"], it), np.array(g["colind"], it), np.array(g["nzval"]))


@pytest.mark.parametrize("it", INDEX_TYPES)
def test_coo_sum_known_answers(oracle, it):
    """test/shared/matrix_coo.jl:388-395 (overlapping A + B) and :276-281 (A + I with no
    diagonal), bit for bit and in the reference's column-major order."""
    g = GOLDEN["coo_add_overlap"]
    r, c, v = oracle.coo_sum(g["m"], g["n"], _coo(g["a"], it), b=_coo(g["b"], it))
    assert (r.tolist(), c.tolist(), v.tolist()) == (g["expected"]["rowind"], g["expected"]["colind"],
                                                    g["expected"]["nzval"])
    g = GOLDEN["coo_add_identity_nodiag"]
    r, c, v = oracle.coo_sum(3, 3, _coo(g["a"], it), n_diag=3, lam=g["lambda"])
    assert (r.tolist(), c.tolist(), v.tolist()) == (g["expected"]["rowind"], g["expected"]["colind"],
                                                    g["expected"]["nzval"])


@pytest.mark.parametrize("dt", VALUE_TYPES)
def test_coo_sum_matches_scipy(oracle, dt):
    """A + B, A' + B, A - A and duplicates inside one source against scipy (which sums
    duplicates too); the result is column-major, zero sums dropped."""
    import scipy.sparse as sp
    rng = np.random.default_rng(7)
    m, n = 40, 40
    A, B = sprand(rng, m, n, 0.1, dt), sprand(rng, m, n, 0.15, dt)
    a, b = parts(A, "coo", np.int64), parts(B, "coo", np.int64)
    for op_a in ("N", "T", "C"):
        r, c, v = oracle.coo_sum(m, n, a, op_a=op_a, b=b)
        Aop = {"N": A, "T": A.T, "C": A.conj().T}[op_a]
        want = (sp.csr_matrix(Aop) + sp.csr_matrix(B)).toarray()
        got = np.zeros((m, n), dtype=v.dtype)
        np.add.at(got, (r - 1, c - 1), v)
        assert np.allclose(got, want, rtol=tol(dt), atol=0)
        keys = (c - 1) * m + (r - 1)
        assert np.all(np.diff(keys) > 0) and np.all(v != 0)
    r, c, v = oracle.coo_sum(m, n, a, b=a, neg_b=True)
    assert r.size == 0
    # duplicates inside A are summed in storage order
    dup = tuple(np.concatenate([x, x[:5]]) for x in a)
    r, c, v = oracle.coo_sum(m, n, dup)
    sums = {}
    for ri, ci, vi in zip(*dup):
        sums[(ci, ri)] = sums.get((ci, ri), 0) + vi
    want = sorted((k, s) for k, s in sums.items() if s != 0)
    assert [(ci, ri) for ri, ci in zip(r.tolist(), c.tolist())] == [k for k, _ in want]


@pytest.mark.parametrize("dt", VALUE_TYPES)
@pytest.mark.parametrize("fmt", ["csr", "csc"])
def test_spgemm_matches_scipy(oracle, dt, fmt):
    """The SpGEMM restatement against scipy: scipy drops sums that cancel to zero and the
    reference keeps every reached position, so values are compared densely and the oracle's
    structure is checked to be a superset of scipy's, with zeros only where scipy has none."""
    import scipy.sparse as sp
    rng = np.random.default_rng(66)
    SA, SB = sprand(rng, 40, 30, 0.12, dt), sprand(rng, 30, 45, 0.12, dt)
    a, b = parts(SA, fmt, np.int64), parts(SB, fmt, np.int64)
    ptr, idx, val = oracle.spgemm(fmt, 40, 30, 45, a, b)
    M = (sp.csr_matrix if fmt == "csr" else sp.csc_matrix)((val, idx - 1, ptr - 1), shape=(40, 45))
    want = (SA @ SB).toarray()
    assert np.allclose(M.toarray(), want, rtol=tol(dt), atol=tol(dt) if not is_int(dt) else 0)
    pattern = lambda S: sp.csr_matrix((np.ones(S.nnz), S.indices, S.indptr), shape=S.shape)
    structure = (pattern(SA) @ pattern(SB)) != 0  # positions reached by a stored product
    assert M.nnz == structure.nnz
    for o in range(ptr.size - 1):  # indices increasing in every outer entry
        assert np.all(np.diff(idx[ptr[o] - 1:ptr[o + 1] - 1]) > 0)


def test_golden_fixtures_are_current():
    """known_answers.json is exactly what tests/golden/make_golden.py writes (so every case in
    it traces back to the cited reference inputs)."""
    import importlib.util
    path = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
    spec = importlib.util.spec_from_file_location("make_golden", path)
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    with open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")) as f:
        assert f.read() == mg.render(mg.build_cases())
    assert all("source" in c for c in mg.build_cases().values())


@pytest.mark.parametrize("dt", VALUE_TYPES)
@pytest.mark.parametrize("fmt", ["csr", "csc", "coo"])
@pytest.mark.parametrize("op", OPS)
def test_dot_matches_numpy(oracle, dt, fmt, op):
    """Three-argument dot(x, op(A), y) = x^H op(A) y (src/matrix_csr/matrix_csr.jl:213-277):
    the oracle's reference-arithmetic value and its double-double value against numpy."""
    from helpers import rand_values
    rng = np.random.default_rng(11)
    S = sprand(rng, 60, 45, 0.1, dt)
    p0, p1, v = parts(S, fmt, np.int64)
    opS = op_apply(S, op)
    x = rand_values(rng, opS.shape[0], dt)
    y = rand_values(rng, opS.shape[1], dt)
    val, exact, scale = oracle.dot(fmt, op, S.shape[0], S.shape[1], p0, p1, v, 1, x, y)
    want = np.vdot(x.astype(np.complex128), opS.astype(np.complex128) @ y.astype(np.complex128))
    if not np.iscomplexobj(v):
        want = want.real
    if is_int(dt):
        assert val == want and exact == want
    else:
        assert abs(exact - want) <= 1e-13 * scale
        assert abs(val - exact) <= tol(dt) * scale


def _canonical(S):
    S = S.copy()
    S.eliminate_zeros()
    S.sort_indices()
    return S


@pytest.mark.parametrize("dt", [np.float64, np.complex64, np.int32])
@pytest.mark.parametrize("it", INDEX_TYPES)
@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("neg_b", [False, True])
def test_compressed_add_matches_scipy(oracle, dt, it, fmt, neg_b):
    """CSR + CSR / CSC + CSC (src/matrix_csr/matrix_csr.jl:290-356, then dropzeros): on sorted,
    duplicate-free operands the sum is scipy's, bit for bit (one add per shared position), and
    positions that cancel are dropped."""
    import scipy.sparse as sp
    rng = np.random.default_rng(5)
    A = sprand(rng, 40, 30, 0.15, dt)
    B = sprand(rng, 40, 30, 0.15, dt)
    # B repeats some of A's entries, so A - B cancels there
    C = sp.coo_matrix(A)
    keep = rng.random(C.nnz) < 0.3
    shared = sp.csr_matrix((C.data[keep], (C.row[keep], C.col[keep])), shape=A.shape)
    B = sp.csr_matrix(B - B.multiply(shared != 0) + shared)
    conv = (lambda X: sp.csr_matrix(X)) if fmt == "csr" else (lambda X: sp.csc_matrix(X))
    a, b = parts(A, fmt, it), parts(B, fmt, it)
    outer = A.shape[0] if fmt == "csr" else A.shape[1]
    ptr, idx, val = oracle.compressed_add(outer, a, b, neg_b=neg_b)
    want = _canonical(conv(A - B if neg_b else A + B))
    assert (ptr - 1).tolist() == want.indptr.tolist()
    assert (idx - 1).tolist() == want.indices.tolist()
    assert val.tobytes() == want.data.astype(dt).tobytes()
    if neg_b:  # the shared positions cancel and are gone
        assert shared.nnz > 0 and len(val) <= A.nnz + B.nnz - 2 * shared.nnz


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.int64])
@pytest.mark.parametrize("fmt", ["csr", "csc"])
def test_compressed_add_diag_matches_scipy(oracle, dt, fmt):
    """A + λI (src/matrix_csr/matrix_csr.jl:358-402): λ added to every stored diagonal, one
    entry inserted in order where none is stored, no dropzeros (a diagonal that sums to zero
    stays stored)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(8)
    A = sp.lil_matrix(sprand(rng, 30, 30, 0.12, dt))
    for i in range(0, 30, 3):
        A[i, i] = 2  # stored diagonals; row 0's sums to zero below
    A = sp.csr_matrix(A)
    lam = -2
    a = parts(A, fmt, np.int64)
    ptr, idx, val = oracle.compressed_add_diag(30, a, lam)
    outer_has_diag = np.array([A[i, i] != 0 for i in range(30)])
    assert ptr[-1] - 1 == A.nnz + int((~outer_has_diag).sum())
    conv = sp.csr_matrix if fmt == "csr" else sp.csc_matrix
    got = conv((val, idx - 1, ptr - 1), shape=(30, 30))
    assert np.array_equal(got.toarray(), (A + lam * sp.identity(30, dtype=dt)).toarray().astype(dt))
    for o in range(30):
        assert np.all(np.diff(idx[ptr[o] - 1:ptr[o + 1] - 1]) > 0)  # rows stay sorted
    assert got[0, 0] == 0 and (idx[ptr[0] - 1:ptr[1] - 1] == 1).any()  # zero sum kept


@pytest.mark.parametrize("fmt", ["csr", "csc"])
@pytest.mark.parametrize("it", INDEX_TYPES)
def test_compressed_to_coo_matches_scipy(oracle, fmt, it):
    """CSR / CSC -> COO (src/conversions/conversions.jl:153-169, 264-280): entries in storage
    order, the outer index expanded."""
    import scipy.sparse as sp
    rng = np.random.default_rng(2)
    S = sprand(rng, 35, 50, 0.1, np.float64)
    p0, p1, v = parts(S, fmt, it)
    if fmt == "csr":
        r, c, vv = oracle.csr_to_coo(35, 50, p0, p1, v)
        X = sp.csr_matrix(S)
    else:
        r, c, vv = oracle.csc_to_coo(35, 50, p0, p1, v)
        X = sp.csc_matrix(S)
    X.sort_indices()
    C = X.tocoo()
    assert (r - 1).tolist() == C.row.tolist() and (c - 1).tolist() == C.col.tolist()
    assert vv.tobytes() == C.data.tobytes()
