"""Size-independent properties of the CPU oracle on generated inputs (CPU only; needs
hypothesis, which the GPU machines do not have, so the module skips there).

These back the oracle with facts that hold for every input rather than for chosen fixtures:
conversion is a stable sort of the triplets, compressed sums commute, and the three-argument
dot is linear in y.
"""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

ORACLE = None


def _oracle():
    global ORACLE
    if ORACLE is None:
        from oracle import oracle as o
        o.build()
        ORACLE = o
    return ORACLE


@st.composite
def triplets(draw, max_dim=12, max_nnz=60):
    """1-based COO triplets, duplicates allowed, in any order."""
    m = draw(st.integers(1, max_dim))
    n = draw(st.integers(1, max_dim))
    k = draw(st.integers(0, max_nnz))
    r = draw(st.lists(st.integers(1, m), min_size=k, max_size=k))
    c = draw(st.lists(st.integers(1, n), min_size=k, max_size=k))
    v = draw(st.lists(st.integers(-5, 5), min_size=k, max_size=k))
    return m, n, np.array(r, np.int64), np.array(c, np.int64), np.array(v, np.float64)


@settings(max_examples=150, deadline=None)
@given(triplets(), st.booleans())
def test_conversion_is_a_stable_sort(t, colmajor):
    """COO -> CSR (CSC) orders the triplets by (row, col) ((col, row)), equal keys in input
    order, keeps duplicates, and CSR -> COO gives the sorted triplets back."""
    o = _oracle()
    m, n, r, c, v = t
    major, minor = (c, r) if colmajor else (r, c)
    order = sorted(range(len(v)), key=lambda i: (major[i], minor[i]))  # sorted() is stable
    conv, back = (o.coo_to_csc, o.csc_to_coo) if colmajor else (o.coo_to_csr, o.csr_to_coo)
    ptr, idx, val = conv(m, n, r, c, v)
    assert idx.tolist() == minor[order].tolist() and val.tolist() == v[order].tolist()
    counts = np.bincount(major - 1, minlength=(n if colmajor else m))
    assert (np.diff(ptr)).tolist() == counts.tolist() and ptr[0] == 1
    r2, c2, v2 = back(m, n, ptr, idx, val)
    assert r2.tolist() == r[order].tolist() and c2.tolist() == c[order].tolist()


def _csr(t):
    m, n, r, c, v = t
    return _oracle().coo_to_csr(m, n, r, c, v)


@settings(max_examples=150, deadline=None)
@given(st.data())
def test_compressed_sum_commutes(data):
    """A + B and B + A have the same entries, bit for bit, for sorted rows without repeats
    (IEEE addition commutes; the merge walks both rows in index order)."""
    o = _oracle()
    m = data.draw(st.integers(1, 10))
    n = data.draw(st.integers(1, 10))

    def draw_matrix():
        cells = data.draw(st.lists(st.tuples(st.integers(1, m), st.integers(1, n)), unique=True, max_size=40))
        vals = data.draw(st.lists(st.floats(-4, 4, allow_nan=False, width=64), min_size=len(cells),
                                  max_size=len(cells)))
        r = np.array([x for x, _ in cells], np.int64)
        c = np.array([y for _, y in cells], np.int64)
        return _csr((m, n, r, c, np.array(vals, np.float64)))

    a, b = draw_matrix(), draw_matrix()
    p1, i1, v1 = o.compressed_add(m, a, b)
    p2, i2, v2 = o.compressed_add(m, b, a)
    assert p1.tolist() == p2.tolist() and i1.tolist() == i2.tolist()
    assert v1.tobytes() == v2.tobytes()
    assert np.all(v1 != 0)  # dropzeros ran


@settings(max_examples=100, deadline=None)
@given(triplets(max_nnz=40), st.integers(-3, 3), st.sampled_from(["N", "T"]))
def test_dot_is_linear_in_y(t, s, op):
    """dot(x, op(A), y1 + s*y2) == dot(x, op(A), y1) + s*dot(x, op(A), y2) exactly for
    integer data (small integers: every double operation is exact)."""
    o = _oracle()
    m, n, r, c, v = t
    ptr, idx, val = o.coo_to_csr(m, n, r, c, v)
    rows, cols = (m, n) if op == "N" else (n, m)
    rng = np.random.default_rng(len(v) * 31 + m * 7 + n)
    x = rng.integers(-3, 4, rows).astype(np.float64)
    y1 = rng.integers(-3, 4, cols).astype(np.float64)
    y2 = rng.integers(-3, 4, cols).astype(np.float64)
    d = lambda y: o.dot("csr", op, m, n, ptr, idx, val, 1, x, y)[0]  # noqa: E731
    assert d(y1 + s * y2) == d(y1) + s * d(y2)
