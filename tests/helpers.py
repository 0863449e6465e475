"""Seeded generators shared by the tests (shapes follow the reference's shared suites)."""
import numpy as np
import scipy.sparse as sp

VALUE_TYPES = [np.float32, np.float64, np.complex64, np.complex128, np.int32, np.int64]
INDEX_TYPES = [np.int32, np.int64]
OPS = ["N", "T", "C"]


def is_complex(dt):
    return np.issubdtype(np.dtype(dt), np.complexfloating)


def is_int(dt):
    return np.issubdtype(np.dtype(dt), np.integer)


def tol(dt):
    """Per-row tolerance relative to sum|a||x| (F64/C64 1e-12, F32/C32 1e-5, ints exact)."""
    dt = np.dtype(dt)
    if is_int(dt):
        return 0.0
    return 1e-5 if dt in (np.dtype(np.float32), np.dtype(np.complex64)) else 1e-12


def rand_values(rng, size, dt):
    dt = np.dtype(dt)
    if is_int(dt):
        return rng.integers(-9, 10, size=size).astype(dt)
    if is_complex(dt):
        return (rng.standard_normal(size) + 1j * rng.standard_normal(size)).astype(dt)
    return rng.uniform(-1, 1, size=size).astype(dt)


def sprand(rng, m, n, density, dt):
    """scipy CSR with sorted indices and ~density*m*n entries of type dt."""
    S = sp.random(m, n, density=density, random_state=rng, format="csr", dtype=np.float64)
    S.sort_indices()
    S = sp.csr_matrix((rand_values(rng, S.nnz, dt), S.indices, S.indptr), shape=(m, n))
    return S


def parts(S, fmt, it, order="storage", rng=None):
    """(p0, p1, val) 1-based arrays of scipy matrix S in format fmt ('csr', 'csc', 'coo').

    COO order: 'storage' = column-major as GenericSparseMatrixCOO(::SparseMatrixCSC) builds it,
    'rows' = row-major, 'shuffle' = a seeded random permutation."""
    if fmt == "csr":
        X = sp.csr_matrix(S)
        X.sort_indices()
        return (X.indptr + 1).astype(it), (X.indices + 1).astype(it), X.data.copy()
    if fmt == "csc":
        X = sp.csc_matrix(S)
        X.sort_indices()
        return (X.indptr + 1).astype(it), (X.indices + 1).astype(it), X.data.copy()
    if order == "rows":
        X = sp.csr_matrix(S)
        X.sort_indices()
        rows = np.repeat(np.arange(X.shape[0]), np.diff(X.indptr))
        r, c, v = rows, X.indices, X.data
    else:
        X = sp.csc_matrix(S)
        X.sort_indices()
        cols = np.repeat(np.arange(X.shape[1]), np.diff(X.indptr))
        r, c, v = X.indices, cols, X.data
    r, c, v = (r + 1).astype(it), (c + 1).astype(it), v.copy()
    if order == "shuffle":
        p = rng.permutation(v.size)
        r, c, v = r[p], c[p], v[p]
    return r, c, v


def op_apply(S, op):
    if op == "N":
        return S
    if op == "T":
        return S.T
    return S.conj().T


def dense_parent(rng, rows, cols, op, dt):
    """Parent P of op(P) with op(P) of shape rows x cols, Fortran-ordered."""
    shape = (rows, cols) if op == "N" else (cols, rows)
    return np.asfortranarray(rand_values(rng, shape, dt))


def laplacian_2d(g, it=np.int32, dt=np.float64):
    """5-point Laplacian on a g x g grid: 4 on the diagonal, -1 to the four neighbours."""
    n = g * g
    idx = np.arange(n)
    i, j = idx // g, idx % g
    rows, cols = [idx], [idx]
    for di, dj in ((-1, 0), (0, -1), (0, 1), (1, 0)):
        ok = (i + di >= 0) & (i + di < g) & (j + dj >= 0) & (j + dj < g)
        rows.append(idx[ok])
        cols.append(((i + di) * g + (j + dj))[ok])
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = np.where(r == c, 4.0, -1.0).astype(dt)
    S = sp.csr_matrix((v, (r, c)), shape=(n, n))
    S.sort_indices()
    return S


_C_SCALARS = {"int64_t": 8, "uint64_t": 8, "size_t": 8, "int32_t": 4, "uint32_t": 4, "int": 4,
              "unsigned char": 1, "char": 1, "double": 8, "float": 4}


def c_struct_layout(header_text, name):
    """[(field, offset, size)] and the total size of `typedef struct { ... } name;` in a C
    header, on an LP64 target with natural alignment (pointers 8 bytes)."""
    import re
    text = re.sub(r"/\*.*?\*/", "", header_text, flags=re.S)
    m = re.search(r"typedef\s+struct\s*\{([^}]*)\}\s*" + name + r"\s*;", text)
    assert m, f"struct {name} not found"
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        base = re.match(r"^((?:const\s+)?(?:unsigned\s+)?[A-Za-z_]\w*)", decl).group(1)
        for d in decl[len(base):].split(","):
            d = d.strip()
            ptr = d.startswith("*")
            dm = re.match(r"^\**\s*(\w+)\s*(?:\[(\d+)\])?$", d)
            assert dm, f"cannot parse {d!r} in {name}"
            scalar = base.replace("const ", "").strip()
            size = 8 if ptr else _C_SCALARS[scalar]
            fields.append((dm.group(1), size, size, int(dm.group(2) or 1)))
    out, off, align_max = [], 0, 1
    for fname, size, align, count in fields:
        off = (off + align - 1) // align * align
        out.append((fname, off, size * count))
        off += size * count
        align_max = max(align_max, align)
    return out, (off + align_max - 1) // align_max * align_max
