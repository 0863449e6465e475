"""Writes tests/golden/known_answers.json: the known-answer cases that the reference's own
tests and docs hold for the sparse x dense mul! path and the conversions.

The reference (Julia) cannot be run (no Julia installation), so each case is rebuilt here
from the inputs written in the reference source (cited per case) and its expected output is
computed with scipy.sparse, which stands in for the SparseArrays results those tests compare
against.  Indices are 1-based, as in the reference.  Run:  python tests/golden/make_golden.py
(`--check`: exit 1 if the committed file differs from what the script writes).
"""
import json
import os
import sys

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))


def sparse(I, J, V, m, n):
    """SparseArrays.sparse(I, J, V, m, n) for duplicate-free 1-based triplets."""
    return sp.csc_matrix((np.asarray(V, dtype=float), (np.asarray(I) - 1, np.asarray(J) - 1)),
                         shape=(m, n))


def csc_arrays(S):
    S = sp.csc_matrix(S)
    S.sort_indices()
    return {"colptr": (S.indptr + 1).tolist(), "rowval": (S.indices + 1).tolist(),
            "nzval": S.data.tolist()}


def csr_arrays(S):
    S = sp.csr_matrix(S)
    S.sort_indices()
    return {"rowptr": (S.indptr + 1).tolist(), "colval": (S.indices + 1).tolist(),
            "nzval": S.data.tolist()}


def coo_from_csc(S):
    """GenericSparseMatrixCOO(::SparseMatrixCSC): column-major walk
    (src/matrix_coo/matrix_coo.jl:64-83)."""
    S = sp.csc_matrix(S)
    S.sort_indices()
    cols = np.repeat(np.arange(S.shape[1]), np.diff(S.indptr))
    return {"rowind": (S.indices + 1).tolist(), "colind": (cols + 1).tolist(),
            "nzval": S.data.tolist()}


def build_cases():
    """The known-answer cases, keyed by name (what known_answers.json holds)."""
    cases = {}

    # docs/src/index.md:47-58 -- A_sparse = sparse([1,2,1,3],[1,1,2,3],[2.0,3.0,4.0,5.0],3,3),
    # A_device = GenericSparseMatrixCSC(A_sparse), b = [1.0,2.0,3.0], c = A_device * b
    A = sparse([1, 2, 1, 3], [1, 1, 2, 3], [2.0, 3.0, 4.0, 5.0], 3, 3)
    b = np.array([1.0, 2.0, 3.0])
    cases["docs_spmv_3x3"] = {
        "source": "docs/src/index.md:47-58", "m": 3, "n": 3, "csc": csc_arrays(A),
        "csr": csr_arrays(A), "coo": coo_from_csc(A), "b": b.tolist(), "c": (A @ b).tolist()}

    # test/shared/matrix_csr.jl:34-58 -- B = sparse([1,2,1],[1,1,2],[1.0,2.0,3.0],2,2);
    # the CSR arrays must equal SparseMatrixCSC(transpose(B))'s colptr/rowval/nzval.
    B = sparse([1, 2, 1], [1, 1, 2], [1.0, 2.0, 3.0], 2, 2)
    Bt = sp.csc_matrix(B.T)
    Bt.sort_indices()
    cases["csr_2x2_structure"] = {
        "source": "test/shared/matrix_csr.jl:34-58", "m": 2, "n": 2, "coo": coo_from_csc(B),
        "csc": csc_arrays(B),
        "expected_csr": {"rowptr": (Bt.indptr + 1).tolist(), "colval": (Bt.indices + 1).tolist(),
                         "nzval": Bt.data.tolist()},
        "dense": B.toarray().tolist()}

    # test/shared/matrix_csr.jl:61-67 -- rowptr of the wrong length -> ArgumentError
    cases["csr_ctor_error"] = {
        "source": "test/shared/matrix_csr.jl:61-67", "m": 2, "n": 2, "rowptr": [1, 3],
        "colval": [1], "nzval": [1.0], "error": "ArgumentError"}

    # test/shared/conversions.jl:128-152 -- single element, full row, full column
    edge = {
        "single": sparse([1], [2], [5.0], 3, 4),
        "full_row": sparse([1, 1, 1, 1], [1, 2, 3, 4], [1, 2, 3, 4], 3, 4),
        "full_col": sparse([1, 2, 3], [2, 2, 2], [1, 2, 3], 3, 4),
    }
    for name, S in edge.items():
        cases[f"conversion_edge_{name}"] = {
            "source": "test/shared/conversions.jl:128-152", "m": 3, "n": 4, "csc": csc_arrays(S),
            "coo": coo_from_csc(S), "expected_csr": csr_arrays(S), "dense": S.toarray().tolist()}

    # test/shared/matrix_csr.jl:32 -- spzeros(Float32, 0, 0): the empty matrix
    cases["empty_0x0"] = {"source": "test/shared/matrix_csr.jl:32", "m": 0, "n": 0,
                          "expected_csr": {"rowptr": [1], "colval": [], "nzval": []}}

    # test/shared/matrix_coo.jl:388-395 -- A_overlap = sparse([1,2,3],[1,2,3],T[1,2,3],50,40),
    # B_overlap = sparse([1,2,4],[1,2,4],T[4,5,6],50,40); A + B of their COO forms
    Ao = sparse([1, 2, 3], [1, 2, 3], [1, 2, 3], 50, 40)
    Bo = sparse([1, 2, 4], [1, 2, 4], [4, 5, 6], 50, 40)
    cases["coo_add_overlap"] = {
        "source": "test/shared/matrix_coo.jl:388-395", "m": 50, "n": 40, "a": coo_from_csc(Ao),
        "b": coo_from_csc(Bo), "expected": coo_from_csc(Ao + Bo)}

    # test/shared/matrix_coo.jl:276-281 -- A_nodiag = sparse([1,2],[2,1],T[1,2],3,3); A + I
    An = sparse([1, 2], [2, 1], [1, 2], 3, 3)
    cases["coo_add_identity_nodiag"] = {
        "source": "test/shared/matrix_coo.jl:276-281", "m": 3, "n": 3, "a": coo_from_csc(An),
        "lambda": 1.0, "expected": coo_from_csc(An + sp.identity(3))}

    return cases


def render(cases):
    return json.dumps(cases, indent=1, sort_keys=True) + "\n"


def main(argv):
    path = os.path.join(HERE, "known_answers.json")
    text = render(build_cases())
    if "--check" in argv:  # exit 1 when the committed file is not what this script writes
        with open(path) as f:
            return 0 if f.read() == text else 1
    with open(path, "w") as f:
        f.write(text)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
