"""The Julia extension's `ccall`s agree with include/gsa.h (CPU only; no Julia needed).

Julia is not part of this toolchain, so the extension source cannot be run here; this test
parses every `ccall((:gsa_..., libgsa), Ret, (T1, T2, ...), args...)` in it and checks, against
the header's declaration of the same function: the number of argument types, the number of
arguments passed, and that each Julia type has the C parameter's width and kind (pointer,
32-bit integer, 64-bit integer, float, double).  Names chosen at run time (`_planned_entry(A)`,
`$(QuoteNode(entry))` in a `for` over entry symbols) are resolved from the source and every
candidate is checked.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gsa.h")
EXT = os.path.join(ROOT, "genericsparsearrays.jl_gb300", "julia", "GenericSparseArraysCUDAExt.jl")


def _split_top(s):
    """Split s at commas outside (), {} and []."""
    out, depth, cur = [], 0, []
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    tail = "".join(cur).strip()
    if tail:
        out.append(tail)
    return out


def _balanced(text, i):
    """text[i] == '('; the index just past its matching ')'."""
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "(":
            depth += 1
        elif text[j] == ")":
            depth -= 1
            if depth == 0:
                return j + 1
    raise ValueError("unbalanced parentheses")


def c_kind(decl, enums=()):
    t = decl.strip()
    if "*" in t:
        return "ptr"
    if t.split() and t.split()[-1] in enums:
        return "i32"
    t = re.sub(r"\b(const|unsigned|signed)\b", lambda m: "u" if m.group(1) == "unsigned" else "", t)
    t = t.split()[0] if t.split() else t
    if t in ("int64_t", "uint64_t", "size_t", "ptrdiff_t", "long"):
        return "i64"
    if t in ("int", "int32_t", "uint32_t", "u"):
        return "i32"
    if t == "double":
        return "f64"
    if t == "float":
        return "f32"
    if t == "void":
        return "void"
    raise AssertionError(f"unknown C type {decl!r}")


def jl_kind(t):
    t = t.strip()
    if re.match(r"^(Ptr|CuPtr|Ref|PtrOrCuPtr)\{", t) or t in ("CUstream", "Cstring", "CuStream"):
        return "ptr"
    if t in ("Cint", "Int32", "Cuint", "UInt32"):
        return "i32"
    if t in ("Int64", "UInt64", "Csize_t", "Clonglong", "Culonglong", "Cssize_t", "Clong", "Culong"):
        return "i64"
    if t in ("Float64", "Cdouble"):
        return "f64"
    if t in ("Float32", "Cfloat"):
        return "f32"
    if t == "Cvoid":
        return "void"
    raise AssertionError(f"unknown Julia type {t!r}")


def header_decls():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"^\s*#[^\n]*", "", text, flags=re.M)
    text = text.replace('extern "C" {', "")
    enums = set(re.findall(r"typedef\s+enum\s*\{[^}]*\}\s*(\w+)\s*;", text))
    text = re.sub(r"typedef[^;{]*\{[^}]*\}[^;]*;", "", text)  # enum and struct typedefs
    decls = {}
    for stmt in text.split(";"):
        m = re.match(r"^\s*([A-Za-z_][\w\s\*]*?)\b(gsa_\w+)\s*\((.*)\)\s*$", stmt, flags=re.S)
        if not m or "typedef" in m.group(1):
            continue
        ret, name, params = m.group(1), m.group(2), " ".join(m.group(3).split())
        kinds = [] if params in ("", "void") else [c_kind(re.sub(r"\w+\s*$", "", p) or p, enums)
                                                    for p in _split_top(params)]
        decls[name] = (c_kind(ret, enums), kinds)
    return decls


def _resolve(target, text, pos):
    """gsa_ names a ccall target can take."""
    m = re.match(r"^\(\s*:(gsa_\w+)\s*,", target)
    if m:
        return [m.group(1)]
    m = re.match(r"^\(\s*(_\w+)\(", target)
    if m:  # a function mapping a matrix type to an entry symbol
        return re.findall(rf"^{m.group(1)}\([^)]*\)\s*=\s*:(gsa_\w+)", text, flags=re.M)
    m = re.match(r"^\(\s*\$\(QuoteNode\((\w+)\)\)", target)
    if m:  # a `for (..., entry, ...) in ((...), ...)` loop around an @eval
        head = text.rfind("\nfor ", 0, pos)
        body = text.find("@eval", head)
        return re.findall(r":(gsa_\w+)", text[head:body])
    raise AssertionError(f"cannot resolve ccall target {target!r}")


def ext_ccalls(text=None):
    text = open(EXT).read() if text is None else text
    calls = []
    for m in re.finditer(r"\bccall\(", text):
        start = m.end() - 1
        parts = _split_top(text[start + 1:_balanced(text, start) - 1])
        target, ret, types, args = parts[0], parts[1], parts[2], parts[3:]
        assert types.startswith("(") and types.endswith(")"), types
        tlist = _split_top(types[1:-1])
        line = text.count("\n", 0, start) + 1
        for name in _resolve(target, text, start):
            calls.append((line, name, ret, tlist, args))
    return calls


def test_extension_calls_match_header():
    decls = header_decls()
    calls = ext_ccalls()
    assert len(calls) >= 25
    seen = set()
    for line, name, ret, tlist, args in calls:
        where = f"{os.path.basename(EXT)}:{line} {name}"
        assert name in decls, f"{where}: not declared in gsa.h"
        cret, ckinds = decls[name]
        assert len(tlist) == len(ckinds), f"{where}: {len(tlist)} argument types, gsa.h has {len(ckinds)}"
        # `size(A)...` splats a matrix's two dimensions; any other splat only bounds the count
        nargs = sum(2 if re.match(r"^size\(\w+\)\.\.\.$", a) else 1 for a in args)
        if any(a.endswith("...") and not re.match(r"^size\(\w+\)\.\.\.$", a) for a in args):
            assert nargs <= len(tlist), f"{where}: {nargs} arguments for {len(tlist)} types"
        else:
            assert nargs == len(tlist), f"{where}: {nargs} arguments for {len(tlist)} types"
        for i, (jt, ck) in enumerate(zip(tlist, ckinds)):
            assert jl_kind(jt) == ck, f"{where}: argument {i + 1} is {jt}, gsa.h wants {ck}"
        assert jl_kind(ret) == cret or (cret == "ptr" and ret.strip() == "Cstring"), \
            f"{where}: returns {ret}, gsa.h returns {cret}"
        seen.add(name)
    # the extension reaches the hot path's entry points
    for name in ("gsa_csr_mul_planned", "gsa_csc_mul_planned", "gsa_coo_mul_planned", "gsa_coo_to_csr",
                 "gsa_coo_to_csc", "gsa_csr_to_coo", "gsa_csc_to_coo", "gsa_spgemm_compute"):
        assert name in seen, f"the extension never calls {name}"


def test_parser_catches_a_mismatch(tmp_path, monkeypatch):
    """A ccall with one argument type dropped is reported (the check is not vacuous)."""
    text = open(EXT).read()
    bad = text.replace("(CUstream, Cint, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint,\n"
                       "             CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}),",
                       "(CUstream, Cint, Int64, Int64, Int64, CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}, Cint,\n"
                       "             CuPtr{Ti}, CuPtr{Ti}, CuPtr{T}),", 1)
    assert bad != text
    p = tmp_path / "ext.jl"
    p.write_text(bad)
    monkeypatch.setattr(__import__(__name__), "EXT", str(p))
    with pytest.raises(AssertionError, match="argument types"):
        test_extension_calls_match_header()


def _header_enum():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return {k: int(v) for k, v in re.findall(r"\b(GSA_[A-Z0-9_]+)\s*=\s*(\d+)", text)}


def test_extension_codes_match_header():
    """The extension's value-type, index-type and op codes, and its status -> exception map,
    are the header's (and the Python binding's)."""
    e = _header_enum()
    text = open(EXT).read()
    dt = dict(re.findall(r"^gsa_dtype\(::Type\{(\w+)\}\)\s*=\s*Cint\((\d+)\)", text, flags=re.M))
    assert {k: int(v) for k, v in dt.items()} == {
        "Float32": e["GSA_F32"], "Float64": e["GSA_F64"], "ComplexF32": e["GSA_C32"],
        "ComplexF64": e["GSA_C64"], "Int32": e["GSA_I32"], "Int64": e["GSA_I64"]}
    it = dict(re.findall(r"^gsa_itype\(::Type\{(\w+)\}\)\s*=\s*Cint\((\d+)\)", text, flags=re.M))
    assert {k: int(v) for k, v in it.items()} == {"Int32": e["GSA_IDX32"], "Int64": e["GSA_IDX64"]}
    ops = re.findall(r"^_opA\(A(?:::(\w+)(?:\{[^}]*\})?)?\)\s*=\s*\([^,]+,\s*Cint\((\d+)\)\)", text, flags=re.M)
    assert ("", str(e["GSA_OP_N"])) in ops and ("Transpose", str(e["GSA_OP_T"])) in ops
    assert ("Adjoint", str(e["GSA_OP_C"])) in ops
    fmt = dict(re.findall(r"^_fmt\(::GenericSparseMatrix(\w+)\)\s*=\s*Cint\((\d+)\)", text, flags=re.M))
    assert {k: int(v) for k, v in fmt.items()} == {"CSR": 0, "CSC": 1, "COO": 2}
    assert re.search(rf"status == {e['GSA_ERR_DIM']} && throw\(DimensionMismatch", text)
    m = re.search(r"status in \(([\d, ]+)\) && throw\(ArgumentError", text)
    assert m and {int(x) for x in m.group(1).split(",")} == {
        e["GSA_ERR_INVALID_ARG"], e["GSA_ERR_UNSUPPORTED"], e["GSA_ERR_STRUCTURE"]}


_JL_SIZES = {"Int64": 8, "UInt64": 8, "Int32": 4, "UInt32": 4, "Float64": 8, "Float32": 4}


def test_julia_group_item_matches_header():
    """GsaGroupItem in the extension (handed to gsa_batch_create as raw bytes) has the field
    order, offsets and size of gsa_group_item."""
    from helpers import c_struct_layout
    text = open(EXT).read()
    m = re.search(r"struct GsaGroupItem\b[^\n]*\n(.*?)\nend", text, flags=re.S)
    assert m
    fields = []
    for decl in re.split(r"[;\n]", m.group(1)):
        decl = decl.split("#")[0].strip()
        if not decl:
            continue
        name, jt = [x.strip() for x in decl.split("::", 1)]
        tm = re.match(r"^NTuple\{(\d+),\s*UInt8\}$", jt)
        if tm:
            size, align = int(tm.group(1)), 1
        elif re.match(r"^(Cu)?Ptr\{", jt):
            size = align = 8
        else:
            size = align = _JL_SIZES[jt]
        fields.append((name, size, align))
    off, got = 0, []
    for name, size, align in fields:
        off = (off + align - 1) // align * align
        got.append((name, off, size))
        off += size
    layout, total = c_struct_layout(open(HEADER).read(), "gsa_group_item")
    assert got == layout
    assert (off + 7) // 8 * 8 == total == 144


def test_integration_guide_snippets_match_header():
    """The `ccall`s shown in the ```julia blocks of INTEGRATION.md match gsa.h too."""
    guide = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = "\n".join(re.findall(r"```julia\n(.*?)```", guide, flags=re.S))
    decls = header_decls()
    calls = ext_ccalls(blocks)
    assert {c[1] for c in calls} >= {"gsa_csr_mul", "gsa_batch_create", "gsa_batch_run"}
    for line, name, ret, tlist, args in calls:
        cret, ckinds = decls[name]
        assert len(tlist) == len(ckinds) == len(args), (name, len(tlist), len(ckinds), len(args))
        for i, (jt, ck) in enumerate(zip(tlist, ckinds)):
            assert jl_kind(jt) == ck, f"{name}: argument {i + 1} is {jt}, gsa.h wants {ck}"


def test_invoke_fallbacks_name_reference_methods():
    """Every `invoke(Base.:+, Tuple{Parent, UniformScaling}, ...)` of the extension (its fallback
    when lambda does not promote to the matrix's element type) names a method the reference
    defines: tests/golden/reference_methods.json lists the reference's `Base.:+(::Matrix,
    ::UniformScaling)` methods with their file:line.  The `@eval` loop's `$Parent` is resolved
    from the loop's `(Fmt, Parent)` pairs.  (The fallback itself has not run: no Julia here.)"""
    import json
    src = open(EXT).read()
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_methods.json")))
    defined = {(r["method"], tuple(r["args"])) for r in ref}
    assert len(defined) == 3
    loop = re.search(r"for \(Fmt, Parent\) in \(([^\n]*)\)\n", src)
    parents = re.findall(r"\(:\w+, :(\w+)\)", loop.group(1)) if loop else []
    assert parents == ["GenericSparseMatrixCSR", "GenericSparseMatrixCSC"]
    calls = re.findall(r"invoke\((Base\.:\+), Tuple\{(\$?\w+), (\w+)\}", src)
    assert calls, "no invoke fallback found"
    seen = set()
    for method, first, second in calls:
        for parent in (parents if first == "$Parent" else [first]):
            assert (method, (parent, second)) in defined, (method, parent, second)
            seen.add(parent)
    assert seen == {"GenericSparseMatrixCOO", "GenericSparseMatrixCSR", "GenericSparseMatrixCSC"}
