"""Writes tests/golden/reference_methods.json: the reference's ``Base.:+`` methods that take a
sparse matrix and a ``UniformScaling`` -- file:line, the parent type of the first argument and
the type of the second, as written in the reference source.  The Julia extension falls back
to these methods through ``invoke`` when lambda does not promote to the matrix's element type;
tests/test_julia_ext_abi.py checks that every such ``invoke`` names one of them.

Run:  python tests/golden/make_reference_methods.py [REFERENCE_ROOT]   (default /root/reference)
      (`--check`: exit 1 if the committed file differs from what the script writes)
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_methods.json")
FILES = ["src/matrix_coo/matrix_coo.jl", "src/matrix_csr/matrix_csr.jl", "src/matrix_csc/matrix_csc.jl"]
SIG = re.compile(r"^function Base\.:\+\(\s*\w+::(GenericSparseMatrix\w+)(?:\{[^}]*\})?\s*,\s*\w+::(UniformScaling)\b")


def collect(root):
    out = []
    for rel in FILES:
        with open(os.path.join(root, rel)) as f:
            for no, line in enumerate(f, 1):
                m = SIG.match(line.strip())
                if m:
                    out.append({"file": rel, "line": no, "method": "Base.:+", "args": [m.group(1), m.group(2)]})
    return out


def main(argv):
    args = [a for a in argv if not a.startswith("--")]
    root = args[0] if args else "/root/reference"
    text = json.dumps(collect(root), indent=1) + "\n"
    if "--check" in argv:
        with open(OUT) as f:
            return 0 if f.read() == text else 1
    with open(OUT, "w") as f:
        f.write(text)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
