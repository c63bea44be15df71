"""Extract the literal known answers of SkewLinearAlgebra.jl's own test file
(test/runtests.jl) into tests/golden/reference_known_answers.json.

The Julia reference cannot run in this environment, so its deterministic
literals are the golden vectors: they are read here as TEXT from the reference
checkout and stored as JSON, which the tests load (the reference checkout is
not needed at test time).

Usage:  python tests/golden/make_known_answers.py path/to/SkewLinearAlgebra.jl/test/runtests.jl
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _nums(s: str):
    return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?(?:e-?\d+)?", s)]


def _matrix(s: str):
    """Julia matrix literal '[a b; c d]' -> list of rows."""
    body = s.strip()[1:-1]
    return [_nums(r) for r in body.split(";")]


def _sparse(call: str):
    """sparse([I], [J], [V], m, n) -> dense list of rows (1-based I, J)."""
    arrs = re.findall(r"\[([^\]]*)\]", call)
    I, J, V = (_nums(a) for a in arrs[:3])
    tail = call[call.rindex("]") + 1:]
    m, n = (int(x) for x in re.findall(r"\d+", tail)[:2])
    M = [[0.0] * n for _ in range(m)]
    for i, j, v in zip(I, J, V):
        M[int(i) - 1][int(j) - 1] += v
    return M


def extract(src: str) -> dict:
    lines = open(src).read().split("\n")

    def line(k):  # 1-based line numbers of runtests.jl
        return lines[k - 1]

    out = {"source": "SkewLinearAlgebra.jl test/runtests.jl", "cases": {}}
    C = out["cases"]
    # README testset (:9-30)
    C["readme_A"] = {"lines": "10", "A": _matrix(re.search(r"A = (\[.*\])", line(10)).group(1))}
    C["readme_hessenberg_v"] = {"lines": "18-19", "v": _nums(re.search(r"\[(.*)\]", line(18)).group(1))}
    ev = re.search(r"iλ₁,iλ₂ = (.*)", line(20)).group(1)
    C["readme_eigs"] = {"lines": "20-23", "ilambda": _nums(ev)}
    C["readme_Q"] = {"lines": "24", "Q": _matrix(re.search(r"≈ (\[.*\])", line(24)).group(1))}
    C["readme_inv_times9"] = {"lines": "16", "Ainv9": _matrix(re.search(r"≈ (\[.*\])/9", line(16)).group(1))}
    C["readme_det"] = {"lines": "14", "det": 81.0}
    # pfaffian known answers (:422-433)
    m49 = re.search(r"big\.\((\[.*\])\)\) == (-?\d+)", line(423))
    C["issue49"] = {"lines": "423", "A": _matrix(m49.group(1)), "pfaffian": float(m49.group(2))}
    m121 = re.search(r"pfaffian\((\[.*\])\) == (-?\d+)", line(433))
    C["issue121"] = {"lines": "433", "A": _matrix(m121.group(1)), "pfaffian": float(m121.group(2))}
    # issue #116 tridiagonal edge cases (:490, :499)
    ev116 = re.search(r"for ev in \((.*)\)$", line(490)).group(1)
    ev116b = re.search(r"for ev in \((.*)\)$", line(499)).group(1)
    C["issue116"] = {"lines": "490,499",
                     "ev_lists": [_nums(x) for x in re.findall(r"\[([^\]]*)\]", ev116 + "," + ev116b)]}
    # issue #130 / #118 (:512, :516, :521)
    C["issue130_10x10"] = {"lines": "512", "A": _sparse(re.search(r"sparse\((.*)\)", line(512)).group(0))}
    C["issue130_66x66"] = {"lines": "516", "A": _sparse(re.search(r"sparse\((.*)\)", line(516)).group(0))}
    ev118 = re.search(r"for v ∈ \((.*)\)$", line(521)).group(1)
    C["issue118"] = {"lines": "521", "ev_lists": [_nums(x) for x in re.findall(r"\[([^\]]*)\]", ev118)]}
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_known_answers.py path/to/SkewLinearAlgebra.jl/test/runtests.jl")
    src = sys.argv[1]
    data = extract(src)
    dst = os.path.join(HERE, "reference_known_answers.json")
    with open(dst, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main()
