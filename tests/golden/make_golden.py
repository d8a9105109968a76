"""Extracts known-answer tests from Finch.jl's own test fixtures.

Reads (text only) the Finch.jl checkout given as the one argument and writes tests/golden/finch_kats.json plus the
MatrixMarket test matrices as tests/golden/mtx_<name>.npz.  Every value in
the JSON is parsed out of the file named beside it; nothing is typed in by
hand.  Run once where the reference is mounted; the outputs are committed so
tests never need the reference at run time.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _floats(s: str) -> list[float]:
    return [float(t) for t in re.findall(r"-?\d+(?:\.\d+)?(?:e-?\d+)?", s)]


def _matrix(lit: str) -> list[list[float]]:
    """Julia matrix literal `[a b c; d e f]` -> rows."""
    body = lit.strip().lstrip("[").rstrip("]")
    return [_floats(row) for row in body.split(";")]


def _result_vector(text: str, prefix: str) -> list[float]:
    m = re.search(re.escape(prefix) + r"\[([^\]]*)\]", text)
    assert m, prefix
    return _floats(m.group(1))


def main(ref: Path) -> None:
    out: dict = {"source": "Finch.jl v1.2.12 test fixtures", "kats": {}}
    kats = out["kats"]

    # 1. CSC SpMV (typical_spmv_csc.txt:1-17 inputs, :92 result)
    f = ref / "test/reference64/typical/typical_spmv_csc.txt"
    t = f.read_text()
    a_lit = re.search(r"A = Tensor\(Dense\(SparseList\(Element\(0\.0\)\)\), (\[[^\]]*\])\)", t).group(1)
    x_lit = re.search(r"x = Tensor\((\[[^\]]*\])\)", t).group(1)
    y = _result_vector(t.split("julia> @finch begin")[1], "Element{0.0, Float64, Int64}(")
    kats["spmv_csc"] = {"file": "test/reference64/typical/typical_spmv_csc.txt",
                        "A": _matrix(a_lit), "x": _floats(x_lit), "y": y,
                        "program": "y .= 0; for j=_, i=_; y[i] += A[i,j] * x[j]"}
    # same KAT through SparseMatrixCSC (typical_spmv_sparsematrixcsc.txt:85)
    f2 = ref / "test/reference64/typical/typical_spmv_sparsematrixcsc.txt"
    t2 = f2.read_text()
    kats["spmv_sparsematrixcsc"] = {
        "file": "test/reference64/typical/typical_spmv_sparsematrixcsc.txt",
        "A": _matrix(re.search(r"A = sparse\((\[[^\]]*\])\)", t2).group(1)),
        "y": _floats(re.search(r"\(y = \[([^\]]*)\],\)", t2).group(1))}

    # 2. Transposed Int SpMV (parallel_tests.jl:414-415 inputs,
    #    parallel_spmv_atomics.txt:117 result)
    pt = (ref / "test/suites/parallel_tests.jl").read_text()
    blk = pt[pt.index("parallel/parallel_spmv_atomics.txt") - 1500:pt.index("parallel/parallel_spmv_atomics.txt")]
    a_lit = re.findall(r"A = Tensor\(Dense\(SparseList\(Element\(0\)\)\), (\[[^\]]*\])\)", blk)[-1]
    x_lit = re.findall(r"x = Tensor\(Dense\(Element\(0\)\), (\[[^\]]*\])\)", blk)[-1]
    t3 = (ref / "test/reference64/parallel/parallel_spmv_atomics.txt").read_text()
    kats["spmv_transposed_int"] = {
        "file": "test/reference64/parallel/parallel_spmv_atomics.txt",
        "A": _matrix(a_lit), "x": _floats(x_lit),
        "y": _result_vector(t3.split("(y = Tensor")[-1], "Element{0, Int64, Int64}("),
        "program": "y .= 0; for i=_, j=_; y[j] += x[i] * A[i,j]"}

    # 3. Two-finger sparse + sparse (typical_tests.jl inputs,
    #    typical_merge_twofinger.txt:194 result)
    tt = (ref / "test/suites/typical_tests.jl").read_text()
    sl = re.findall(r"SparseList\(\s*Element\{0\.0,\s*Float64\}\((\[[^\]]*\])\),\s*(\d+),\s*(\[[^\]]*\]),\s*(\[[^\]]*\])\)", tt)
    (xv, xn, xp, xi), (yv, yn, yp, yi) = sl[0], sl[1]
    t4 = (ref / "test/reference64/typical/typical_merge_twofinger.txt").read_text()
    m = re.search(r"\(z = Tensor\(SparseList\{Int64\}\(Element\{0\.0, Float64, Int64\}\((\[[^\]]*\])\), (\d+), (\[[^\]]*\]), (\[[^\]]*\])\)\),\)", t4)
    kats["merge_twofinger_add"] = {
        "file": "test/reference64/typical/typical_merge_twofinger.txt",
        "x": {"n": int(xn), "ptr": _floats(xp), "idx": _floats(xi), "val": _floats(xv)},
        "y": {"n": int(yn), "ptr": _floats(yp), "idx": _floats(yi), "val": _floats(yv)},
        "z": {"n": int(m.group(2)), "ptr": _floats(m.group(3)), "idx": _floats(m.group(4)),
              "val": _floats(m.group(1))},
        "program": "z .= 0; for i=_; z[i] = x[i] + y[i]"}

    # 4. einsum matmul and reduction (interface_tests.jl:13-24)
    it = (ref / "test/suites/interface_tests.jl").read_text()
    a = _matrix(re.search(r"A = (\[1 2; 3 4\])", it).group(1))
    b = _matrix(re.search(r"B = (\[5 6; 7 8\])", it).group(1))
    s = int(re.search(r"@test s\[\] == (\d+)", it).group(1))
    c = _matrix(re.search(r"@test C == (\[[^\]]*\])", it).group(1))
    kats["einsum_matmul"] = {"file": "test/suites/interface_tests.jl", "A": a, "B": b, "C": c,
                             "s_abs": s,
                             "program": "@einsum C[i,j] += A[i,k]*B[k,j]; "
                                        "@einsum s[] += abs(A[i,k]*B[k,j])"}

    # 5. reduce(+, A; dims) (reference64/interface/reduce_default.txt)
    t5 = (ref / "test/reference64/interface/reduce_default.txt").read_text()
    a_lit = re.search(r"A = Tensor\(Dense\(SparseList\(Element\(0\.0\)\)\), (\[[^\]]*\])\)", t5).group(1)
    parts = t5.split("julia> ")
    def _after(header):
        blk = next(p for p in parts if p.startswith(header))
        return _floats("\n".join(blk.splitlines()[2:]))
    kats["reduce"] = {"file": "test/reference64/interface/reduce_default.txt",
                      "A": _matrix(a_lit), "dims1": _after("reduce(+, A, dims = 1)"),
                      "dims2": _after("reduce(+, A, dims = 2)"),
                      "all": _floats(next(p for p in parts if p.startswith("reduce(+, A, dims = (:))")).splitlines()[1])[0]}

    # 6. fwrite of Trec4 read from its .mtx: the canonical TensorMarket text
    #    (test/suites/fileio_tests.jl:164-168 checks it against this fixture)
    kats["trec4_ttx"] = {"file": "test/reference64/fileio/Trec4.ttx",
                         "text": (ref / "test/reference64/fileio/Trec4.ttx").read_text()}

    (HERE / "finch_kats.json").write_text(json.dumps(out, indent=1))

    # 7. MatrixMarket matrices used by Finch's kernel tests (kernel_tests.jl)
    for rel in ["HB/west0132", "LPnetlib/lpi_itest6", "LPnetlib/lp_blend", "JGD_Kocay/Trec4"]:
        lines = [ln for ln in (ref / "test/data" / f"{rel}.mtx").read_text().splitlines()
                 if ln and not ln.startswith("%")]
        m_, n_, nnz = (int(v) for v in lines[0].split())
        trip = np.array([[float(v) for v in ln.split()[:3]] for ln in lines[1:1 + nnz]])
        np.savez_compressed(HERE / f"mtx_{rel.split('/')[-1]}.npz", shape=np.array([m_, n_]),
                            i=trip[:, 0].astype(np.int64), j=trip[:, 1].astype(np.int64),
                            v=trip[:, 2])
    print("wrote", HERE / "finch_kats.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of a Finch.jl checkout>")
    main(Path(sys.argv[1]))
