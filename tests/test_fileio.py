"""fread / fwrite (src/interface/fileio): the TensorMarket text of Trec4
against the reference's own golden output, and round trips of every format
and tensor kind the reference's fileio tests cover."""
import json
from pathlib import Path

import numpy as np
import pytest

from finchgb import (Dense, Element, FinchExtensionError, Pattern, SparseCOO, SparseList, Tensor,
                     fread, fwrite, swizzle)

GOLDEN = Path(__file__).parent / "golden"
KATS = json.loads((GOLDEN / "finch_kats.json").read_text())["kats"]
A = np.array([[0.0, 1.0, 2.0, 2.0], [0.0, 0.0, 0.0, 0.0], [1.0, 1.0, 2.0, 0.0], [0.0, 0.0, 0.0, 1.0]])


def test_trec4_ttx_matches_reference_text(tmp_path):
    # the reference reads Trec4.mtx and writes it back as .ttx (fileio_tests.jl:164-168)
    z = np.load(GOLDEN / "mtx_Trec4.npz")
    src = tmp_path / "Trec4.mtx"
    lines = ["%%MatrixMarket matrix coordinate integer general", "% a comment",
             f"{z['shape'][0]} {z['shape'][1]} {len(z['i'])}"]
    lines += [f"{i} {j} {int(v)}" for i, j, v in zip(z["i"], z["j"], z["v"])]
    src.write_text("\n".join(lines) + "\n")
    t = fread(str(src))
    out = tmp_path / "test.ttx"
    fwrite(str(out), t)
    assert out.read_text().rstrip("\n") == KATS["trec4_ttx"]["text"].rstrip("\n")


@pytest.mark.parametrize("ext", [".ttx", ".mtx", ".tns", ".bspnpy"])
def test_coo_round_trip(tmp_path, ext):
    t = Tensor(SparseCOO(2, Element(0.0)), A)
    f = str(tmp_path / f"A_COO{ext}")
    fwrite(f, t)
    back = fread(f)
    # .tns records no shape: the largest coordinates (here the full 4 x 4)
    assert back.shape == (4, 4) and back == t


@pytest.mark.parametrize("dtype", [np.float64, np.int64, np.bool_])
@pytest.mark.parametrize("fill", [0, 1])
def test_binsparse_formats(tmp_path, dtype, fill):
    D = (A if dtype != np.bool_ else A != 0).astype(dtype)
    fv = np.asarray(fill).astype(dtype)[()]
    el = Element(fv, dtype)
    cases = {
        "dense": swizzle(Tensor(Dense(Dense(el)), D.T), 2, 1),
        "denseC": Tensor(Dense(Dense(el)), D),
        "CSC": Tensor(Dense(SparseList(el)), D),
        "CSR": swizzle(Tensor(Dense(SparseList(el)), D.T), 2, 1),
        "COOC": Tensor(SparseCOO(2, el), D),
    }
    for name, t in cases.items():
        f = str(tmp_path / f"A_{name}_{fill}.bspnpy")
        fwrite(f, t)
        back = fread(f)
        assert np.array_equal(back.todense(), t.todense()), name
        assert type(back) is type(t), name  # swizzled stays swizzled


def test_dense_vector_and_errors(tmp_path):
    # the reference's issue #500 case: a Dense vector through .bspnpy
    v = Tensor(Dense(Element(0.0)), np.random.default_rng(0).random(4))
    f = str(tmp_path / "test.bspnpy")
    fwrite(f, v)
    assert fread(f) == v
    with pytest.raises(FinchExtensionError):
        fread(str(tmp_path / "x.bsp.h5"))
    with pytest.raises(ValueError):
        fwrite(str(tmp_path / "x.unknown"), v)
