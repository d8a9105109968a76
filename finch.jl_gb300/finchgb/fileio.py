"""fread / fwrite: Finch's file formats, read straight into HBM when asked.

Formats by extension, as in src/interface/fileio/fileio.jl:
  .bspnpy     Binsparse, NumPy + JSON directory (binsparse.jl; NPZExt.jl)
  .mtx .ttx   MatrixMarket / TensorMarket coordinate text (TensorMarketExt.jl)
  .tns        FROSTT coordinate text
  .bsp.h5     Binsparse HDF5: needs an HDF5 module, which this environment
              lacks -- the same error the reference raises without HDF5.jl.

With `device` given, level buffers go to the GPU directly: a compressed
(CSC/CSR) tensor's ptr/idx/values are uploaded as they are (idx narrowed to
int32), and coordinate (COO) data are sorted and folded in HBM by
fgb_coo_assemble -- no host-side conversion between formats.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from .tensors import (GPU, Dense, Element, Pattern, SparseList, SwizzleArray, Tensor,
                      fsparse, swizzle, transfer)
from .workloads import SparseBuffers

BINSPARSE_VERSION = "0.1"

_BSP_TYPES = {"uint8": np.uint8, "uint16": np.uint16, "uint32": np.uint32, "uint64": np.uint64,
              "int8": np.int8, "int16": np.int16, "int32": np.int32, "int64": np.int64,
              "float32": np.float32, "float64": np.float64, "bint8": np.bool_}
_BSP_NAMES = {np.dtype(v): k for k, v in _BSP_TYPES.items()}


class FinchExtensionError(RuntimeError):
    """A format whose reader needs a module this environment does not have."""


def fwrite(filename: str, t) -> str:
    name = str(filename)
    if name.endswith(".tns"):
        _tns_write(name, t)
    elif name.endswith(".ttx") or name.endswith(".mtx"):
        _tt_write(name, t)
    elif name.endswith(".bspnpy"):
        _bsp_write(name, t)
    elif name.endswith(".bsp.h5") or name.endswith(".bsp.hdf5"):
        raise FinchExtensionError("HDF5 must be available to write .bsp.h5 files")
    else:
        raise ValueError(f"Unknown file extension for file {name}")
    return name


def fread(filename: str, device=None):
    name = str(filename)
    if name.endswith(".tns"):
        t = _tns_read(name)
    elif name.endswith(".ttx") or name.endswith(".mtx"):
        t = _tt_read(name)
    elif name.endswith(".bspnpy"):
        t = _bsp_read(name)
    elif name.endswith(".bsp.h5") or name.endswith(".bsp.hdf5"):
        raise FinchExtensionError("HDF5 must be available to read .bsp.h5 files")
    else:
        raise ValueError(f"Unknown file extension for file {name}")
    if device is not None:
        transfer(device if isinstance(device, GPU) else GPU(int(device)), t)
    return t


# ---------------------------------------------------------------- coordinates


def _findnz(t):
    """Coordinates (1-based, column-major order -- Finch's ffindnz) and values."""
    if isinstance(t, SwizzleArray):
        I, J, V = _findnz(t.body)
        if tuple(t.dims) == (2, 1):
            I, J = J, I
            order = np.lexsort((I, J))
            return I[order], J[order], V[order]
        return I, J, V
    if t.kind == "coo" and t.coo is not None:
        I, J, V = (np.asarray(a) for a in t.coo)
        key = (J - 1) * t.shape[0] + (I - 1)
        order = np.argsort(key, kind="stable")
        key, V = key[order], V[order]
        heads = np.flatnonzero(np.r_[True, key[1:] != key[:-1]])
        if heads.size != key.size:  # duplicates fold with the tensor's combine
            from .tensors import _fold

            ends = np.r_[heads[1:], key.size]
            V = np.array([_fold(t.combine, V[a:b]) for a, b in zip(heads, ends)], dtype=V.dtype)
            key = key[heads]
        return key % t.shape[0] + 1, key // t.shape[0] + 1, V
    elif t.kind in ("dense1", "dense2"):
        D = t.todense()
        if D.ndim == 1:
            nz = np.flatnonzero(D != t.fill_value)
            return (nz + 1,), None, D[nz]
    else:
        b = t.host_buffers()
        f = np.repeat(np.arange(b.nfibers), np.diff(b.ptr))
        inner = np.asarray(b.idx, dtype=np.int64) - b.base
        I, J = (inner, f) if b.orient == "csc" else (f, inner)
        V = np.ones(b.nnz, dtype=np.bool_) if b.val is None else np.asarray(b.val)
        order = np.lexsort((I, J))
        return I[order] + 1, J[order] + 1, V[order]
    J, I = np.nonzero(D.T != t.fill_value)  # column-major
    return I + 1, J + 1, D[I, J]


def _field(V) -> str:
    kind = np.asarray(V).dtype.kind
    return {"b": "pattern", "i": "integer", "u": "integer", "f": "real", "c": "complex"}[kind]


def _fmt_value(v) -> str:
    if isinstance(v, (np.floating, float)):
        return repr(float(v))
    return str(int(v))


def _tt_write(name: str, t) -> None:
    I, J, V = _findnz(t)
    shape = tuple(t.shape)
    field = _field(V)
    lines = [f"%%MatrixMarket matrix coordinate {field} general",
             f"{shape[0]} {shape[1]} {len(I)}"]
    for a, b, v in zip(I, J, V):
        lines.append(f"{a} {b}" if field == "pattern" else f"{a} {b} {_fmt_value(v)}")
    Path(name).write_text("\n".join(lines) + "\n")


def _tt_read(name: str) -> Tensor:
    """MatrixMarket/TensorMarket coordinate file -> a COO tensor (fsparse!)."""
    with open(name) as f:
        header = f.readline().split()
        if len(header) < 5 or header[0].lower() not in ("%%matrixmarket", "%%tensormarket"):
            raise ValueError(f"{name}: not a MatrixMarket/TensorMarket file")
        fmt, field, symm = header[2].lower(), header[3].lower(), header[4].lower()
        if fmt != "coordinate":
            raise ValueError(f"{name}: only coordinate files are read")
        line = f.readline()
        while line.startswith("%") or not line.strip():
            line = f.readline()
        m, n, nnz = (int(x) for x in line.split()[:3])
        data = np.loadtxt(f, ndmin=2, max_rows=nnz) if nnz else np.zeros((0, 3))
    I = data[:, 0].astype(np.int64)
    J = data[:, 1].astype(np.int64)
    if field == "pattern":
        V = np.ones(len(I), dtype=np.bool_)
    elif field == "integer":
        V = data[:, 2].astype(np.int64)
    elif field == "real":
        V = data[:, 2].astype(np.float64)
    else:
        raise ValueError(f"{name}: field {field} is not supported")
    if symm in ("symmetric", "skew-symmetric", "hermitian"):
        off = I != J
        sign = -1 if symm == "skew-symmetric" else 1
        I, J, V = (np.r_[I, J[off]], np.r_[J, I[off]],
                   np.r_[V, (V[off] * sign) if field != "pattern" else V[off]])
    return fsparse(I, J, V, (m, n))


def _tns_write(name: str, t) -> None:
    I, J, V = _findnz(t)
    Path(name).write_text("".join(f"{a} {b} {_fmt_value(v)}\n" for a, b, v in zip(I, J, V)))


def _tns_read(name: str) -> Tensor:
    data = np.loadtxt(name, ndmin=2)
    I, J = data[:, 0].astype(np.int64), data[:, 1].astype(np.int64)
    raw = data[:, 2]
    V = raw.astype(np.int64) if np.all(raw == np.round(raw)) else raw
    return fsparse(I, J, V)


# ---------------------------------------------------------------- binsparse


def _bsp_write(name: str, t) -> None:
    """A tensor as a binsparse directory: binsparse.json + one .npy per array
    (src/interface/fileio/binsparse.jl:275-298, NPZExt.jl)."""
    d = Path(name)
    d.mkdir(parents=True, exist_ok=True)
    arrays: dict[str, np.ndarray] = {}
    desc: dict = {"version": BINSPARSE_VERSION, "fill": True, "data_types": {},
                  "attrs": {}}
    swz = isinstance(t, SwizzleArray) and tuple(t.dims) == (2, 1)
    body = t.body if isinstance(t, SwizzleArray) else t
    fill = body.fill_value
    if body.kind == "dense1":
        desc["format"], desc["shape"] = "DVEC", [int(body.shape[0])]
        arrays["values"] = np.asarray(body.todense())
    elif body.kind == "dense2":
        D = np.asarray(body.todense())
        if swz:  # rows outer
            desc["format"], desc["shape"] = "DMATR", list(map(int, t.shape))
            arrays["values"] = np.ascontiguousarray(D.T).reshape(-1)
        else:
            desc["format"], desc["shape"] = "DMATC", list(map(int, D.shape))
            arrays["values"] = np.asfortranarray(D).reshape(-1, order="F")
    elif body.kind == "csc":
        b = body.host_buffers()
        desc["format"] = "CSR" if swz else "CSC"
        desc["shape"] = list(map(int, t.shape if swz else body.shape))
        arrays["pointers_to_1"] = np.asarray(b.ptr, dtype=np.int64) - b.base
        arrays["indices_1"] = np.asarray(b.idx, dtype=np.int64) - b.base
        if b.val is not None:
            arrays["values"] = np.asarray(b.val)
    elif body.kind == "coo":
        I, J, V = _findnz(body)
        desc["format"], desc["shape"] = "COOC", list(map(int, body.shape))
        arrays["indices_1"], arrays["indices_0"] = I - 1, J - 1
        arrays["values"] = np.asarray(V)
    else:
        raise NotImplementedError(f"binsparse writer: tensor kind {body.kind}")
    if "values" in arrays:
        arrays["fill_value"] = np.array([fill], dtype=arrays["values"].dtype)
    desc["number_of_stored_values"] = int(len(arrays.get("values", arrays.get("indices_1", []))))
    for k, v in arrays.items():
        v = np.ascontiguousarray(v)
        desc["data_types"][k] = _BSP_NAMES[v.dtype]
        np.save(d / f"{k}.npy", v)
    (d / "binsparse.json").write_text(json.dumps({"binsparse": desc}, indent=4))


def _bsp_read(name: str):
    """binsparse directory -> tensor, following bspread (binsparse.jl:329-353):
    CSC/COOC come back as plain tensors, CSR/COO/COOR/DMATR as the swizzle of
    the transposed storage."""
    d = Path(name)
    desc = json.loads((d / "binsparse.json").read_text())["binsparse"]
    if desc.get("version") != BINSPARSE_VERSION:
        raise ValueError(f"{name}: binsparse version {desc.get('version')} (expected {BINSPARSE_VERSION})")
    if "structure" in desc:
        raise ValueError("binsparse structure field currently unsupported")
    fmt = desc.get("format")
    shape = [int(x) for x in desc["shape"]]

    def arr(key):
        t = desc["data_types"][key]
        if t.startswith("iso[") or t.startswith("complex["):
            raise ValueError(f"binsparse type {t} is not supported")
        return np.load(d / f"{key}.npy").astype(_BSP_TYPES[t], copy=False)

    vals = arr("values") if "values" in desc["data_types"] else None
    fill = arr("fill_value")[0] if "fill_value" in desc["data_types"] else (
        np.zeros((), vals.dtype)[()] if vals is not None else False)
    if fmt == "DVEC":
        return Tensor(Dense(Element(fill, vals.dtype)), vals)
    if fmt in ("DMAT", "DMATR"):  # rows outer, no transpose: the swizzle of the storage
        D = vals.reshape(shape)
        return swizzle(Tensor(Dense(Dense(Element(fill, vals.dtype))), D.T), 2, 1)
    if fmt == "DMATC":
        D = vals.reshape(shape, order="F")
        return Tensor(Dense(Dense(Element(fill, vals.dtype))), D)
    if fmt in ("CSC", "CSR"):
        ptr = arr("pointers_to_1").astype(np.int64) + 1
        idx = arr("indices_1").astype(np.int64) + 1
        m, n = shape
        lvl = Pattern() if vals is None else Element(fill, vals.dtype)
        if fmt == "CSC":
            b = SparseBuffers(m, n, ptr, idx, vals, "csc")
            return Tensor.from_buffers(Dense(SparseList(lvl)), b)
        # CSR: the CSC storage of the transpose (n x m), swizzled back
        b = SparseBuffers(n, m, ptr, idx, vals, "csc")
        return swizzle(Tensor.from_buffers(Dense(SparseList(lvl)), b), 2, 1)
    if fmt in ("COO", "COOR", "COOC"):
        i1 = arr("indices_1").astype(np.int64) + 1
        i0 = arr("indices_0").astype(np.int64) + 1
        if vals is None:
            vals = np.ones(len(i0), dtype=np.bool_)
        if fmt == "COOC":  # transpose [1, 0]: tbl = (indices_1, indices_0) on the given shape
            return fsparse(i1, i0, vals, tuple(shape), fill_value=fill)
        # no transpose: the reversed shape, swizzled back
        return swizzle(fsparse(i1, i0, vals, (shape[1], shape[0]), fill_value=fill), 2, 1)
    raise ValueError(f"binsparse format {fmt} is not supported")
