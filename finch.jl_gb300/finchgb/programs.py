"""Matchers for whole @finch loop programs with several statements: the
`choose` and `minby` graph programs of Finch's examples, mapped onto the
graph kernels of libfinchgb.

  BFS round (docs/examples/bfs.jl:25-34)
      _F .= false
      for j=_, k=_
        if F[j] && edges[k, j] && !(V[k])
          _F[k] |= true
          P[k] <<choose(0)>>= j
        end
      end
  -> fgb_bfs_pull over the CSR of `edges` (row k lists its j)

  BFS bookkeeping (bfs.jl:35-42)
      for k=_; let _f = _F[k]; V[k] |= _f; c[] += _f; end; end
  -> fgb_or_count

  Relaxation, first loop (docs/examples/shortest_paths.jl:22-27)
      for j=_; if active_prev[j]; dists[j] <<minby>>= dists_prev[j]; end; end
  -> fgb_minby_map

  Relaxation, second loop (shortest_paths.jl:29-40)
      active .= false
      for j=_; if active_prev[j]; for i=_
        let d = first(dists_prev[j]) + edges[i, j]
          dists[i] <<minby>>= (d, j)
          active[i] |= d < first(dists_prev[i])
      end; end; end; end
  -> fgb_minby_relax over the CSR of `edges` (row i lists its j)

  Transition matrix of PageRank (docs/examples/pagerank.jl:18-25)
      scaled_edges .= 0
      for j=_, i=_
        if out_degree[i] != 0
          scaled_edges[i, j] = edges[i, j] / out_degree[j]
        end
      end
  -> fgb_sparse_scale over the stored entries of `edges` (the condition may
     test either index, the divisor run over either, and `*` stands for `/`)

The matchers bind the program's own tensor and index names, so any names
work; the shapes of the statements must be these.  Vertex numbers are
Finch's, 1-based.
"""
from __future__ import annotations

import numpy as np
import torch

from . import device as dev
from .notation import Assign, Call, Define, Index, Init, Lit, Loop, Sieve, Tup, Var, single, stmts


def _is_idx(e, name, *idxs) -> bool:
    return (isinstance(e, Index) and (name is None or e.tns == name)
            and len(e.idxs) == len(idxs) and all(isinstance(a, Var) and a.name == b for a, b in zip(e.idxs, idxs)))


def _and_terms(e) -> list:
    if isinstance(e, Call) and e.fn == "&&":
        return _and_terms(e.args[0]) + _and_terms(e.args[1])
    return [e]


def _nested(node, n):
    """n nested single loops: (indices outer first, body) or None."""
    idxs = []
    for _ in range(n):
        node = single(node)
        if not isinstance(node, Loop):
            return None
        idxs.append(node.idx)
        node = node.body
    return idxs, node


def match_bfs_round(prog) -> dict | None:
    s = stmts(prog)
    if len(s) != 2 or not isinstance(s[0], Init) or not isinstance(s[1], Loop):
        return None
    nf = s[0].name
    if not (isinstance(s[0].value, Lit) and s[0].value.value is False):
        return None
    nest = _nested(s[1], 2)
    if nest is None:
        return None
    (j, k), body = nest
    sv = single(body)
    if not isinstance(sv, Sieve):
        return None
    terms = _and_terms(sv.cond)
    if len(terms) != 3:
        return None
    F = E = V = None
    for t in terms:
        if _is_idx(t, None, j):
            F = t.tns
        elif _is_idx(t, None, k, j):
            E = t.tns
        elif isinstance(t, Call) and t.fn == "!" and _is_idx(t.args[0], None, k):
            V = t.args[0].tns
    if not (F and E and V):
        return None
    body_s = stmts(sv.body)
    if len(body_s) != 2:
        return None
    setf = next((a for a in body_s if isinstance(a, Assign) and a.op == "|" and _is_idx(a.lhs, nf, k)), None)
    par = next((a for a in body_s if isinstance(a, Assign) and isinstance(a.op, Call) and a.op.fn == "choose"
                and _is_idx(a.lhs, None, k)), None)
    if setf is None or par is None or not (isinstance(setf.rhs, Lit) and setf.rhs.value is True):
        return None
    if not (isinstance(par.rhs, Var) and par.rhs.name == j) or len(par.op.args) != 1 or \
            not isinstance(par.op.args[0], Lit):
        return None
    return {"next": nf, "frontier": F, "edges": E, "visited": V, "parent": par.lhs.tns,
            "fill": par.op.args[0].value}


def match_or_count(prog) -> dict | None:
    nest = _nested(prog, 1)
    if nest is None:
        return None
    (k,), body = nest
    d = single(body)
    if not isinstance(d, Define) or not _is_idx(d.value, None, k):
        return None
    f = d.name
    body_s = stmts(d.body)
    if len(body_s) != 2:
        return None
    vis = next((a for a in body_s if isinstance(a, Assign) and a.op == "|" and _is_idx(a.lhs, None, k)
                and isinstance(a.rhs, Var) and a.rhs.name == f), None)
    cnt = next((a for a in body_s if isinstance(a, Assign) and a.op == "+" and isinstance(a.lhs, Index)
                and a.lhs.idxs == () and isinstance(a.rhs, Var) and a.rhs.name == f), None)
    if vis is None or cnt is None:
        return None
    return {"next": d.value.tns, "visited": vis.lhs.tns, "count": cnt.lhs.tns}


def match_minby_map(prog) -> dict | None:
    nest = _nested(prog, 1)
    if nest is None:
        return None
    (j,), body = nest
    sv = single(body)
    mask = None
    if isinstance(sv, Sieve):
        if not _is_idx(sv.cond, None, j):
            return None
        mask = sv.cond.tns
        sv = single(sv.body)
    if not (isinstance(sv, Assign) and sv.op == "minby" and _is_idx(sv.lhs, None, j) and _is_idx(sv.rhs, None, j)):
        return None
    return {"mask": mask, "dst": sv.lhs.tns, "src": sv.rhs.tns}


def _first_of(e, i):
    return isinstance(e, Call) and e.fn == "first" and len(e.args) == 1 and _is_idx(e.args[0], None, i)


def match_minby_relax(prog) -> dict | None:
    s = stmts(prog)
    if len(s) != 2 or not isinstance(s[0], Init) or not isinstance(s[1], Loop):
        return None
    act = s[0].name
    if not (isinstance(s[0].value, Lit) and s[0].value.value is False):
        return None
    outer = s[1]
    j = outer.idx
    sv = single(outer.body)
    if not (isinstance(sv, Sieve) and _is_idx(sv.cond, None, j)):
        return None
    aprev = sv.cond.tns
    inner = single(sv.body)
    if not isinstance(inner, Loop):
        return None
    i = inner.idx
    d = single(inner.body)
    if not isinstance(d, Define):
        return None
    v = d.value
    if not (isinstance(v, Call) and v.fn == "+" and len(v.args) == 2):
        return None
    a, b = v.args
    if _first_of(b, j):
        a, b = b, a
    if not (_first_of(a, j) and _is_idx(b, None, i, j)):
        return None
    dprev, edges = a.args[0].tns, b.tns
    body_s = stmts(d.body)
    if len(body_s) != 2:
        return None
    upd = next((x for x in body_s if isinstance(x, Assign) and x.op == "minby" and _is_idx(x.lhs, None, i)), None)
    flag = next((x for x in body_s if isinstance(x, Assign) and x.op == "|" and _is_idx(x.lhs, act, i)), None)
    if upd is None or flag is None:
        return None
    if not (isinstance(upd.rhs, Tup) and len(upd.rhs.items) == 2 and isinstance(upd.rhs.items[0], Var)
            and upd.rhs.items[0].name == d.name and isinstance(upd.rhs.items[1], Var)
            and upd.rhs.items[1].name == j):
        return None
    c = flag.rhs
    if not (isinstance(c, Call) and c.fn == "<" and isinstance(c.args[0], Var) and c.args[0].name == d.name
            and _first_of(c.args[1], i) and c.args[1].args[0].tns == dprev):
        return None
    return {"active": act, "active_prev": aprev, "dist_prev": dprev, "edges": edges, "dist": upd.lhs.tns}


def match_masked_scale(prog) -> dict | None:
    s = stmts(prog)
    if len(s) != 2 or not isinstance(s[0], Init) or not isinstance(s[1], Loop):
        return None
    out = s[0].name
    if not (isinstance(s[0].value, Lit) and s[0].value.value == 0 and not isinstance(s[0].value.value, bool)):
        return None
    nest = _nested(s[1], 2)
    if nest is None:
        return None
    (j, i), body = nest
    keep = None
    sv = single(body)
    if isinstance(sv, Sieve):
        c = sv.cond
        if not (isinstance(c, Call) and c.fn == "!=" and len(c.args) == 2 and isinstance(c.args[1], Lit)
                and c.args[1].value == 0 and isinstance(c.args[0], Index) and len(c.args[0].idxs) == 1
                and isinstance(c.args[0].idxs[0], Var) and c.args[0].idxs[0].name in (i, j)):
            return None
        keep = (c.args[0].tns, "row" if c.args[0].idxs[0].name == i else "col")
        sv = single(sv.body)
    if not (isinstance(sv, Assign) and sv.op is None and _is_idx(sv.lhs, out, i, j)):
        return None
    rhs = sv.rhs
    if not (isinstance(rhs, Call) and rhs.fn in ("/", "*") and len(rhs.args) == 2):
        return None
    pairs = [rhs.args] if rhs.fn == "/" else [rhs.args, rhs.args[::-1]]
    for a, b in pairs:
        if (_is_idx(a, None, i, j) and isinstance(b, Index) and len(b.idxs) == 1 and isinstance(b.idxs[0], Var)
                and b.idxs[0].name in (i, j) and b.tns != a.tns):
            return {"out": out, "init": s[0].value.value, "edges": a.tns, "by": b.tns,
                    "by_axis": "row" if b.idxs[0].name == i else "col", "op": rhs.fn,
                    "keep": None if keep is None else keep[0], "keep_axis": None if keep is None else keep[1]}
    return None


# ---------------------------------------------------------------- execution


MATCHERS = (("bfs_round", match_bfs_round), ("or_count", match_or_count), ("minby_map", match_minby_map),
            ("masked_scale", match_masked_scale), ("minby_relax", match_minby_relax))


def match(prog) -> tuple | None:
    """(kind, bindings) of the first whole-program matcher that binds prog,
    or None.  Depends on the program alone, so callers may keep it."""
    for kind, fn in MATCHERS:
        m = fn(prog)
        if m is not None:
            return kind, m
    return None


def run(prog, tensors: dict, adjacency_rows) -> dict | None:
    """Runs a matched program on the device; returns {name: tensor} of the
    outputs, or None if no graph program matches.  adjacency_rows(t) gives
    the CSR of a matrix tensor whose row i lists the j with t[i, j] stored."""
    found = match(prog)
    return None if found is None else run_matched(found[0], found[1], tensors, adjacency_rows)


def run_matched(kind: str, m: dict, tensors: dict, adjacency_rows) -> dict:
    """Runs a program that match() bound, on the given tensors."""
    from .tensors import dense_from_device
    from .scheduler import FinchGBUnsupported, Scalar, _device_vector

    if kind == "bfs_round":
        A = adjacency_rows(tensors[m["edges"]])
        F = _device_vector(tensors[m["frontier"]], torch.uint8)
        V = _device_vector(tensors[m["visited"]], torch.uint8)
        P = _device_vector(tensors[m["parent"]], None)
        if P.dtype not in (torch.int32, torch.int64):
            raise FinchGBUnsupported("choose: the parent vector must hold Int32 or Int64")
        nxt = dev.bfs_pull(A, F, V, P, choose_fill=int(m["fill"]), index_offset=1)
        return {m["next"]: dense_from_device(nxt, False), m["parent"]: tensors[m["parent"]]}
    if kind == "or_count":
        nxt = _device_vector(tensors[m["next"]], torch.uint8)
        V = _device_vector(tensors[m["visited"]], torch.uint8)
        c = tensors[m["count"]]
        if not isinstance(c, Scalar):
            raise FinchGBUnsupported("the count must be a Scalar")
        cnt = c.device_value(torch.int64)
        dev.or_count(V, nxt, cnt)
        return {m["visited"]: tensors[m["visited"]], m["count"]: c}
    if kind == "minby_map":
        mask = None if m["mask"] is None else _device_vector(tensors[m["mask"]], torch.uint8)
        src = tensors[m["src"]].pair_device()
        dst = tensors[m["dst"]].pair_device()
        dev.minby_map(mask, src, dst)
        return {m["dst"]: tensors[m["dst"]]}
    if kind == "masked_scale":
        return _run_masked_scale(m, tensors)
    if kind == "minby_relax":
        A = adjacency_rows(tensors[m["edges"]])
        dprev = tensors[m["dist_prev"]].pair_device()
        aprev = _device_vector(tensors[m["active_prev"]], torch.uint8)
        dst = tensors[m["dist"]].pair_device()
        if A.val is None or A.val.dtype != dprev[0].dtype:
            raise FinchGBUnsupported("minby: the edge weights and distances must share one type")
        act = dev.minby_relax(A, dprev[0], aprev, dst, index_offset=1)
        return {m["active"]: dense_from_device(act, False), m["dist"]: tensors[m["dist"]]}
    raise ValueError(f"unknown program kind {kind!r}")


def _run_masked_scale(m: dict, tensors: dict) -> dict:
    """fgb_sparse_scale for a matched masked scale.  The kernel visits the
    stored entries of the sparse operand; Finch's nest also writes
    `0 op by[l]` where it stores nothing, since `/` has no annihilator
    (src/symbolic/symbolic.jl:145-153).  Those values equal the fill 0
    unless an element of `by` is 0 or NaN (Inf or NaN for `*`), which the
    library counts: such a program is refused rather than answered
    differently."""
    from . import _lib as L
    from .scheduler import FinchGBUnsupported, _device_vector, sparse_operand
    from .tensors import sparse_from_device

    e = tensors[m["edges"]]
    fill = (e.body if hasattr(e, "body") else e).fill_value
    if np.any(np.asarray(fill)):
        raise FinchGBUnsupported(f"{m['edges']}: a scale of stored entries needs a zero fill, not {fill!r}")
    A = sparse_operand(e, ("i", "j"), ("i", "j"))
    by = _device_vector(tensors[m["by"]], None)
    keep = None if m["keep"] is None else _device_vector(tensors[m["keep"]], None)
    prev = tensors.get(m["out"])
    out_dtype = torch.float32 if prev is not None and np.dtype(prev.dtype) == np.float32 else torch.float64
    axis = {"row": L.AXIS_ROW, "col": L.AXIS_COL}
    res, changed = dev.sparse_scale(A, by, axis[m["by_axis"]], keep, axis.get(m["keep_axis"], L.AXIS_ROW),
                                    L.MAP_DIV if m["op"] == "/" else L.MAP_MUL, out_dtype)
    if changed:
        raise FinchGBUnsupported(
            f"{changed} element(s) of {m['by']} make `0 {m['op']} {m['by']}` non-zero (0/0 is NaN): Finch's "
            f"nest writes that value wherever {m['edges']} stores nothing, so visiting its stored entries "
            f"alone would give another result")
    return {m["out"]: sparse_from_device(res, fill_value=float(m["init"]))}
