"""Exact Delaunay checker -- TEST INFRASTRUCTURE ONLY.

Checks a triangle list against its points with the oracle's exact
predicates (floating-point filter plus expansion arithmetic, a different
method from the GPU's integer arithmetic), in the spirit of the reference
harness's verify() (qdt_verify.cpp:535-725):

* every triangle strictly counter-clockwise, no repeated index;
* every directed edge used at most once (a manifold mesh);
* every distinct point used, duplicates unused;
* the boundary is one closed counter-clockwise convex cycle, and the
  triangle count is 2 V - 2 - h (V used points, h boundary points), which
  with the above means the triangles tile the convex hull;
* every interior edge locally Delaunay: the opposite vertex is not strictly
  inside the circumcircle (exact in-circle <= 0).

Returns a dict of violation counts; all zero means a valid Delaunay
triangulation.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import oracle as O


def _lib():
    L = O.lib()
    if not getattr(L, "_batch_bound", False):
        for name in ("qdo_orient_batch", "qdo_incircle_batch"):
            f = getattr(L, name)
            f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
            f.restype = None
        L._batch_bound = True
    return L


def orient_signs(pts, idx3):
    idx3 = np.ascontiguousarray(idx3, dtype=np.int64)
    out = np.zeros(idx3.shape[0], dtype=np.int8)
    if idx3.shape[0]:
        _lib().qdo_orient_batch(pts.ctypes.data, idx3.ctypes.data, idx3.shape[0], out.ctypes.data)
    return out


def incircle_signs(pts, idx4):
    idx4 = np.ascontiguousarray(idx4, dtype=np.int64)
    out = np.zeros(idx4.shape[0], dtype=np.int8)
    if idx4.shape[0]:
        _lib().qdo_incircle_batch(pts.ctypes.data, idx4.ctypes.data, idx4.shape[0], out.ctypes.data)
    return out


def check(pts, tris, rep=None) -> dict:
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
    T = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    n = pts.shape[0]
    v = {"not_ccw": 0, "repeated_index": 0, "edge_reuse": 0, "unused_point": 0, "used_duplicate": 0,
         "boundary": 0, "count": 0, "not_delaunay": 0}
    if rep is None:
        from . import oracle
        rep = oracle.triangulate(pts).rep if n else np.zeros(0, np.uint32)
    rep = np.asarray(rep, dtype=np.int64)
    if T.shape[0] == 0:
        return v
    v["repeated_index"] = int(np.sum((T[:, 0] == T[:, 1]) | (T[:, 1] == T[:, 2]) | (T[:, 0] == T[:, 2])))
    v["not_ccw"] = int(np.sum(orient_signs(pts, T) <= 0))
    # directed edges
    E = np.concatenate([T[:, [0, 1]], T[:, [1, 2]], T[:, [2, 0]]], axis=0)
    opp = np.concatenate([T[:, 2], T[:, 0], T[:, 1]])
    key = E[:, 0] * n + E[:, 1]
    order = np.argsort(key, kind="stable")
    ks = key[order]
    v["edge_reuse"] = int(np.sum(ks[1:] == ks[:-1]))
    # used points
    used = np.zeros(n, dtype=bool)
    used[T.ravel()] = True
    is_rep = rep == np.arange(n)
    v["unused_point"] = int(np.sum(is_rep & ~used))
    v["used_duplicate"] = int(np.sum(~is_rep & used))
    # twins
    rkey = E[:, 1] * n + E[:, 0]
    pos = np.searchsorted(ks, rkey)
    pos = np.minimum(pos, ks.shape[0] - 1)
    has_twin = ks[pos] == rkey
    twin = order[pos]
    # boundary: directed edges without twin form one ccw convex cycle
    b = np.nonzero(~has_twin)[0]
    h = b.shape[0]
    V = int(used.sum())
    if T.shape[0] != 2 * V - 2 - h:
        v["count"] = 1
    bu, bv = E[b, 0], E[b, 1]
    nxt = {int(a): int(c) for a, c in zip(bu, bv)}
    if len(nxt) != h:
        v["boundary"] += 1
    else:
        start = int(bu[0])
        cyc = [start]
        cur = nxt[start]
        while cur != start and len(cyc) <= h:
            cyc.append(cur)
            cur = nxt.get(cur, start)
        if len(cyc) != h:
            v["boundary"] += 1
        else:
            c = np.array(cyc, dtype=np.int64)
            trip = np.stack([c, np.roll(c, -1), np.roll(c, -2)], axis=1)
            v["boundary"] += int(np.sum(orient_signs(pts, trip) < 0))
    # local Delaunay on interior edges (each undirected edge once)
    inter = np.nonzero(has_twin & (E[:, 0] < E[:, 1]))[0]
    if inter.shape[0]:
        q = np.stack([E[inter, 0], E[inter, 1], opp[inter], opp[twin[inter]]], axis=1)
        v["not_delaunay"] = int(np.sum(incircle_signs(pts, q) > 0))
    return v


def ok(res: dict) -> bool:
    return all(x == 0 for x in res.values())
