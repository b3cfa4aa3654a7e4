"""Constraint tracing on the GPU (qdtg_trace_constraints).

For every edge, on its own against the current triangulation, the status
must be exactly what qdt_insert_constraint returns when that edge is the
next call (checked on an identical copy of the context), and the crossed
count must equal the number of mesh edges the open segment properly
crosses (brute force with the oracle's exact orientation predicate).
"""
import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from libqdt_gb300 import workloads as W
from oracle import delaunay_check as D

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return G.load()


def state(t):
    n = t.points_size()
    pts = np.array([t.point(i)[1] for i in range(n)])
    return pts, t.triangles_array().astype(np.int64), t.rep_array().astype(np.int64)


def undirected_edges(tris):
    E = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    E = np.sort(E, axis=1)
    return np.unique(E, axis=0)


def crossings(pts, edges, u, w):
    """Mesh edges the open segment u-w properly crosses."""
    k = len(edges)
    a, b = edges[:, 0], edges[:, 1]
    U, Wv = np.full(k, u), np.full(k, w)
    o1 = D.orient_signs(pts, np.stack([U, Wv, a], 1)).astype(int)
    o2 = D.orient_signs(pts, np.stack([U, Wv, b], 1)).astype(int)
    o3 = D.orient_signs(pts, np.stack([a, b, U], 1)).astype(int)
    o4 = D.orient_signs(pts, np.stack([a, b, Wv], 1)).astype(int)
    return int(((o1 * o2 < 0) & (o3 * o4 < 0)).sum())


def make(lib, base, pre):
    t = G.Triangulation(lib)
    assert t.execute(base) == Q.QDT_OK
    if len(pre):
        t.insert_constraints_batch(pre)
    return t


def test_trace_equals_insert_constraint(lib):
    rng = np.random.default_rng(17)
    base = rng.integers(0, 24, size=(260, 2)).astype(np.float64)   # collinear runs and duplicates
    pre = rng.integers(0, len(base), size=(12, 2))
    t = make(lib, base, pre)
    pts, tris, rep = state(t)
    n = len(base)
    E = undirected_edges(tris)
    entries = [rng.integers(0, n, size=(150, 2)),                   # random pairs
               E[rng.integers(0, len(E), 30)],                       # existing edges
               np.array([[0, n + 3], [n, 1], [5, 5]])]               # invalid index, same point
    dup = np.nonzero(rep != np.arange(n))[0]
    if dup.size:
        entries.append(np.stack([dup[:5], rep[dup[:5]]], 1))        # a point and its duplicate
    entries = np.concatenate(entries).astype(np.uint64)
    st, status, crossed = t.trace_constraints(entries)
    assert st == Q.QDT_OK
    seen = set()
    for (a, b), s, c in zip(entries, status, crossed):
        u = make(lib, base, pre)
        want = u.insert_constraint(int(a), int(b))
        u.close()
        assert s == want, "edge %d-%d: traced %d, inserted %d" % (a, b, s, want)
        seen.add(int(s))
        if s == Q.QDT_OK:
            ra, rb = int(rep[a]), int(rep[b])
            exists = ((E[:, 0] == min(ra, rb)) & (E[:, 1] == max(ra, rb))).any()
            assert c == (0 if exists else crossings(pts, E, ra, rb))
    assert {Q.QDT_OK, Q.QDT_ERR_THROUGH_POINT, Q.QDT_ERR_INVALID_INDEX, Q.QDT_ERR_SAME_POINT} <= seen
    t.close()


def test_trace_crossing_constraints_uniform(lib):
    """General position: no vertex lies on a segment, so an edge is rejected
    exactly when it properly crosses an accepted constraint."""
    rng = np.random.default_rng(19)
    base = W.uniform(100_000, 4)
    n = len(base)
    with G.Triangulation(lib) as t:
        assert t.execute(base) == Q.QDT_OK
        pre = rng.integers(0, n, size=(40, 2))
        # short constraints between near neighbours of a sorted order
        order = np.argsort(base[:, 0])
        pre = np.stack([order[pre[:, 0] % (n - 3)], order[pre[:, 0] % (n - 3) + 3]], 1)
        st, res = t.insert_constraints_batch(pre)
        acc = pre[res == Q.QDT_OK]
        assert len(acc) > 0
        segs = rng.integers(0, n, size=(300, 2))
        segs = segs[segs[:, 0] != segs[:, 1]]
        st, status, crossed = t.trace_constraints(segs)
        assert st == Q.QDT_OK
        pts = base
        for (a, b), s in zip(segs, status):
            hits = crossings(pts, acc, int(a), int(b)) if len(acc) else 0
            assert s == (Q.QDT_ERR_CROSSES_CONSTRAINT if hits else Q.QDT_OK)
        # crossed counts against brute force on a few segments
        E = undirected_edges(t.triangles_array().astype(np.int64))
        ok = np.nonzero(status == Q.QDT_OK)[0][:6]
        for i in ok:
            assert crossed[i] == crossings(pts, E, int(segs[i, 0]), int(segs[i, 1]))
        # the device copy follows later edits
        t.insert_constraint(int(segs[ok[0], 0]), int(segs[ok[0], 1]))
        st, s2, c2 = t.trace_constraints(segs[ok[:1]])
        assert st == Q.QDT_OK and s2[0] == Q.QDT_OK and c2[0] == 0


def test_trace_edge_cases(lib):
    with G.Triangulation(lib) as t:
        st, s, c = t.trace_constraints(np.array([[0, 1]]))
        assert st == Q.QDT_OK and s[0] == Q.QDT_ERR_INVALID_INDEX
        assert t.execute(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]])) == Q.QDT_OK
        st, s, c = t.trace_constraints(np.array([[0, 2], [0, 0]]))
        assert st == Q.QDT_OK and s.tolist() == [Q.QDT_ERR_NO_TRIANGLES, Q.QDT_ERR_SAME_POINT]
        sq = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0], [1.0, 1.0], [1.0, 1.0]])
        assert t.execute(sq) == Q.QDT_OK
        st, s, c = t.trace_constraints(np.array([[0, 2], [1, 3], [0, 1], [4, 5], [0, 4]]))
        assert st == Q.QDT_OK
        # 0-2 and 1-3 pass through the centre point 4; 0-1 is a hull edge;
        # 4 and 5 are the same point; 0-4 is an edge
        assert s.tolist() == [Q.QDT_ERR_THROUGH_POINT, Q.QDT_ERR_THROUGH_POINT, Q.QDT_OK,
                              Q.QDT_ERR_SAME_POINT, Q.QDT_OK]
        assert c.tolist() == [0, 0, 0, 0, 0]
