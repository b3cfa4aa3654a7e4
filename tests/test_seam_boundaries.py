"""The geometric facts the split merges' seam segments rest on
(libqdt_gb300/csrc/seam_split.cuh, "segment boundaries"), checked on the
CPU against an independent Delaunay triangulation (scipy's Qhull) of points
in general position, where the triangulation is unique:

* a pair (l, r) of mutually nearest vertices across the cut (l the unique
  left vertex nearest to r, r the unique right vertex nearest to l) is an
  edge of the merged triangulation;
* steepest descent over a half's own triangulation reaches the vertex of
  that half nearest to a point (what seam_nearest does);
* the edges of a half's triangulation that cross lr are exactly the ones the
  merge deletes there (none of them is an edge of the merged triangulation),
  and the walk from l towards r across the half's faces (seam_crossed) meets
  each of them.

These are properties of the algorithm, restated here in numpy; the CUDA
code that implements them is checked on the GPU against the reference
(tests/test_gpu_parity.py::test_split_segments_same_result).
"""
import numpy as np
import pytest

spatial = pytest.importorskip("scipy.spatial")


def edges_of(tri):
    e = set()
    for a, b, c in tri.simplices:
        for u, v in ((a, b), (b, c), (c, a)):
            e.add((min(u, v), max(u, v)))
    return e


def neighbours(tri):
    nb = {}
    for u, v in edges_of(tri):
        nb.setdefault(u, set()).add(v)
        nb.setdefault(v, set()).add(u)
    return nb


def nearest_by_descent(pts, nb, start, t):
    v = start
    for _ in range(len(pts)):
        best = min(nb[v], key=lambda u: np.sum((pts[u] - t) ** 2))
        if np.sum((pts[best] - t) ** 2) < np.sum((pts[v] - t) ** 2):
            v = best
        else:
            return v
    raise AssertionError("descent did not settle")


def segments_cross(p1, p2, q1, q2):
    def o(a, b, c):
        return np.sign((b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0]))
    return o(p1, p2, q1) * o(p1, p2, q2) < 0 and o(q1, q2, p1) * o(q1, q2, p2) < 0


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mutual_nearest_pairs_are_seam_edges(seed):
    rng = np.random.default_rng(seed)
    pts = rng.random((3000, 2))
    left = np.flatnonzero(pts[:, 0] < 0.5)
    right = np.flatnonzero(pts[:, 0] >= 0.5)
    full = edges_of(spatial.Delaunay(pts))
    tl, tr = spatial.Delaunay(pts[left]), spatial.Delaunay(pts[right])
    nbl, nbr = neighbours(tl), neighbours(tr)
    el, er = edges_of(tl), edges_of(tr)
    pl, pr = pts[left], pts[right]
    found = 0
    for y in np.linspace(0.1, 0.9, 9):
        # start vertices: the ones nearest to the cut near height y
        sl = int(np.argmin(np.abs(pl[:, 0] - 0.5) + 4 * np.abs(pl[:, 1] - y)))
        sr = int(np.argmin(np.abs(pr[:, 0] - 0.5) + 4 * np.abs(pr[:, 1] - y)))
        l, r = sl, sr
        for _ in range(12):
            l = nearest_by_descent(pl, nbl, l, pr[r])
            assert l == int(np.argmin(np.sum((pl - pr[r]) ** 2, axis=1)))   # descent finds the nearest
            r2 = nearest_by_descent(pr, nbr, r, pl[l])
            assert r2 == int(np.argmin(np.sum((pr - pl[l]) ** 2, axis=1)))
            if r2 == r:
                break
            r = r2
        else:
            continue
        found += 1
        gl, gr = int(left[l]), int(right[r])
        # the boundary is an edge of the merged triangulation
        assert (min(gl, gr), max(gl, gr)) in full
        # the halves' edges it crosses are all deleted by the merge
        for (u, v) in el:
            if segments_cross(pl[u], pl[v], pl[l], pr[r]):
                gu, gv = int(left[u]), int(left[v])
                assert (min(gu, gv), max(gu, gv)) not in full
        for (u, v) in er:
            if segments_cross(pr[u], pr[v], pl[l], pr[r]):
                gu, gv = int(right[u]), int(right[v])
                assert (min(gu, gv), max(gu, gv)) not in full
    assert found >= 6


def test_face_walk_meets_every_crossed_edge():
    """Walking from l towards r over the left half's triangles (the face
    across each crossed edge, then out through the edge the segment leaves
    by) meets exactly the left edges the segment crosses."""
    rng = np.random.default_rng(7)
    pts = rng.random((2000, 2))
    left = pts[pts[:, 0] < 0.5]
    right = pts[pts[:, 0] >= 0.5]
    tl = spatial.Delaunay(left)
    el = edges_of(tl)
    tri_of_edge = {}
    for t in tl.simplices:
        for u, v in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
            tri_of_edge.setdefault((min(u, v), max(u, v)), []).append(tuple(t))
    for trial in range(20):
        l = int(rng.integers(0, left.shape[0]))
        r = int(rng.integers(0, right.shape[0]))
        a, b = left[l], right[r]
        want = {e for e in el if l not in e and segments_cross(left[e[0]], left[e[1]], a, b)}
        # the walk: the triangle at l that the segment enters, then across
        got = set()
        start = None
        for t in tl.simplices:
            if l in t:
                u, v = [x for x in t if x != l]
                if segments_cross(left[u], left[v], a, b):
                    start = (min(u, v), max(u, v))
                    prev = tuple(t)
                    break
        e = start
        steps = 0
        while e is not None:
            steps += 1
            assert steps <= len(el), "the walk revisits an edge"
            got.add(e)
            nxt = None
            across = [t for t in tri_of_edge[e] if t != prev]
            if across:   # no face across a hull edge: the segment leaves the half
                t = across[0]
                c = [x for x in t if x not in e][0]
                for f in ((min(e[0], c), max(e[0], c)), (min(e[1], c), max(e[1], c))):
                    if segments_cross(left[f[0]], left[f[1]], a, b):
                        nxt = f
                prev = t
            e = nxt
        assert got == want, trial
