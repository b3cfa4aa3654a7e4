"""Batch point location on the GPU and batch insertion that uses it.

qdtg_locate_points extends the reference's single-point locate_
(GuibasStolfiDwyer_Wrapper.cpp:423-486): every query gets the smallest index
of a triangle containing it (border included) and its class. The oracle is a
brute force over all triangles with the oracle's exact orientation
predicate: a point's class is the same in every triangle that contains it,
so the smallest containing triangle and its zero count give the answer.

qdtg_insert_points must give exactly what qdt_insert_point gives called for
each point in order: statuses, indices, points, representatives and the
triangle list in the same order.
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


def brute_locate(pts, tris, q):
    """(tri, where) per query by testing every triangle."""
    pts = np.asarray(pts, dtype=np.float64)
    tris = np.asarray(tris, dtype=np.int64)
    q = np.asarray(q, dtype=np.float64)
    T, K = len(tris), len(q)
    tri = np.full(K, -1, dtype=np.int64)
    where = np.full(K, -1, dtype=np.int32)
    if T == 0 or K == 0:
        return tri, where
    P = np.concatenate([pts, q])
    n = len(pts)
    step = max(1, 400_000 // T)
    for s in range(0, K, step):
        qi = np.arange(s, min(K, s + step)) + n
        kk = len(qi)
        a = np.repeat(tris[:, 0][None, :], kk, 0).ravel()
        b = np.repeat(tris[:, 1][None, :], kk, 0).ravel()
        c = np.repeat(tris[:, 2][None, :], kk, 0).ravel()
        qq = np.repeat(qi, T)
        o = np.stack([D.orient_signs(P, np.stack([a, b, qq], 1)),
                      D.orient_signs(P, np.stack([b, c, qq], 1)),
                      D.orient_signs(P, np.stack([c, a, qq], 1))], 1).reshape(kk, T, 3)
        inside = (o >= 0).all(2)
        has = inside.any(1)
        first = np.argmax(inside, 1)
        for j in range(kk):
            if has[j]:
                tri[s + j] = first[j]
                where[s + j] = int((o[j, first[j]] == 0).sum())
    return tri, where


def state(t):
    n = t.points_size()
    pts = np.array([t.point(i)[1] for i in range(n)]) if n else np.zeros((0, 2))
    return pts, t.triangles_array().astype(np.int64), t.rep_array()


def queries(pts, tris, rng, k_rand=400):
    """Vertices, edge midpoints, centroids, random points and far points."""
    P = np.asarray(pts, dtype=np.float64)
    used = np.unique(tris.ravel())
    qs = [P[used[rng.integers(0, len(used), 60)]]]
    e = tris[rng.integers(0, len(tris), 120)]
    qs.append((P[e[:, 0]] + P[e[:, 1]]) / 2)
    qs.append((P[e[:, 0]] + P[e[:, 1]] + P[e[:, 2]]) / 3)
    lo, hi = P[used].min(0), P[used].max(0)
    span = hi - lo
    qs.append(lo + rng.random((k_rand, 2)) * span)
    qs.append(lo - 0.5 * span + rng.random((80, 2)) * 2.0 * span)
    return np.concatenate(qs)


def check_locate(t, rng, **kw):
    pts, tris, _ = state(t)
    q = queries(pts, tris, rng, **kw)
    st, tri, where = t.locate(q)
    assert st == Q.QDT_OK
    bt, bw = brute_locate(pts, tris, q)
    bad = np.nonzero((tri != bt) | (where != bw))[0]
    assert bad.size == 0, "query %s: got (%d, %d) want (%d, %d)" % (
        q[bad[0]], tri[bad[0]], where[bad[0]], bt[bad[0]], bw[bad[0]])
    return where


@pytest.mark.parametrize("kind", ["integer", "uniform", "clustered", "circle"])
def test_locate_equals_brute_force(lib, kind):
    rng = np.random.default_rng(11)
    if kind == "integer":
        p = rng.integers(0, 40, size=(600, 2)).astype(np.float64)   # duplicates, collinear and cocircular runs
    elif kind == "uniform":
        p = W.uniform(3000, 5)
    elif kind == "clustered":
        p = W.gaussian_mixture(3000, 8, 5)
    else:
        p = W.unit_circle(500, 5)   # all points on the hull: long thin triangles
    with G.Triangulation(lib) as t:
        assert t.execute(p) == Q.QDT_OK
        where = check_locate(t, rng)
        assert {-1, 0, 1, 2} <= set(where.tolist())


@pytest.mark.parametrize("mesh_on_gpu", [True, False])
def test_locate_after_insertions_and_constraints(lib, mesh_on_gpu):
    """The device copy follows the host mesh: after insertions and
    constraints the next location uploads it again."""
    rng = np.random.default_rng(3)
    p = rng.integers(0, 64, size=(800, 2)).astype(np.float64)
    with G.Triangulation(lib) as t:
        t.set_mesh_on_gpu(mesh_on_gpu)
        assert t.execute(p) == Q.QDT_OK
        check_locate(t, rng)
        for x, y in rng.random((30, 2)) * 70 - 3:
            assert t.insert_point(float(x), float(y))[0] == Q.QDT_OK
        check_locate(t, rng)
        n = t.points_size()
        ok = 0
        for a, b in rng.integers(0, n, size=(40, 2)):
            ok += t.insert_constraint(int(a), int(b)) == Q.QDT_OK
        assert ok > 0
        check_locate(t, rng)


def test_locate_edge_cases(lib):
    with G.Triangulation(lib) as t:
        st, tri, where = t.locate(np.array([[0.0, 0.0]]))
        assert st == Q.QDT_OK and tri[0] == -1 and where[0] == -1   # no triangles yet
        assert t.execute(np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]])) == Q.QDT_OK   # collinear: none
        st, tri, where = t.locate(np.array([[1.0, 1.0], [5.0, 0.0]]))
        assert st == Q.QDT_OK and (tri == -1).all() and (where == -1).all()
        assert t.execute(np.array([[0.0, 0.0], [4.0, 0.0], [0.0, 4.0]])) == Q.QDT_OK
        q = np.array([[1.0, 1.0], [2.0, 0.0], [0.0, 0.0], [4.0, 0.0], [3.0, 3.0], [-1e300, 1e300], [2.0, 2.0]])
        st, tri, where = t.locate(q)
        assert st == Q.QDT_OK
        assert tri.tolist() == [0, 0, 0, 0, -1, -1, 0]
        assert where.tolist() == [0, 1, 2, 2, -1, -1, 1]
        st, _, _ = t.locate(np.array([[np.nan, 0.0]]))
        assert st == Q.QDT_ERR_NOT_FINITE
        st, tri, where = t.locate(np.zeros((0, 2)))
        assert st == Q.QDT_OK and tri.size == 0


def insert_cases(rng, base, k):
    lo, hi = base.min(0), base.max(0)
    span = hi - lo
    q = [lo + rng.random((k, 2)) * span]                       # inside
    q.append(base[rng.integers(0, len(base), k // 20 + 1)])    # duplicates of input points
    q.append(lo - 0.3 * span + rng.random((k // 20 + 1, 2)) * 1.6 * span)   # some beyond the hull
    q = np.concatenate(q)
    rng.shuffle(q)
    q[rng.integers(0, len(q), 3)] = np.nan                     # rejected entries
    return q


def sequential(t, q):
    res, idx = [], []
    for x, y in q:
        st, i = t.insert_point(float(x), float(y))
        res.append(st)
        idx.append(i if st == Q.QDT_OK else np.iinfo(np.uint64).max)
    return np.array(res), np.array(idx, dtype=np.uint64)


@pytest.mark.parametrize("n,k", [(2000, 400), (200_000, 4000)])
def test_insert_points_equals_sequential(lib, n, k):
    rng = np.random.default_rng(n)
    base = W.uniform(n, 9)
    q = insert_cases(rng, base, k)
    with G.Triangulation(lib) as a, G.Triangulation(lib) as b:
        assert a.execute(base) == Q.QDT_OK and b.execute(base) == Q.QDT_OK
        # two rounds: the first uses the mirror the mesh build left, the
        # second uploads the changed mesh
        for r in range(2):
            qq = q if r == 0 else insert_cases(rng, base, k // 2)
            ra, ia = sequential(a, qq)
            st, rb, ib = b.insert_points(qq)
            assert st == (Q.QDT_ERR_NOT_FINITE if (ra != 0).any() else Q.QDT_OK)
            np.testing.assert_array_equal(ra, rb)
            np.testing.assert_array_equal(ia, ib)
            pa, ta, repa = state(a)
            pb, tb, repb = state(b)
            np.testing.assert_array_equal(pa, pb)
            np.testing.assert_array_equal(repa, repb)
            np.testing.assert_array_equal(ta, tb)   # same triangles in the same order
        res = D.check(pb, tb, repb)
        assert D.ok(res), res


def test_insert_points_integer_grid_with_constraints(lib):
    """Points on edges and vertices of a mesh with constrained edges (a point
    on a constrained edge splits it)."""
    rng = np.random.default_rng(5)
    base = rng.integers(0, 50, size=(700, 2)).astype(np.float64)
    with G.Triangulation(lib) as a, G.Triangulation(lib) as b:
        for t in (a, b):
            assert t.execute(base) == Q.QDT_OK
        edges = rng.integers(0, len(base), size=(30, 2))
        for t in (a, b):
            st, _ = t.insert_constraints_batch(edges)
        pts, tris, _ = state(a)
        e = tris[rng.integers(0, len(tris), 200)]
        q = np.concatenate([(pts[e[:, 0]] + pts[e[:, 1]]) / 2, pts[e[:, 2]], rng.integers(-5, 55, (200, 2))])
        q = q.astype(np.float64)
        ra, ia = sequential(a, q)
        st, rb, ib = b.insert_points(q)
        np.testing.assert_array_equal(ra, rb)
        np.testing.assert_array_equal(ia, ib)
        for x, y in zip(state(a), state(b)):
            np.testing.assert_array_equal(x, y)


def test_insert_points_on_empty_context_rebuilds(lib):
    with G.Triangulation(lib) as a, G.Triangulation(lib) as b:
        q = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.5, 0.5]])
        ra, ia = sequential(a, q)
        st, rb, ib = b.insert_points(q)
        assert st == Q.QDT_OK
        np.testing.assert_array_equal(ra, rb)
        np.testing.assert_array_equal(ia, ib)
        for x, y in zip(state(a), state(b)):
            np.testing.assert_array_equal(x, y)
