"""The handle operations' host code (insertion and constrained edges,
mesh.cu) on the CPU, without a GPU: each case's starting triangulation is
the oracle's, loaded into a context with qdtg_set_triangulation, and the
reference's own operation sequences (tests/golden/mesh_cases.npz) are
replayed on it. Statuses, returned indices and used flags must equal the
reference's; the final triangle set too where the input is in general
position (the constrained Delaunay triangulation is unique there), and
elsewhere the triangle count and the validity of the constrained Delaunay
result. Integer outputs: exact comparisons.
"""
import os

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from oracle import delaunay_check as D
from oracle import oracle as O
from tests import mesh_check as MC
from tests.golden import cases as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    return G.load()


def loaded(lib, pts):
    """A context holding the oracle's triangulation of pts."""
    r = O.triangulate(pts)
    t = G.Triangulation(lib)
    assert t.set_triangulation(pts, r.tris, r.rep) == Q.QDT_OK
    return t


def test_mesh_cases_equal_reference_on_host(lib):
    d = np.load(os.path.join(GOLDEN, "mesh_cases.npz"))
    for name, pts, ops in C.mesh_cases():
        key = "%s/ser" % name
        with loaded(lib, pts) as t:
            st = MC.run_ops(t, ops)
            assert np.array_equal(st, d[key + "/status"]), (name, st, d[key + "/status"])
            used = np.array([t.point_is_used(i) for i in range(t.points_size())], dtype=np.uint8)
            assert np.array_equal(used, d[key + "/used"]), name
            got = O.canonical(t.triangles_array())
            if MC.general_position_case(name):
                assert np.array_equal(got, d[key + "/tris"]), name
            else:
                assert got.shape == d[key + "/tris"].shape, name
            res = MC.constrained_valid(t, MC.accepted_constraints(ops, st))
            assert D.ok(res), (name, res)


def test_insertions_equal_batch_of_all_points(lib):
    for s in range(4):
        rng = np.random.default_rng(910 + s)
        base = rng.random((int(rng.integers(50, 2000)), 2))
        extra = rng.random((80, 2)) * 1.6 - 0.3          # inside and outside the hull
        with loaded(lib, base) as t:
            for x, y in extra:
                assert t.insert_point(float(x), float(y))[0] == 0
            allp = np.concatenate([base, extra])
            assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(O.triangulate(allp).tris))


def test_constraints_give_the_constrained_delaunay_triangulation(lib):
    """Random long constraints between points in general position: every
    accepted edge present, every other edge locally Delaunay, statuses
    consistent with the geometry (a segment through a point is refused)."""
    for s in range(3):
        rng = np.random.default_rng(930 + s)
        pts = rng.random((1500, 2))
        ops = []
        for _ in range(25):
            a, b = rng.integers(0, pts.shape[0], size=2)
            ops.append(("constraint", int(a), int(b)))
        for _ in range(20):
            ops.append(("insert", float(rng.random()), float(rng.random())))
        with loaded(lib, pts) as t:
            st = MC.run_ops(t, ops)
            cons = MC.accepted_constraints(ops, st)
            assert len(cons) >= 3
            res = MC.constrained_valid(t, cons)
            assert D.ok(res), (s, res)


def test_constraint_statuses_on_a_grid(lib):
    g = np.array([[float(i), float(j)] for i in range(4) for j in range(4)])
    with loaded(lib, g) as t:
        assert t.insert_constraint(0, 15) == Q.QDT_ERR_THROUGH_POINT    # through (1,1) and (2,2)
        assert t.insert_constraint(1, 4) == 0                           # (0,1)-(1,0)
        assert t.insert_constraint(0, 5) == Q.QDT_ERR_CROSSES_CONSTRAINT
        assert t.insert_constraint(3, 3) == Q.QDT_ERR_SAME_POINT
        assert t.insert_constraint(3, 30) == Q.QDT_ERR_INVALID_INDEX
    quad = np.array([[0.0, 0.0], [4.0, 0.0], [3.0, 1.0], [1.0, 1.0]])
    with loaded(lib, quad) as t:
        assert t.insert_constraint(0, 2) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(np.array([[2, 0, 1], [0, 2, 3]])))


def test_insert_on_constrained_edge_splits_it(lib):
    sq = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0], [1.0, 3.0], [1.0, -1.0]])
    with loaded(lib, sq) as t:
        assert t.insert_constraint(0, 2) == 0                 # the diagonal (0,0)-(2,2)
        st, idx = t.insert_point(1.0, 1.0)                    # on it
        assert st == 0 and idx == 6
        res = MC.constrained_valid(t, [(0, 6), (6, 2)])
        assert D.ok(res), res
        # the halves are constrained: a segment across one is refused, one
        # through the new point too
        assert t.insert_constraint(5, 3) == Q.QDT_ERR_CROSSES_CONSTRAINT   # (1,-1)-(0,2) crosses (0,0)-(1,1)
        assert t.insert_constraint(1, 3) == Q.QDT_ERR_THROUGH_POINT        # (2,0)-(0,2) runs through (1,1)


def test_split_constrained_hull_edge_keeps_both_halves(lib):
    """A point on a constrained hull edge splits it into two constrained
    halves; a point added outside then sees both, hidden behind them, and
    a segment from it across either half is refused."""
    sq = np.array([[0.0, 0.0], [4.0, 0.0], [4.0, 4.0], [0.0, 4.0], [2.0, 2.5]])
    with loaded(lib, sq) as t:
        assert t.insert_constraint(0, 1) == 0                      # the bottom hull edge
        assert t.insert_point(2.0, 0.0) == (0, 5)                  # on it
        assert t.insert_point(2.0, -3.0) == (0, 6)                 # below the hull
        res = MC.constrained_valid(t, [(0, 5), (5, 1)])
        assert D.ok(res), res
        assert t.insert_constraint(6, 2) == Q.QDT_ERR_CROSSES_CONSTRAINT   # across (2,0)-(4,0)
        assert t.insert_constraint(6, 3) == Q.QDT_ERR_CROSSES_CONSTRAINT   # across (0,0)-(2,0)
        assert t.insert_constraint(6, 4) == Q.QDT_ERR_THROUGH_POINT        # through (2,0)


def test_constraint_around_a_constrained_antenna(lib):
    """(0, 3.5) has three neighbours, the corners of the triangle around it;
    the segment (-20,4)-(20,4) passes just above it and crosses its whole
    fan. The constrained edge (0,0)-(0,3.5), which it does not cross, stays
    an edge and stays constrained (a segment across it is refused), as in
    the reference."""
    pts = np.array([[0, 0], [-5, 10], [5, 10], [0, 3.5], [-20, 4], [20, 4], [0, -6], [0, 16]], dtype=np.float64)
    with loaded(lib, pts) as t:
        nb = {int(x) for tri in t.triangles_array() for x in tri if 3 in tri} - {3}
        assert nb == {0, 1, 2}
        assert t.insert_constraint(0, 3) == 0
        assert t.insert_constraint(4, 5) == 0
        assert t.insert_point(-1.0, 1.0) == (0, 8)
        assert t.insert_point(1.0, 2.0) == (0, 9)
        assert t.insert_constraint(8, 9) == Q.QDT_ERR_CROSSES_CONSTRAINT
        res = MC.constrained_valid(t, [(0, 3), (4, 5)])
        assert D.ok(res), res


def test_set_triangulation_checks(lib):
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 0.0]])
    with G.Triangulation(lib) as t:
        assert t.set_triangulation(pts, np.array([[0, 1, 2]]), np.array([0, 1, 2, 1])) == Q.QDT_OK
        assert t.triangles_size() == 1 and t.points_size() == 4
        assert t.point_is_used(3) == 0 and t.point_is_used(1) == 1
        assert t.set_triangulation(pts, np.array([[0, 2, 1]]), np.array([0, 1, 2, 1])) == Q.QDT_ERR_INVALID_INDEX
        assert t.triangles_size() == 0 and t.points_size() == 0       # a rejected load empties the context
        assert t.set_triangulation(pts, np.array([[0, 3, 2]]), np.array([0, 1, 2, 1])) == Q.QDT_ERR_INVALID_INDEX
        assert t.set_triangulation(pts, np.array([[0, 1, 2]]), np.array([0, 1, 2, 3])) == Q.QDT_ERR_INVALID_INDEX
        assert t.set_triangulation(pts, np.array([[0, 1, 2], [0, 1, 2]]), np.array([0, 1, 2, 1])) == \
            Q.QDT_ERR_INVALID_INDEX
        bad = pts.copy()
        bad[2, 0] = np.nan
        assert t.set_triangulation(bad, np.array([[0, 1, 2]]), np.array([0, 1, 2, 1])) == Q.QDT_ERR_NOT_FINITE
    # the triangles must cover the convex hull of the distinct points once
    sq = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 2.0], [0.0, 2.0], [1.0, 1.0]])
    fan = np.array([[0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4]])
    with G.Triangulation(lib) as t:
        assert t.set_triangulation(sq, fan) == Q.QDT_OK
        assert t.set_triangulation(sq, fan[:3]) == Q.QDT_ERR_INVALID_INDEX         # a reflex corner at (1,1)
        assert t.set_triangulation(sq, fan[[0, 2]]) == Q.QDT_ERR_INVALID_INDEX     # two pieces
        assert t.set_triangulation(sq, np.array([[0, 1, 2], [0, 2, 3]])) == Q.QDT_ERR_INVALID_INDEX   # (1,1) unused
        ring = np.array([[0.0, 0.0], [6.0, 0.0], [6.0, 6.0], [0.0, 6.0], [2.0, 2.0], [4.0, 2.0], [4.0, 4.0],
                         [2.0, 4.0]])
        holed = np.array([[0, 1, 5], [0, 5, 4], [1, 2, 6], [1, 6, 5], [2, 3, 7], [2, 7, 6], [3, 0, 4], [3, 4, 7]])
        assert t.set_triangulation(ring, holed) == Q.QDT_ERR_INVALID_INDEX        # a hole in the middle
        assert t.set_triangulation(ring, np.concatenate([holed, [[4, 5, 6], [4, 6, 7]]])) == Q.QDT_OK


@pytest.mark.parametrize("seed", range(4))
def test_batch_insertion_equals_sequential_on_host(lib, seed):
    """qdtg_insert_points without a GPU (each walk starts from the host's own
    seeds instead of a device location) gives what qdt_insert_point gives
    point by point: statuses, indices, triangles and representatives."""
    rng = np.random.default_rng(60 + seed)
    if seed % 2:
        pts = rng.integers(0, 20, size=(300, 2)).astype(np.float64)
        q = rng.integers(-2, 22, size=(200, 2)) + 0.5 * rng.integers(0, 2, size=(200, 2))
    else:
        pts = rng.random((400, 2))
        q = rng.random((200, 2)) * 1.3 - 0.15
    with loaded(lib, pts) as a, loaded(lib, pts) as b:
        st, res, idx = a.insert_points(q)
        assert st == Q.QDT_OK
        seq = [b.insert_point(float(x), float(y)) for x, y in q]
        assert [int(v) for v in res] == [s for s, _ in seq]
        assert [int(v) for v in idx] == [i for _, i in seq]
        assert np.array_equal(O.canonical(a.triangles_array()), O.canonical(b.triangles_array()))
        assert np.array_equal(a.rep_array(), b.rep_array())
