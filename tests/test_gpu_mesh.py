"""Incremental insertion and constrained edges on the handle the GPU batch
path returns (the calls qdt.h keeps on the same context).

The fixtures (tests/golden/mesh_cases.npz) are the reference library's own
results for the same call sequences: every status, every returned index, the
final canonical triangle set and the used-point flags. Where the input is in
general position the constrained Delaunay triangulation is unique, so the
triangle sets must be identical; on integer inputs with cocircular points the
reference documents that equally valid results may differ, so there the
statuses, the point bookkeeping and the validity of the result are checked.
"""
import os

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from libqdt_gb300 import workloads as W
from oracle import delaunay_check as D
from oracle import oracle as O
from tests.golden import cases as C

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def lib():
    return G.load()


def run_ops(lib, pts, ops, par):
    t = G.Triangulation(lib)
    assert t.execute(pts, parallel=par) == 0
    statuses = []
    for op in ops:
        if op[0] == "insert":
            st, idx = t.insert_point(op[1], op[2], parallel=par)
            statuses += [st, idx]
        else:
            statuses.append(t.insert_constraint(op[1], op[2]))
    return t, np.array(statuses, dtype=np.int64)


def constrained_valid(t, cons):
    """Triangulation valid; every accepted constraint present; every other
    interior edge locally Delaunay."""
    n = t.points_size()
    pts = np.array([t.point(i)[1] for i in range(n)])
    tris = t.triangles_array().astype(np.int64)
    rep = t.rep_array()
    res = D.check(pts, tris, rep)
    E = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    und = {(min(a, b), max(a, b)) for a, b in E}
    for a, b in cons:
        a, b = int(rep[a]), int(rep[b])
        assert (min(a, b), max(a, b)) in und, "constraint %d-%d missing" % (a, b)
    if res["not_delaunay"]:
        # allowed only on constrained edges: recount without them
        opp = np.concatenate([tris[:, 2], tris[:, 0], tris[:, 1]])
        key = {(int(a), int(b)): int(o) for (a, b), o in zip(E, opp)}
        consset = {(min(int(rep[a]), int(rep[b])), max(int(rep[a]), int(rep[b]))) for a, b in cons}
        quads = []
        for (a, b), o in key.items():
            if a < b and (b, a) in key and (a, b) not in consset:
                quads.append((a, b, o, key[(b, a)]))
        if quads:
            bad = int(np.sum(D.incircle_signs(pts, np.array(quads)) > 0))
        else:
            bad = 0
        res["not_delaunay"] = bad
    return res


def test_mesh_cases_equal_reference(lib):
    d = np.load(os.path.join(GOLDEN, "mesh_cases.npz"))
    for name, pts, ops in C.mesh_cases():
        general = name.startswith(("six_point", "quad", "long_uniform")) or (name.startswith("mixed_") and
                                                            int(name.split("_")[1]) % 3 == 0)
        for par in (False, True):
            key = "%s/%s" % (name, "par" if par else "ser")
            t, st = run_ops(lib, pts, ops, par)
            with t:
                assert np.array_equal(st, d[key + "/status"]), (name, st, d[key + "/status"])
                used = np.array([t.point_is_used(i) for i in range(t.points_size())], dtype=np.uint8)
                assert np.array_equal(used, d[key + "/used"]), name
                got = O.canonical(t.triangles_array())
                if general:
                    assert np.array_equal(got, d[key + "/tris"]), name
                else:
                    assert got.shape == d[key + "/tris"].shape, name
                cons = [(op[1], op[2]) for op, s in zip([o for o in ops if o[0] == "constraint"],
                                                        [x for x in _constraint_statuses(ops, st)]) if s == 0]
                res = constrained_valid(t, cons)
                assert D.ok(res), (name, res)


def _constraint_statuses(ops, st):
    out, i = [], 0
    for op in ops:
        if op[0] == "insert":
            i += 2
        else:
            out.append(int(st[i]))
            i += 1
    return out


def test_readme_listings(lib):
    # six-point example (README "Example"), quad before/after the constraint
    listing = {(1, 3, 4), (0, 1, 4), (2, 0, 5), (0, 4, 5), (4, 3, 5), (3, 2, 5)}
    sq = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]])
    with G.Triangulation(lib) as t:
        assert t.execute(sq) == 0
        assert t.insert_point(0.5, 0.5) == (0, 4)
        assert t.insert_point(0.25, 0.75) == (0, 5)
        assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(np.array(sorted(listing))))
    quad = np.array([[0.0, 0.0], [4.0, 0.0], [3.0, 1.0], [1.0, 1.0]])
    with G.Triangulation(lib) as t:
        assert t.execute(quad) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(np.array([[3, 0, 1], [1, 2, 3]])))
        assert t.insert_constraint(0, 2) == 0
        assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(np.array([[2, 0, 1], [0, 2, 3]])))
        assert t.insert_constraint(0, 9) == Q.QDT_ERR_INVALID_INDEX


def test_insertions_match_batch(lib):
    # in general position the triangulation after insertions is the batch
    # triangulation of all points
    for s in range(4):
        rng = np.random.default_rng(900 + s)
        base = rng.random((int(rng.integers(50, 3000)), 2))
        extra = rng.random((60, 2)) * 1.6 - 0.3
        with G.Triangulation(lib) as t:
            assert t.execute(base) == 0
            for x, y in extra:
                st, idx = t.insert_point(float(x), float(y), parallel=bool(s & 1))
                assert st == 0
            allp = np.concatenate([base, extra])
            assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(O.triangulate(allp).tris))


def test_constraint_errors(lib):
    line = np.array([[float(i), 0.0] for i in range(10)])
    with G.Triangulation(lib) as t:
        assert t.execute(line) == 0
        assert t.insert_constraint(0, 5) == Q.QDT_ERR_NO_TRIANGLES
        assert t.insert_constraint(3, 3) == Q.QDT_ERR_SAME_POINT
        assert t.insert_constraint(3, 30) == Q.QDT_ERR_INVALID_INDEX
    g = np.array([[float(i), float(j)] for i in range(4) for j in range(4)])
    with G.Triangulation(lib) as t:
        assert t.execute(g) == 0
        # (0,0)-(3,3) passes through (1,1) and (2,2)
        assert t.insert_constraint(0, 15) == Q.QDT_ERR_THROUGH_POINT
        assert t.insert_constraint(1, 4) == 0          # (0,1)-(1,0)
        assert t.insert_constraint(0, 5) == Q.QDT_ERR_CROSSES_CONSTRAINT   # (0,0)-(1,1) crosses it
        st, res = t.insert_constraints_batch(np.array([[3, 6], [0, 5], [3, 3]]))
        assert list(res) == [0, Q.QDT_ERR_CROSSES_CONSTRAINT, Q.QDT_ERR_SAME_POINT]
        assert st == Q.QDT_ERR_CROSSES_CONSTRAINT


def test_insert_into_empty_and_duplicates(lib):
    with G.Triangulation(lib) as t:
        assert t.execute(np.zeros((0, 2))) == 0
        assert t.insert_point(0.0, 0.0) == (0, 0)
        assert t.insert_point(1.0, 0.0) == (0, 1)
        assert t.triangles_size() == 0
        assert t.insert_point(0.0, 1.0) == (0, 2)
        assert t.triangles_size() == 1
        assert t.insert_point(1.0, 0.0) == (0, 3)    # duplicate
        assert t.point_is_used(3) == 0 and t.point_is_used(1) == 1
        assert t.triangles_size() == 1
        p = W.uniform(100, 5)
        for x, y in p:
            assert t.insert_point(float(x), float(y))[0] == 0
        allp = np.concatenate([[[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 0.0]], p])
        assert np.array_equal(O.canonical(t.triangles_array()), O.canonical(O.triangulate(allp).tris))


def _ops_sequence(pts, seed):
    """Insertions (inside, on an existing point, outside the hull, on a
    lattice line) and constraints between existing points."""
    rng = np.random.default_rng(seed)
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    ops = []
    for k in range(40):
        r = rng.random()
        if r < 0.5:
            x, y = lo + (hi - lo) * rng.random(2)
            ops.append(("insert", float(x), float(y)))
        elif r < 0.6:
            x, y = pts[int(rng.integers(0, len(pts)))]
            ops.append(("insert", float(x), float(y)))
        elif r < 0.7:
            x, y = lo - 0.2 * (hi - lo) + 1.4 * (hi - lo) * rng.random(2)
            ops.append(("insert", float(x), float(y)))
        else:
            a, b = rng.integers(0, len(pts), size=2)
            ops.append(("constraint", int(a), int(b)))
    return ops


def test_mesh_built_on_gpu_equals_host(lib):
    """The first insertion or constraint builds the half-edge mesh on the GPU
    (k_mesh.cu) or on the host; the two meshes are the same arrays, so every
    status and the triangle list itself (order included) must agree after a
    sequence of operations."""
    inputs = [W.uniform(20000, 41), W.lattice_with_duplicates(48, 0.05, 42), W.unit_circle(500, 43),
              np.concatenate([W.uniform(3000, 44), W.uniform(3000, 44)[:500]]), W.uniform(5, 45)]
    for i, pts in enumerate(inputs):
        ops = _ops_sequence(pts, 500 + i)
        results = []
        for on_gpu in (1, 0):
            with G.Triangulation(lib) as t:
                assert t.set_mesh_on_gpu(on_gpu)
                assert t.execute(pts) == 0
                sts = []
                for op in ops:
                    if op[0] == "insert":
                        sts.append(t.insert_point(op[1], op[2]))
                    else:
                        sts.append(t.insert_constraint(op[1], op[2]))
                results.append((sts, t.triangles_array().copy(), t.points_size()))
        assert results[0][0] == results[1][0], i
        assert results[0][2] == results[1][2], i
        assert np.array_equal(results[0][1], results[1][1]), i


# Small edits around constrained hull edges and enclosed fans, after a batch
# call on the GPU: the statuses (and triangle counts) the reference library
# returns for the same calls, serial and parallel alike.
_EDIT_CASES = [
    # a point on a constrained hull edge splits it; a point below sees both halves
    ("split_hull", [[0, 0], [4, 0], [4, 4], [0, 4], [2, 2.5]],
     [("constraint", 0, 1), ("insert", 2.0, 0.0), ("insert", 2.0, -3.0), ("constraint", 6, 2),
      ("constraint", 6, 3), ("constraint", 6, 4)], [0, 0, 5, 0, 6, -8, -8, -9], 7),
    # a segment crossing the whole fan of (0, 3.5) keeps the constrained edge to (0, 0)
    ("antenna", [[0, 0], [-5, 10], [5, 10], [0, 3.5], [-20, 4], [20, 4], [0, -6], [0, 16]],
     [("constraint", 0, 3), ("constraint", 4, 5), ("insert", -1.0, 1.0), ("insert", 1.0, 2.0),
      ("constraint", 8, 9)], [0, 0, 0, 8, 0, 9, -8], 14),
    # a point outside the hull, then a constraint from the end of the open border
    ("open_border", [[3, 8], [5, 3], [1, 1], [6, 9], [8, 1], [7, 2], [3, 8], [8, 0]],
     [("insert", 0.0, 6.0), ("constraint", 6, 5)], [0, 8, 0], 8),
    # a constrained hull edge hides the triangle behind it from a point outside
    ("hidden_hull", [[0, 0], [4, 0], [4, 4], [0, 4], [2, 1]],
     [("constraint", 0, 1), ("insert", 2.0, -1.0), ("constraint", 5, 4), ("constraint", 5, 2)],
     [0, 0, 5, -8, -8], 5),
]


@pytest.mark.parametrize("case", _EDIT_CASES, ids=[c[0] for c in _EDIT_CASES])
def test_edits_at_constrained_hull_edges(lib, case):
    name, pts, ops, want, ntri = case
    for par in (False, True):
        t, st = run_ops(lib, np.array(pts, dtype=np.float64), ops, par)
        with t:
            assert st.tolist() == want, (name, par, st)
            assert t.triangles_size() == ntri, name
