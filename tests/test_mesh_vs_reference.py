"""The handle operations' host code (mesh.cu) against the reference library
itself, on operation sequences that are not in the committed fixtures.

Where the reference was compiled from its own sources into oracle/_ref, each
case triangulates fresh seeded points in both libraries (ours is loaded with
the oracle's triangulation through qdtg_set_triangulation, so no GPU is
needed), applies the same insertions and constraints in the same order,
then one qdt_insert_constraints_batch call. Inputs: uniform points; integer
points with duplicates and insertions on vertices, edges and outside the
hull; a few integer points with insertions at midpoints; coordinates from
2^-100 to 2^100. Required: equal statuses, returned indices, used flags
and triangle counts; equal triangle sets where the input is in general
position (the constrained Delaunay triangulation is unique there); and
everywhere a valid constrained Delaunay triangulation that holds every
accepted constraint (as the pieces later insertions on it split it into).
Skipped where the reference is not compiled.
"""
import os

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from oracle import delaunay_check as D
from oracle import oracle as O
from tests import mesh_check as MC

pytestmark = pytest.mark.skipif(
    not (O.reference_available() and os.path.exists(os.path.join(O.REF_DIR, "libqdt_dump_ref.so"))),
    reason="the reference is not compiled here (oracle/_ref)")


@pytest.fixture(scope="module")
def libs():
    from tests.golden import make_golden as M
    return G.load(), Q.load(O.REF_LIB_PATH), M.load_dump()


def _case(seed):
    """(points, ops, general position) for one seed."""
    rng = np.random.default_rng(seed)
    kind = seed % 6
    n = int(rng.integers(3, 400))
    ops = []
    if kind == 5:      # coordinates from 2^-100 to 2^100 in one set, insertions alike
        def draw(k):
            return (rng.random((k, 2)) * 2 - 1) * np.ldexp(1.0, rng.integers(-100, 100, size=(k, 2)))
        p = draw(n)
        for _ in range(int(rng.integers(1, 60))):
            if rng.random() < 0.6:
                q = draw(1)[0]
                ops.append(("insert", float(q[0]), float(q[1])))
            else:
                ops.append(("constraint", int(rng.integers(0, n + 3)), int(rng.integers(0, n + 3))))
        return p, ops, True
    if kind == 4:      # a few integer points; insertions at midpoints of point pairs, repeats, far points
        p = rng.integers(0, int(rng.integers(2, 17)), size=(int(rng.integers(3, 12)), 2)).astype(np.float64)
        allp = [tuple(x) for x in p]
        for _ in range(int(rng.integers(1, 200))):
            r = rng.random()
            if r < 0.45:
                if r < 0.3:
                    a, b = allp[int(rng.integers(0, len(allp)))], allp[int(rng.integers(0, len(allp)))]
                    q = ((a[0] + b[0]) / 2, (a[1] + b[1]) / 2)
                elif r < 0.37:
                    q = tuple(float(v) for v in rng.integers(-50, 50, size=2))
                else:
                    q = allp[int(rng.integers(0, len(allp)))]
                ops.append(("insert", float(q[0]), float(q[1])))
                allp.append(q)
            else:
                ops.append(("constraint", int(rng.integers(0, len(allp))), int(rng.integers(0, len(allp)))))
        return p, ops, False
    if kind == 0:      # uniform doubles, insertions inside and around the hull
        p = rng.random((n, 2))
        for _ in range(int(rng.integers(1, 60))):
            if rng.random() < 0.6:
                ops.append(("insert", float(rng.random() * 1.4 - 0.2), float(rng.random() * 1.4 - 0.2)))
            else:
                ops.append(("constraint", int(rng.integers(0, n + 3)), int(rng.integers(0, n + 3))))
        return p, ops, True
    # integer points: duplicates, insertions on vertices, edges and outside
    R = int(rng.choice([4, 10, 40]))
    p = rng.integers(0, R, size=(n, 2)).astype(np.float64)
    for _ in range(int(rng.integers(1, 60))):
        r = rng.random()
        if r < 0.2:
            q = p[int(rng.integers(0, n))]
            ops.append(("insert", float(q[0]), float(q[1])))
        elif r < 0.5:
            q = rng.integers(-2, R + 2, size=2) + (0.5 if kind == 2 else 0.0) * rng.integers(0, 2, size=2)
            ops.append(("insert", float(q[0]), float(q[1])))
        else:
            ops.append(("constraint", int(rng.integers(0, n + 3)), int(rng.integers(0, n + 3))))
    return p, ops, False


def _split_constraints(t, cons):
    """The accepted constraints as the edges they consist of now: a point
    inserted later on a constrained edge splits it. For the integer cases
    (coordinates below 64 in magnitude on a grid of 2^-20: scaled by 2^20
    they are exact integers, and the products below fit in 64 bits)."""
    rep = t.rep_array()
    P = np.array([t.point(i)[1] for i in range(t.points_size())])
    Q2 = np.rint(P * (1 << 20)).astype(np.int64)
    assert np.array_equal(Q2, P * (1 << 20)) and np.abs(P).max() < 64
    V = np.unique(rep)
    out = []
    for a, b in cons:
        a, b = int(rep[a]), int(rep[b])
        d = Q2[b] - Q2[a]
        r = Q2[V] - Q2[a]
        s = r[:, 0] * d[0] + r[:, 1] * d[1]
        on = (d[0] * r[:, 1] - d[1] * r[:, 0] == 0) & (s > 0) & (s < d[0] * d[0] + d[1] * d[1])
        chain = [a] + [int(v) for v in V[on][np.argsort(s[on])]] + [b]
        out += list(zip(chain[:-1], chain[1:]))
    return out


def _batch_edges(seed, m):
    """The qdt_insert_constraints_batch call that ends a sequence: random
    end points among the m points (some invalid, some equal)."""
    rng = np.random.default_rng(seed + 7)
    return rng.integers(0, m + 2, size=(int(rng.integers(0, 30)), 2))


def _apply(c, ops, par, edges):
    """The operations, then one batch of constraints: every status as one
    array (the batch's return value, then its per-edge results)."""
    st = MC.run_ops(c, ops, par)
    bst, bres = c.insert_constraints_batch(edges)
    return st, np.concatenate([[bst], bres]).astype(np.int64)


def _reference(lib, dump, pts, ops, par, edges):
    with Q.Context(lib) as c:
        assert c.execute(pts, parallel=par) == 0
        st = _apply(c, ops, par, edges)
        tris = np.zeros((c.triangles_size(), 3), dtype=np.int64)
        dump.qdt_dump_triangles(c.ptr, tris.ctypes.data)
        used = np.zeros(c.points_size(), dtype=np.uint8)
        dump.qdt_dump_used(c.ptr, used.ctypes.data)
    return st, O.canonical(tris), used


@pytest.mark.parametrize("block", range(4))
def test_mesh_operations_equal_reference_on_fresh_sequences(libs, block):
    ours, ref, dump = libs
    checked = 0
    for seed in range(880000 + 500 * block, 880000 + 500 * (block + 1)):
        pts, ops, general = _case(seed)
        r = O.triangulate(pts)
        if r.tris.shape[0] == 0:
            continue   # collinear points: an insertion re-runs the batch call, on the GPU
        par = bool(seed & 1)
        edges = _batch_edges(seed, pts.shape[0] + len(ops))
        (want_st, want_bst), want_tris, want_used = _reference(ref, dump, pts, ops, par, edges)
        with G.Triangulation(ours) as t:
            assert t.set_triangulation(pts, r.tris, r.rep) == Q.QDT_OK
            st, bst = _apply(t, ops, par, edges)
            assert np.array_equal(st, want_st), (seed, st, want_st)
            assert np.array_equal(bst, want_bst), (seed, bst, want_bst)
            used = np.array([t.point_is_used(i) for i in range(t.points_size())], dtype=np.uint8)
            assert np.array_equal(used, want_used), seed
            got = O.canonical(t.triangles_array())
            assert got.shape == want_tris.shape, seed
            if general:
                assert np.array_equal(got, want_tris), seed
            cons = MC.accepted_constraints(ops, st)
            cons += [(int(a), int(b)) for (a, b), s in zip(edges, bst[1:]) if s == 0]
            res = MC.constrained_valid(t, cons if general else _split_constraints(t, cons))
            assert D.ok(res), (seed, res)
        checked += 1
    assert checked > 450
