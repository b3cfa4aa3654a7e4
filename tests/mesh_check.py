"""Shared checks of the handle operations (insertion, constraints) for the
GPU tests and the CPU tests of the host mesh code. TEST INFRASTRUCTURE."""
import numpy as np

from oracle import delaunay_check as D


def run_ops(t, ops, par=False):
    """Applies ("insert", x, y) / ("constraint", i, j) operations in order;
    returns every status (and inserted index) as one array."""
    statuses = []
    for op in ops:
        if op[0] == "insert":
            st, idx = t.insert_point(op[1], op[2], parallel=par)
            statuses += [st, idx]
        else:
            statuses.append(t.insert_constraint(op[1], op[2]))
    return np.array(statuses, dtype=np.int64)


def constraint_statuses(ops, st):
    out, i = [], 0
    for op in ops:
        if op[0] == "insert":
            i += 2
        else:
            out.append(int(st[i]))
            i += 1
    return out


def accepted_constraints(ops, st):
    cons_ops = [o for o in ops if o[0] == "constraint"]
    return [(op[1], op[2]) for op, s in zip(cons_ops, constraint_statuses(ops, st)) if s == 0]


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
        res["not_delaunay"] = int(np.sum(D.incircle_signs(pts, np.array(quads)) > 0)) if quads else 0
    return res


def general_position_case(name):
    """Mesh fixtures whose inputs are in general position: there the
    constrained Delaunay triangulation is unique and the triangle sets must
    equal the reference's."""
    return name.startswith(("six_point", "quad", "long_uniform")) or (
        name.startswith("mixed_") and int(name.split("_")[1]) % 3 == 0)
