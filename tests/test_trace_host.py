"""The constraint trace and the point location of the GPU path
(mesh_walk.cuh: trace_segment, which the kernel k_mesh_trace runs for
qdtg_trace_constraints; walk and classify, which k_mesh_locate runs for
qdtg_locate_points) run on the CPU: the harness tests/mesh_trace_check.cu is
compiled with nvcc as a host program from the same source. On
triangulations edited by insertions and constraints through the library
(loaded with the oracle's triangulation, no GPU needed), every traced status must equal what qdt_insert_constraint
returns for the same segment on the same state, and for a segment that is
accepted, the count of crossed edges must equal the edges of the
triangulation the open segment crosses (counted with the oracle's exact
orientation). Points located from random start half-edges (at vertices, on
edges, inside, outside the hull) must get the brute-force answer: the
smallest triangle that holds the point, border included, and whether it
lies inside, on an edge or on a vertex. The GPU tests compare the kernels
with the same calls on the device (tests/test_gpu_trace.py,
tests/test_gpu_locate.py)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import libqdt_gb300 as G
from libqdt_gb300 import qdt_api as Q
from oracle import oracle as O
from tests import mesh_check as MC

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "libqdt_gb300", "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
STATUS = {0: Q.QDT_OK, 1: Q.QDT_ERR_THROUGH_POINT, 2: Q.QDT_ERR_CROSSES_CONSTRAINT}


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if not nvcc:
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("trace") / "mesh_trace_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, "-I", INCLUDE,
                        os.path.join(HERE, "mesh_trace_check.cu"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _case(seed):
    rng = np.random.default_rng(seed)
    if seed % 2 == 0:      # uniform doubles: no insertion lands on an edge
        p = rng.random((int(rng.integers(20, 300)), 2))
        ops = []
        for _ in range(int(rng.integers(5, 40))):
            if rng.random() < 0.5:
                ops.append(("insert", float(rng.random() * 1.4 - 0.2), float(rng.random() * 1.4 - 0.2)))
            else:
                ops.append(("constraint", int(rng.integers(0, len(p))), int(rng.integers(0, len(p)))))
        return p, ops
    R = int(rng.choice([5, 12, 30]))   # integer points: through-points and collinear constraints
    p = rng.integers(0, R, size=(int(rng.integers(20, 300)), 2)).astype(np.float64)
    ops = []
    for _ in range(int(rng.integers(5, 40))):
        if rng.random() < 0.3:
            q = rng.integers(-2, R + 2, size=2) + 0.5 * rng.integers(0, 2, size=2)
            ops.append(("insert", float(q[0]), float(q[1])))
        else:
            ops.append(("constraint", int(rng.integers(0, len(p))), int(rng.integers(0, len(p)))))
    return p, ops


def _state(lib, pts, ops, r):
    t = G.Triangulation(lib)
    assert t.set_triangulation(pts, r.tris, r.rep) == Q.QDT_OK
    st = MC.run_ops(t, ops)
    return t, st


def _constrained_edges(t, ops, st):
    """The accepted constraints as edges now: the pieces a later insertion
    on a constrained edge split it into (exact on a half-integer grid; the
    uniform doubles put no point on an edge)."""
    rep = t.rep_array()
    P = np.array([t.point(i)[1] for i in range(t.points_size())])
    V = np.unique(rep)
    out = []
    for a, b in MC.accepted_constraints(ops, st):
        a, b = int(rep[a]), int(rep[b])
        chain = [a]
        if np.array_equal(np.rint(2 * P), 2 * P):
            Q2 = np.rint(2 * P).astype(np.int64)
            d, r_ = Q2[b] - Q2[a], Q2[V] - Q2[a]
            s = r_ @ d
            on = (d[0] * r_[:, 1] - d[1] * r_[:, 0] == 0) & (s > 0) & (s < d @ d)
            chain += [int(v) for v in V[on][np.argsort(s[on])]]
        chain.append(b)
        out += list(zip(chain[:-1], chain[1:]))
    return out


def _crossed_edges(P, tris, u, w):
    """Edges of the triangulation the open segment u-w crosses properly."""
    E = {(min(a, b), max(a, b)) for t in tris for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0]))}
    lo, hi = np.minimum(P[u], P[w]), np.maximum(P[u], P[w])
    n = 0
    for a, b in E:
        if a in (u, w) or b in (u, w):
            continue
        if max(P[a][0], P[b][0]) < lo[0] or min(P[a][0], P[b][0]) > hi[0] or \
                max(P[a][1], P[b][1]) < lo[1] or min(P[a][1], P[b][1]) > hi[1]:
            continue
        if O.orient2d(P[u], P[w], P[a]) * O.orient2d(P[u], P[w], P[b]) < 0 and \
                O.orient2d(P[a], P[b], P[u]) * O.orient2d(P[a], P[b], P[w]) < 0:
            n += 1
    return n


def _locate_brute(P, tris, x):
    """(smallest triangle holding x, border included; 0 inside, 1 on an
    edge, 2 on a vertex), or (-1, -1) outside the hull."""
    for k, t3 in enumerate(tris):
        o = [O.orient2d(P[t3[i]], P[t3[(i + 1) % 3]], x) for i in range(3)]
        if min(o) >= 0:
            return k, 3 - sum(1 for s in o if s != 0)
    return -1, -1


@pytest.mark.parametrize("seed", range(12))
def test_trace_and_locate_on_the_cpu(harness, tmp_path, seed):
    lib = G.load()
    pts, ops = _case(seed)
    r = O.triangulate(pts)
    if r.tris.shape[0] == 0:
        pytest.skip("collinear input")
    t, st = _state(lib, pts, ops, r)
    with t:
        rep = t.rep_array()
        P = np.array([t.point(i)[1] for i in range(t.points_size())])
        tris = t.triangles_array().astype(np.int64)
        cons = _constrained_edges(t, ops, st)
    used = np.unique(rep)
    rng = np.random.default_rng(1000 + seed)
    qs = []
    while len(qs) < 60:
        u, w = (int(x) for x in rng.choice(used, size=2))
        if u != w:
            qs.append((u, w))
    # points to locate: vertices, edge midpoints, random points in and around the hull
    lo, hi = P[used].min(axis=0), P[used].max(axis=0)
    locs = [P[int(v)] for v in rng.choice(used, size=20)]
    for t3 in tris[rng.integers(0, len(tris), size=20)]:
        locs.append((P[t3[0]] + P[t3[1]]) / 2)
    locs += list(lo - 0.1 * (hi - lo) + rng.random((40, 2)) * 1.2 * (hi - lo))
    locs = np.array(locs, dtype=np.float64)
    starts = rng.integers(0, 3 * len(tris), size=len(locs)).astype(np.int32)
    blob = (np.int32(len(P)).tobytes() + P.astype(np.float64).tobytes()
            + np.int32(len(tris)).tobytes() + tris.astype(np.int32).tobytes()
            + np.int32(len(cons)).tobytes() + np.array(cons, dtype=np.int32).reshape(-1, 2).tobytes()
            + np.int32(len(qs)).tobytes() + np.array(qs, dtype=np.int32).tobytes()
            + np.int32(len(locs)).tobytes() + locs.tobytes() + starts.tobytes())
    f = tmp_path / "mesh.bin"
    f.write_bytes(blob)
    out = subprocess.run([harness, str(f)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    got = [tuple(int(x) for x in line.split()) for line in out.stdout.split("\n") if line.strip()]
    assert len(got) == len(qs) + len(locs)
    for x, (tri, where) in zip(locs, got[len(qs):]):
        assert (tri, where) == _locate_brute(P, tris, x), (seed, x)
    for (u, w), (status, crossed) in zip(qs, got[:len(qs)]):
        assert status in STATUS, (seed, u, w, status)
        t2, _ = _state(lib, pts, ops, r)
        with t2:
            want = t2.insert_constraint(u, w)
        assert STATUS[status] == want, (seed, u, w, status, want)
        if status == 0:
            assert crossed == _crossed_edges(P, tris, u, w), (seed, u, w)
