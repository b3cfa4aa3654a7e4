// Point location in the half-edge mesh, shared by the host (insertion, the
// fallback of the batch location) and the GPU batch location (k_locate.cu).
//
// walk(): the visibility walk of the reference's locate_
// (GuibasStolfiDwyer_Wrapper.cpp:423-486): from a triangle, cross an edge
// whose line separates the triangle from p until p lies in the triangle
// (border included) or beyond a hull edge. When two edges separate, the one
// crossed is picked by a hash of the step, which ends the cycles a fixed
// choice can run into in a constrained (non-Delaunay) mesh.
//
// classify(): the canonical answer for a point in a triangle: the point lies
// inside it, on an edge or on a vertex, and the triangle reported is the
// smallest index among all triangles containing the point (border
// included): the triangle itself, the smaller of the two triangles of the
// edge, or the smallest triangle around the vertex. The answer therefore
// depends only on the mesh and the point, not on where the walk started.
#pragma once

#include <cstdint>

#include "mesh_layout.hpp"
#include "predicates.cuh"

namespace qdtg {

enum LocClass : int
{
    kLocUnresolved = -2,   // the walk gave up (step limit or a damaged mesh)
    kLocOutside = -1,      // beyond the hull, or no triangles
    kLocInside = 0,
    kLocEdge = 1,
    kLocVertex = 2,
};

struct LocResult
{
    int tri;     // canonical triangle, -1 outside
    int where;   // LocClass
    int he;      // the half-edge the walk ended on (in the triangle, or the hull edge p sees)
};

QDT_HD inline bool he_ok(const MeshHalfEdge* h, int nh, int nv, int e)
{
    return e >= 0 && e < nh && h[e].org >= 0 && h[e].org < nv && h[e].next >= 0 && h[e].next < nh;
}

QDT_HD inline int edge_orient(const MeshVertex* v, const MeshHalfEdge* h, int e, double x, double y)
{
    const MeshVertex& a = v[h[e].org];
    const MeshVertex& b = v[h[h[e].next].org];
    return orient2d_sign(a.x, a.y, b.x, b.y, x, y);
}

// Walks from half-edge `start` toward (x, y). Returns the half-edge of a
// triangle containing the point (border included) with where = kLocInside,
// or the hull half-edge the point lies beyond with where = kLocOutside, or
// where = kLocUnresolved after `cap` steps or on an index out of range.
// *nsteps (when given) receives the triangles visited.
QDT_HD inline LocResult walk(const MeshVertex* v, const MeshHalfEdge* h, int nv, int nh, int start, double x,
    double y, int cap, int* nsteps = nullptr)
{
    LocResult r{ -1, kLocUnresolved, -1 };
    int       e = start;
    int       entered = -1;   // the edge the walk came in through: the point is strictly left of it
    for (int step = 0; step < cap; ++step)
    {
        if (nsteps) *nsteps = step + 1;
        if (!he_ok(h, nh, nv, e)) return r;
        const int e1 = h[e].next;
        if (!he_ok(h, nh, nv, e1)) return r;
        const int e2 = h[e1].next;
        if (!he_ok(h, nh, nv, e2) || h[e2].next != e) return r;
        const int o0 = e == entered ? 1 : edge_orient(v, h, e, x, y);
        const int o1 = edge_orient(v, h, e1, x, y);
        const int o2 = edge_orient(v, h, e2, x, y);
        if (o0 >= 0 && o1 >= 0 && o2 >= 0)
        {
            r.where = kLocInside;
            r.he = e;
            r.tri = h[e].tri;
            return r;
        }
        int cross;
        const int neg = (o0 < 0) + (o1 < 0) + (o2 < 0);
        if (neg == 1)
            cross = o0 < 0 ? e : (o1 < 0 ? e1 : e2);
        else
        {
            const uint32_t hs = ((uint32_t)step * 2654435761u) ^ ((uint32_t)e * 40503u);
            const bool     second = (hs >> 16) & 1u;
            const int      a = o0 < 0 ? e : e1;          // the first separating edge
            const int      b = o2 < 0 ? e2 : e1;         // the last one
            cross = second ? b : a;
        }
        const int tw = h[cross].twin;
        if (tw < 0)
        {
            r.where = kLocOutside;
            r.he = cross;
            return r;
        }
        e = tw;
        entered = tw;
    }
    return r;
}

// Canonical class and triangle of a point in the triangle of half-edge e
// (border included). ring_cap bounds the walk around a vertex.
QDT_HD inline LocResult classify(const MeshVertex* v, const MeshHalfEdge* h, int nv, int nh, int e, double x,
    double y, int ring_cap)
{
    LocResult r{ -1, kLocUnresolved, e };
    int       hh[3];
    hh[0] = e;
    hh[1] = h[e].next;
    hh[2] = h[hh[1]].next;
    int o[3];
    for (int i = 0; i < 3; ++i) o[i] = edge_orient(v, h, hh[i], x, y);
    const int zeros = (o[0] == 0) + (o[1] == 0) + (o[2] == 0);
    int       best = h[e].tri;
    if (zeros == 0)
    {
        r.where = kLocInside;
        r.tri = best;
        return r;
    }
    if (zeros == 1)
    {
        const int z = o[0] == 0 ? hh[0] : (o[1] == 0 ? hh[1] : hh[2]);
        const int tw = h[z].twin;
        if (tw >= 0 && tw < nh && h[tw].tri >= 0 && h[tw].tri < best) best = h[tw].tri;
        r.where = kLocEdge;
        r.tri = best;
        return r;
    }
    // two edges through the point: it is their common vertex, the origin of
    // the second edge; visit the triangles around it
    int s = -1;
    for (int i = 0; i < 3; ++i)
        if (o[i] == 0 && o[(i + 1) % 3] == 0) s = hh[(i + 1) % 3];
    if (s < 0) return r;   // three zero orientations: a degenerate triangle
    // counter-clockwise: the half-edge into the vertex, then its twin
    int  k = s;
    bool closed = false;
    for (int step = 0; step < ring_cap; ++step)
    {
        const int in = h[h[k].next].next;
        if (in < 0 || in >= nh) return r;
        const int t = h[in].twin;
        if (t < 0) break;
        if (t >= nh) return r;
        k = t;
        if (k == s)
        {
            closed = true;
            break;
        }
        if (h[k].tri >= 0 && h[k].tri < best) best = h[k].tri;
        if (step + 1 == ring_cap) return r;
    }
    if (!closed)
    {
        // a hull vertex: clockwise from s as well
        k = s;
        for (int step = 0; step < ring_cap; ++step)
        {
            const int t = h[k].twin;
            if (t < 0) break;
            if (t >= nh) return r;
            k = h[t].next;
            if (k < 0 || k >= nh) return r;
            if (h[k].tri >= 0 && h[k].tri < best) best = h[k].tri;
            if (step + 1 == ring_cap) return r;
        }
    }
    r.where = kLocVertex;
    r.tri = best;
    return r;
}

// Outcome of tracing a constraint segment through the mesh: what
// qdt_insert_constraint decides for it before any flip
// (GuibasStolfiDwyer_Wrapper.cpp:1050-1106 and the existing-edge check
// before it).
enum TraceClass : int
{
    kTraceOk = 0,                 // the edge exists, or the segment crosses only unconstrained edges
    kTraceThroughPoint = 1,       // a vertex lies on the open segment
    kTraceCrossesConstraint = 2,  // a constrained edge crosses it first
    kTraceBroken = 3,             // the mesh around the start vertex is inconsistent
    kTraceUnresolved = 4,         // the step limit ran out
};

QDT_HD inline bool same_direction(const MeshVertex& a, const MeshVertex& b, const MeshVertex& c)
{
    auto      sg = [](double d) { return d > 0 ? 1 : (d < 0 ? -1 : 0); };
    const int sx = sg(b.x - a.x) * sg(c.x - a.x);
    const int sy = sg(b.y - a.y) * sg(c.y - a.y);
    return sx >= 0 && sy >= 0 && (sx > 0 || sy > 0);
}

QDT_HD inline int orient_v(const MeshVertex* v, int a, int b, int c)
{
    return orient2d_sign(v[a].x, v[a].y, v[b].x, v[b].y, v[c].x, v[c].y);
}

// Traces the segment from mesh vertex u to mesh vertex w (u != w). Visits
// u's fan counter-clockwise from u's stored half-edge, then clockwise for a
// hull vertex: an edge u-w in either direction means kTraceOk with nothing
// crossed; otherwise the fan triangle the segment leaves through, or a
// neighbour on the segment, decides the start (at most one of the two
// exists, so the outcome does not depend on which half-edge u stores), and
// the march counts the edges crossed until w, a vertex on the segment, or a
// constrained edge. *crossed = edges crossed before the outcome. Each fan
// visit and each crossing is one step of cap.
QDT_HD inline int trace_segment(const MeshVertex* v, const MeshHalfEdge* h, int nv, int nh, int u, int w, int cap,
    int* crossed)
{
    *crossed = 0;
    if (u < 0 || u >= nv || w < 0 || w >= nv) return kTraceBroken;
    const int h0 = v[u].he;
    if (!he_ok(h, nh, nv, h0) || h[h0].org != u) return kTraceBroken;
    int  steps = 0;
    int  start = -1;
    bool blocked = false, exists = false;
    // one fan visit: the existing-edge check over the whole fan, and the
    // first start / blocking neighbour in fan order
    auto visit = [&](int e) -> bool {
        const int hn = h[e].next;
        if (!he_ok(h, nh, nv, hn) || !he_ok(h, nh, nv, h[hn].next)) return false;
        const int y = h[hn].org, z = h[h[hn].next].org;
        if (y == w || z == w)
        {
            exists = true;
            return false;
        }
        if (start < 0 && !blocked)
        {
            const int oy = orient_v(v, u, y, w), oz = orient_v(v, u, z, w);
            if (oy > 0 && oz < 0)
                start = hn;
            else if ((oy == 0 && same_direction(v[u], v[y], v[w])) || (oz == 0 && same_direction(v[u], v[z], v[w])))
                blocked = true;
        }
        return true;
    };
    bool ok = true, closed = false;
    int  e = h0;
    for (;;)
    {
        if (++steps > cap) return kTraceUnresolved;
        if (!visit(e))
        {
            ok = exists;
            break;
        }
        const int prev = h[h[e].next].next;
        const int tw = h[prev].twin;
        if (tw < 0) break;
        if (tw == h0)
        {
            closed = true;
            break;
        }
        if (!he_ok(h, nh, nv, tw))
        {
            ok = false;
            break;
        }
        e = tw;
    }
    if (exists) return kTraceOk;
    if (!ok) return kTraceBroken;
    if (!closed)
    {
        e = h0;
        for (;;)
        {
            const int tw = h[e].twin;
            if (tw < 0) break;
            if (!he_ok(h, nh, nv, tw)) return kTraceBroken;
            e = h[tw].next;
            if (e == h0) break;
            if (!he_ok(h, nh, nv, e)) return kTraceBroken;
            if (++steps > cap) return kTraceUnresolved;
            if (!visit(e))
            {
                if (exists) return kTraceOk;
                return kTraceBroken;
            }
        }
    }
    if (exists) return kTraceOk;
    if (blocked) return kTraceThroughPoint;
    if (start < 0) return kTraceBroken;
    e = start;
    for (;;)
    {
        if (++steps > cap) return kTraceUnresolved;
        if (h[e].cons) return kTraceCrossesConstraint;
        ++*crossed;
        const int tw = h[e].twin;
        if (!he_ok(h, nh, nv, tw)) return kTraceBroken;
        const int a = h[tw].next;
        if (!he_ok(h, nh, nv, a)) return kTraceBroken;
        const int b = h[a].next;
        if (!he_ok(h, nh, nv, b)) return kTraceBroken;
        const int x = h[b].org;
        if (x == w) return kTraceOk;
        const int o = orient_v(v, u, w, x);
        if (o == 0) return kTraceThroughPoint;
        e = o > 0 ? a : b;
    }
}

}  // namespace qdtg
