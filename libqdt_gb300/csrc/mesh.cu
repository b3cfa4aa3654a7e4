// Incremental point insertion and constrained edges on the handle returned by
// the batch path (host code; not on the GPU hot path).
//
// The batch engine leaves triangles, representatives and points in the
// context. The first insertion or constraint builds a half-edge mesh from
// them (reference GuibasStolfiDwyer_Wrapper.cpp:99-202); afterwards the mesh
// and the context's triangle list are kept in step. The algorithms are the
// published ones the reference uses, written here from their definitions:
//
// * insertion (Wrapper.cpp:531-876): locate the point by a visibility walk
//   with a scan as fallback; split the triangle it lies in (or the two
//   triangles of the edge it lies on, or join it to the visible hull edges
//   when it lies outside); restore the Delaunay property with Lawson flips
//   that never flip a constrained edge;
// * constraints (Wrapper.cpp:878-1285): trace the segment through the mesh,
//   reject it when it crosses a constrained edge or passes through a vertex,
//   flip the crossed edges away (Sloan 1993), mark the new edge constrained,
//   and re-legalise with Lawson flips.
//
// All geometric decisions use the exact predicates of predicates.cuh.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <deque>
#include <unordered_map>
#include <vector>

#include "context.hpp"
#include "mesh_layout.hpp"
#include "mesh_walk.cuh"
#include "predicates.cuh"
#include "qdt.h"

namespace qdtg {

using MV = MeshVertex;
using HE = MeshHalfEdge;

// Start points of the host walks: a uniform grid over the vertices' bounding
// box, about two vertices per cell, holding one vertex of each cell.
// Vertices are never removed, so a seed never goes stale. Built once the
// walks without it have taken about as many steps as building it costs.
struct SeedGrid
{
    int              gx = 0, gy = 0;
    double           x0 = 0, y0 = 0, ix = 0, iy = 0;
    std::vector<int> cell;         // vertex per cell, -1 when none
    size_t           walked = 0;   // walk steps taken before the grid existed
};

struct Mesh
{
    MeshVec<MV>      v;
    MeshVec<HE>      h;
    std::vector<int> free_h;
    MeshVec<int>     o2l;    // point index -> mesh vertex, -1 when none
    std::vector<int> t2h;    // triangle -> one of its half-edges
    SeedGrid         grid;
    int              last = 0;
    uint64_t         id = next_id();   // identifies this mesh to the device mirror
    uint64_t         version = 0;      // bumped by every call that may change the mesh

    static uint64_t next_id()
    {
        static std::atomic<uint64_t> n{ 0 };
        return ++n;
    }
};

void mesh_destroy(Mesh* m) noexcept { delete m; }

namespace {

inline int orient(const Mesh& M, int a, int b, double px, double py)
{
    const MV &A = M.v[a], &B = M.v[b];
    return orient2d_sign(A.x, A.y, B.x, B.y, px, py);
}
inline int orient3(const Mesh& M, int a, int b, int c) { return orient(M, a, b, M.v[c].x, M.v[c].y); }
inline int incircle4(const Mesh& M, int a, int b, int c, int d)
{
    const MV &A = M.v[a], &B = M.v[b], &C = M.v[c], &D = M.v[d];
    return incircle_sign(A.x, A.y, B.x, B.y, C.x, C.y, D.x, D.y);
}

// Builds the half-edge mesh from the context's triangles (Wrapper.cpp:99-202).
void build_mesh(Context& c, Mesh& M)
{
    const size_t T = c.ntris();
    M.v.clear();
    M.h.clear();
    M.free_h.clear();
    M.t2h.clear();
    M.last = 0;
    M.o2l.assign(c.npoints(), -1);
    M.v.reserve(T / 2 + 8);
    for (size_t t = 0; t < 3 * T; ++t)
    {
        const uint32_t o = c.tris[t];
        if (M.o2l[o] < 0)
        {
            M.o2l[o] = (int)M.v.size();
            M.v.push_back(MV{ c.points[2 * o], c.points[2 * o + 1], o, -1 });
        }
    }
    M.h.resize(3 * T);
    M.t2h.resize(T);
    for (size_t t = 0; t < T; ++t)
    {
        const int base = (int)(3 * t);
        for (int i = 0; i < 3; ++i)
        {
            const int a = M.o2l[c.tris[3 * t + i]];
            M.h[base + i] = HE{ a, -1, base + (i + 1) % 3, (int)t, false };
            if (M.v[a].he < 0) M.v[a].he = base + i;
        }
        M.t2h[t] = base;
    }
    // twins: outgoing half-edges grouped by origin (CSR), then for u->w look
    // among w's outgoing ones for w->u
    const int        nV = (int)M.v.size();
    std::vector<int> off(nV + 1, 0), adj(3 * T);
    for (size_t i = 0; i < 3 * T; ++i) ++off[M.h[i].org + 1];
    for (int i = 0; i < nV; ++i) off[i + 1] += off[i];
    {
        std::vector<int> cur(off.begin(), off.end() - 1);
        for (size_t i = 0; i < 3 * T; ++i) adj[cur[M.h[i].org]++] = (int)i;
    }
    for (size_t i = 0; i < 3 * T; ++i)
    {
        if (M.h[i].twin >= 0) continue;
        const int u = M.h[i].org, w = M.h[M.h[i].next].org;
        for (int k = off[w]; k < off[w + 1]; ++k)
        {
            const int j = adj[k];
            if (M.h[M.h[j].next].org == u)
            {
                M.h[i].twin = j;
                M.h[j].twin = (int)i;
                break;
            }
        }
    }
}

// The same mesh built on the GPU from the batch result the engine still
// holds (k_mesh.cu); false when it cannot (then the host builds it).
bool build_mesh_on_device(Context& c, Mesh& M)
{
    if (!c.mesh_on_gpu || !c.engine) return false;
    const size_t T = c.ntris();
    if (c.engine->build_mesh(c.npoints(), T, M.o2l, M.v, M.h) != 0) return false;
    M.free_h.clear();
    M.last = 0;
    M.t2h.reserve(T + std::max<size_t>(T / 8, 1024));
    M.t2h.resize(T);
    for (size_t t = 0; t < T; ++t) M.t2h[t] = (int)(3 * t);
    MeshMirror& mr = c.engine->mirror();
    mr.mesh_id = M.id;
    mr.mesh_version = M.version;
    return true;
}

// Brings the engine's device mirror to the mesh's current state (an upload
// when the host changed it since). false when there is no engine or the
// upload failed.
bool sync_mirror(Context& c, const Mesh& M)
{
    if (!c.engine || !c.engine->activate()) return false;
    MeshMirror& mr = c.engine->mirror();
    if (mr.mesh_id == M.id && mr.mesh_version == M.version && mr.nv == M.v.size() && mr.nh == M.h.size())
        return true;
    if (mirror_upload(mr, M.v.data(), M.v.size(), M.h.data(), M.h.size(), c.engine->stream()) != 0) return false;
    mr.mesh_id = M.id;
    mr.mesh_version = M.version;
    return true;
}

Mesh& ensure_mesh(Context& c)
{
    if (!c.mesh)
    {
        Mesh* m = new Mesh();
        try
        {
            if (!build_mesh_on_device(c, *m)) build_mesh(c, *m);
        }
        catch (...)
        {
            delete m;
            throw;
        }
        c.mesh = m;
    }
    return *c.mesh;
}

int alloc_he(Mesh& M)
{
    if (!M.free_h.empty())
    {
        const int k = M.free_h.back();
        M.free_h.pop_back();
        return k;
    }
    M.h.push_back(HE{ -1, -1, -1, -1, false });
    return (int)M.h.size() - 1;
}

void free_he(Mesh& M, int k)
{
    M.h[k] = HE{ -1, -1, -1, -1, false };
    M.free_h.push_back(k);
}

size_t add_tri(Context& c, Mesh& M, int a, int b, int d, int h0)
{
    const size_t t = c.ntris();
    c.tris.push_back(M.v[a].orig);
    c.tris.push_back(M.v[b].orig);
    c.tris.push_back(M.v[d].orig);
    M.t2h.push_back(h0);
    return t;
}

// removes triangle idx by moving the last triangle into its slot
void remove_tri(Context& c, Mesh& M, size_t idx)
{
    const size_t last = c.ntris() - 1;
    if (idx != last)
    {
        for (int i = 0; i < 3; ++i) c.tris[3 * idx + i] = c.tris[3 * last + i];
        const int moved = M.t2h[last];
        M.t2h[idx] = moved;
        int e = moved;
        do
        {
            M.h[e].tri = (int)idx;
            e = M.h[e].next;
        } while (e != moved);
    }
    c.tris.resize(3 * last);
    M.t2h.pop_back();
}

// Visibility walk (Wrapper.cpp:423-486), scan as fallback (:491-521).
// Returns a half-edge of the triangle containing p (border included), or -1
// with *hull set to a hull half-edge that p sees. The walk starts at the
// half-edge `start` when it is alive, else at the last insertion.
int locate(const Mesh& M, size_t ntri, double px, double py, int* hull, int start = -1, size_t* steps = nullptr)
{
    *hull = -1;
    if (M.h.empty() || ntri == 0) return -1;
    int h = (start >= 0 && start < (int)M.h.size() && M.h[start].org >= 0) ? start : M.last;
    if (h < 0 || h >= (int)M.h.size() || M.h[h].org < 0)
    {
        h = 0;
        while (h < (int)M.h.size() && M.h[h].org < 0) ++h;
        if (h >= (int)M.h.size()) return -1;
    }
    for (size_t step = 0; step < ntri + 16; ++step)
    {
        if (steps) *steps = step + 1;
        const int h0 = h, h1 = M.h[h0].next, h2 = M.h[h1].next;
        if (M.h[h2].next != h0) break;
        const int o0 = orient(M, M.h[h0].org, M.h[h1].org, px, py);
        const int o1 = orient(M, M.h[h1].org, M.h[h2].org, px, py);
        const int o2 = orient(M, M.h[h2].org, M.h[h0].org, px, py);
        if (o0 >= 0 && o1 >= 0 && o2 >= 0) return h0;
        const int cross = o0 < 0 ? h0 : (o1 < 0 ? h1 : h2);
        const int tw = M.h[cross].twin;
        if (tw < 0)
        {
            *hull = cross;
            return -1;
        }
        h = tw;
    }
    for (size_t t = 0; t < M.t2h.size(); ++t)
    {
        const int h0 = M.t2h[t], h1 = M.h[h0].next, h2 = M.h[h1].next;
        if (orient(M, M.h[h0].org, M.h[h1].org, px, py) >= 0 && orient(M, M.h[h1].org, M.h[h2].org, px, py) >= 0 &&
            orient(M, M.h[h2].org, M.h[h0].org, px, py) >= 0)
            return h0;
    }
    for (size_t i = 0; i < M.h.size(); ++i)
    {
        const HE& e = M.h[i];
        if (e.org < 0 || e.twin >= 0) continue;
        if (orient(M, e.org, M.h[e.next].org, px, py) < 0)
        {
            *hull = (int)i;
            return -1;
        }
    }
    return -1;
}

size_t seed_cell(const SeedGrid& g, double x, double y)
{
    const double fx = (x - g.x0) * g.ix, fy = (y - g.y0) * g.iy;
    const int    cx = fx >= g.gx - 1 ? g.gx - 1 : (fx > 0 ? (int)fx : 0);
    const int    cy = fy >= g.gy - 1 ? g.gy - 1 : (fy > 0 ? (int)fy : 0);
    return (size_t)cy * (size_t)g.gx + (size_t)cx;
}

void seed_build(Mesh& M)
{
    SeedGrid& g = M.grid;
    if (M.v.empty()) return;
    double x0 = M.v[0].x, x1 = x0, y0 = M.v[0].y, y1 = y0;
    for (const MV& p : M.v)
    {
        x0 = std::min(x0, p.x), x1 = std::max(x1, p.x);
        y0 = std::min(y0, p.y), y1 = std::max(y1, p.y);
    }
    const double w = x1 - x0, hgt = y1 - y0;
    const double cells = std::max(1.0, std::min((double)M.v.size() / 2.0, (double)(1 << 24)));
    int          gx = 1, gy = 1;
    if (w > 0 && hgt > 0 && std::isfinite(w) && std::isfinite(hgt))
    {
        gx = (int)std::clamp(std::sqrt(cells * w / hgt), 1.0, cells);
        gy = (int)std::clamp(cells / gx, 1.0, cells);
    }
    else if (w > 0 && std::isfinite(w))
        gx = (int)cells;
    else if (hgt > 0 && std::isfinite(hgt))
        gy = (int)cells;
    g.gx = gx;
    g.gy = gy;
    g.x0 = x0;
    g.y0 = y0;
    g.ix = (gx > 1 && w > 0 && std::isfinite(gx / w)) ? gx / w : 0.0;
    g.iy = (gy > 1 && hgt > 0 && std::isfinite(gy / hgt)) ? gy / hgt : 0.0;
    g.cell.assign((size_t)gx * (size_t)gy, -1);
    for (size_t i = 0; i < M.v.size(); ++i) g.cell[seed_cell(g, M.v[i].x, M.v[i].y)] = (int)i;
    // an empty cell (about one in seven at two vertices per cell) takes the
    // nearest seed along its row, or of the nearest row that has one
    std::vector<char> row_has(gy, 0);
    for (int y = 0; y < gy; ++y)
    {
        int* row = g.cell.data() + (size_t)y * gx;
        int  last = -1;
        for (int x = 0; x < gx; ++x)
        {
            if (row[x] >= 0)
                last = row[x];
            else
                row[x] = last;
        }
        last = -1;
        for (int x = gx - 1; x >= 0; --x)
        {
            if (row[x] >= 0)
                last = row[x];
            else
                row[x] = last;
        }
        row_has[y] = row[0] >= 0;
    }
    for (int pass = 0; pass < 2; ++pass)
    {
        int src = -1;
        for (int k = 0; k < gy; ++k)
        {
            const int y = pass ? gy - 1 - k : k;
            if (row_has[y])
                src = y;
            else if (src >= 0)
            {
                std::copy_n(g.cell.data() + (size_t)src * gx, gx, g.cell.data() + (size_t)y * gx);
                row_has[y] = 1;
            }
        }
    }
}

// A half-edge out of the seed vertex of p's cell, or -1 (no grid yet, empty
// cell); any live half-edge is a valid start for locate()
int seed_start(const Mesh& M, double x, double y)
{
    if (M.grid.cell.empty()) return -1;
    const int v = M.grid.cell[seed_cell(M.grid, x, y)];
    if (v < 0 || v >= (int)M.v.size()) return -1;
    const int he = M.v[v].he;
    return (he >= 0 && he < (int)M.h.size() && M.h[he].org == v) ? he : -1;
}

// counts a walk's steps while there is no grid; builds the grid once the
// walks have cost about as much as the build (one pass over the vertices)
void seed_account(Mesh& M, size_t steps)
{
    if (!M.grid.cell.empty()) return;
    M.grid.walked += steps;
    if (M.grid.walked > M.v.size() / 32 + 64) seed_build(M);
}

// Flips the diagonal h (Wrapper.cpp:942-1009). Before: triangles
// (a, b, c) with h = a->b and (b, a, d) with twin = b->a. After: (d, c, a)
// and (c, d, b). Refused unless both new triangles are strictly
// counter-clockwise, or when h is constrained or on the hull.
bool flip(Context& c, Mesh& M, int h)
{
    const int tw = M.h[h].twin;
    if (tw < 0 || M.h[h].cons) return false;
    const int hn = M.h[h].next, hp = M.h[hn].next;
    const int tn = M.h[tw].next, tp = M.h[tn].next;
    const int a = M.h[h].org, b = M.h[hn].org, cc = M.h[hp].org, d = M.h[tp].org;
    if (orient3(M, d, cc, a) <= 0 || orient3(M, cc, d, b) <= 0) return false;
    // triangle 1: h = d->c, hp = c->a, tn = a->d
    M.h[h].org = d;
    M.h[h].next = hp;
    M.h[hp].next = tn;
    M.h[tn].next = h;
    // triangle 2: tw = c->d, tp = d->b, hn = b->c
    M.h[tw].org = cc;
    M.h[tw].next = tp;
    M.h[tp].next = hn;
    M.h[hn].next = tw;
    const int t1 = M.h[h].tri, t2 = M.h[tw].tri;
    M.h[tn].tri = t1;
    M.h[hn].tri = t2;
    c.tris[3 * t1 + 0] = M.v[d].orig;
    c.tris[3 * t1 + 1] = M.v[cc].orig;
    c.tris[3 * t1 + 2] = M.v[a].orig;
    c.tris[3 * t2 + 0] = M.v[cc].orig;
    c.tris[3 * t2 + 1] = M.v[d].orig;
    c.tris[3 * t2 + 2] = M.v[b].orig;
    M.t2h[t1] = h;
    M.t2h[t2] = tw;
    M.v[a].he = tn;
    M.v[b].he = hn;
    M.v[cc].he = hp;
    M.v[d].he = h;
    return true;
}

// Calls f(h) for every half-edge h leaving x until f returns true
// (Wrapper.cpp:885-923): counter-clockwise from the stored one, then
// clockwise for hull vertices.
template <class F>
void for_each_out(const Mesh& M, int x, F&& f)
{
    const int h0 = M.v[x].he;
    if (h0 < 0) return;
    const size_t limit = M.h.size();
    size_t       steps = 0;
    int          h = h0;
    for (;;)
    {
        if (f(h)) return;
        if (++steps > limit) return;
        const int prev = M.h[M.h[h].next].next;
        const int tw = M.h[prev].twin;
        if (tw < 0) break;
        if (tw == h0) return;
        h = tw;
    }
    h = h0;
    for (;;)
    {
        const int tw = M.h[h].twin;
        if (tw < 0) return;
        h = M.h[tw].next;
        if (h == h0) return;
        if (f(h)) return;
        if (++steps > limit) return;
    }
}

int find_he(const Mesh& M, int u, int w)
{
    int found = -1;
    for_each_out(M, u, [&](int h) {
        if (M.h[M.h[h].next].org == w)
        {
            found = h;
            return true;
        }
        return false;
    });
    return found;
}

void mark_cons(Mesh& M, int h)
{
    M.h[h].cons = true;
    if (M.h[h].twin >= 0) M.h[M.h[h].twin].cons = true;
}

bool segments_cross(const Mesh& M, int a, int b, int c, int d)
{
    const int o1 = orient3(M, a, b, c), o2 = orient3(M, a, b, d);
    const int o3 = orient3(M, c, d, a), o4 = orient3(M, c, d, b);
    return ((o1 > 0 && o2 < 0) || (o1 < 0 && o2 > 0)) && ((o3 > 0 && o4 < 0) || (o3 < 0 && o4 > 0));
}

// Lists the edges the open segment u-w crosses, each as the half-edge from
// the vertex right of u->w to the one on its left (Wrapper.cpp:1050-1106).
int trace(const Mesh& M, size_t ntri, int u, int w, std::vector<int>& crossed)
{
    int  start = -1;
    bool blocked = false;
    for_each_out(M, u, [&](int h) {
        const int hn = M.h[h].next;
        const int y = M.h[hn].org, z = M.h[M.h[hn].next].org;
        const int oy = orient3(M, u, y, w), oz = orient3(M, u, z, w);
        if (oy > 0 && oz < 0)
        {
            start = hn;
            return true;
        }
        if ((oy == 0 && same_direction(M.v[u], M.v[y], M.v[w])) ||
            (oz == 0 && same_direction(M.v[u], M.v[z], M.v[w])))
        {
            blocked = true;
            return true;
        }
        return false;
    });
    if (blocked) return QDT_ERR_THROUGH_POINT;
    if (start < 0) return QDT_ERR_INTERNAL;
    int e = start;
    for (size_t guard = 0; guard <= ntri; ++guard)
    {
        if (M.h[e].cons) return QDT_ERR_CROSSES_CONSTRAINT;
        crossed.push_back(e);
        const int tw = M.h[e].twin;
        if (tw < 0) return QDT_ERR_INTERNAL;
        const int a = M.h[tw].next, b = M.h[a].next;
        const int x = M.h[b].org;
        if (x == w) return QDT_OK;
        const int o = orient3(M, u, w, x);
        if (o == 0) return QDT_ERR_THROUGH_POINT;
        e = o > 0 ? a : b;
    }
    return QDT_ERR_INTERNAL;
}

// Lawson's flips over a stack of half-edges (Wrapper.cpp:1111-1142).
void legalize(Context& c, Mesh& M, std::vector<int>& stack)
{
    while (!stack.empty())
    {
        const int h = stack.back();
        stack.pop_back();
        if (M.h[h].org < 0) continue;
        const int tw = M.h[h].twin;
        if (tw < 0 || M.h[h].cons) continue;
        const int hn = M.h[h].next, hp = M.h[hn].next;
        const int tn = M.h[tw].next, tp = M.h[tn].next;
        const int a = M.h[h].org, b = M.h[hn].org, cc = M.h[hp].org, d = M.h[tp].org;
        if (incircle4(M, a, b, cc, d) <= 0) continue;
        if (!flip(c, M, h)) continue;
        stack.push_back(hp);
        stack.push_back(hn);
        stack.push_back(tn);
        stack.push_back(tp);
    }
}

int insert_by_rebuild(Context& c, double x, double y)
{
    c.points.push_back(x);
    c.points.push_back(y);
    return rebuild_from_points(c);
}

}  // namespace

int mesh_insert_point(Context& c, double x, double y, bool, int hint)
{
    if (c.ntris() == 0) return insert_by_rebuild(c, x, y);
    Mesh& M = ensure_mesh(c);
    if (M.h.empty()) return insert_by_rebuild(c, x, y);
    ++M.version;

    int    hull = -1;
    size_t steps = 0;
    if (hint < 0) hint = seed_start(M, x, y);
    int h_start = locate(M, c.ntris(), x, y, &hull, hint, &steps);
    seed_account(M, steps);
    if (h_start < 0 && hull < 0) return insert_by_rebuild(c, x, y);
    const bool outside = h_start < 0;
    if (!outside)
    {
        // a vertex equal to p is a corner of the triangle that contains it
        int e = h_start;
        do
        {
            const MV& q = M.v[M.h[e].org];
            if (q.x == x && q.y == y)
            {
                c.points.push_back(x);
                c.points.push_back(y);
                c.rep.push_back(q.orig);
                return QDT_OK;
            }
            e = M.h[e].next;
        } while (e != h_start);
        // start from the canonical containing triangle (the smaller index of
        // the two when p lies on an edge), so that the result does not depend
        // on where the walk began
        const LocResult cl =
            classify(M.v.data(), M.h.data(), (int)M.v.size(), (int)M.h.size(), h_start, x, y, INT_MAX);
        if ((cl.where == kLocInside || cl.where == kLocEdge) && cl.tri >= 0 && cl.tri < (int)M.t2h.size())
            h_start = M.t2h[cl.tri];
    }
    M.last = outside ? hull : h_start;

    const uint32_t id = (uint32_t)c.npoints();
    c.points.push_back(x);
    c.points.push_back(y);
    c.rep.push_back(id);
    ++c.unique_points;
    const int nv = (int)M.v.size();
    M.v.push_back(MV{ x, y, id, -1 });
    if (M.o2l.size() <= id) M.o2l.resize(id + 1, -1);
    M.o2l[id] = nv;
    if (!M.grid.cell.empty()) M.grid.cell[seed_cell(M.grid, x, y)] = nv;

    // visible hull edges (outside case)
    std::vector<int> visible;
    if (outside)
    {
        auto vis = [&](int e) { return orient(M, M.h[e].org, M.h[M.h[e].next].org, x, y) < 0; };
        auto next_hull = [&](int e) {
            int k = M.h[e].next;
            while (M.h[k].twin >= 0) k = M.h[M.h[k].twin].next;
            return k;
        };
        auto prev_hull = [&](int e) {
            int k = M.h[M.h[e].next].next;
            while (M.h[k].twin >= 0)
            {
                const int t = M.h[k].twin;
                k = M.h[M.h[t].next].next;
            }
            return k;
        };
        // the visible hull edges form one chain; list it from its first edge
        // (in hull order), whichever edge the walk found
        int s = hull;
        for (int e = prev_hull(hull); e != hull && vis(e); e = prev_hull(e)) s = e;
        visible.push_back(s);
        for (int e = next_hull(s); e != s && vis(e); e = next_hull(e)) visible.push_back(e);
        M.last = s;
    }

    // the cavity: the triangle that contains p, and the one across the edge p
    // lies on, if any
    std::vector<int> cav_he, cav_tri;
    auto             in_cav = [&](int t) { return std::find(cav_tri.begin(), cav_tri.end(), t) != cav_tri.end(); };
    int              split_a = -1, split_b = -1;
    if (!outside)
    {
        auto add = [&](int e) {
            const int t = M.h[e].tri;
            if (t >= 0 && !in_cav(t))
            {
                cav_tri.push_back(t);
                cav_he.push_back(e);
            }
        };
        add(h_start);
        int e = h_start;
        do
        {
            const int en = M.h[e].next;
            if (orient(M, M.h[e].org, M.h[en].org, x, y) == 0)
            {
                if (M.h[e].twin >= 0) add(M.h[e].twin);
                if (M.h[e].cons)
                {
                    split_a = M.h[e].org;
                    split_b = M.h[en].org;
                }
            }
            e = en;
        } while (e != h_start);
    }

    struct Bnd
    {
        int  a, b, ext;
        bool cons;
    };
    std::vector<Bnd> bnd;
    for (int h0 : cav_he)
    {
        int e = h0;
        do
        {
            const int tw = M.h[e].twin;
            const int twt = tw >= 0 ? M.h[tw].tri : -1;
            if (!(twt >= 0 && in_cav(twt)))
            {
                const int a = M.h[e].org, b = M.h[M.h[e].next].org;
                if (tw >= 0 || orient(M, a, b, x, y) > 0) bnd.push_back(Bnd{ a, b, tw, M.h[e].cons != 0 });
            }
            e = M.h[e].next;
        } while (e != h0);
    }
    for (int e : visible)
    {
        const int t = M.h[e].tri;
        if (t >= 0 && in_cav(t)) continue;
        const int a = M.h[e].org, b = M.h[M.h[e].next].org;
        bnd.push_back(Bnd{ b, a, e, M.h[e].cons != 0 });
    }

    std::sort(cav_tri.rbegin(), cav_tri.rend());
    for (int t : cav_tri) remove_tri(c, M, (size_t)t);
    for (int h0 : cav_he)
    {
        int e = h0;
        do
        {
            const int en = M.h[e].next;
            free_he(M, e);
            e = en;
        } while (e != h0);
    }

    struct NT
    {
        int h0, h1, h2;
    };
    std::vector<NT> nts;
    for (const Bnd& q : bnd)
    {
        const int h0 = alloc_he(M), h1 = alloc_he(M), h2 = alloc_he(M);
        M.h[h0] = HE{ q.a, q.ext, h1, -1, q.cons };
        M.h[h1] = HE{ q.b, -1, h2, -1, false };
        M.h[h2] = HE{ nv, -1, h0, -1, false };
        if (q.ext >= 0)
        {
            M.h[q.ext].twin = h0;
            M.h[q.ext].cons = q.cons;
        }
        const int t = (int)add_tri(c, M, q.a, q.b, nv, h0);
        M.h[h0].tri = M.h[h1].tri = M.h[h2].tri = t;
        nts.push_back(NT{ h0, h1, h2 });
    }
    if (nts.empty())
    {
        // cannot happen with exact predicates; start over from the points
        c.points.resize(c.points.size() - 2);
        c.rep.pop_back();
        return insert_by_rebuild(c, x, y);
    }
    {
        std::unordered_map<int, int> by_b, by_a;   // b -> (b->p), a -> (p->a)
        for (const NT& t : nts)
        {
            by_b[M.h[t.h1].org] = t.h1;
            by_a[M.h[t.h0].org] = t.h2;
        }
        for (const auto& kv : by_b)
        {
            const auto it = by_a.find(kv.first);
            if (it != by_a.end())
            {
                M.h[kv.second].twin = it->second;
                M.h[it->second].twin = kv.second;
            }
        }
    }
    M.v[nv].he = nts[0].h2;
    M.last = nts[0].h0;
    for (size_t i = 0; i < nts.size(); ++i)
    {
        M.v[bnd[i].a].he = nts[i].h0;
        M.v[bnd[i].b].he = nts[i].h1;
    }
    if (split_a >= 0)
    {
        for (size_t i = 0; i < nts.size(); ++i)
        {
            if (bnd[i].b == split_a || bnd[i].b == split_b) mark_cons(M, nts[i].h1);
            if (bnd[i].a == split_a || bnd[i].a == split_b) mark_cons(M, nts[i].h2);
        }
    }

    // Lawson flips around p: h0 of every new triangle faces p
    std::vector<int> pending;
    for (const NT& t : nts) pending.push_back(t.h0);
    while (!pending.empty())
    {
        const int h = pending.back();
        pending.pop_back();
        const int tw = M.h[h].twin;
        if (tw < 0 || M.h[h].cons) continue;
        const int hn = M.h[h].next, hp = M.h[hn].next;
        if (M.h[hp].org != nv) continue;
        const int tn = M.h[tw].next, tp = M.h[tn].next;
        const int a = M.h[h].org, b = M.h[hn].org, d = M.h[tp].org;
        if (incircle4(M, a, b, nv, d) <= 0) continue;
        if (flip(c, M, h))
        {
            pending.push_back(tn);
            pending.push_back(tp);
        }
    }
    return QDT_OK;
}

int mesh_insert_constraint(Context& c, size_t v0, size_t v1)
{
    if (v0 >= c.rep.size() || v1 >= c.rep.size()) return QDT_ERR_INVALID_INDEX;
    v0 = c.rep[v0];
    v1 = c.rep[v1];
    if (v0 == v1) return QDT_ERR_SAME_POINT;
    Mesh& M = ensure_mesh(c);
    ++M.version;
    const int u = v0 < M.o2l.size() ? M.o2l[v0] : -1;
    const int w = v1 < M.o2l.size() ? M.o2l[v1] : -1;
    if (u < 0 || w < 0) return QDT_ERR_NO_TRIANGLES;

    int e = find_he(M, u, w);
    if (e < 0) e = find_he(M, w, u);
    if (e >= 0)
    {
        mark_cons(M, e);
        return QDT_OK;
    }
    std::vector<int> crossed;
    const int        tr = trace(M, c.ntris(), u, w, crossed);
    if (tr != QDT_OK) return tr;

    std::deque<int>  queue(crossed.begin(), crossed.end());
    std::vector<int> fresh;
    size_t           stalled = 0;
    while (!queue.empty())
    {
        const int h = queue.front();
        queue.pop_front();
        if (flip(c, M, h))
        {
            stalled = 0;
            const int a = M.h[h].org, b = M.h[M.h[h].next].org;
            if (segments_cross(M, u, w, a, b)) queue.push_back(h);
            else fresh.push_back(h);
        }
        else
        {
            queue.push_back(h);
            if (++stalled >= queue.size()) break;
        }
    }
    bool ok = false;
    if (queue.empty())
    {
        e = -1;
        for (int h : fresh)
        {
            const int a = M.h[h].org, b = M.h[M.h[h].next].org;
            if ((a == u && b == w) || (a == w && b == u))
            {
                e = h;
                break;
            }
        }
        if (e < 0) e = find_he(M, u, w);
        if (e < 0) e = find_he(M, w, u);
        if (e >= 0)
        {
            mark_cons(M, e);
            ok = true;
        }
    }
    std::vector<int> stack;
    auto             around = [&](int h) {
        if (M.h[h].org < 0) return;
        const int n = M.h[h].next;
        stack.push_back(h);
        stack.push_back(n);
        stack.push_back(M.h[n].next);
        const int tw = M.h[h].twin;
        if (tw >= 0)
        {
            const int tn = M.h[tw].next;
            stack.push_back(tn);
            stack.push_back(M.h[tn].next);
        }
    };
    for (int h : fresh) around(h);
    for (int h : queue) around(h);
    legalize(c, M, stack);
    return ok ? QDT_OK : QDT_ERR_INTERNAL;
}

int mesh_locate(Context& c, const double* xy, size_t k, int* tri, int* where, int* he)
{
    if (k == 0) return QDT_OK;
    auto none = [&](size_t i) {
        tri[i] = -1;
        where[i] = kLocOutside;
        if (he) he[i] = -1;
    };
    if (c.ntris() == 0)
    {
        for (size_t i = 0; i < k; ++i) none(i);
        return QDT_OK;
    }
    Mesh& M = ensure_mesh(c);
    if (M.h.empty() || M.h.size() > (size_t)INT_MAX || M.v.size() > (size_t)INT_MAX)
    {
        for (size_t i = 0; i < k; ++i) none(i);
        return QDT_OK;
    }
    std::vector<int> hev;
    int*             hp = he;
    if (!hp)
    {
        hev.resize(k);
        hp = hev.data();
    }
    if (!sync_mirror(c, M)) return QDT_ERR_OUT_OF_MEMORY;
    if (mirror_locate(c.engine->mirror(), xy, k, tri, where, hp, c.engine->stream()) != 0)
        return QDT_ERR_OUT_OF_MEMORY;
    // the walks the device gave up on, on the host
    const int nv = (int)M.v.size(), nh = (int)M.h.size();
    for (size_t i = 0; i < k; ++i)
    {
        if (where[i] != kLocUnresolved) continue;
        int       hull = -1;
        const int h0 = locate(M, c.ntris(), xy[2 * i], xy[2 * i + 1], &hull);
        if (h0 >= 0)
        {
            const LocResult r = classify(M.v.data(), M.h.data(), nv, nh, h0, xy[2 * i], xy[2 * i + 1], INT_MAX);
            tri[i] = r.tri;
            where[i] = r.where;
            hp[i] = h0;
        }
        else
        {
            tri[i] = -1;
            where[i] = kLocOutside;
            hp[i] = hull;
        }
    }
    return QDT_OK;
}

int mesh_trace_segments(Context& c, const size_t* v01, size_t k, int* status, int64_t* crossed)
{
    if (k == 0) return QDT_OK;
    // the checks of mesh_insert_constraint, in its order
    std::vector<int>    uw;
    std::vector<size_t> at;
    Mesh*               M = nullptr;
    for (size_t i = 0; i < k; ++i)
    {
        size_t v0 = v01[2 * i], v1 = v01[2 * i + 1];
        crossed[i] = 0;
        if (v0 >= c.rep.size() || v1 >= c.rep.size())
        {
            status[i] = QDT_ERR_INVALID_INDEX;
            continue;
        }
        v0 = c.rep[v0];
        v1 = c.rep[v1];
        if (v0 == v1)
        {
            status[i] = QDT_ERR_SAME_POINT;
            continue;
        }
        if (c.ntris() == 0)
        {
            status[i] = QDT_ERR_NO_TRIANGLES;
            continue;
        }
        if (!M) M = &ensure_mesh(c);
        const int u = v0 < M->o2l.size() ? M->o2l[v0] : -1;
        const int w = v1 < M->o2l.size() ? M->o2l[v1] : -1;
        if (u < 0 || w < 0)
        {
            status[i] = QDT_ERR_NO_TRIANGLES;
            continue;
        }
        uw.push_back(u);
        uw.push_back(w);
        at.push_back(i);
    }
    const size_t m = at.size();
    if (m == 0) return QDT_OK;
    if (M->h.size() > (size_t)INT_MAX || M->v.size() > (size_t)INT_MAX) return QDT_ERR_INTERNAL;
    std::vector<int> out(m), cr(m);
    if (!sync_mirror(c, *M)) return QDT_ERR_OUT_OF_MEMORY;
    if (mirror_trace(c.engine->mirror(), uw.data(), m, out.data(), cr.data(), c.engine->stream()) != 0)
        return QDT_ERR_OUT_OF_MEMORY;
    const int nv = (int)M->v.size(), nh = (int)M->h.size();
    for (size_t j = 0; j < m; ++j)
    {
        if (out[j] == kTraceUnresolved)
            out[j] = trace_segment(M->v.data(), M->h.data(), nv, nh, uw[2 * j], uw[2 * j + 1], INT_MAX, &cr[j]);
        static const int map[4] = { QDT_OK, QDT_ERR_THROUGH_POINT, QDT_ERR_CROSSES_CONSTRAINT, QDT_ERR_INTERNAL };
        status[at[j]] = (out[j] >= 0 && out[j] < 4) ? map[out[j]] : QDT_ERR_INTERNAL;
        crossed[at[j]] = cr[j];
    }
    return QDT_OK;
}

std::vector<int> mesh_insert_hints(Context& c, const double* xy, size_t k)
{
    std::vector<int> hints(k, -1);
    if (k < 2 || c.ntris() == 0 || !c.engine) return hints;
    Mesh& M = ensure_mesh(c);
    if (M.h.empty() || M.h.size() > (size_t)INT_MAX) return hints;
    // Without hints each walk crosses about sqrt(half-edges) triangles; a
    // stale mirror costs an upload of the whole mesh. Locate on the device
    // when the mirror is current, or when the walks saved outweigh the upload.
    const MeshMirror& mr = c.engine->mirror();
    const bool current = mr.mesh_id == M.id && mr.mesh_version == M.version && mr.nh == M.h.size();
    if (!current && (double)k < std::sqrt((double)M.h.size()) / 8.0) return hints;
    std::vector<double> q;
    std::vector<size_t> at;
    q.reserve(2 * k);
    at.reserve(k);
    for (size_t i = 0; i < k; ++i)
        if (std::isfinite(xy[2 * i]) && std::isfinite(xy[2 * i + 1]))
        {
            q.push_back(xy[2 * i]);
            q.push_back(xy[2 * i + 1]);
            at.push_back(i);
        }
    const size_t     m = at.size();
    std::vector<int> tri(m), where(m), he(m);
    if (m == 0 || mesh_locate(c, q.data(), m, tri.data(), where.data(), he.data()) != QDT_OK) return hints;
    for (size_t j = 0; j < m; ++j) hints[at[j]] = he[j];
    return hints;
}

}  // namespace qdtg
