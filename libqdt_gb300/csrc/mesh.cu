// Incremental point insertion and constrained edges on the handle returned by
// the batch path (host code; not on the GPU hot path).
//
// The batch engine leaves triangles, representatives and points in the
// context. The first insertion or constraint builds a half-edge mesh from
// them (on the GPU when the engine still holds the result, k_mesh.cu; else
// here); afterwards the mesh and the context's triangle list change
// together. Both operations produce the constrained Delaunay triangulation
// of the new input directly, each with a published method:
//
// * insertion: the Bowyer-Watson cavity -- the triangles whose circumcircle
//   holds the new point strictly, grown from the triangle(s) that contain
//   it across unconstrained edges (and, for a point beyond the hull, the
//   hull edges it sees) -- replaced by the fan of the point over the
//   cavity's border. A constrained edge the point lies on is split into two
//   constrained edges.
// * constraints: the channel of triangles the open segment crosses (it is
//   refused when it runs through a vertex or crosses a constrained edge) is
//   removed and the two pseudo-polygons on either side of the segment are
//   triangulated by Anglada's recursion (1997): the base edge takes the
//   polygon vertex whose circle with it holds no other polygon vertex, and
//   the two sub-polygons it leaves are filled the same way.
//
// The results are the ones the reference's insertion and constraint calls
// produce (GuibasStolfiDwyer_Wrapper.cpp:531-876 and :878-1285: statuses,
// indices, and in general position the same triangles, the constrained
// Delaunay triangulation being unique there). An edit gives back exactly
// the triangle slots and half-edges it frees and appends the rest, so the
// triangle list stays dense and every half-edge of the mesh is in use. All
// geometric decisions use the exact predicates of predicates.cuh.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <utility>
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

// Directed edges of one edit looked up by their end points: open addressing
// with linear probing, at most half full, its storage kept from edit to
// edit.
struct EdgeTable
{
    static constexpr uint64_t kEmpty = ~0ull;   // no edge key: vertex ids are below 2^31
    std::vector<uint64_t>     key;
    std::vector<int>          val;
    int                       shift = 64;

    void reset(size_t n)
    {
        int bits = 4;
        while (((size_t)1 << bits) < 2 * n) ++bits;
        key.assign((size_t)1 << bits, kEmpty);
        val.resize((size_t)1 << bits);
        shift = 64 - bits;
    }
    size_t home(uint64_t k) const { return (size_t)((k * 0x9E3779B97F4A7C15ull) >> shift); }
    void   put(uint64_t k, int v)
    {
        const size_t m = key.size() - 1;
        size_t       i = home(k);
        while (key[i] != kEmpty && key[i] != k) i = (i + 1) & m;
        key[i] = k;
        val[i] = v;
    }
    int get(uint64_t k) const   // -1 when absent
    {
        const size_t m = key.size() - 1;
        for (size_t i = home(k);; i = (i + 1) & m)
        {
            if (key[i] == k) return val[i];
            if (key[i] == kEmpty) return -1;
        }
    }
};

struct Mesh
{
    MeshVec<MV>           v;
    MeshVec<HE>           h;        // every entry in use
    MeshVec<int>          o2l;      // point index -> mesh vertex, -1 when none
    std::vector<int>      t2h;      // triangle -> one of its half-edges
    std::vector<uint32_t> mark;     // per triangle: the stamp of the last edit that took it
    uint32_t              stamp = 0;
    SeedGrid              grid;
    int                   last = 0;   // a half-edge near the last edit: the next walk's default start
    uint64_t              id = next_id();   // identifies this mesh to the device mirror
    uint64_t              version = 0;      // bumped by every call that may change the mesh
    EdgeTable             fresh_edges, outer_edges;   // scratch of the constraint fill

    static uint64_t next_id()
    {
        static std::atomic<uint64_t> n{ 0 };
        return ++n;
    }
};

void mesh_destroy(Mesh* m) noexcept { delete m; }

namespace {

// ---- mesh navigation -------------------------------------------------------

inline int nxt(const Mesh& M, int e) { return M.h[e].next; }
inline int prv(const Mesh& M, int e) { return M.h[M.h[e].next].next; }
inline int dst(const Mesh& M, int e) { return M.h[M.h[e].next].org; }

// orientation of p against the half-edge e (> 0: p on its triangle's side)
inline int side(const Mesh& M, int e, double px, double py)
{
    const MV &A = M.v[M.h[e].org], &B = M.v[dst(M, e)];
    return orient2d_sign(A.x, A.y, B.x, B.y, px, py);
}
inline int orient3(const Mesh& M, int a, int b, int c)
{
    const MV &A = M.v[a], &B = M.v[b], &C = M.v[c];
    return orient2d_sign(A.x, A.y, B.x, B.y, C.x, C.y);
}
// > 0 when d lies strictly inside the circle through a, b, c (counter-clockwise)
inline int circle4(const Mesh& M, int a, int b, int c, int d)
{
    const MV &A = M.v[a], &B = M.v[b], &C = M.v[c], &D = M.v[d];
    return incircle_sign(A.x, A.y, B.x, B.y, C.x, C.y, D.x, D.y);
}
// > 0 when (px, py) lies strictly inside the circumcircle of triangle slot t
inline int circle_holds(const Mesh& M, int t, double px, double py)
{
    const int  e = M.t2h[t];
    const MV&  A = M.v[M.h[e].org];
    const MV&  B = M.v[dst(M, e)];
    const MV&  C = M.v[M.h[prv(M, e)].org];
    return incircle_sign(A.x, A.y, B.x, B.y, C.x, C.y, px, py);
}

// Visits the outgoing half-edges of vertex x, one per triangle around it:
// counter-clockwise from the stored one until the fan closes, and around a
// hull vertex then clockwise from the stored one to the hull. f returns true
// to stop; the result says whether it did.
template <class F>
bool around(const Mesh& M, int x, F&& f)
{
    const int s = M.v[x].he;
    if (s < 0) return false;
    const size_t cap = M.h.size() + 1;
    size_t       n = 0;
    for (int k = s;;)
    {
        if (f(k)) return true;
        const int t = M.h[prv(M, k)].twin;   // counter-clockwise neighbour
        if (t == s) return false;            // the fan closed: all visited
        if (t < 0 || ++n > cap) break;
        k = t;
    }
    for (int k = s;;)
    {
        const int t = M.h[k].twin;   // clockwise neighbour: the half-edge after the twin
        if (t < 0) return false;
        k = M.h[t].next;
        if (k == s || ++n > cap) return false;
        if (f(k)) return true;
    }
}

// A half-edge of the edge u-w (u -> w, or w -> u where only that side has a
// triangle), or -1.
int edge_between(const Mesh& M, int u, int w)
{
    int found = -1;
    around(M, u, [&](int k) {
        if (dst(M, k) == w) found = k;
        else if (M.h[prv(M, k)].org == w) found = prv(M, k);
        return found >= 0;
    });
    return found;
}

void set_constrained(Mesh& M, int e)
{
    M.h[e].cons = 1;
    if (M.h[e].twin >= 0) M.h[M.h[e].twin].cons = 1;
}

// the hull half-edge after / before hull half-edge e (interior on its left)
int hull_after(const Mesh& M, int e)
{
    int k = nxt(M, e);   // out of e's end; turn clockwise until the hull
    for (size_t n = 0; M.h[k].twin >= 0 && n <= M.h.size(); ++n) k = M.h[M.h[k].twin].next;
    return k;
}
int hull_before(const Mesh& M, int e)
{
    int k = prv(M, e);   // into e's start; turn counter-clockwise until the hull
    for (size_t n = 0; M.h[k].twin >= 0 && n <= M.h.size(); ++n) k = prv(M, M.h[k].twin);
    return k;
}

// A fresh stamp for marking the triangles one edit takes.
uint32_t new_stamp(Mesh& M, size_t ntri)
{
    if (M.mark.size() < ntri) M.mark.resize(ntri, 0);
    if (++M.stamp == 0)
    {
        std::fill(M.mark.begin(), M.mark.end(), 0u);
        M.stamp = 1;
    }
    return M.stamp;
}

// ---- writing triangles -----------------------------------------------------

// Triangle slots and half-edge ids for the triangles an edit makes: first
// the ones it removed, then new ones at the end of the arrays.
struct Reuse
{
    std::vector<int> slots, hes;
    size_t           ns = 0, nh = 0;

    size_t slot(const Context& c) { return ns < slots.size() ? (size_t)slots[ns++] : c.ntris(); }
    int    he(Mesh& M)
    {
        if (nh < hes.size()) return hes[nh++];
        M.h.push_back(HE{ -1, -1, -1, -1, 0 });
        return (int)M.h.size() - 1;
    }
    bool all_used() const { return ns == slots.size() && nh == hes.size(); }
};

// Triangle slot t (t == ntris() appends) becomes e0 -> e1 -> e2 with origins
// a, b, d, counter-clockwise; twins and constraint flags are left to the
// caller.
void put_triangle(Context& c, Mesh& M, size_t t, int e0, int e1, int e2, int a, int b, int d)
{
    const int ti = (int)t;
    M.h[e0].org = a, M.h[e0].next = e1, M.h[e0].tri = ti;
    M.h[e1].org = b, M.h[e1].next = e2, M.h[e1].tri = ti;
    M.h[e2].org = d, M.h[e2].next = e0, M.h[e2].tri = ti;
    const uint32_t o[3] = { M.v[a].orig, M.v[b].orig, M.v[d].orig };
    if (t == c.ntris())
    {
        c.tris.insert(c.tris.end(), o, o + 3);
        M.t2h.push_back(e0);
    }
    else
    {
        std::copy(o, o + 3, c.tris.begin() + 3 * t);
        M.t2h[t] = e0;
    }
}

// Gives the triangles in `slots` to r: their slots and half-edges.
void reuse_triangles(const Mesh& M, const std::vector<int>& slots, Reuse& r)
{
    r.slots = slots;
    r.hes.clear();
    for (int t : slots)
    {
        const int e = M.t2h[t];
        r.hes.push_back(e);
        r.hes.push_back(nxt(M, e));
        r.hes.push_back(prv(M, e));
    }
}

inline uint64_t edge_key(int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

// ---- point location --------------------------------------------------------

// A half-edge of a triangle that contains (x, y) (border included), or -1
// with *seen set to a hull half-edge whose outer side the point lies
// strictly on. The walk of mesh_walk.cuh first; a scan of every triangle,
// then of every hull edge, when it gives up.
int find_point(const Mesh& M, int start, double x, double y, int* seen, size_t* steps)
{
    *seen = -1;
    const int nv = (int)M.v.size(), nh = (int)M.h.size();
    if (nh == 0) return -1;
    if (start < 0 || start >= nh) start = (M.last >= 0 && M.last < nh) ? M.last : 0;
    int             n = 0;
    const int       cap = (int)std::min<size_t>(M.t2h.size() + 16, (size_t)INT_MAX);
    const LocResult r = walk(M.v.data(), M.h.data(), nv, nh, start, x, y, cap, &n);
    if (steps) *steps = (size_t)n;
    if (r.where == kLocInside) return r.he;
    if (r.where == kLocOutside)
    {
        *seen = r.he;
        return -1;
    }
    for (size_t t = 0; t < M.t2h.size(); ++t)
    {
        const int e = M.t2h[t];
        if (side(M, e, x, y) >= 0 && side(M, nxt(M, e), x, y) >= 0 && side(M, prv(M, e), x, y) >= 0) return e;
    }
    for (int e = 0; e < nh; ++e)
        if (M.h[e].twin < 0 && side(M, e, x, y) < 0)
        {
            *seen = e;
            return -1;
        }
    return -1;
}

// Builds the half-edge mesh from the context's triangles (what the reference
// builds at Wrapper.cpp:99-202): vertices numbered by first appearance in the
// triangle list, three half-edges per triangle, twins matched through the
// outgoing half-edges grouped by origin.
void build_mesh(Context& c, Mesh& M)
{
    const size_t T = c.ntris();
    M.v.clear();
    M.h.clear();
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

int insert_by_rebuild(Context& c, double x, double y)
{
    c.points.push_back(x);
    c.points.push_back(y);
    return rebuild_from_points(c);
}

// One border edge of an insertion cavity: the new triangle (a, b, p) takes
// it, and its half-edge a -> b faces `ext` (-1 on the hull).
struct Border
{
    int a, b, ext, cons;
};

// The Bowyer-Watson cavity of (x, y): `in` is a half-edge of a triangle that
// contains the point (or -1 with `seen` a hull edge the point sees). The
// cavity grows from the triangle(s) that contain the point (or from the
// triangles behind the hull edges it sees) into neighbours whose
// circumcircle holds the point strictly, crossing an edge only outward (the
// point strictly on the near side) and never a constrained edge. Its border
// must be strictly visible from the point; a triangle whose border edge is
// not (one hidden behind a constrained edge) is excluded and the cavity is
// grown again. Fills the cavity's triangle slots, its border in a fixed
// order, and the constrained edge the point splits (split_a, split_b; -1
// when none). false when no star-shaped cavity is found, which exact
// predicates rule out; the mesh is not changed here.
bool insertion_cavity(Context& c, Mesh& M, int in, int seen, double x, double y, std::vector<int>& cav,
    std::vector<Border>& border, int& split_a, int& split_b)
{
    std::vector<int> sees;   // hull edges the point sees from outside, in hull order
    if (in < 0)
    {
        // they form one chain: listed from its first edge in hull order
        auto sees_it = [&](int e) { return side(M, e, x, y) < 0; };
        int  first = seen;
        for (int e = hull_before(M, seen); e != seen && sees_it(e); e = hull_before(M, e)) first = e;
        sees.push_back(first);
        for (int e = hull_after(M, first); e != first && sees_it(e); e = hull_after(M, e)) sees.push_back(e);
    }
    std::vector<int> excluded;
    auto             is_excluded = [&](int t) { return std::find(excluded.begin(), excluded.end(), t) != excluded.end(); };
    for (int round = 0; round < 256; ++round)
    {
        cav.clear();
        border.clear();
        split_a = split_b = -1;
        const uint32_t stamp = new_stamp(M, c.ntris());
        auto           taken = [&](int t) { return M.mark[t] == stamp; };
        auto           take = [&](int t) {
            M.mark[t] = stamp;
            cav.push_back(t);
        };
        size_t seeds = 0;
        if (in >= 0)
        {
            take(M.h[in].tri);
            // a point on an edge takes the triangle across it too, across a
            // constrained edge as well (which it splits)
            for (int k = 0, e = in; k < 3; ++k, e = nxt(M, e))
                if (side(M, e, x, y) == 0)
                {
                    const int tw = M.h[e].twin;
                    if (tw >= 0 && !taken(M.h[tw].tri)) take(M.h[tw].tri);
                    if (M.h[e].cons)
                    {
                        split_a = M.h[e].org;
                        split_b = dst(M, e);
                    }
                }
            seeds = cav.size();
        }
        else
            for (int e : sees)
            {
                // a constrained hull edge hides the triangle behind it
                const int t = M.h[e].tri;
                if (!M.h[e].cons && !taken(t) && !is_excluded(t) && circle_holds(M, t, x, y) > 0) take(t);
            }
        for (size_t i = 0; i < cav.size(); ++i)
        {
            const int e0 = M.t2h[cav[i]];
            for (int k = 0, e = e0; k < 3; ++k, e = nxt(M, e))
            {
                const int tw = M.h[e].twin;
                if (tw < 0 || M.h[e].cons) continue;
                const int t = M.h[tw].tri;
                if (taken(t) || is_excluded(t) || side(M, e, x, y) <= 0) continue;
                if (circle_holds(M, t, x, y) > 0) take(t);
            }
        }
        // the border: edges of cavity triangles whose other side stays, in
        // the order the triangles joined; then the seen hull edges whose
        // triangle stays, crossed from outside
        int hidden = -1;
        for (size_t i = 0; i < cav.size() && hidden < 0; ++i)
        {
            const int e0 = M.t2h[cav[i]];
            for (int k = 0, e = e0; k < 3; ++k, e = nxt(M, e))
            {
                const int tw = M.h[e].twin;
                if (tw >= 0 && taken(M.h[tw].tri)) continue;
                const int s = side(M, e, x, y);
                if (s > 0)
                    border.push_back(Border{ M.h[e].org, dst(M, e), tw, M.h[e].cons });
                else if (tw < 0 && ((s == 0 && i < seeds) ||
                                    (s < 0 && std::find(sees.begin(), sees.end(), e) != sees.end())))
                    continue;   // a hull edge the point splits, or one it sees: inside the cavity
                else
                {
                    hidden = cav[i];
                    break;
                }
            }
        }
        if (hidden >= 0)
        {
            if (in >= 0 && std::find(cav.begin(), cav.begin() + seeds, hidden) != cav.begin() + seeds) return false;
            excluded.push_back(hidden);
            continue;
        }
        for (int e : sees)
            if (!taken(M.h[e].tri)) border.push_back(Border{ dst(M, e), M.h[e].org, e, M.h[e].cons });
        return !border.empty();
    }
    return false;
}

}  // namespace

int mesh_insert_point(Context& c, double x, double y, bool, int hint)
{
    if (c.ntris() == 0) return insert_by_rebuild(c, x, y);
    Mesh& M = ensure_mesh(c);
    if (M.h.empty()) return insert_by_rebuild(c, x, y);
    ++M.version;

    int    seen = -1;
    size_t steps = 0;
    if (hint < 0) hint = seed_start(M, x, y);
    int in = find_point(M, hint, x, y, &seen, &steps);
    seed_account(M, steps);
    if (in < 0 && seen < 0) return insert_by_rebuild(c, x, y);
    if (in >= 0)
    {
        // a point equal to a vertex is a corner of the triangle it was found in
        for (int k = 0, e = in; k < 3; ++k, e = nxt(M, e))
        {
            const MV& q = M.v[M.h[e].org];
            if (q.x == x && q.y == y)
            {
                c.points.push_back(x);
                c.points.push_back(y);
                c.rep.push_back(q.orig);
                return QDT_OK;
            }
        }
        // the cavity grows from the canonical containing triangle (the
        // smaller one when the point is on an edge): the triangle order of
        // the result does not depend on where the walk began
        const LocResult cl = classify(M.v.data(), M.h.data(), (int)M.v.size(), (int)M.h.size(), in, x, y, INT_MAX);
        if ((cl.where == kLocInside || cl.where == kLocEdge) && cl.tri >= 0 && cl.tri < (int)M.t2h.size())
            in = M.t2h[cl.tri];
    }

    std::vector<int>    cav;
    std::vector<Border> border;
    int                 split_a = -1, split_b = -1;
    if (!insertion_cavity(c, M, in, seen, x, y, cav, border, split_a, split_b)) return QDT_ERR_INTERNAL;

    // the new vertex
    const uint32_t id = (uint32_t)c.npoints();
    c.points.push_back(x);
    c.points.push_back(y);
    c.rep.push_back(id);
    ++c.unique_points;
    const int p = (int)M.v.size();
    M.v.push_back(MV{ x, y, id, -1 });
    if (M.o2l.size() <= id) M.o2l.resize(id + 1, -1);
    M.o2l[id] = p;
    if (!M.grid.cell.empty()) M.grid.cell[seed_cell(M.grid, x, y)] = p;

    // the fan of p over the border; spokes b -> p and p -> b pair up by b
    Reuse r;
    reuse_triangles(M, cav, r);
    std::vector<std::pair<int, int>> into, out;   // (b, b -> p), (a, p -> a)
    into.reserve(border.size());
    out.reserve(border.size());
    int first_spoke = -1;
    for (const Border& q : border)
    {
        const size_t t = r.slot(c);
        const int    e0 = r.he(M), e1 = r.he(M), e2 = r.he(M);
        put_triangle(c, M, t, e0, e1, e2, q.a, q.b, p);
        M.h[e0].twin = q.ext;
        M.h[e0].cons = q.cons;
        if (q.ext >= 0) M.h[q.ext].twin = e0;
        M.h[e1].twin = M.h[e2].twin = -1;
        M.h[e1].cons = M.h[e2].cons = 0;
        // both ends get a half-edge that survives: the old one may lie in a
        // cavity slot now reused (the last end of an open border, after a
        // point outside the hull, starts no border edge)
        M.v[q.b].he = e1;
        M.v[q.a].he = e0;
        into.emplace_back(q.b, e1);
        out.emplace_back(q.a, e2);
        if (first_spoke < 0) first_spoke = e2;
    }
    if (!r.all_used()) return QDT_ERR_INTERNAL;
    std::sort(into.begin(), into.end());
    std::sort(out.begin(), out.end());
    for (size_t i = 0, j = 0; i < into.size() && j < out.size();)
    {
        if (into[i].first < out[j].first) ++i;
        else if (out[j].first < into[i].first) ++j;
        else
        {
            M.h[into[i].second].twin = out[j].second;
            M.h[out[j].second].twin = into[i].second;
            ++i, ++j;
        }
    }
    M.v[p].he = first_spoke;
    // the two halves of a split constrained edge stay constrained; on the
    // hull one half is an outgoing spoke only (p -> split end, no twin)
    if (split_a >= 0)
    {
        for (const auto& s : into)
            if (s.first == split_a || s.first == split_b) set_constrained(M, s.second);
        for (const auto& s : out)
            if (s.first == split_a || s.first == split_b) set_constrained(M, s.second);
    }
    M.last = M.t2h[M.h[first_spoke].tri];
    return QDT_OK;
}

namespace {

// The triangles the open segment u-w crosses, from u to w, and the vertices
// on either side of it in the same order.
struct Channel
{
    std::vector<int> tris;
    std::vector<int> left, right;
};

// Finds the triangle at u that the segment leaves through, then crosses one
// edge at a time to w. QDT_OK, QDT_ERR_THROUGH_POINT (a vertex on the open
// segment), QDT_ERR_CROSSES_CONSTRAINT, or QDT_ERR_INTERNAL on a broken
// mesh; whichever comes first along the segment decides.
int open_channel(const Mesh& M, int u, int w, Channel& ch)
{
    int  leave = -1;
    bool through = false;
    around(M, u, [&](int k) {
        // triangle (u, x, y): the segment leaves through x-y when it runs
        // strictly between u->x and u->y
        const int x = dst(M, k), y = M.h[prv(M, k)].org;
        const int ox = orient3(M, u, x, w), oy = orient3(M, u, y, w);
        if (ox > 0 && oy < 0) leave = nxt(M, k);
        else if ((ox == 0 && same_direction(M.v[u], M.v[x], M.v[w])) ||
                 (oy == 0 && same_direction(M.v[u], M.v[y], M.v[w])))
            through = true;
        return leave >= 0 || through;
    });
    if (through) return QDT_ERR_THROUGH_POINT;
    if (leave < 0) return QDT_ERR_INTERNAL;
    ch.tris.push_back(M.h[leave].tri);
    // `leave` runs from the vertex right of u->w to the one on its left
    for (size_t n = 0; n <= M.t2h.size(); ++n)
    {
        if (M.h[leave].cons) return QDT_ERR_CROSSES_CONSTRAINT;
        const int rv = M.h[leave].org, lv = dst(M, leave);
        if (ch.right.empty() || ch.right.back() != rv) ch.right.push_back(rv);
        if (ch.left.empty() || ch.left.back() != lv) ch.left.push_back(lv);
        const int back = M.h[leave].twin;   // lv -> rv in the next triangle
        if (back < 0) return QDT_ERR_INTERNAL;
        ch.tris.push_back(M.h[back].tri);
        const int q = M.h[prv(M, back)].org;
        if (q == w) return QDT_OK;
        const int o = orient3(M, u, w, q);
        if (o == 0) return QDT_ERR_THROUGH_POINT;
        leave = o > 0 ? nxt(M, back) : prv(M, back);   // rv -> q, or q -> lv
    }
    return QDT_ERR_INTERNAL;
}

struct Tri3
{
    int a, b, c;
};

// Anglada's triangulation of the pseudo-polygon a, b, poly[0], ...,
// poly[k-1] (counter-clockwise, a -> b its base edge): the base takes the
// vertex whose circle with it holds no other polygon vertex (the first one
// on ties), and the polygons on its two sides are filled the same way.
// false if a triangle would not be strictly counter-clockwise.
bool fill_polygon(const Mesh& M, int a, int b, const std::vector<int>& poly, std::vector<Tri3>& out)
{
    struct Part
    {
        int    a, b;
        size_t lo, hi;
    };
    // the polygon's coordinates side by side, as the scans read them
    std::vector<double> px(poly.size()), py(poly.size());
    for (size_t i = 0; i < poly.size(); ++i)
    {
        px[i] = M.v[poly[i]].x;
        py[i] = M.v[poly[i]].y;
    }
    std::vector<Part> todo{ Part{ a, b, 0, poly.size() } };
    while (!todo.empty())
    {
        const Part q = todo.back();
        todo.pop_back();
        if (q.lo >= q.hi) continue;
        const MV& A = M.v[q.a];
        const MV& B = M.v[q.b];
        size_t    best = q.lo;
        for (size_t i = q.lo + 1; i < q.hi; ++i)
            if (incircle_sign(A.x, A.y, B.x, B.y, px[best], py[best], px[i], py[i]) > 0) best = i;
        const int c = poly[best];
        if (orient3(M, q.a, q.b, c) <= 0) return false;
        out.push_back(Tri3{ q.a, q.b, c });
        todo.push_back(Part{ c, q.b, q.lo, best });      // b, poly[lo..best), c
        todo.push_back(Part{ q.a, c, best + 1, q.hi });  // c, poly(best..hi), a
    }
    return true;
}

// Replaces the channel by the triangulations of its two sides with the
// edge u-w between them, constrained.
int fill_channel(Context& c, Mesh& M, int u, int w, const Channel& ch)
{
    // left side: u, w, then its vertices back from w; right side: w, u, then
    // its vertices from u
    std::vector<int>  lpoly(ch.left.rbegin(), ch.left.rend());
    std::vector<Tri3> made;
    if (!fill_polygon(M, u, w, lpoly, made) || !fill_polygon(M, w, u, ch.right, made)) return QDT_ERR_INTERNAL;
    if (made.size() != ch.tris.size()) return QDT_ERR_INTERNAL;

    // the channel's border half-edges, each with the half-edge facing it
    // from outside and its constraint flag, keyed as the new triangles run
    // them
    const uint32_t stamp = new_stamp(M, c.ntris());
    for (int t : ch.tris) M.mark[t] = stamp;
    struct Outer
    {
        uint64_t key;
        int      ext, cons;
    };
    std::vector<Outer> outer;
    // Constrained edges with channel triangles on both sides. The segment
    // crosses none of them (open_channel refuses that): each joins a vertex
    // whose whole fan lies in the channel to a neighbour on the same side of
    // the segment, an antenna of that side's pseudo-polygon. The fill keeps
    // the edge (a polygon edge); it must keep the flag too.
    std::vector<uint64_t> antennas;
    for (int t : ch.tris)
    {
        const int e0 = M.t2h[t];
        for (int k = 0, e = e0; k < 3; ++k, e = nxt(M, e))
        {
            const int tw = M.h[e].twin;
            if (tw >= 0 && M.mark[M.h[tw].tri] == stamp)
            {
                if (M.h[e].cons) antennas.push_back(edge_key(M.h[e].org, dst(M, e)));
                continue;
            }
            outer.push_back(Outer{ edge_key(M.h[e].org, dst(M, e)), tw, M.h[e].cons });
        }
    }
    EdgeTable& ot = M.outer_edges;
    ot.reset(outer.size());
    for (size_t i = 0; i < outer.size(); ++i) ot.put(outer[i].key, (int)i);

    Reuse r;
    reuse_triangles(M, ch.tris, r);
    EdgeTable& ft = M.fresh_edges;   // key of a -> b: its new half-edge
    ft.reset(3 * made.size());
    std::vector<int> made_he(3 * made.size());
    for (size_t i = 0; i < made.size(); ++i)
    {
        const Tri3&  q = made[i];
        const size_t t = r.slot(c);
        const int    e0 = r.he(M), e1 = r.he(M), e2 = r.he(M);
        put_triangle(c, M, t, e0, e1, e2, q.a, q.b, q.c);
        const int v3[3] = { q.a, q.b, q.c }, e3[3] = { e0, e1, e2 };
        for (int k = 0; k < 3; ++k)
        {
            ft.put(edge_key(v3[k], v3[(k + 1) % 3]), e3[k]);
            made_he[3 * i + k] = e3[k];
            M.h[e3[k]].twin = -1;
            M.h[e3[k]].cons = 0;
            M.v[v3[k]].he = e3[k];
        }
    }
    if (!r.all_used()) return QDT_ERR_INTERNAL;
    for (size_t i = 0; i < made.size(); ++i)
    {
        const int v3[3] = { made[i].a, made[i].b, made[i].c };
        for (int k = 0; k < 3; ++k)
        {
            const int a = v3[k], b = v3[(k + 1) % 3];
            const int e = made_he[3 * i + k];
            const int in = ft.get(edge_key(b, a));
            if (in >= 0)
            {
                M.h[e].twin = in;   // a diagonal, or the new edge u-w
                continue;
            }
            const int o = ot.get(edge_key(a, b));
            if (o < 0) return QDT_ERR_INTERNAL;
            M.h[e].twin = outer[o].ext;
            M.h[e].cons = outer[o].cons;
            if (outer[o].ext >= 0) M.h[outer[o].ext].twin = e;
        }
    }
    for (const uint64_t k : antennas)
    {
        const int e = ft.get(k);
        if (e < 0) return QDT_ERR_INTERNAL;
        set_constrained(M, e);
    }
    const int uw = ft.get(edge_key(u, w));
    if (uw < 0) return QDT_ERR_INTERNAL;
    set_constrained(M, uw);
    M.last = uw;
    return QDT_OK;
}

}  // namespace

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
    const int e = edge_between(M, u, w);
    if (e >= 0)
    {
        set_constrained(M, e);
        return QDT_OK;
    }
    Channel   ch;
    const int st = open_channel(M, u, w, ch);
    if (st != QDT_OK) return st;
    return fill_channel(c, M, u, w, ch);
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
        const int h0 = find_point(M, -1, xy[2 * i], xy[2 * i + 1], &hull, nullptr);
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
