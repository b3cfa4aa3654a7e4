// Host harness of the constraint trace and the point location the GPU runs
// (mesh_walk.cuh: trace_segment, walk and classify; tests/test_trace_host.py).
// Compiled with nvcc as a host program: the same source the device kernels
// k_mesh_trace and k_mesh_locate are built from, run here on the CPU. It
// builds the half-edge mesh of a triangulation the way the mesh builders lay
// it out (half-edges 3t, 3t+1, 3t+2 of triangle t, each vertex storing its
// first outgoing half-edge in triangle order),
// flags the constrained edges it is given, traces the queried segments and
// locates the queried points (a walk from a given half-edge, then the
// canonical answer).
//
// Input (binary file): int32 nv; float64 xy[2 nv]; int32 ntri;
// int32 tri[3 ntri]; int32 ncons; int32 cons[2 ncons]; int32 nq;
// int32 q[2 nq]; int32 nl; float64 p[2 nl]; int32 start[nl]. Output: one
// line "status crossed" per segment, then one line "tri where" per point.
#include <climits>
#include <cstdio>
#include <map>
#include <utility>
#include <vector>

#include "mesh_walk.cuh"

using namespace qdtg;

template <class T>
static bool get(FILE* f, T* p, size_t n)
{
    return fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char** argv)
{
    if (argc != 2) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int nv = 0, nt = 0, nc = 0, nq = 0;
    if (!get(f, &nv, 1) || nv < 0) return 3;
    std::vector<double> xy(2 * (size_t)nv);
    if (!get(f, xy.data(), xy.size()) || !get(f, &nt, 1) || nt < 0) return 3;
    std::vector<int> tri(3 * (size_t)nt);
    if (!get(f, tri.data(), tri.size()) || !get(f, &nc, 1) || nc < 0) return 3;
    std::vector<int> cons(2 * (size_t)nc);
    if (!get(f, cons.data(), cons.size()) || !get(f, &nq, 1) || nq < 0) return 3;
    std::vector<int> q(2 * (size_t)nq);
    if (!get(f, q.data(), q.size())) return 3;
    int nl = 0;
    if (!get(f, &nl, 1) || nl < 0) return 3;
    std::vector<double> p(2 * (size_t)nl);
    std::vector<int>    start(nl);
    if (!get(f, p.data(), p.size()) || !get(f, start.data(), start.size())) return 3;
    fclose(f);

    std::vector<MeshVertex>   v(nv);
    std::vector<MeshHalfEdge> h(3 * (size_t)nt);
    for (int i = 0; i < nv; ++i) v[i] = MeshVertex{ xy[2 * i], xy[2 * i + 1], (uint32_t)i, -1 };
    std::map<std::pair<int, int>, int> dir;
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
        {
            const int a = tri[3 * t + k], b = tri[3 * t + (k + 1) % 3], e = 3 * t + k;
            if (a < 0 || a >= nv || b < 0 || b >= nv) return 4;
            h[e] = MeshHalfEdge{ a, -1, 3 * t + (k + 1) % 3, t, 0 };
            if (v[a].he < 0) v[a].he = e;
            dir[{ a, b }] = e;
        }
    for (auto& [ab, e] : dir)
    {
        const auto tw = dir.find({ ab.second, ab.first });
        if (tw != dir.end()) h[e].twin = tw->second;
    }
    for (int i = 0; i < nc; ++i)
    {
        const int a = cons[2 * i], b = cons[2 * i + 1];
        const auto e1 = dir.find({ a, b }), e2 = dir.find({ b, a });
        if (e1 == dir.end() && e2 == dir.end()) return 5;   // a constrained edge that is no edge
        if (e1 != dir.end()) h[e1->second].cons = 1;
        if (e2 != dir.end()) h[e2->second].cons = 1;
    }
    for (int i = 0; i < nq; ++i)
    {
        int       crossed = 0;
        const int st = trace_segment(v.data(), h.data(), nv, (int)h.size(), q[2 * i], q[2 * i + 1], INT_MAX, &crossed);
        printf("%d %d\n", st, crossed);
    }
    const int nh = (int)h.size();
    for (int i = 0; i < nl; ++i)
    {
        LocResult r = walk(v.data(), h.data(), nv, nh, start[i], p[2 * i], p[2 * i + 1], INT_MAX);
        if (r.where == kLocInside) r = classify(v.data(), h.data(), nv, nh, r.he, p[2 * i], p[2 * i + 1], INT_MAX);
        printf("%d %d\n", r.where == kLocOutside ? -1 : r.tri, r.where);
    }
    return 0;
}
