// The half-edge mesh of the last batch result, built on the GPU for the first
// insertion or constraint on the handle (reference Wrapper.cpp:99-202, whose
// host builder mesh.cu also has). The arrays are those the host builder makes:
//
// * vertices are numbered in the order of their first appearance in the
//   triangle list: the first position of every point (atomicMin), a flag at
//   each first position, and an exclusive scan of the flags give the number;
//   a vertex's outgoing half-edge is its first position;
// * half-edge i is corner i of triangle i / 3, next = the following corner;
// * twins: the outgoing half-edges of every vertex are grouped (counts, scan,
//   a fill by atomic cursors; the order inside a group does not matter), and
//   the half-edge u -> w finds w -> u among w's outgoing half-edges. In a
//   triangulation the reverse of a directed edge is unique, so the result is
//   the host builder's.
#include <climits>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "engine.hpp"
#include "engine_kernels.hpp"
#include "mesh_layout.hpp"
#include "mesh_mirror.hpp"
#include "scan.cuh"

namespace qdtg {

namespace {

__global__ void k_mesh_first(const uint32_t* __restrict__ tris, uint32_t n3, uint32_t n, int* __restrict__ first)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const uint32_t o = tris[i];
    if (o < n) atomicMin(&first[o], (int)i);
}

struct FirstFlag
{
    const uint32_t* tris;
    const int*      first;
    uint32_t        n;
    __device__ __forceinline__ uint32_t operator()(size_t i) const
    {
        const uint32_t o = tris[i];
        return (o < n && first[o] == (int)i) ? 1u : 0u;
    }
};

__global__ void k_mesh_vertices(const int* __restrict__ first, const uint32_t* __restrict__ lid,
    const double2* __restrict__ pts, uint32_t n, uint32_t n3, int* __restrict__ o2l, MeshVertex* __restrict__ v)
{
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int f = first[o];
    if (f < 0 || (uint32_t)f >= n3)   // still the fill value: the point is in no triangle
    {
        o2l[o] = -1;
        return;
    }
    const uint32_t l = lid[f];
    o2l[o] = (int)l;
    const double2 p = pts[o];
    v[l] = MeshVertex{ p.x, p.y, o, f };
}

__global__ void k_mesh_halfedges(const uint32_t* __restrict__ tris, uint32_t n3, uint32_t n,
    const int* __restrict__ o2l, MeshHalfEdge* __restrict__ h, uint32_t* __restrict__ deg, uint32_t nv)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const uint32_t o = tris[i];
    const int      a = o < n ? o2l[o] : -1;
    const uint32_t c = i % 3, base = i - c;
    h[i] = MeshHalfEdge{ a, -1, (int)(base + (c + 1) % 3), (int)(i / 3), 0 };
    if (a >= 0 && (uint32_t)a < nv) atomicAdd(&deg[a], 1u);
}

__global__ void k_mesh_fill(const MeshHalfEdge* __restrict__ h, uint32_t n3, const uint32_t* __restrict__ off,
    uint32_t* __restrict__ cursor, uint32_t nv, uint32_t* __restrict__ adj)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const int a = h[i].org;
    if (a < 0 || (uint32_t)a >= nv) return;
    const uint32_t k = off[a] + atomicAdd(&cursor[a], 1u);
    if (k < n3) adj[k] = i;
}

__global__ void k_mesh_twins(MeshHalfEdge* __restrict__ h, uint32_t n3, const uint32_t* __restrict__ off,
    const uint32_t* __restrict__ deg, uint32_t nv, const uint32_t* __restrict__ adj)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const int u = h[i].org;
    const int nx = h[i].next;
    if (u < 0 || nx < 0 || (uint32_t)nx >= n3) return;
    const int w = h[nx].org;
    if (w < 0 || (uint32_t)w >= nv) return;
    const uint32_t b = off[w], e = min(b + deg[w], n3);
    for (uint32_t k = b; k < e; ++k)
    {
        const uint32_t j = adj[k];
        const int      jn = h[j].next;
        if (jn >= 0 && (uint32_t)jn < n3 && h[jn].org == u)
        {
            h[i].twin = (int)j;
            return;
        }
    }
}

inline unsigned grid(size_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

int mesh_build_device(const uint32_t* tris, const double2* pts, size_t n, size_t T, cudaStream_t s,
    MeshMirror& mir, MeshVec<int>& o2l, MeshVec<MeshVertex>& v, MeshVec<MeshHalfEdge>& h)
{
    if (T == 0 || 3 * T > 0x7FFFFFFFull || n > 0x7FFFFFFFull) return -1;
    const uint32_t n3 = (uint32_t)(3 * T), un = (uint32_t)n;
    // the vertices and half-edges are built in the mirror, which keeps them
    // for the batch point location
    mir.mesh_version = ~0ull;
    mir.nv = mir.nh = 0;
    if (mirror_reserve(mir, n, n3) != 0) return -1;
    // working memory: first[n], lid[3T], o2l[n], deg[n], off[n+1], cursor[n], adj[3T], scan scratch
    const size_t sw = scan_scratch_words(std::max<size_t>(n3, n + 1)) + 8;
    size_t       bytes = 0;
    auto         take = [&](size_t b) {
        const size_t o = bytes;
        bytes += (b + 255) & ~(size_t)255;
        return o;
    };
    const size_t o_first = take(n * 4), o_lid = take((size_t)n3 * 4), o_o2l = take(n * 4), o_deg = take(n * 4),
                 o_off = take((n + 1) * 4), o_cur = take(n * 4), o_adj = take((size_t)n3 * 4), o_scr = take(sw * 4),
                 o_tot = take(16);
    char* base = nullptr;
    if (cudaMalloc(&base, bytes) != cudaSuccess)
    {
        cudaGetLastError();
        return -1;
    }
    int*          first = reinterpret_cast<int*>(base + o_first);
    uint32_t*     lid = reinterpret_cast<uint32_t*>(base + o_lid);
    int*          d_o2l = reinterpret_cast<int*>(base + o_o2l);
    MeshVertex*   d_v = mir.v;
    MeshHalfEdge* d_h = mir.h;
    uint32_t*     deg = reinterpret_cast<uint32_t*>(base + o_deg);
    uint32_t*     off = reinterpret_cast<uint32_t*>(base + o_off);
    uint32_t*     cur = reinterpret_cast<uint32_t*>(base + o_cur);
    uint32_t*     adj = reinterpret_cast<uint32_t*>(base + o_adj);
    uint32_t*     scr = reinterpret_cast<uint32_t*>(base + o_scr);
    uint32_t*     tot = reinterpret_cast<uint32_t*>(base + o_tot);

    cudaMemsetAsync(first, 0x7F, n * 4, s);   // 0x7F7F7F7F: above every position (3 T < 2^31)
    cudaMemsetAsync(deg, 0, n * 4, s);
    cudaMemsetAsync(cur, 0, n * 4, s);
    cudaMemsetAsync(tot, 0, 16, s);
    k_mesh_first<<<grid(n3), 256, 0, s>>>(tris, n3, un, first);
    scan_exclusive(FirstFlag{ tris, first, un }, n3, lid, scr, tot, s);
    uint32_t nv = 0;
    int      rc = 0;
    if (cudaMemcpyAsync(&nv, tot, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess ||
        nv > n)
        rc = -1;
    if (rc == 0)
    {
        k_mesh_vertices<<<grid(n), 256, 0, s>>>(first, lid, pts, un, n3, d_o2l, d_v);
        k_mesh_halfedges<<<grid(n3), 256, 0, s>>>(tris, n3, un, d_o2l, d_h, deg, nv);
        scan_exclusive(ArrayIn{ deg }, nv, off, scr, nullptr, s);
        k_mesh_fill<<<grid(n3), 256, 0, s>>>(d_h, n3, off, cur, nv, adj);
        k_mesh_twins<<<grid(n3), 256, 0, s>>>(d_h, n3, off, deg, nv, adj);
        try
        {
            // capacity for later insertions (untouched pages cost nothing):
            // growing would copy the whole array
            auto room = [](size_t s) { return s + std::max<size_t>(s / 8, 1024); };
            o2l.reserve(room(n));
            v.reserve(room(nv));
            h.reserve(room(n3));
            o2l.resize(n);
            v.resize(nv);
            h.resize(n3);
        }
        catch (...)
        {
            rc = -2;
        }
        if (rc == 0)
        {
            cudaMemcpyAsync(o2l.data(), d_o2l, n * 4, cudaMemcpyDeviceToHost, s);
            if (nv) cudaMemcpyAsync(v.data(), d_v, (size_t)nv * sizeof(MeshVertex), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(h.data(), d_h, (size_t)n3 * sizeof(MeshHalfEdge), cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess) rc = -1;
        }
        if (rc == 0)
        {
            mir.nv = nv;
            mir.nh = n3;
        }
    }
    cudaGetLastError();
    cudaFree(base);
    return rc;
}

}  // namespace qdtg
