// Batch point location on the GPU (an extension of the reference's
// single-point locate_, GuibasStolfiDwyer_Wrapper.cpp:423-486): one thread
// per query point walks the mirrored half-edge mesh (mesh_walk.cuh) from a
// seed next to the point, then classifies it canonically. Walks that give up
// (a step limit, kept far above the expected walk length) are returned as
// unresolved and finished on the host.
//
// Index: the bounding box of the vertices (order keys, one atomic per warp),
// a grid of about two vertices per cell, and per cell the largest alive
// half-edge whose origin lies in it (atomicMax, so the index does not depend
// on the schedule).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "mesh_mirror.hpp"
#include "mesh_walk.cuh"

namespace qdtg {

namespace {

constexpr int kWalkCap = 1 << 16;   // steps before a device walk is handed to the host
constexpr int kRingCap = 4096;      // triangles around a vertex visited by classify

__device__ __forceinline__ unsigned long long order_key(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

inline double key_value(unsigned long long k)
{
    const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    double v;
    std::memcpy(&v, &b, 8);
    return v;
}

__global__ void k_mesh_box(const MeshVertex* __restrict__ v, size_t nv, unsigned long long* __restrict__ box)
{
    unsigned long long mnx = ~0ull, mny = ~0ull, mxx = 0, mxy = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x)
    {
        const unsigned long long kx = order_key(v[i].x), ky = order_key(v[i].y);
        mnx = min(mnx, kx), mny = min(mny, ky), mxx = max(mxx, kx), mxy = max(mxy, ky);
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicMin(&box[0], mnx);
        atomicMin(&box[1], mny);
        atomicMax(&box[2], mxx);
        atomicMax(&box[3], mxy);
    }
}

struct Grid
{
    int    gx, gy;
    double x0, y0, ix, iy;
    __device__ __forceinline__ int cx(double x) const
    {
        const double f = floor((x - x0) * ix);
        return f < 0.0 ? 0 : (f >= (double)(gx - 1) ? gx - 1 : (int)f);
    }
    __device__ __forceinline__ int cy(double y) const
    {
        const double f = floor((y - y0) * iy);
        return f < 0.0 ? 0 : (f >= (double)(gy - 1) ? gy - 1 : (int)f);
    }
};

__global__ void k_mesh_seed(const MeshVertex* __restrict__ v, const MeshHalfEdge* __restrict__ h, int nv, int nh,
    Grid g, int* __restrict__ seed, unsigned long long* __restrict__ any)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nh) return;
    const MeshHalfEdge he = h[e];
    if (he.org < 0 || he.org >= nv || he.next < 0 || he.next >= nh || he.tri < 0) return;
    const MeshVertex p = v[he.org];
    atomicMax(&seed[g.cy(p.y) * g.gx + g.cx(p.x)], e);
    if ((e & 1023) == 0) atomicMax(any, (unsigned long long)e + 1ull);
}

__global__ void k_mesh_locate(const MeshVertex* __restrict__ v, const MeshHalfEdge* __restrict__ h, int nv, int nh,
    Grid g, const int* __restrict__ seed, const unsigned long long* __restrict__ any, const double2* __restrict__ q,
    size_t k, int4* __restrict__ out)
{
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= k) return;
    const double2 p = q[i];
    const int     cx = g.cx(p.x), cy = g.cy(p.y);
    int           s = seed[cy * g.gx + cx];
    // an empty cell: the nearest non-empty cell within two rings
    for (int r = 1; s < 0 && r <= 2; ++r)
        for (int dy = -r; dy <= r && s < 0; ++dy)
            for (int dx = -r; dx <= r && s < 0; ++dx)
            {
                const int x = cx + dx, y = cy + dy;
                if (x >= 0 && y >= 0 && x < g.gx && y < g.gy) s = seed[y * g.gx + x];
            }
    if (s < 0)
    {
        const unsigned long long a = *any;
        s = a == 0ull ? 0 : (int)(a - 1);
    }
    LocResult r = walk(v, h, nv, nh, s, p.x, p.y, kWalkCap);
    if (r.where == kLocInside) r = classify(v, h, nv, nh, r.he, p.x, p.y, kRingCap);
    out[i] = make_int4(r.tri, r.where, r.he, 0);
}

// one thread per constraint segment (mesh vertices u, w): the trace outcome
// and the edges crossed
__global__ void k_mesh_trace(const MeshVertex* __restrict__ v, const MeshHalfEdge* __restrict__ h, int nv, int nh,
    const int2* __restrict__ uw, size_t k, int2* __restrict__ out)
{
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= k) return;
    const int2 s = uw[i];
    int        crossed = 0;
    const int  r = trace_segment(v, h, nv, nh, s.x, s.y, kWalkCap, &crossed);
    out[i] = make_int2(r, crossed);
}

inline unsigned blocks(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

template <class T>
int grow(T*& p, size_t& cap, size_t need)
{
    if (need <= cap && p) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const size_t want = std::max<size_t>(need + need / 4, 1024);
    if (cudaMalloc(&p, want * sizeof(T)) != cudaSuccess)
    {
        cudaGetLastError();
        p = nullptr;
        return -1;
    }
    cap = want;
    return 0;
}

int build_index(MeshMirror& m, cudaStream_t s)
{
    if (m.nv == 0 || m.nh == 0 || m.nh > 0x7FFFFFFFull) return -1;
    if (!m.box && cudaMalloc(&m.box, 8 * sizeof(unsigned long long)) != cudaSuccess)
    {
        cudaGetLastError();
        m.box = nullptr;
        return -1;
    }
    const unsigned long long init[5] = { ~0ull, ~0ull, 0ull, 0ull, 0ull };
    unsigned long long       hb[5];
    cudaMemcpyAsync(m.box, init, sizeof(init), cudaMemcpyHostToDevice, s);
    k_mesh_box<<<std::min<unsigned>(blocks(m.nv, 256), 152 * 4), 256, 0, s>>>(m.v, m.nv, m.box);
    ++launch_counter();
    cudaMemcpyAsync(hb, m.box, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    const double x0 = key_value(hb[0]), y0 = key_value(hb[1]), x1 = key_value(hb[2]), y1 = key_value(hb[3]);
    if (!(x1 >= x0) || !(y1 >= y0)) return -1;
    const double w = x1 - x0, hgt = y1 - y0;
    // about two vertices per cell, cells close to square
    const double cells = std::max(1.0, std::min((double)m.nv / 2.0, (double)(1 << 26)));
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
    const size_t nc = (size_t)gx * gy;
    if (grow(m.seed, m.cap_seed, nc) != 0) return -1;
    m.gx = gx;
    m.gy = gy;
    m.x0 = x0;
    m.y0 = y0;
    m.ix = (gx > 1 && w > 0) ? gx / w : 0.0;
    m.iy = (gy > 1 && hgt > 0) ? gy / hgt : 0.0;
    if (!std::isfinite(m.ix)) m.ix = 0.0;
    if (!std::isfinite(m.iy)) m.iy = 0.0;
    const Grid g{ m.gx, m.gy, m.x0, m.y0, m.ix, m.iy };
    cudaMemsetAsync(m.seed, 0xFF, nc * sizeof(int), s);
    // any alive half-edge, stored + 1 (0: none)
    k_mesh_seed<<<blocks(m.nh, 256), 256, 0, s>>>(m.v, m.h, (int)m.nv, (int)m.nh, g, m.seed, m.box + 4);
    ++launch_counter();
    m.indexed = cudaGetLastError() == cudaSuccess;
    return m.indexed ? 0 : -1;
}

}  // namespace

int mirror_reserve(MeshMirror& m, size_t nv, size_t nh)
{
    m.indexed = false;
    if (grow(m.v, m.cap_v, nv) != 0 || grow(m.h, m.cap_h, nh) != 0) return -1;
    return 0;
}

void mirror_free(MeshMirror& m) noexcept
{
    if (m.v) cudaFree(m.v);
    if (m.h) cudaFree(m.h);
    if (m.seed) cudaFree(m.seed);
    if (m.box) cudaFree(m.box);
    if (m.q) cudaFree(m.q);
    if (m.out) cudaFree(m.out);
    m = MeshMirror{};
}

int mirror_upload(MeshMirror& m, const MeshVertex* v, size_t nv, const MeshHalfEdge* h, size_t nh, cudaStream_t s)
{
    m.mesh_version = ~0ull;
    if (mirror_reserve(m, nv, nh) != 0) return -1;
    if (nv) cudaMemcpyAsync(m.v, v, nv * sizeof(MeshVertex), cudaMemcpyHostToDevice, s);
    if (nh) cudaMemcpyAsync(m.h, h, nh * sizeof(MeshHalfEdge), cudaMemcpyHostToDevice, s);
    m.nv = nv;
    m.nh = nh;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// k query slots: 16 bytes in (q) and 16 bytes out (out) each
static int query_buffers(MeshMirror& m, size_t k)
{
    if (k > m.cap_q || !m.q || !m.out)
    {
        if (m.q) cudaFree(m.q);
        if (m.out) cudaFree(m.out);
        m.q = nullptr;
        m.out = nullptr;
        m.cap_q = 0;
        const size_t want = std::max<size_t>(k + k / 4, 1024);
        if (cudaMalloc(&m.q, want * sizeof(double2)) != cudaSuccess ||
            cudaMalloc(&m.out, want * sizeof(int4)) != cudaSuccess)
        {
            cudaGetLastError();
            if (m.q) cudaFree(m.q);
            m.q = nullptr;
            m.out = nullptr;
            return -1;
        }
        m.cap_q = want;
    }
    return 0;
}

int mirror_locate(MeshMirror& m, const double* xy, size_t k, int* tri, int* where, int* he, cudaStream_t s)
{
    if (k == 0) return 0;
    if (m.nv > 0x7FFFFFFFull || m.nh > 0x7FFFFFFFull) return -1;
    if (!m.indexed && build_index(m, s) != 0) return -1;
    if (query_buffers(m, k) != 0) return -1;
    std::vector<int4> res(k);
    cudaMemcpyAsync(m.q, xy, k * sizeof(double2), cudaMemcpyHostToDevice, s);
    const Grid g{ m.gx, m.gy, m.x0, m.y0, m.ix, m.iy };
    k_mesh_locate<<<blocks(k, 128), 128, 0, s>>>(m.v, m.h, (int)m.nv, (int)m.nh, g, m.seed, m.box + 4, m.q, k, m.out);
    ++launch_counter();
    cudaMemcpyAsync(res.data(), m.out, k * sizeof(int4), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    for (size_t i = 0; i < k; ++i)
    {
        tri[i] = res[i].x;
        where[i] = res[i].y;
        he[i] = res[i].z;
    }
    return 0;
}

int mirror_trace(MeshMirror& m, const int* uw, size_t k, int* outcome, int* crossed, cudaStream_t s)
{
    if (k == 0) return 0;
    if (m.nv > 0x7FFFFFFFull || m.nh > 0x7FFFFFFFull) return -1;
    if (query_buffers(m, k) != 0) return -1;
    std::vector<int2> res(k);
    int2*             d_uw = reinterpret_cast<int2*>(m.q);     // 8 of the slot's 16 bytes
    int2*             d_out = reinterpret_cast<int2*>(m.out);
    cudaMemcpyAsync(d_uw, uw, k * sizeof(int2), cudaMemcpyHostToDevice, s);
    k_mesh_trace<<<blocks(k, 128), 128, 0, s>>>(m.v, m.h, (int)m.nv, (int)m.nh, d_uw, k, d_out);
    ++launch_counter();
    cudaMemcpyAsync(res.data(), d_out, k * sizeof(int2), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return -1;
    for (size_t i = 0; i < k; ++i)
    {
        outcome[i] = res[i].x;
        crossed[i] = res[i].y;
    }
    return 0;
}

}  // namespace qdtg
