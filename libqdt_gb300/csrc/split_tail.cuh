// The Dwyer split levels of one small node in shared memory.
//
// Once a node holds at most kTailMax points, one thread block runs all of
// its remaining depths with the marks of the per-depth kernels (side = 1 for
// the points at or after the node's middle in the splitting order; seam
// coordinates for the upper depths of a single set) and their stable
// partitions of the other order, on the node's slice of both orders, and
// writes the final orders once. Inside the block the points go by local ids
// (their positions in the slice of the frame-0 order), so the side flags and
// both orders live in shared memory; `loc` (one word per point id of scratch)
// maps a point to its local id once. The input and output orders may be the
// same buffers: a block reads its whole slice before it writes it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "scan.cuh"

namespace qdtg {

constexpr int kTailThreads = 512;
constexpr int kTailItems = 8;
constexpr int kTailMax = kTailThreads * kTailItems;
constexpr int kTailSmem = kTailMax * (4 + 3 * 2 + 2 + 1) + 64 * 4;

// the first depth at which every node of a set of ms points holds at most
// kTailMax points (node sizes at depth d are at most ceil(ms / 2^d))
__host__ __device__ inline int tail_depth(int ms)
{
    int d = 0;
    while ((((long long)ms + (1ll << d) - 1) >> d) > kTailMax) ++d;
    return d;
}

// the depth a set of ms points splits down to (split_levels: the first depth
// whose nodes all hold fewer than 4 points)
__host__ __device__ inline int split_depth(int ms)
{
    int d = 0;
    while ((((long long)ms + (1ll << d) - 1) >> d) >= 4) ++d;
    return d;
}

// the node of depth at most d0 + levels holding set position i, from the
// node [lo, hi) of depth d0 down (the halving of node_of); returns the
// levels descended
__device__ __forceinline__ int node_below(int lo, int hi, int levels, int i, int& nlo, int& nhi)
{
    for (int l = 0; l < levels; ++l)
    {
        if (hi - lo < 4)
        {
            nlo = lo, nhi = hi;
            return l;
        }
        const int mid = lo + (hi - lo) / 2;
        if (i < mid) hi = mid;
        else lo = mid;
    }
    nlo = lo, nhi = hi;
    return levels;
}

// One block: the node [lo, hi) (set positions) at depth d0 of a set of ms
// points that starts at global position base and splits down to depth D.
// Orders hold point ids below nids. seam (single set only, else nullptr)
// receives the cut coordinate of every node of depth at most kSeamDepth.
__device__ inline void split_tail_node(const uint32_t* Ain, const uint32_t* Bin, uint32_t* Aout, uint32_t* Bout,
    uint32_t* __restrict__ loc, const double2* __restrict__ ucoord, double* __restrict__ seam, int ms, int base,
    int lo, int hi, int d0, int D, uint32_t nids, uint32_t* tsm)
{
    uint32_t* gid = tsm;                                            // point of each local id
    uint32_t* ssm = tsm + kTailMax;                                 // block scan
    uint16_t* a = reinterpret_cast<uint16_t*>(ssm + 64);            // frame-0 order (local ids)
    uint16_t* b = a + kTailMax;                                     // frame-1 order
    uint16_t* t = b + kTailMax;                                     // partition target
    uint16_t* r = t + kTailMax;                                     // right-side points before each position
    uint8_t*  side = reinterpret_cast<uint8_t*>(r + kTailMax);      // by local id
    const int sz = hi - lo;
    if (sz > kTailMax || sz < 0) return;   // the host sizes the nodes so that this never holds
    for (int j = threadIdx.x; j < sz; j += blockDim.x)
    {
        const uint32_t p = Ain[base + lo + j];
        gid[j] = p;
        a[j] = (uint16_t)j;
        if (p < nids) loc[p] = (uint32_t)j;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < sz; j += blockDim.x)
    {
        const uint32_t p = Bin[base + lo + j];
        const uint32_t l = p < nids ? loc[p] : 0u;
        b[j] = (uint16_t)(l < (uint32_t)sz ? l : 0u);   // always in range: both orders hold the node's points
    }
    __syncthreads();
    const int rowbase = threadIdx.x * kTailItems;
    for (int d = d0; d < D; ++d)
    {
        uint16_t* S = (d & 1) ? b : a;
        uint16_t* O = (d & 1) ? a : b;
        for (int j = threadIdx.x; j < sz; j += blockDim.x)
        {
            const int i = lo + j;
            int       nlo, nhi;
            const int dep = d0 + node_below(lo, hi, d - d0, i, nlo, nhi);
            uint8_t   s = 0;
            if (dep == d && nhi - nlo >= 4)
            {
                const int mid = nlo + (nhi - nlo) / 2;
                s = (i >= mid) ? 1 : 0;
                if (seam && i == mid && d <= kSeamDepth)
                {
                    long long k = 0;
                    int       x = 0, y = ms;
                    for (int l = 0; l < d; ++l)
                    {
                        const int c = x + (y - x) / 2;
                        if (i < c) y = c, k = 2 * k;
                        else x = c, k = 2 * k + 1;
                    }
                    const double2 p = ucoord[min(gid[S[j]], nids - 1)];
                    seam[(1ll << d) + k] = (d & 1) ? p.y : p.x;
                }
            }
            side[S[j]] = s;
        }
        __syncthreads();
        uint32_t cnt = 0;
        for (int q = 0; q < kTailItems; ++q)
            if (rowbase + q < sz) cnt += side[O[rowbase + q]];
        uint32_t total;
        uint32_t run = block_excl_scan(cnt, ssm, &total);
        for (int q = 0; q < kTailItems; ++q)
            if (rowbase + q < sz)
            {
                r[rowbase + q] = (uint16_t)run;
                run += side[O[rowbase + q]];
            }
        __syncthreads();
        for (int q = 0; q < kTailItems; ++q)
        {
            const int j = rowbase + q;
            if (j >= sz) break;
            int            nlo, nhi;
            const int      dep = d0 + node_below(lo, hi, d - d0, lo + j, nlo, nhi);
            const uint16_t p = O[j];
            if (dep != d || nhi - nlo < 4)
            {
                t[j] = p;
                continue;
            }
            const int l0 = nlo - lo, mid = l0 + (nhi - nlo) / 2;
            const int rb = (int)(uint16_t)(r[j] - r[l0]);
            const int to = side[p] ? mid + rb : l0 + (j - l0 - rb);
            if (to >= 0 && to < sz) t[to] = p;   // always: both orders hold the node's points
        }
        __syncthreads();
        if (d & 1)
        {
            uint16_t* x = a;
            a = t;
            t = x;
        }
        else
        {
            uint16_t* x = b;
            b = t;
            t = x;
        }
    }
    for (int j = threadIdx.x; j < sz; j += blockDim.x)
    {
        Aout[base + lo + j] = gid[a[j]];
        Bout[base + lo + j] = gid[b[j]];
    }
}

// the node k of depth d of a set of ms points, as set positions [lo, hi)
__host__ __device__ inline void node_at(int ms, int d, uint32_t k, int& lo, int& hi)
{
    lo = 0, hi = ms;
    for (int l = 0; l < d; ++l)
    {
        const int mid = lo + (hi - lo) / 2;
        if ((k >> (d - 1 - l)) & 1u) lo = mid;
        else hi = mid;
    }
}

}  // namespace qdtg
