// Distinct points and representatives without any device allocation.
//
// Some callers cannot call cudaMalloc at all: plug-ins whose host
// application owns every device allocation and forbids others, and
// real-time loops that may not take the allocator's locks or its latency.
// For them qdtg_unique_points_noalloc() computes what the batch path's first
// stage computes (reference builder.hxx:356-390: the points sorted by
// (x, y, index), equal coordinates collapsed, rep[i] = the lowest index with
// the same coordinates) for up to kNoAllocMaxPoints points, with one thread
// block and all its working memory in the file-scope array below. The
// caller passes its own device input and output.
//
// The array lives on every GPU that loads the library until the process
// exits. All calls share it, and it keeps the last call's contents: the
// kernel initialises everything it reads, and the host sets the two status
// words to a value no kernel writes before each launch, so a launch that did
// not run can never pass for a result. Calls that overlap on the GPU (on
// different streams, or from different host threads) race on the array:
// serialise them. The call reads its status back into host memory and waits
// for its stream before it returns.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "common.cuh"
#include "qdt.h"
#include "qdt_gpu.h"

namespace qdtg {

constexpr int kNoAllocMaxPoints = 1 << 16;
constexpr int kNoAllocThreads = 1024;

// keys x, keys y (two buffers each), indices (two buffers), status word
constexpr size_t kNoAllocScratchBytes = (size_t)kNoAllocMaxPoints * (2 * 8 + 2 * 8 + 2 * 4) + 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

__device__ __forceinline__ uint64_t na_key(double v)
{
    if (v == 0.0) return 0x8000000000000000ull;   // -0.0 and +0.0 are one value
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void __launch_bounds__(kNoAllocThreads) k_unique_noalloc(const double2* __restrict__ pts, int n,
    unsigned char* __restrict__ scratch, uint32_t* __restrict__ rep)
{
    const int M = kNoAllocMaxPoints;
    uint64_t* kx[2] = { reinterpret_cast<uint64_t*>(scratch), reinterpret_cast<uint64_t*>(scratch) + M };
    uint64_t* ky[2] = { reinterpret_cast<uint64_t*>(scratch) + 2 * M, reinterpret_cast<uint64_t*>(scratch) + 3 * M };
    uint32_t* ix[2] = { reinterpret_cast<uint32_t*>(scratch + (size_t)32 * M),
        reinterpret_cast<uint32_t*>(scratch + (size_t)32 * M) + M };
    uint32_t* status = reinterpret_cast<uint32_t*>(scratch + (size_t)40 * M);   // [0] flags, [1] distinct

    __shared__ uint32_t hist[256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t whist[kNoAllocThreads / 32][256];
    __shared__ uint32_t wsum[kNoAllocThreads / 32];
    __shared__ int      bad;
    __shared__ uint32_t carry_head, carry_count;

    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    constexpr int W = kNoAllocThreads / 32;
    if (t == 0) bad = 0;
    __syncthreads();
    for (int i = t; i < n; i += kNoAllocThreads)
    {
        const double2 p = pts[i];
        if (!isfinite(p.x) || !isfinite(p.y)) bad = 1;
        kx[0][i] = na_key(p.x);
        ky[0][i] = na_key(p.y);
        ix[0][i] = (uint32_t)i;
    }
    __syncthreads();
    if (bad)
    {
        if (t == 0)
        {
            status[0] = 1;
            status[1] = 0;
        }
        return;
    }

    // stable LSD radix sort by (kx, ky): 8 passes over ky, then 8 over kx
    int cur = 0;
    for (int pass = 0; pass < 16; ++pass)
    {
        const uint64_t* key = pass < 8 ? ky[cur] : kx[cur];
        const int       sh = 8 * (pass & 7);
        if (t < 256) hist[t] = 0;
        __syncthreads();
        for (int i = t; i < n; i += kNoAllocThreads) atomicAdd(&hist[(uint32_t)(key[i] >> sh) & 255u], 1u);
        __syncthreads();
        if (t == 0)
        {
            uint32_t run = 0;
            for (int d = 0; d < 256; ++d)
            {
                base[d] = run;
                run += hist[d];
            }
        }
        __syncthreads();
        // tiles in order; inside a tile the rank of an element among equal
        // digits follows its position (warps in order, lanes in order)
        for (int tile = 0; tile < n; tile += kNoAllocThreads)
        {
            const int      i = tile + t;
            const bool     valid = i < n;
            const uint32_t d = valid ? (uint32_t)(key[i] >> sh) & 255u : 256u + (uint32_t)lane;
            for (int q = t; q < W * 256; q += kNoAllocThreads) (&whist[0][0])[q] = 0;
            __syncthreads();
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const unsigned lrank = __popc(peers & ((1u << lane) - 1u));
            if (valid && lane == __ffs(peers) - 1) whist[w][d] = __popc(peers);
            __syncthreads();
            if (t < 256)
            {
                uint32_t run = 0;
                for (int q = 0; q < W; ++q)
                {
                    const uint32_t c = whist[q][t];
                    whist[q][t] = run;
                    run += c;
                }
                hist[t] = run;   // this tile's count of digit t
            }
            __syncthreads();
            if (valid)
            {
                const uint32_t dst = base[d] + whist[w][d] + lrank;
                kx[1 - cur][dst] = kx[cur][i];
                ky[1 - cur][dst] = ky[cur][i];
                ix[1 - cur][dst] = ix[cur][i];
            }
            __syncthreads();
            if (t < 256) base[t] += hist[t];
            __syncthreads();
        }
        cur = 1 - cur;
    }

    // runs of equal keys: the head of a run holds the lowest index (the
    // sort is stable and the indices started in order)
    if (t == 0)
    {
        carry_head = 0;
        carry_count = 0;
    }
    __syncthreads();
    for (int tile = 0; tile < n; tile += kNoAllocThreads)
    {
        const int  i = tile + t;
        const bool valid = i < n;
        const bool head = valid && (i == 0 || kx[cur][i] != kx[cur][i - 1] || ky[cur][i] != ky[cur][i - 1]);
        // inclusive max-scan of head positions across the block
        uint32_t hp = head ? (uint32_t)i + 1u : 0u;   // +1: 0 means "none yet"
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(0xffffffffu, hp, o);
            if (lane >= o) hp = max(hp, v);
        }
        const unsigned hb = __ballot_sync(0xffffffffu, head);
        if (lane == 31) wsum[w] = hp;
        __syncthreads();
        if (w == 0)
        {
            uint32_t v = lane < W ? wsum[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v = max(v, u);
            }
            if (lane < W) wsum[lane] = v;
        }
        __syncthreads();
        uint32_t h = hp;
        if (w > 0) h = max(h, wsum[w - 1]);
        if (h == 0) h = carry_head + 1u;
        if (valid) rep[ix[cur][i]] = ix[cur][h - 1u];
        // count heads of this tile
        if (lane == 0) atomicAdd(&carry_count, (uint32_t)__popc(hb));
        __syncthreads();
        if (t == kNoAllocThreads - 1) carry_head = max(h, carry_head + 1u) - 1u;
        __syncthreads();
    }
    if (t == 0)
    {
        status[0] = 0;
        status[1] = carry_count;
    }
}

namespace {
std::mutex       g_na_mutex;
unsigned char*   g_na_ptr[64] = {};   // device address of the array, per device
}  // namespace

}  // namespace qdtg

extern "C" {

// No counterpart in the reference (see qdt_gpu.h).
QDT_API qdt_status qdtg_unique_points_noalloc(const qdt_vec2d* d_pts, size_t n, uint32_t* d_rep,
    size_t* unique_points, void* cuda_stream)
{
    using namespace qdtg;
    if (n > (size_t)kNoAllocMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
    if (!unique_points) return QDT_ERR_NULL_ARGUMENT;
    if (n > 0 && (!d_pts || !d_rep)) return QDT_ERR_NULL_ARGUMENT;
    *unique_points = 0;
    if (n == 0) return QDT_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    {
        cudaGetLastError();
        return QDT_ERR_INTERNAL;
    }
    unsigned char* scratch = nullptr;
    {
        // once per device, with that device current: the device address of
        // the array (the host-side symbol is only a stand-in)
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[dev])
        {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
            {
                cudaGetLastError();
                return QDT_ERR_INTERNAL;
            }
            g_na_ptr[dev] = static_cast<unsigned char*>(p);
        }
        scratch = g_na_ptr[dev];
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
    if (s)
    {
        // the array's address above is the current device's: a stream of
        // another device would run the kernel on that device's array
        int sdev = -1;
        if (cudaStreamGetDevice(s, &sdev) != cudaSuccess || sdev != dev)
        {
            cudaGetLastError();
            return QDT_ERR_INTERNAL;
        }
    }
    uint32_t* d_status = reinterpret_cast<uint32_t*>(scratch + (size_t)40 * kNoAllocMaxPoints);
    // status words to 0xFFFFFFFF, which the kernel never writes: a launch
    // that did not run leaves them there instead of the last call's result
    if (cudaMemsetAsync(d_status, 0xFF, 2 * sizeof(uint32_t), s) != cudaSuccess)
    {
        cudaGetLastError();
        return QDT_ERR_INTERNAL;
    }
    k_unique_noalloc<<<1, kNoAllocThreads, 0, s>>>(reinterpret_cast<const double2*>(d_pts), (int)n, scratch, d_rep);
    if (cudaGetLastError() != cudaSuccess) return QDT_ERR_INTERNAL;
    uint32_t st[2] = { 0xFFFFFFFFu, 0xFFFFFFFFu };
    if (cudaMemcpyAsync(st, d_status, sizeof st, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
    {
        cudaGetLastError();
        return QDT_ERR_INTERNAL;
    }
    if (st[0] == 1u) return QDT_ERR_NOT_FINITE;
    if (st[0] != 0u || st[1] > (uint32_t)n) return QDT_ERR_INTERNAL;
    *unique_points = st[1];
    return QDT_OK;
}

}  // extern "C"
