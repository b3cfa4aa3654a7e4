// Device-wide exclusive prefix sum of uint32 values produced by a functor
// (reduce-then-scan: per-block sums, a recursive scan of those sums, then a
// block-local scan with the block's offset). Used by the unique-point
// compaction, the split partitions and the triangle compaction.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace qdtg {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive block scan of one value per thread; returns the block total in
// *total (all threads).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* smem, uint32_t* total)
{
    const int      lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t incl = warp_incl_scan(v);
    if (lane == 31) smem[w] = incl;
    __syncthreads();
    if (w == 0)
    {
        const int      nw = blockDim.x >> 5;
        const uint32_t s = lane < nw ? smem[lane] : 0u;
        const uint32_t si = warp_incl_scan(s);
        if (lane < nw) smem[lane] = si - s;
        if (lane == nw - 1) smem[32] = si;
    }
    __syncthreads();
    const uint32_t r = smem[w] + incl - v;
    *total = smem[32];
    __syncthreads();
    return r;
}

template <class F>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(F f, size_t n, uint32_t* sums)
{
    __shared__ uint32_t smem[33];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t     s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += f(base + i);
    uint32_t total;
    block_excl_scan(s, smem, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <class F>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(F f, size_t n, const uint32_t* offs, uint32_t* out,
    uint32_t* grand_total)
{
    __shared__ uint32_t smem[33];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    uint32_t     v[kScanItems];
    uint32_t     s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        v[i] = (base + i < n) ? f(base + i) : 0u;
        s += v[i];
    }
    uint32_t  total;
    uint32_t  run = block_excl_scan(s, smem, &total) + (offs ? offs[blockIdx.x] : 0u);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (grand_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) *grand_total = run;
}

struct ArrayIn
{
    const uint32_t* a;
    __device__ __forceinline__ uint32_t operator()(size_t i) const { return a[i]; }
};

// Scratch words needed by scan_exclusive for n items.
inline size_t scan_scratch_words(size_t n)
{
    size_t total = 0;
    size_t m = n;
    while (m > (size_t)kScanTile)
    {
        m = (m + kScanTile - 1) / kScanTile;
        total += 2 * m + 1;
    }
    return total + 4;
}

// out[i] = sum of f(j) for j < i; *grand_total (device) = sum of all.
template <class F>
void scan_exclusive(F f, size_t n, uint32_t* out, uint32_t* scratch, uint32_t* grand_total, cudaStream_t s)
{
    if (n == 0) return;
    const size_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1)
    {
        k_scan_apply<<<1, kScanThreads, 0, s>>>(f, n, nullptr, out, grand_total);
        ++launch_counter();
        return;
    }
    uint32_t* sums = scratch;
    uint32_t* offs = scratch + nb;
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(f, n, sums);
    ++launch_counter();
    scan_exclusive(ArrayIn{ sums }, nb, offs, scratch + 2 * nb + 1, nullptr, s);
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, s>>>(f, n, offs, out, grand_total);
    ++launch_counter();
}

}  // namespace qdtg
