// Stage K0-K2 of the batch triangulation: input validation and sort keys,
// device radix sort, unique points and representatives, and the Dwyer split
// tree (reference builder.hxx:356-390 load_unique_points and :303-348 build's
// median cuts).
//
// Layout in HBM (n input points, m distinct points):
//   pts      double2[n]  input, AoS 16 B/pt, read with 16-byte vector loads
//   kx, ky   u64[n] x2   order-preserving keys of x and y (-0.0 as +0.0)
//   val      u32[n] x2   input index carried through the sort
//   rep      u32[n]      lowest index with the same coordinates
//   ucoord   double2[m]  distinct points in (x, y) order; uid u32[m] their ids
//   A, B     u32[m] x2   distinct point numbers ordered by frame 0 (x, y) and
//                        by frame 1 (y, -x) inside every node of the tree
//   V        double2[m]  distinct points in leaf order (the builder's V)
//   vid      u32[m]      input index of V[i]
#include "common.cuh"
#include "engine_kernels.hpp"
#include "scan.cuh"
#include "split_tail.cuh"

namespace qdtg {

// ---------------------------------------------------------------------------
// K0: validation + keys
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint64_t order_key(double v)
{
    // -0.0 and +0.0 compare equal (reference builder.hxx:373-380): one key
    if (v == 0.0) return 0x8000000000000000ull;
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_keys(const double2* __restrict__ pts, size_t n, uint64_t* __restrict__ kx, uint64_t* __restrict__ ky,
    uint32_t* __restrict__ idx, DevStatus* st)
{
    bool         bad = false;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const double2 p = pts[i];
        if (!isfinite(p.x) || !isfinite(p.y)) bad = true;
        kx[i] = order_key(p.x);
        ky[i] = order_key(p.y);
        idx[i] = (uint32_t)i;
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&st->flags, (unsigned)ST_NOT_FINITE);
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits, keys of one or two 64-bit words
// ---------------------------------------------------------------------------

constexpr int kSortThreads = 256;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;

template <int KW>
__device__ __forceinline__ uint32_t sort_digit(uint64_t hi, uint64_t lo, int pass)
{
    if (KW == 2 && pass >= 8) return (uint32_t)(hi >> (8 * (pass - 8))) & 255u;
    return (uint32_t)(lo >> (8 * pass)) & 255u;
}

template <int KW>
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint64_t* __restrict__ khi,
    const uint64_t* __restrict__ klo, size_t n, int pass, uint32_t* __restrict__ counts, unsigned nblocks)
{
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const size_t tile = (size_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kSortRounds; ++r)
    {
        const size_t i = tile + (size_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[sort_digit<KW>(KW == 2 ? khi[i] : 0, klo[i], pass)], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

template <int KW>
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const uint64_t* __restrict__ khi,
    const uint64_t* __restrict__ klo, const uint32_t* __restrict__ val, uint64_t* __restrict__ ohi,
    uint64_t* __restrict__ olo, uint32_t* __restrict__ oval, size_t n, int pass, const uint32_t* __restrict__ offs,
    unsigned nblocks)
{
    constexpr int       W = kSortThreads / 32;
    __shared__ uint32_t whist[W][256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t tot[256];
    const int           t = threadIdx.x, lane = t & 31, w = t >> 5;
    base[t] = offs[(size_t)t * nblocks + blockIdx.x];
    tot[t] = 0;
    const size_t tile = (size_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; ++r)
    {
        base[t] += tot[t];
#pragma unroll
        for (int q = 0; q < W; ++q) whist[q][t] = 0;
        const size_t i = tile + (size_t)r * kSortThreads + t;
        const bool   valid = i < n;
        uint64_t     hi = 0, lo = 0;
        uint32_t     v = 0, d;
        if (valid)
        {
            if (KW == 2) hi = khi[i];
            lo = klo[i];
            v = val[i];
            d = sort_digit<KW>(hi, lo, pass);
        }
        else
            d = 256u + (uint32_t)lane;   // alone in its class
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int      leader = __ffs(peers) - 1;
        const unsigned lrank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == leader) whist[w][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = 0;
#pragma unroll
            for (int q = 0; q < W; ++q)
            {
                const uint32_t c = whist[q][t];
                whist[q][t] = run;
                run += c;
            }
            tot[t] = run;
        }
        __syncthreads();
        if (valid)
        {
            const uint32_t dst = base[d] + whist[w][d] + lrank;
            if (KW == 2) ohi[dst] = hi;
            olo[dst] = lo;
            oval[dst] = v;
        }
        __syncthreads();
    }
}

// Sorts (khi, klo, val) by (khi, klo) (KW == 2) or by klo (KW == 1), stably.
// The result ends in buffer index *which (0 or 1) of the ping-pong pairs.
template <int KW>
static void radix_sort(uint64_t* khi[2], uint64_t* klo[2], uint32_t* val[2], size_t n, int* which, uint32_t* counts,
    uint32_t* offs, uint32_t* scratch, cudaStream_t s)
{
    if (n <= 1) return;
    const unsigned nb = (unsigned)((n + kSortTile - 1) / kSortTile);
    int            cur = *which;
    for (int pass = 0; pass < 8 * KW; ++pass)
    {
        k_sort_hist<KW><<<nb, kSortThreads, 0, s>>>(KW == 2 ? khi[cur] : nullptr, klo[cur], n, pass, counts, nb);
        ++launch_counter();
        scan_exclusive(ArrayIn{ counts }, (size_t)256 * nb, offs, scratch, nullptr, s);
        k_sort_scatter<KW><<<nb, kSortThreads, 0, s>>>(KW == 2 ? khi[cur] : nullptr, klo[cur], val[cur],
            KW == 2 ? khi[1 - cur] : nullptr, klo[1 - cur], val[1 - cur], n, pass, offs, nb);
        ++launch_counter();
        cur = 1 - cur;
    }
    *which = cur;
}

size_t sort_count_words(size_t n) { return (size_t)256 * ((n + kSortTile - 1) / kSortTile) + 1; }

// Small inputs: one block sorts in shared memory (bitonic network over the
// next power of two, padded with keys above every real one) and writes the
// result where the radix passes would leave it (an even pass count ends in
// buffer 0). Keys are made unique by the value, so the order is the stable
// radix sort's: (khi, klo, val) ascending for the points; for the frame-1
// order, (klo ascending, val descending), the stable sort of the reversed
// (x, y) order that k_frame1_keys sets up.
constexpr int kSmallSort = 4096;
constexpr int kSmallThreads = 1024;

template <int KW>
__global__ void __launch_bounds__(kSmallThreads) k_small_sort(uint64_t* khi, uint64_t* klo, uint32_t* val, int n)
{
    extern __shared__ uint64_t ssort[];
    int P = 1;
    while (P < n) P <<= 1;
    uint64_t* hi = ssort;
    uint64_t* lo = hi + (KW == 2 ? kSmallSort : 0);
    uint32_t* v = reinterpret_cast<uint32_t*>(lo + kSmallSort);
    for (int i = threadIdx.x; i < P; i += blockDim.x)
    {
        const bool real = i < n;
        if (KW == 2) hi[i] = real ? khi[i] : ~0ull;
        lo[i] = real ? klo[i] : ~0ull;
        // padding sorts last: above every real value in both orders
        v[i] = real ? val[i] : (KW == 2 ? 0xFFFFFFFFu : 0u);
    }
    __syncthreads();
    auto before = [&](int x, int y) -> bool {   // element x precedes element y
        if (KW == 2)
        {
            if (hi[x] != hi[y]) return hi[x] < hi[y];
            if (lo[x] != lo[y]) return lo[x] < lo[y];
            return v[x] < v[y];
        }
        if (lo[x] != lo[y]) return lo[x] < lo[y];
        return v[x] > v[y];
    };
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int t = threadIdx.x; t < P / 2; t += blockDim.x)
            {
                const int  x = 2 * t - (t & (j - 1));   // lower index of the pair (x, x + j)
                const int  y = x + j;
                const bool up = (x & k) == 0;
                if (before(y, x) == up)
                {
                    if (KW == 2)
                    {
                        const uint64_t h = hi[x];
                        hi[x] = hi[y];
                        hi[y] = h;
                    }
                    const uint64_t l = lo[x];
                    lo[x] = lo[y];
                    lo[y] = l;
                    const uint32_t w = v[x];
                    v[x] = v[y];
                    v[y] = w;
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x)
    {
        if (KW == 2) khi[i] = hi[i];
        klo[i] = lo[i];
        val[i] = v[i];
    }
}

template <int KW>
constexpr int small_sort_smem()
{
    return kSmallSort * (KW * 8 + 4);
}

// ---------------------------------------------------------------------------
// K1: unique points, representatives
// ---------------------------------------------------------------------------

struct HeadFlag
{
    const uint64_t* kx;
    const uint64_t* ky;
    __device__ __forceinline__ uint32_t operator()(size_t i) const
    {
        return (i == 0 || kx[i] != kx[i - 1] || ky[i] != ky[i - 1]) ? 1u : 0u;
    }
};

// Also counts the distinct points that share their x with the previous
// distinct point (*xties): integer lattices and snapped grids have them in
// the majority, points in general position almost never, and the build picks
// its merge window by it.
__global__ void k_heads(const uint64_t* __restrict__ kx, const uint64_t* __restrict__ ky,
    const uint32_t* __restrict__ idx, const uint32_t* __restrict__ uexcl, const double2* __restrict__ pts, size_t n,
    uint32_t* __restrict__ head, uint32_t* __restrict__ uid, double2* __restrict__ ucoord, uint32_t* __restrict__ xties)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool         tie = false;
    if (i < n && (i == 0 || kx[i] != kx[i - 1] || ky[i] != ky[i - 1]))
    {
        const uint32_t u = uexcl[i];
        const uint32_t id = idx[i];
        head[u] = (uint32_t)i;
        uid[u] = id;
        ucoord[u] = pts[id];
        tie = i > 0 && kx[i] == kx[i - 1];
    }
    const unsigned t = __ballot_sync(0xffffffffu, tie);
    if ((threadIdx.x & 31) == 0 && t) atomicAdd(xties, (uint32_t)__popc(t));
}

__global__ void k_rep(const uint64_t* __restrict__ kx, const uint64_t* __restrict__ ky,
    const uint32_t* __restrict__ idx, const uint32_t* __restrict__ uexcl, const uint32_t* __restrict__ uid, size_t n,
    uint32_t* __restrict__ rep)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool     h = (i == 0 || kx[i] != kx[i - 1] || ky[i] != ky[i - 1]);
    const uint32_t u = uexcl[i] + (h ? 1u : 0u) - 1u;
    rep[idx[i]] = uid[u];
}

// Frame-1 keys: the distinct points in reverse (x, y) order, keyed by y; a
// stable sort by y then orders equal y by decreasing x (reference
// builder.hxx:75, frame 1 = (y, -x)).
__global__ void k_frame1_keys(const uint64_t* __restrict__ ky_sorted, const uint32_t* __restrict__ head, size_t m,
    uint64_t* __restrict__ key, uint32_t* __restrict__ val)
{
    const size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const uint32_t u = (uint32_t)(m - 1 - j);
    key[j] = ky_sorted[head[u]];
    val[j] = u;
}

__global__ void k_iota(uint32_t* a, size_t m)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) a[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------
// K2: Dwyer split levels
// ---------------------------------------------------------------------------

// side[point] = 1 if the point goes to the right child at depth d
// side[point] = 1 if the point goes to the right child at depth d. For the
// upper depths (d <= kSeamDepth) the first point of every right child also
// records the node's seam: the cut coordinate (x for even d, y for odd d)
// that separates the children, used to prefetch the seam's records before
// the node merges.
__global__ void k_split_mark(const uint32_t* __restrict__ S, uint8_t* __restrict__ side, int m, int d,
    const double2* __restrict__ ucoord, double* __restrict__ seam)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int       lo, hi;
    const int dep = node_of(m, d, i, lo, hi);
    uint8_t   s = 0;
    if (dep == d && hi - lo >= 4)
    {
        const int mid = lo + (hi - lo) / 2;
        s = (i >= mid) ? 1 : 0;
        if (i == mid && d <= kSeamDepth)
        {
            long long k = 0;
            int       a = 0, b = m;
            for (int l = 0; l < d; ++l)
            {
                const int c = a + (b - a) / 2;
                if (i < c) b = c, k = 2 * k;
                else a = c, k = 2 * k + 1;
            }
            const double2 p = ucoord[S[i]];
            seam[(1ll << d) + k] = (d & 1) ? p.y : p.x;
        }
    }
    side[S[i]] = s;
}

struct SideOf
{
    const uint32_t* O;
    const uint8_t*  side;
    __device__ __forceinline__ uint32_t operator()(size_t j) const { return side[O[j]]; }
};

// stable partition of O inside every node at depth d by side
__global__ void k_split_scatter(const uint32_t* __restrict__ O, uint32_t* __restrict__ O2,
    const uint8_t* __restrict__ side, const uint32_t* __restrict__ R, int m, int d)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    int            lo, hi;
    const int      dep = node_of(m, d, j, lo, hi);
    const uint32_t p = O[j];
    if (dep != d || hi - lo < 4)
    {
        O2[j] = p;
        return;
    }
    const int mid = lo + (hi - lo) / 2;
    const int rb = (int)(R[j] - R[lo]);
    if (side[p]) O2[mid + rb] = p;
    else O2[lo + (j - lo - rb)] = p;
}

// The levels below the first depth d0 whose nodes hold at most kTailMax
// points: one block per node of depth d0 (split_tail.cuh), seam
// coordinates included.
__global__ void __launch_bounds__(kTailThreads) k_split_tail(const uint32_t* Ain, const uint32_t* Bin, uint32_t* Aout,
    uint32_t* Bout, uint32_t* __restrict__ loc, const double2* __restrict__ ucoord, double* __restrict__ seam, int m,
    int d0, int D)
{
    extern __shared__ uint32_t tsm[];
    int lo, hi;
    node_at(m, d0, blockIdx.x, lo, hi);
    split_tail_node(Ain, Bin, Aout, Bout, loc, ucoord, seam, m, 0, lo, hi, d0, D, (uint32_t)m, tsm);
}

// V in leaf order: inside a leaf the points follow the frame of its parent's
// cut (reference builder.hxx:177-180 sorts a leaf by outAxis).
__global__ void k_finalize(const uint32_t* __restrict__ A, const uint32_t* __restrict__ B,
    const double2* __restrict__ ucoord, const uint32_t* __restrict__ uid, int m, double2* __restrict__ V,
    uint32_t* __restrict__ vid)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int       lo, hi;
    const int dep = node_of(m, 64, i, lo, hi);
    const int frame = dep == 0 ? 0 : ((dep - 1) & 1);
    const uint32_t u = frame ? B[i] : A[i];
    V[i] = ucoord[u];
    vid[i] = uid[u];
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

static inline unsigned grid_for(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

void launch_keys(const PrepBuffers& b, size_t n, cudaStream_t s)
{
    const unsigned g = (unsigned)std::min<size_t>(grid_for(n, 256), (size_t)152 * 16);
    k_keys<<<g, 256, 0, s>>>(b.pts, n, b.kx[0], b.ky[0], b.val[0], b.status);
    ++launch_counter();
}

void launch_sort_points(PrepBuffers& b, size_t n, cudaStream_t s)
{
    int which = 0;
    if (n > 1 && n <= (size_t)kSmallSort)
    {
        cudaFuncSetAttribute(k_small_sort<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, small_sort_smem<2>());
        k_small_sort<2><<<1, kSmallThreads, small_sort_smem<2>(), s>>>(b.kx[0], b.ky[0], b.val[0], (int)n);
        ++launch_counter();
    }
    else
        radix_sort<2>(b.kx, b.ky, b.val, n, &which, b.counts, b.offs, b.scratch, s);
    b.sorted = which;
}

void launch_unique(const PrepBuffers& b, size_t n, cudaStream_t s)
{
    const int w = b.sorted;
    scan_exclusive(HeadFlag{ b.kx[w], b.ky[w] }, n, b.uexcl, b.scratch, &b.status_u32[0], s);
    k_heads<<<grid_for(n, 256), 256, 0, s>>>(b.kx[w], b.ky[w], b.val[w], b.uexcl, b.pts, n, b.head, b.uid, b.ucoord,
        &b.status_u32[2]);
    ++launch_counter();
    k_rep<<<grid_for(n, 256), 256, 0, s>>>(b.kx[w], b.ky[w], b.val[w], b.uexcl, b.uid, n, b.rep);
    ++launch_counter();
}

void launch_frames(PrepBuffers& b, size_t m, cudaStream_t s)
{
    // frame 0 order: the distinct points are already in (x, y) order
    k_iota<<<grid_for(m, 256), 256, 0, s>>>(b.A[0], m);
    ++launch_counter();
    // frame 1 order: stable sort by y of the reversed (x, y) order; the keys
    // go to the free key buffers
    const int w = b.sorted;
    uint64_t* k1[2] = { b.kx[1 - w], b.ky[1 - w] };
    uint32_t* v1[2] = { b.B[0], b.B[1] };
    k_frame1_keys<<<grid_for(m, 256), 256, 0, s>>>(b.ky[w], b.head, m, k1[0], v1[0]);
    ++launch_counter();
    int which = 0;
    if (m > 1 && m <= (size_t)kSmallSort)
    {
        cudaFuncSetAttribute(k_small_sort<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, small_sort_smem<1>());
        k_small_sort<1><<<1, kSmallThreads, small_sort_smem<1>(), s>>>(nullptr, k1[0], v1[0], (int)m);
        ++launch_counter();
    }
    else
        radix_sort<1>(nullptr, k1, v1, m, &which, b.counts, b.offs, b.scratch, s);
    b.bcur = which;
    b.acur = 0;
}

int split_levels(int m)
{
    int d = 0;
    while (true)
    {
        const long long maxsz = ((long long)m + (1ll << d) - 1) >> d;
        if (maxsz < 4) break;
        ++d;
    }
    return d;
}

void launch_split(PrepBuffers& b, int m, cudaStream_t s)
{
    const int D = split_levels(m);
    // the first depth whose nodes all fit one shared-memory block (D: none)
    int d0 = 0;
    if (b.split_tail)
        d0 = std::min(D, tail_depth(m));
    else
        d0 = D;
    for (int d = 0; d < d0; ++d)
    {
        const int axis = d & 1;
        uint32_t* S = axis == 0 ? b.A[b.acur] : b.B[b.bcur];
        int&      ocur = axis == 0 ? b.bcur : b.acur;
        uint32_t* O = axis == 0 ? b.B[ocur] : b.A[ocur];
        uint32_t* O2 = axis == 0 ? b.B[1 - ocur] : b.A[1 - ocur];
        k_split_mark<<<grid_for(m, 256), 256, 0, s>>>(S, b.side, m, d, b.ucoord, b.seam);
        ++launch_counter();
        scan_exclusive(SideOf{ O, b.side }, (size_t)m, b.uexcl, b.scratch, nullptr, s);
        k_split_scatter<<<grid_for(m, 256), 256, 0, s>>>(O, O2, b.side, b.uexcl, m, d);
        ++launch_counter();
        ocur = 1 - ocur;
    }
    if (d0 < D)
    {
        const uint32_t* Ain = b.A[b.acur];
        const uint32_t* Bin = b.B[b.bcur];
        // end in the buffers the level-by-level form ends in
        for (int d = d0; d < D; ++d)
        {
            int& ocur = (d & 1) == 0 ? b.bcur : b.acur;
            ocur = 1 - ocur;
        }
        cudaFuncSetAttribute(k_split_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem);
        // the unique-point numbering in uexcl is spent: it holds the local ids
        k_split_tail<<<1u << d0, kTailThreads, kTailSmem, s>>>(Ain, Bin, b.A[b.acur], b.B[b.bcur], b.uexcl, b.ucoord,
            b.seam, m, d0, D);
        ++launch_counter();
    }
}

// order-preserving key of a double (larger double, larger key)
__device__ __forceinline__ unsigned long long box_key(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// bounding box of the distinct points, as order keys: box = {min x, min y,
// max x, max y}, preset to {~0, ~0, 0, 0}
__global__ void k_bbox(const double2* __restrict__ P, int m, unsigned long long* __restrict__ box)
{
    unsigned long long mnx = ~0ull, mny = ~0ull, mxx = 0, mxy = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    {
        const double2            p = P[i];
        const unsigned long long kx = box_key(p.x), ky = box_key(p.y);
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

void launch_finalize(const PrepBuffers& b, int m, cudaStream_t s)
{
    k_finalize<<<grid_for(m, 256), 256, 0, s>>>(b.A[b.acur], b.B[b.bcur], b.ucoord, b.uid, m, b.V, b.vid);
    ++launch_counter();
    if (b.box)
    {
        // the seam prefetch scales its band by the mean point spacing
        cudaMemsetAsync(b.box, 0xFF, 2 * sizeof(unsigned long long), s);
        cudaMemsetAsync(b.box + 2, 0x00, 2 * sizeof(unsigned long long), s);
        k_bbox<<<(unsigned)std::min<size_t>(grid_for(m, 256), 152 * 4), 256, 0, s>>>(b.ucoord, m, b.box);
        ++launch_counter();
    }
}

}  // namespace qdtg
