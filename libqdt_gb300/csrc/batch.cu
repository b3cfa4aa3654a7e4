// The many-set engine: thousands of independent point sets of uneven size
// triangulated by one pipeline on the device.
//
// Every stage of the single-set engine runs once for all sets together:
//  * keys carry the set: the radix sort orders by (set, x, y), index order
//    breaking ties (reference builder.hxx:371-376 within each set);
//  * distinct points and representatives per set (builder.hxx:377-389);
//  * the Dwyer split levels: each set has its own tree (its shape depends
//    only on the set's distinct count), but the partition of a level is one
//    global stable partition, because no node straddles two sets;
//  * the build: one launch per depth over the nodes of every set that has
//    that depth (the shared builder of builder.cuh, node per warp or per
//    thread by the size of the depth), so the 4,096 root merges of a batch
//    run at the same time;
//  * extraction writes every set's triangles with the set's own indices.
// The launches after the one host synchronisation (the distinct counts decide
// the tree shapes) are recorded once into a CUDA graph per batch shape and
// replayed while the same shape comes back.
#include <algorithm>
#include <cstring>
#include <functional>
#include <new>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "batch_kernels.hpp"
#include "builder.cuh"
#include "common.cuh"
#include "context.hpp"
#include "engine.hpp"
#include "engine_kernels.hpp"
#include "host_copy.hpp"
#include "qdt.h"
#include "qdt_gpu.h"
#include "scan.cuh"
#include "split_tail.cuh"

namespace qdtg {

namespace {

// words per set for the per-height entry lists: at most 2 entries per set and
// height, heights < 28 (sets of at most 1e8 points), plus one offset per height
constexpr size_t kEntWords = 64;

constexpr int kBThreads = 256;
constexpr int kBRounds = 8;
constexpr int kBTile = kBThreads * kBRounds;

__device__ __forceinline__ uint64_t bkey(double v)
{
    if (v == 0.0) return 0x8000000000000000ull;
    const uint64_t b = (uint64_t)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_bkeys(const double2* __restrict__ pts, uint32_t n, const uint32_t* __restrict__ in_off, int S,
    uint64_t* __restrict__ kx, uint64_t* __restrict__ ky, uint32_t* __restrict__ idx, uint32_t* __restrict__ seg,
    uint8_t* __restrict__ set_bad)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2  p = pts[i];
    const uint32_t s = find_set(in_off, S, i);
    if (!isfinite(p.x) || !isfinite(p.y)) set_bad[s] = 1;
    kx[i] = bkey(p.x);
    ky[i] = bkey(p.y);
    idx[i] = i;
    seg[i] = s;
}

// digit sources of the two sorts
struct DigitXYS   // passes 0-7: y, 8-15: x, 16-: set of the element's input index
{
    const uint64_t* kx;
    const uint64_t* ky;
    const uint32_t* val;
    const uint32_t* seg;
    __device__ __forceinline__ uint32_t operator()(size_t i, int pass) const
    {
        if (pass < 8) return (uint32_t)(ky[i] >> (8 * pass)) & 255u;
        if (pass < 16) return (uint32_t)(kx[i] >> (8 * (pass - 8))) & 255u;
        return (seg[val[i]] >> (8 * (pass - 16))) & 255u;
    }
};
struct DigitYS   // passes 0-7: y, 8-: set of the distinct point
{
    const uint64_t* ky;
    const uint32_t* val;
    const uint32_t* useg;
    __device__ __forceinline__ uint32_t operator()(size_t i, int pass) const
    {
        if (pass < 8) return (uint32_t)(ky[i] >> (8 * pass)) & 255u;
        return (useg[val[i]] >> (8 * (pass - 8))) & 255u;
    }
};

template <class DF>
__global__ void __launch_bounds__(kBThreads) k_bhist(DF f, size_t n, int pass, uint32_t* __restrict__ counts,
    unsigned nb)
{
    __shared__ uint32_t hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const size_t tile = (size_t)blockIdx.x * kBTile;
    for (int r = 0; r < kBRounds; ++r)
    {
        const size_t i = tile + (size_t)r * kBThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[f(i, pass)], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nb + blockIdx.x] = hist[threadIdx.x];
}

// stable scatter of (kx?, ky, val) by the digit of pass
template <class DF, bool TWO>
__global__ void __launch_bounds__(kBThreads) k_bscatter(DF f, const uint64_t* __restrict__ kx,
    const uint64_t* __restrict__ ky, const uint32_t* __restrict__ val, uint64_t* __restrict__ okx,
    uint64_t* __restrict__ oky, uint32_t* __restrict__ oval, size_t n, int pass, const uint32_t* __restrict__ offs,
    unsigned nb)
{
    constexpr int       W = kBThreads / 32;
    __shared__ uint32_t whist[W][256];
    __shared__ uint32_t base[256];
    __shared__ uint32_t tot[256];
    const int           t = threadIdx.x, lane = t & 31, w = t >> 5;
    base[t] = offs[(size_t)t * nb + blockIdx.x];
    tot[t] = 0;
    const size_t tile = (size_t)blockIdx.x * kBTile;
    for (int r = 0; r < kBRounds; ++r)
    {
        base[t] += tot[t];
#pragma unroll
        for (int q = 0; q < W; ++q) whist[q][t] = 0;
        const size_t i = tile + (size_t)r * kBThreads + t;
        const bool   valid = i < n;
        uint64_t     a = 0, b = 0;
        uint32_t     v = 0, d;
        if (valid)
        {
            if (TWO) a = kx[i];
            b = ky[i];
            v = val[i];
            d = f(i, pass);
        }
        else
            d = 256u + (uint32_t)lane;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lrank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) whist[w][d] = __popc(peers);
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
            if (TWO) okx[dst] = a;
            oky[dst] = b;
            oval[dst] = v;
        }
        __syncthreads();
    }
}

struct BHeadFlag
{
    const uint64_t* kx;
    const uint64_t* ky;
    const uint32_t* val;
    const uint32_t* seg;
    __device__ __forceinline__ uint32_t operator()(size_t i) const
    {
        return (i == 0 || seg[val[i]] != seg[val[i - 1]] || kx[i] != kx[i - 1] || ky[i] != ky[i - 1]) ? 1u : 0u;
    }
};

__global__ void k_bheads(BHeadFlag h, const uint32_t* __restrict__ uexcl, const double2* __restrict__ pts, size_t n,
    uint32_t* __restrict__ head, uint32_t* __restrict__ uid, double2* __restrict__ ucoord)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !h(i)) return;
    const uint32_t u = uexcl[i], id = h.val[i];
    head[u] = (uint32_t)i;
    uid[u] = id;
    ucoord[u] = pts[id];
}

__global__ void k_brep(BHeadFlag h, const uint32_t* __restrict__ uexcl, const uint32_t* __restrict__ uid,
    const uint32_t* __restrict__ in_off, size_t n, uint32_t* __restrict__ rep)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t u = uexcl[i] + h(i) - 1u, id = h.val[i];
    rep[id] = uid[u] - in_off[h.seg[id]];   // in the set's own numbering
}

// u_off[s] = first distinct number of set s (the exclusive head count at the
// set's first sorted position; the sort keeps every set in its input range)
__global__ void k_uoff(const uint32_t* __restrict__ uexcl, const uint32_t* __restrict__ in_off, int S, uint32_t n,
    const uint32_t* __restrict__ total, uint32_t* __restrict__ u_off)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > S) return;
    u_off[s] = (s == S || in_off[s] >= n) ? *total : uexcl[in_off[s]];
}

__global__ void k_useg(const uint32_t* __restrict__ u_off, int S, uint32_t M, uint32_t* __restrict__ useg)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < M) useg[j] = find_set(u_off, S, j);
}

__global__ void k_bframe1_keys(const uint64_t* __restrict__ ky_sorted, const uint32_t* __restrict__ head,
    const uint32_t* __restrict__ useg, const uint32_t* __restrict__ u_off, uint32_t M, uint64_t* __restrict__ key,
    uint32_t* __restrict__ val, uint32_t* __restrict__ A)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M) return;
    const uint32_t s = useg[j];
    const uint32_t u = u_off[s] + u_off[s + 1] - 1u - j;   // reversed inside the set
    key[j] = ky_sorted[head[u]];
    val[j] = u;
    A[j] = j;
}

struct BNode
{
    int lo, hi;   // global positions
    int dep;
    int tail;     // the set's tail depth: the depths from there run in k_bsplit_tail
};
__device__ __forceinline__ BNode bnode_of(const uint32_t* __restrict__ useg, const uint32_t* __restrict__ u_off,
    int i, int d)
{
    const uint32_t s = useg[i];
    const int      base = (int)u_off[s], ms = (int)(u_off[s + 1] - u_off[s]);
    int            lo, hi;
    BNode          b;
    b.dep = node_of(ms, d, i - base, lo, hi);
    b.lo = lo + base;
    b.hi = hi + base;
    b.tail = tail_depth(ms);
    return b;
}

__global__ void k_bsplit_mark(const uint32_t* __restrict__ S, uint8_t* __restrict__ side,
    const uint32_t* __restrict__ useg, const uint32_t* __restrict__ u_off, uint32_t M, int d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)M) return;
    const BNode b = bnode_of(useg, u_off, i, d);
    uint8_t     s = 0;
    if (b.dep == d && d < b.tail && b.hi - b.lo >= 4) s = (i >= b.lo + (b.hi - b.lo) / 2) ? 1 : 0;
    side[S[i]] = s;
}

// the split depths of a set from its tail depth down (or, for a set the
// build skips, a copy of its slice), one block per entry (split_tail.cuh)
constexpr uint32_t kTailCopy = 0xFFFFFFFFu;
__global__ void __launch_bounds__(kTailThreads) k_bsplit_tail(const uint32_t* Ain, const uint32_t* Bin,
    uint32_t* Aout, uint32_t* Bout, uint32_t* __restrict__ loc, const uint2* __restrict__ ent,
    const uint32_t* __restrict__ u_off, uint32_t M)
{
    extern __shared__ uint32_t tsm[];
    const uint2 e = ent[blockIdx.x];
    const int   base = (int)u_off[e.x], ms = (int)(u_off[e.x + 1] - u_off[e.x]);
    if (e.y == kTailCopy)
    {
        for (int j = threadIdx.x; j < ms; j += blockDim.x)
        {
            if (Ain != Aout) Aout[base + j] = Ain[base + j];
            if (Bin != Bout) Bout[base + j] = Bin[base + j];
        }
        return;
    }
    const int t = tail_depth(ms);
    int       lo, hi;
    node_at(ms, t, e.y, lo, hi);
    split_tail_node(Ain, Bin, Aout, Bout, loc, nullptr, nullptr, ms, base, lo, hi, t, split_depth(ms), M, tsm);
}

struct BSideOf
{
    const uint32_t* O;
    const uint8_t*  side;
    __device__ __forceinline__ uint32_t operator()(size_t j) const { return side[O[j]]; }
};

__global__ void k_bsplit_scatter(const uint32_t* __restrict__ O, uint32_t* __restrict__ O2,
    const uint8_t* __restrict__ side, const uint32_t* __restrict__ R, const uint32_t* __restrict__ useg,
    const uint32_t* __restrict__ u_off, uint32_t M, int d)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (int)M) return;
    const BNode    b = bnode_of(useg, u_off, j, d);
    const uint32_t p = O[j];
    if (b.dep != d || d >= b.tail || b.hi - b.lo < 4)
    {
        O2[j] = p;
        return;
    }
    const int mid = b.lo + (b.hi - b.lo) / 2;
    const int rb = (int)(R[j] - R[b.lo]);
    if (side[p]) O2[mid + rb] = p;
    else O2[b.lo + (j - b.lo - rb)] = p;
}

__global__ void k_bfinalize(const uint32_t* __restrict__ A, const uint32_t* __restrict__ B,
    const double2* __restrict__ ucoord, const uint32_t* __restrict__ uid, const uint32_t* __restrict__ useg,
    const uint32_t* __restrict__ u_off, uint32_t M, double2* __restrict__ V, uint32_t* __restrict__ vid)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)M) return;
    const BNode    b = bnode_of(useg, u_off, i, 64);
    const int      frame = b.dep == 0 ? 0 : ((b.dep - 1) & 1);
    const uint32_t u = frame ? B[i] : A[i];
    V[i] = ucoord[u];
    vid[i] = uid[u];
}


struct BMaskCount
{
    const uint8_t* m;
    __device__ __forceinline__ uint32_t operator()(size_t i) const { return __popc((unsigned)m[i]); }
};

__global__ void k_btri_write(const Rec* __restrict__ R, int nrec, const uint8_t* __restrict__ mask,
    const uint32_t* __restrict__ off, const uint32_t* __restrict__ vid, const uint32_t* __restrict__ useg,
    const uint32_t* __restrict__ in_off, uint32_t* __restrict__ tris)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrec) return;
    const uint8_t mk = mask[k];
    if (!mk) return;
    const uint32_t base = in_off[useg[k / 3]];
    uint32_t       o = off[k];
    for (int s = 0; s < 2; ++s)
    {
        if (!(mk & (1 << s))) continue;
        const int e = 2 * k + s;
        const int f = R[(e ^ 1) >> 1].prev[(e ^ 1) & 1];
        const int g = R[(f ^ 1) >> 1].prev[(f ^ 1) & 1];
        tris[3 * (size_t)o + 0] = vid[R[e >> 1].org[e & 1]] - base;
        tris[3 * (size_t)o + 1] = vid[R[f >> 1].org[f & 1]] - base;
        tris[3 * (size_t)o + 2] = vid[R[g >> 1].org[g & 1]] - base;
        ++o;
    }
}

__global__ void k_tri_base(const uint32_t* __restrict__ tri_off, const uint32_t* __restrict__ u_off, int S,
    uint32_t nrec, const uint32_t* __restrict__ total, uint32_t* __restrict__ tri_base)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > S) return;
    const uint32_t r = 3u * u_off[s];
    tri_base[s] = (s == S || r >= nrec) ? *total : tri_off[r];
}

inline unsigned gridn(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct BatchEngine
{
    int          device = 0;
    cudaStream_t stream = nullptr;
    void*        block = nullptr;
    size_t       capN = 0, capS = 0;
    // device buffers
    double2*  pts = nullptr;
    uint32_t* in_off = nullptr;
    uint64_t *kx[2] = {}, *ky[2] = {};
    uint32_t *val[2] = {}, *seg = nullptr, *uexcl = nullptr, *head = nullptr, *uid = nullptr, *rep = nullptr;
    double2*  ucoord = nullptr;
    uint32_t *useg = nullptr, *u_off = nullptr, *A[2] = {}, *Bv[2] = {};
    uint8_t * side = nullptr, *set_bad = nullptr, *skip = nullptr, *mask = nullptr;
    double2*  V = nullptr;
    uint32_t* vid = nullptr;
    Rec*      recs = nullptr;
    NodeOut*  nodes = nullptr;
    uint32_t *noff = nullptr, *ents = nullptr, *eoffs = nullptr, *tri_off = nullptr, *tris = nullptr,
             *tri_base = nullptr;
    uint32_t* cell_off = nullptr;
    uint32_t *counts = nullptr, *offs = nullptr, *scratch = nullptr, *words = nullptr;
    DevStatus* status = nullptr;
    size_t     nodes_cap = 0;
    // split tails: one entry (set, node of the set's tail depth, or
    // kTailCopy) per block; the per-depth launches run the depths above
    uint2*             tail = nullptr;
    size_t             tail_cap = 0;
    std::vector<uint2> h_tail;
    int                tail_levels = 0;   // depths of the per-depth launches
    // host results (pinned)
    PinnedVec<uint32_t> h_tris, h_rep, h_tri_base, h_u_off, h_in_off;
    PinnedVec<double>   h_pts;   // staging of host input
    PinnedVec<uint8_t>  h_bad;
    std::vector<uint32_t> h_noff, h_ents, h_eoffs;
    // per height: first entry, number of entries, first offset word
    std::vector<int>      h_ent0, h_nent, h_eoff0;
    DevStatus*            h_status = nullptr;
    uint32_t*             h_words = nullptr;
    size_t                nsets = 0, npts = 0, ntri = 0;
    bool                  host_results = false;   // h_tris and h_rep hold the last call's results
    RunInfo               info;
    bool                  count_filter = false, timing = false, use_graph = true;
    int                   warp_min_points = 512;   // heights whose nodes have at least this many points: a warp per node
    int                   warp_nodes = 4096;       // heights with at most this many nodes: a warp per node
    int                   cell_points = 0;         // largest cell built in shared memory (0: none)
    bool                  persistent = false;      // the build as one persistent launch (k_bbuild_persist)
    uint32_t*             done = nullptr;          // per node slot: set once the node is built (persistent form)
    uint32_t*             pcounter = nullptr;      // the persistent form's unit counter
    PersistPlan*          plan = nullptr;          // its schedule (device copy of h_plan)
    PersistPlan           h_plan{};
    int                   persist_grid = 0;        // its resident blocks
    std::vector<uint32_t> h_cell_off;
    uint32_t              ncells = 0;
    cudaEvent_t           ev[8] = {};
    // CUDA graphs of the post-synchronisation part, by batch shape
    struct GraphEntry
    {
        cudaGraphExec_t       exec;
        int                   launches;
        std::vector<uint32_t> shape;   // everything the key hashes, compared on a hit
    };
    static constexpr size_t                  kMaxGraphs = 8;
    std::unordered_map<uint64_t, GraphEntry> graphs;

    ~BatchEngine()
    {
        if (!stream && !block && !h_status && !h_words) return;   // never set up (a sizing probe)
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        if (block) cudaFree(block);
        if (h_status) cudaFreeHost(h_status);
        if (h_words) cudaFreeHost(h_words);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }

    int ensure(size_t N, size_t S);
    int run(size_t N, size_t S, bool host_io);
    // a warp per node at height h >= 1 when its nodes are large (they have more
    // than 3 * 2^(h-1) points) or few (the launch is then bound by the
    // latency of each merge, not by throughput)
    bool height_warp(int h, long long nodes) const
    {
        return h >= 1 && (3ll * (1ll << (h - 1)) + 1 >= warp_min_points || nodes <= warp_nodes);
    }
    void post_sync_work(size_t N, size_t S, uint32_t M, int Dmax, bool wide);
    // this batch's build as one persistent launch (not with cells)
    bool persist_now() const
    {
        return persistent && persist_grid > 0 && !(cell_points > 0 && ncells > 0) &&
               (int)h_nent.size() <= kMaxHeights;
    }
};

namespace {

struct Carve
{
    char*  base;
    size_t off = 0;
    template <class T>
    T* take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += count * sizeof(T);
        return p;
    }
};

size_t bcarve(BatchEngine& g, char* base, size_t N, size_t S)
{
    Carve c{ base };
    const size_t tiles = (size_t)256 * ((N + kBTile - 1) / kBTile) + 1;
    g.pts = c.take<double2>(N);
    g.in_off = c.take<uint32_t>(S + 1);
    for (int i = 0; i < 2; ++i)
    {
        g.kx[i] = c.take<uint64_t>(N);
        g.ky[i] = c.take<uint64_t>(N);
        g.val[i] = c.take<uint32_t>(N);
        g.A[i] = c.take<uint32_t>(N);
        g.Bv[i] = c.take<uint32_t>(N);
    }
    g.seg = c.take<uint32_t>(N);
    g.uexcl = c.take<uint32_t>(N);
    g.head = c.take<uint32_t>(N);
    g.uid = c.take<uint32_t>(N);
    g.rep = c.take<uint32_t>(N);
    g.ucoord = c.take<double2>(N);
    g.useg = c.take<uint32_t>(N);
    g.u_off = c.take<uint32_t>(S + 1);
    g.side = c.take<uint8_t>(N);
    g.set_bad = c.take<uint8_t>(S);
    g.skip = c.take<uint8_t>(S);
    g.V = c.take<double2>(N);
    g.vid = c.take<uint32_t>(N);
    g.recs = c.take<Rec>(3 * N);
    g.mask = c.take<uint8_t>(3 * N);
    g.tri_off = c.take<uint32_t>(3 * N);
    g.tris = c.take<uint32_t>(6 * N + 3);
    g.tri_base = c.take<uint32_t>(S + 1);
    g.noff = c.take<uint32_t>(S + 1);
    g.cell_off = c.take<uint32_t>(S + 1);
    g.ents = c.take<uint32_t>(kEntWords * (S + 1));
    g.eoffs = c.take<uint32_t>(kEntWords * (S + 1));
    g.counts = c.take<uint32_t>(tiles);
    g.offs = c.take<uint32_t>(tiles);
    g.scratch = c.take<uint32_t>(std::max(scan_scratch_words(3 * N), scan_scratch_words(tiles)));
    g.status = c.take<DevStatus>(1);
    g.words = c.take<uint32_t>(8);
    // node heaps: sum over sets of 2^(D+1) <= 4 N + 2 S
    g.nodes_cap = 4 * N + 2 * S + 16;
    g.nodes = c.take<NodeOut>(g.nodes_cap);
    g.done = c.take<uint32_t>(g.nodes_cap);
    g.pcounter = c.take<uint32_t>(8);
    g.plan = c.take<PersistPlan>(1);
    // split tails: a set of m points has 2^tail_depth(m) < 2 m / kTailMax
    // tail nodes when it has more than one
    g.tail_cap = S + 2 * N / kTailMax + 16;
    g.tail = c.take<uint2>(g.tail_cap);
    return c.off + 256;
}

}  // namespace

// device bytes of a workspace for N points in S sets
size_t bcarve_bytes(size_t N, size_t S)
{
    BatchEngine probe;
    return bcarve(probe, nullptr, N, S);
}

int BatchEngine::ensure(size_t N, size_t S)
{
    if (block && N <= capN && S <= capS) return QDT_OK;
    size_t n2 = std::max<size_t>(N, 4096), s2 = std::max<size_t>(S, 64);
    if (capN) n2 = std::max(n2, capN + capN / 4);
    if (capS) s2 = std::max(s2, capS + capS / 4);
    if (block)
    {
        cudaStreamSynchronize(stream);
        for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
        cudaFree(block);
        block = nullptr;
        capN = capS = 0;
    }
    const size_t bytes = bcarve(*this, nullptr, n2, s2);
    void*        p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess)
    {
        cudaGetLastError();
        return QDT_ERR_OUT_OF_MEMORY;
    }
    block = p;
    capN = n2;
    capS = s2;
    bcarve(*this, static_cast<char*>(p), n2, s2);
    return QDT_OK;
}

// Everything after the distinct counts are known: frames, split levels,
// finalize, build, extraction. Shapes depend on the counts only, so the
// launches can be recorded once per shape.
void BatchEngine::post_sync_work(size_t N, size_t S, uint32_t M, int Dmax, bool wide)
{
    cudaStream_t s = stream;
    // the flags and predicate counters of a first pass of the same batch
    cudaMemsetAsync(status, 0, sizeof(DevStatus), s);
    const int    segp = S <= 1 ? 0 : (S <= 256 ? 1 : (S <= 65536 ? 2 : 3));
    // frames
    k_useg<<<gridn(M, 256), 256, 0, s>>>(u_off, (int)S, M, useg);
    ++launch_counter();
    k_bframe1_keys<<<gridn(M, 256), 256, 0, s>>>(ky[0], head, useg, u_off, M, kx[1], val[1], A[0]);
    ++launch_counter();
    {
        uint64_t* k1[2] = { kx[1], ky[1] };
        uint32_t* v1[2] = { val[1], Bv[1] };
        int       cur = 0;
        const unsigned nb = gridn(M, kBTile);
        for (int pass = 0; pass < 8 + segp; ++pass)
        {
            DigitYS f{ k1[cur], v1[cur], useg };
            k_bhist<DigitYS><<<nb, kBThreads, 0, s>>>(f, M, pass, counts, nb);
            ++launch_counter();
            scan_exclusive(ArrayIn{ counts }, (size_t)256 * nb, offs, scratch, nullptr, s);
            k_bscatter<DigitYS, false><<<nb, kBThreads, 0, s>>>(f, nullptr, k1[cur], v1[cur], nullptr, k1[1 - cur],
                v1[1 - cur], M, pass, offs, nb);
            ++launch_counter();
            cur = 1 - cur;
        }
        if (v1[cur] != Bv[0])
        {
            cudaMemcpyAsync(Bv[0], v1[cur], M * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
        }
    }
    // split levels: per depth down to the deepest tail depth, then the tails
    int       acur = 0, bcur = 0;
    const int Dper = std::min(tail_levels, Dmax);
    for (int d = 0; d < Dper; ++d)
    {
        const int axis = d & 1;
        uint32_t* Sa = axis == 0 ? A[acur] : Bv[bcur];
        int&      ocur = axis == 0 ? bcur : acur;
        uint32_t* O = axis == 0 ? Bv[ocur] : A[ocur];
        uint32_t* O2 = axis == 0 ? Bv[1 - ocur] : A[1 - ocur];
        k_bsplit_mark<<<gridn(M, 256), 256, 0, s>>>(Sa, side, useg, u_off, M, d);
        ++launch_counter();
        scan_exclusive(BSideOf{ O, side }, (size_t)M, uexcl, scratch, nullptr, s);
        k_bsplit_scatter<<<gridn(M, 256), 256, 0, s>>>(O, O2, side, uexcl, useg, u_off, M, d);
        ++launch_counter();
        ocur = 1 - ocur;
    }
    if (!h_tail.empty())
    {
        const uint32_t* Ain = A[acur];
        const uint32_t* Bin = Bv[bcur];
        // end in the buffers the depth-by-depth form ends in
        for (int d = Dper; d < Dmax; ++d)
        {
            int& ocur = (d & 1) == 0 ? bcur : acur;
            ocur = 1 - ocur;
        }
        cudaFuncSetAttribute(k_bsplit_tail, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem);
        // the split ranks in uexcl are spent: it holds the local ids
        k_bsplit_tail<<<(unsigned)h_tail.size(), kTailThreads, kTailSmem, s>>>(Ain, Bin, A[acur], Bv[bcur], uexcl,
            tail, u_off, M);
        ++launch_counter();
    }
    k_bfinalize<<<gridn(M, 256), 256, 0, s>>>(A[acur], Bv[bcur], ucoord, uid, useg, u_off, M, V, vid);
    ++launch_counter();
    if (timing) cudaEventRecord(ev[4], s);
    const int nrec = 3 * (int)M;
    BatchBuildArgs a;
    a.recs = recs;
    a.nrec = nrec;
    a.V = V;
    a.nodes = nodes;
    a.noff = noff;
    a.ents = ents;
    a.eoffs = eoffs;
    a.u_off = u_off;
    a.cell_off = cell_off;
    a.S = (int)S;
    a.cell_points = cell_points;
    a.ncells = ncells;
    a.status = status;
    a.count = count_filter ? 1 : 0;
    a.counter = pcounter;
    a.done = done;
    a.useg = useg;
    a.skip = skip;
    a.mask = mask;
    // the bottom of every set's tree in shared-memory cells
    if (cell_points > 0 && ncells > 0)
    {
        if (wide) wide::launch_bbuild_cells(a, s);
        else narrow::launch_bbuild_cells(a, s);
        ++launch_counter();
    }
    // the nodes above: one launch per height, from the leaves up; a warp per
    // node for the heights whose nodes have at least warp_min_points points
    // -- or all heights in one persistent launch
    if (persist_now())
    {
        cudaMemsetAsync(done, 0, (size_t)h_noff[S] * sizeof(uint32_t), s);
        cudaMemsetAsync(pcounter, 0, sizeof(uint32_t), s);
        // (mostly thread-per-node merges: the build with the widest tier)
        wide::launch_bbuild_persist(a, plan, persist_grid, s);
        ++launch_counter();
    }
    else
        for (int h = 0; h < (int)h_nent.size(); ++h)
        {
            const int nent = h_nent[h];
            if (nent == 0) continue;
            const long long slots = h_eoffs[h_eoff0[h] + nent];
            if (slots == 0) continue;
            const uint32_t* en = ents + h_ent0[h];
            const uint32_t* eo = eoffs + h_eoff0[h];
            const bool      w = height_warp(h, slots);
            // the thread-per-node merges always from the build with the
            // widest tier: measured twice as fast as the build without it
            // (same instructions, a quarter of the waits on loads)
            if (wide || (h > 0 && !w)) wide::launch_bbuild_height(a, h, en, eo, nent, slots, w, s);
            else narrow::launch_bbuild_height(a, h, en, eo, nent, slots, w, s);
            ++launch_counter();
        }
    if (timing) cudaEventRecord(ev[5], s);
    if (wide) wide::launch_btri_mask(a, s);
    else narrow::launch_btri_mask(a, s);
    ++launch_counter();
    scan_exclusive(BMaskCount{ mask }, (size_t)nrec, tri_off, scratch, words + 1, s);
    k_btri_write<<<gridn(nrec, 256), 256, 0, s>>>(recs, nrec, mask, tri_off, vid, useg, in_off, tris);
    ++launch_counter();
    k_tri_base<<<gridn(S + 1, 256), 256, 0, s>>>(tri_off, u_off, (int)S, (uint32_t)nrec, words + 1, tri_base);
    ++launch_counter();
}

int BatchEngine::run(size_t N, size_t S, bool host_io)
{
    cudaStream_t s = stream;
    info = RunInfo();
    info.n = N;
    launch_counter() = 0;
    if (timing) cudaEventRecord(ev[1], s);
    cudaMemsetAsync(status, 0, sizeof(DevStatus), s);
    cudaMemsetAsync(words, 0, 8 * sizeof(uint32_t), s);
    cudaMemsetAsync(set_bad, 0, S, s);
    k_bkeys<<<gridn(N, 256), 256, 0, s>>>(pts, (uint32_t)N, in_off, (int)S, kx[0], ky[0], val[0], seg, set_bad);
    ++launch_counter();
    // sort by (set, x, y); stable, so equal points keep index order
    const int segp = S <= 1 ? 0 : (S <= 256 ? 1 : (S <= 65536 ? 2 : 3));
    int       cur = 0;
    {
        const unsigned nb = gridn(N, kBTile);
        for (int pass = 0; pass < 16 + segp; ++pass)
        {
            DigitXYS f{ kx[cur], ky[cur], val[cur], seg };
            k_bhist<DigitXYS><<<nb, kBThreads, 0, s>>>(f, N, pass, counts, nb);
            ++launch_counter();
            scan_exclusive(ArrayIn{ counts }, (size_t)256 * nb, offs, scratch, nullptr, s);
            k_bscatter<DigitXYS, true><<<nb, kBThreads, 0, s>>>(f, kx[cur], ky[cur], val[cur], kx[1 - cur],
                ky[1 - cur], val[1 - cur], N, pass, offs, nb);
            ++launch_counter();
            cur = 1 - cur;
        }
    }
    if (cur != 0)
    {
        cudaMemcpyAsync(kx[0], kx[1], N * 8, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(ky[0], ky[1], N * 8, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(val[0], val[1], N * 4, cudaMemcpyDeviceToDevice, s);
    }
    if (timing) cudaEventRecord(ev[2], s);
    BHeadFlag hf{ kx[0], ky[0], val[0], seg };
    scan_exclusive(hf, N, uexcl, scratch, words, s);
    k_bheads<<<gridn(N, 256), 256, 0, s>>>(hf, uexcl, pts, N, head, uid, ucoord);
    ++launch_counter();
    k_brep<<<gridn(N, 256), 256, 0, s>>>(hf, uexcl, uid, in_off, N, rep);
    ++launch_counter();
    k_uoff<<<gridn(S + 1, 256), 256, 0, s>>>(uexcl, in_off, (int)S, (uint32_t)N, words, u_off);
    ++launch_counter();
    if (timing) cudaEventRecord(ev[3], s);
    h_u_off.resize(S + 1);
    h_bad.resize(S);
    cudaMemcpyAsync(h_u_off.data(), u_off, (S + 1) * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(h_bad.data(), set_bad, S, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess)
    {
        cudaGetLastError();
        return QDT_ERR_INTERNAL;
    }
    const uint32_t M = h_u_off[S];
    info.unique_points = M;
    // plan the trees: node heaps, cells, per-height entry lists
    // Each set of m distinct points splits down to depth split_levels(m); the
    // cells cover the depths from cell_depth(m, C) down, the height launches
    // the nodes above (all nodes without cells).
    const int            C = cell_points;
    std::vector<uint8_t> skipv(S);
    std::vector<int>     top(S, -1);   // deepest depth built by the height launches
    int                  Dmax = 0;     // deepest split
    h_noff.assign(S + 1, 0);
    h_cell_off.assign(S + 1, 0);
    size_t nacc = 0, cacc = 0;
    for (size_t i = 0; i < S; ++i)
    {
        const int ms = (int)(h_u_off[i + 1] - h_u_off[i]);
        skipv[i] = (ms < 3 || h_bad[i]) ? 1 : 0;
        h_noff[i] = (uint32_t)nacc;
        h_cell_off[i] = (uint32_t)cacc;
        if (!skipv[i])
        {
            const int Ds = split_levels(ms);
            Dmax = std::max(Dmax, Ds);
            nacc += (size_t)2 << Ds;
            if (C > 0)
            {
                const int dc = cell_depth(ms, C);
                cacc += (size_t)1 << dc;
                top[i] = dc - 1;
            }
            else
                top[i] = Ds;
        }
    }
    h_noff[S] = (uint32_t)nacc;
    h_cell_off[S] = (uint32_t)cacc;
    ncells = (uint32_t)cacc;
    if (nacc > nodes_cap || cacc > 0xFFFFFFFFull) return QDT_ERR_INTERNAL;
    // split tails: every set's slice is written by its entries (a copy for
    // the sets the build skips)
    h_tail.clear();
    tail_levels = 0;
    for (size_t i = 0; i < S; ++i)
    {
        if (skipv[i])
        {
            h_tail.push_back(make_uint2((uint32_t)i, kTailCopy));
            continue;
        }
        const int t = tail_depth((int)(h_u_off[i + 1] - h_u_off[i]));
        tail_levels = std::max(tail_levels, t);
        for (uint32_t k = 0; k < (1u << t); ++k) h_tail.push_back(make_uint2((uint32_t)i, k));
    }
    if (h_tail.size() > tail_cap || h_tail.size() > 0x7FFFFFFFull) return QDT_ERR_INTERNAL;
    // per height the entries (set, depth) that hold nodes of that height (at
    // depths D - h and D - h - 1, above the cells), with their slot offsets
    int Hmax = -1;
    for (size_t i = 0; i < S; ++i)
        if (!skipv[i]) Hmax = std::max(Hmax, split_levels((int)(h_u_off[i + 1] - h_u_off[i])));
    h_ent0.assign(Hmax + 1, 0);
    h_nent.assign(Hmax + 1, 0);
    h_eoff0.assign(Hmax + 1, 0);
    h_ents.clear();
    h_eoffs.clear();
    for (int h = 0; h <= Hmax; ++h)
    {
        h_ent0[h] = (int)h_ents.size();
        h_eoff0[h] = (int)h_eoffs.size();
        uint64_t acc = 0;
        for (size_t i = 0; i < S; ++i)
        {
            if (skipv[i]) continue;
            const int Ds = split_levels((int)(h_u_off[i + 1] - h_u_off[i]));
            for (int d = Ds - h; d >= Ds - h - 1; --d)
            {
                if (d < 0 || d > top[i]) continue;
                h_ents.push_back(((uint32_t)i << 5) | (uint32_t)d);
                h_eoffs.push_back((uint32_t)acc);
                acc += (uint64_t)1 << d;
            }
        }
        if (acc > 0xFFFFFFFFull) return QDT_ERR_INTERNAL;
        h_nent[h] = (int)h_ents.size() - h_ent0[h];
        h_eoffs.push_back((uint32_t)acc);
    }
    if (h_ents.size() > kEntWords * (capS + 1) || h_eoffs.size() > kEntWords * (capS + 1) || S >= (1u << 27))
        return QDT_ERR_INTERNAL;
    cudaMemcpyAsync(skip, skipv.data(), S, cudaMemcpyHostToDevice, s);
    if (!h_tail.empty()) cudaMemcpyAsync(tail, h_tail.data(), h_tail.size() * sizeof(uint2), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(noff, h_noff.data(), (S + 1) * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(cell_off, h_cell_off.data(), (S + 1) * 4, cudaMemcpyHostToDevice, s);
    if (!h_ents.empty()) cudaMemcpyAsync(ents, h_ents.data(), h_ents.size() * 4, cudaMemcpyHostToDevice, s);
    if (!h_eoffs.empty()) cudaMemcpyAsync(eoffs, h_eoffs.data(), h_eoffs.size() * 4, cudaMemcpyHostToDevice, s);
    if (persist_now())
    {
        // the persistent build's units, heights in increasing order
        h_plan = PersistPlan{};
        h_plan.nh = (int)h_nent.size();
        uint64_t units = 0;
        for (int h = 0; h < h_plan.nh; ++h)
        {
            const long long slots = h_nent[h] ? h_eoffs[h_eoff0[h] + h_nent[h]] : 0;
            h_plan.unit_off[h] = (uint32_t)units;
            h_plan.ent0[h] = (uint32_t)h_ent0[h];
            h_plan.eoff0[h] = (uint32_t)h_eoff0[h];
            h_plan.nent[h] = h_nent[h];
            h_plan.warp[h] = height_warp(h, slots) ? 1 : 0;
            units += (uint64_t)(h_plan.warp[h] ? slots : (slots + 31) / 32);
        }
        if (units > 0xFFFFFFFFull) return QDT_ERR_INTERNAL;
        h_plan.unit_off[h_plan.nh] = (uint32_t)units;
        cudaMemcpyAsync(plan, &h_plan, sizeof(PersistPlan), cudaMemcpyHostToDevice, s);
    }

    // the post-synchronisation launches, replayed from a graph per shape
    auto post = [&](bool wide) {
        bool ran = false;
        if (use_graph && !timing)
        {
            std::vector<uint32_t> shape;
            shape.reserve(2 * S + 9);
            shape.insert(shape.end(), { (uint32_t)N, (uint32_t)((uint64_t)N >> 32), (uint32_t)S,
                                          count_filter ? 1u : 0u, (uint32_t)warp_min_points, (uint32_t)warp_nodes,
                                          (uint32_t)cell_points, persistent ? 1u : 0u, wide ? 1u : 0u });
            shape.insert(shape.end(), h_u_off.begin(), h_u_off.begin() + S + 1);
            shape.insert(shape.end(), skipv.begin(), skipv.end());
            uint64_t key = 1469598103934665603ull;
            for (uint32_t v : shape) key = (key ^ v) * 1099511628211ull;
            auto it = graphs.find(key);
            if (it != graphs.end() && it->second.shape != shape)
                it = graphs.end();   // another shape with the same hash: launch by launch
            else if (it == graphs.end() && graphs.size() < kMaxGraphs)
            {
                cudaGraph_t graph = nullptr;
                cudaGetLastError();   // an error left by an earlier call is not this one's
                if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
                {
                    const int before = launch_counter();
                    post_sync_work(N, S, M, Dmax, wide);
                    // a launch refused while recording: no graph, the
                    // launches run directly below and report it
                    const bool recorded = cudaGetLastError() == cudaSuccess;
                    const int  added = launch_counter() - before;
                    if (cudaStreamEndCapture(s, &graph) == cudaSuccess && graph)
                    {
                        cudaGraphExec_t exec = nullptr;
                        if (recorded && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess)
                            it = graphs.emplace(key, GraphEntry{ exec, added, std::move(shape) }).first;
                        cudaGraphDestroy(graph);
                    }
                    cudaGetLastError();
                    launch_counter() = before;   // nothing ran during the capture
                }
                else
                    cudaGetLastError();
            }
            if (it != graphs.end())
            {
                if (cudaGraphLaunch(it->second.exec, s) == cudaSuccess)
                {
                    ran = true;
                    launch_counter() += it->second.launches;   // the kernels recorded in the graph
                }
                else
                    cudaGetLastError();
            }
        }
        if (!ran)
        {
            cudaGetLastError();
            post_sync_work(N, S, M, Dmax, wide);
            if (cudaGetLastError() != cudaSuccess) return false;
        }
        if (timing) cudaEventRecord(ev[6], s);
        cudaMemcpyAsync(h_status, status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(h_words, words, 8 * 4, cudaMemcpyDeviceToHost, s);
        h_tri_base.resize(S + 1);
        cudaMemcpyAsync(h_tri_base.data(), tri_base, (S + 1) * 4, cudaMemcpyDeviceToHost, s);
        if (host_io)
        {
            // the count is at most 2 M: copy that bound, not a round trip
            h_tris.resize(6 * (size_t)M + 3);
            h_rep.resize(N);
            if (M) cudaMemcpyAsync(h_tris.data(), tris, 6 * (size_t)M * 4, cudaMemcpyDeviceToHost, s);
            if (N) cudaMemcpyAsync(h_rep.data(), rep, N * 4, cudaMemcpyDeviceToHost, s);
        }
        if (timing) cudaEventRecord(ev[7], s);
        if (cudaStreamSynchronize(s) == cudaSuccess) return true;
        cudaGetLastError();
        return false;
    };
    if (!post(false)) return QDT_ERR_INTERNAL;
    bool need_wide = false;
    for (int sg = 0; sg < kPredStages; ++sg) need_wide = need_wide || h_status->pc[sg].wide;
    if (need_wide)
    {
        // a predicate needed the widest exact tier, which the default
        // kernels leave out: the stages after the synchronisation once more
        // with the kernels that have it
        info.wide = 1;
        if (!post(true)) return QDT_ERR_INTERNAL;
    }
    ntri = h_words[1];
    info.ntri = ntri;
    info.device_status = (int)h_status->flags;
    take_pred_stats(info, *h_status);
    info.launches = launch_counter();
    if (timing)
    {
        auto el = [&](int a, int z) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[a], ev[z]);
            return ms;
        };
        info.ms.keys_sort = el(1, 2);
        info.ms.unique = el(2, 3);
        info.ms.split = el(3, 4);
        info.ms.build = el(4, 5);
        info.ms.extract = el(5, 6);
        info.ms.d2h = el(6, 7);
        info.ms.total = el(0, 7);
    }
    if (h_status->flags & (ST_POOL_EMPTY | ST_GUARD | ST_BAD_INDEX)) return QDT_ERR_INTERNAL;
    return QDT_OK;
}

}  // namespace qdtg

// ---------------------------------------------------------------------------
// C ABI (qdt_gpu.h)
// ---------------------------------------------------------------------------

struct qdtg_batch
{
    qdtg::BatchEngine e;
};

namespace {

qdt_status batch_prepare(qdtg_batch* b, const size_t* offsets, size_t nsets, size_t* N)
{
    if (!b) return QDT_ERR_NULL_CONTEXT;
    if (nsets > 0 && !offsets) return QDT_ERR_NULL_ARGUMENT;
    *N = nsets ? offsets[nsets] : 0;
    if (*N > qdtg::kMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
    for (size_t i = 0; i < nsets; ++i)
        if (offsets[i + 1] < offsets[i] || (i == 0 && offsets[0] != 0)) return QDT_ERR_NULL_ARGUMENT;
    return QDT_OK;
}

qdt_status batch_run(qdtg_batch* b, const qdt_vec2d* pts, bool device_in, const size_t* offsets, size_t nsets,
    void* stream)
{
    size_t     N = 0;
    qdt_status st = batch_prepare(b, offsets, nsets, &N);
    if (st != QDT_OK) return st;
    qdtg::BatchEngine& e = b->e;
    e.nsets = 0;
    e.ntri = 0;
    e.host_results = false;
    if (nsets == 0) return QDT_OK;
    if (N > 0 && !pts) return QDT_ERR_NULL_ARGUMENT;
    try
    {
        if (cudaSetDevice(e.device) != cudaSuccess)
        {
            cudaGetLastError();
            return QDT_ERR_INTERNAL;
        }
        const int rc = e.ensure(std::max<size_t>(N, 1), nsets);
        if (rc != QDT_OK) return (qdt_status)rc;
        e.h_in_off.resize(nsets + 1);
        for (size_t i = 0; i <= nsets; ++i) e.h_in_off[i] = (uint32_t)offsets[i];
        if (N == 0)
        {
            // only empty sets: nothing to run
            e.h_u_off.assign(nsets + 1, 0);
            e.h_bad.assign(nsets, 0);
            e.h_tri_base.assign(nsets + 1, 0);
            e.h_rep.clear();
            e.h_tris.clear();
            e.info = qdtg::RunInfo();
            e.npts = 0;
            e.nsets = nsets;
            e.host_results = true;
            return QDT_OK;
        }
        if (e.timing) cudaEventRecord(e.ev[0], e.stream);
        if (stream)
        {
            cudaEventRecord(e.ev[7], reinterpret_cast<cudaStream_t>(stream));
            cudaStreamWaitEvent(e.stream, e.ev[7], 0);
        }
        cudaMemcpyAsync(e.in_off, e.h_in_off.data(), (nsets + 1) * 4, cudaMemcpyHostToDevice, e.stream);
        cudaPointerAttributes attr{};
        const bool pinned = !device_in && N && cudaPointerGetAttributes(&attr, pts) == cudaSuccess &&
                            attr.type == cudaMemoryTypeHost;
        cudaGetLastError();
        if (N && (device_in || pinned))
            cudaMemcpyAsync(e.pts, pts, N * sizeof(double2), device_in ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                e.stream);
        else if (N)
        {
            // through page-locked staging in chunks: the host copy of a chunk
            // overlaps the upload of the previous one
            e.h_pts.resize(2 * N);
            const size_t chunk = (size_t)1 << 20;   // 16 MiB, each copied by the host pool
            const double* src = reinterpret_cast<const double*>(pts);
            for (size_t o = 0; o < N; o += chunk)
            {
                const size_t c = std::min(chunk, N - o);
                qdtg::parallel_copy(e.h_pts.data() + 2 * o, src + 2 * o, c * sizeof(double2));
                cudaMemcpyAsync(e.pts + o, e.h_pts.data() + 2 * o, c * sizeof(double2), cudaMemcpyHostToDevice,
                    e.stream);
            }
        }
        e.npts = N;
        e.nsets = nsets;
        const int r = e.run(N, nsets, !device_in);
        if (r != QDT_OK)
        {
            e.nsets = 0;
            return (qdt_status)r;
        }
        e.host_results = !device_in;
        return QDT_OK;
    }
    catch (const std::bad_alloc&)
    {
        e.nsets = 0;
        return QDT_ERR_OUT_OF_MEMORY;
    }
    catch (...)
    {
        e.nsets = 0;
        return QDT_ERR_INTERNAL;
    }
}

}  // namespace

extern "C" {

QDT_API qdtg_batch* qdtg_batch_create(void)
{
    qdtg_batch* b = new (std::nothrow) qdtg_batch();
    if (!b) return nullptr;
    qdtg::BatchEngine& e = b->e;
    if (cudaGetDevice(&e.device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaHostAlloc((void**)&e.h_status, sizeof(qdtg::DevStatus), cudaHostAllocPortable) != cudaSuccess ||
        cudaHostAlloc((void**)&e.h_words, 8 * sizeof(uint32_t), cudaHostAllocPortable) != cudaSuccess)
    {
        cudaGetLastError();
        delete b;
        return nullptr;
    }
    for (auto& ev : e.ev) cudaEventCreate(&ev);
    e.cell_points = qdtg::tuning().batch_cell_points;
    e.warp_min_points = qdtg::tuning().batch_warp_min_points;
    e.warp_nodes = qdtg::tuning().batch_warp_nodes;
    return b;
}

QDT_API void qdtg_batch_destroy(qdtg_batch* b) { delete b; }

QDT_API qdt_status qdtg_batch_execute(qdtg_batch* b, const qdt_vec2d* pts, const size_t* offsets, size_t nsets)
{
    return batch_run(b, pts, false, offsets, nsets, nullptr);
}

QDT_API qdt_status qdtg_batch_execute_device(qdtg_batch* b, const qdt_vec2d* d_pts, const size_t* offsets,
    size_t nsets, void* cuda_stream)
{
    return batch_run(b, d_pts, true, offsets, nsets, cuda_stream);
}

QDT_API size_t qdtg_batch_set_count(const qdtg_batch* b) { return b ? b->e.nsets : 0; }

QDT_API qdt_status qdtg_batch_set_status(const qdtg_batch* b, size_t set)
{
    if (!b) return QDT_ERR_NULL_CONTEXT;
    if (set >= b->e.nsets) return QDT_ERR_INVALID_INDEX;
    return b->e.h_bad[set] ? QDT_ERR_NOT_FINITE : QDT_OK;
}

QDT_API size_t qdtg_batch_triangles(const qdtg_batch* b, size_t set, const uint32_t** tris)
{
    if (!b || set >= b->e.nsets || b->e.h_bad[set]) return 0;
    const qdtg::BatchEngine& e = b->e;
    const size_t             lo = e.h_tri_base[set], hi = e.h_tri_base[set + 1];
    if (tris) *tris = (e.host_results && hi > lo) ? e.h_tris.data() + 3 * lo : nullptr;
    return hi - lo;
}

QDT_API size_t qdtg_batch_unique_points(const qdtg_batch* b, size_t set)
{
    if (!b || set >= b->e.nsets || b->e.h_bad[set]) return 0;
    return b->e.h_u_off[set + 1] - b->e.h_u_off[set];
}

QDT_API const uint32_t* qdtg_batch_rep(const qdtg_batch* b, size_t set)
{
    if (!b || set >= b->e.nsets || b->e.h_bad[set] || !b->e.host_results || b->e.npts == 0) return nullptr;
    return b->e.h_rep.data() + b->e.h_in_off[set];
}

QDT_API size_t qdtg_batch_device_triangles(const qdtg_batch* b, const uint32_t** d_tris, const uint32_t** d_offsets)
{
    if (!b) return 0;
    if (d_tris) *d_tris = b->e.tris;
    if (d_offsets) *d_offsets = b->e.tri_base;
    return b->e.ntri;
}

QDT_API size_t qdtg_batch_download_device_triangles(const qdtg_batch* b, uint32_t* out, size_t cap,
    uint32_t* offsets_out)
{
    if (!b || b->e.nsets == 0) return 0;
    const qdtg::BatchEngine& e = b->e;
    if (cudaSetDevice(e.device) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    const size_t k = std::min(cap, e.ntri);
    if (out && k && cudaMemcpy(out, e.tris, 3 * k * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    if (offsets_out) std::memcpy(offsets_out, e.h_tri_base.data(), (e.nsets + 1) * sizeof(uint32_t));
    return out ? k : 0;
}

QDT_API void qdtg_batch_set_options(qdtg_batch* b, int count_filter_failures, int stage_timing, int use_graphs,
    int warp_min_points)
{
    if (!b) return;
    b->e.count_filter = count_filter_failures != 0;
    b->e.timing = stage_timing != 0;
    b->e.use_graph = use_graphs != 0;
    if (warp_min_points > 0) b->e.warp_min_points = warp_min_points;
}

QDT_API qdt_status qdtg_batch_reserve(qdtg_batch* b, size_t points, size_t sets)
{
    if (!b) return QDT_ERR_NULL_CONTEXT;
    if (points > qdtg::kMaxPoints) return QDT_ERR_TOO_MANY_POINTS;
    if (cudaSetDevice(b->e.device) != cudaSuccess)
    {
        cudaGetLastError();
        return QDT_ERR_INTERNAL;
    }
    return (qdt_status)b->e.ensure(std::max<size_t>(points, 1), std::max<size_t>(sets, 1));
}

QDT_API size_t qdtg_batch_workspace_bytes(const qdtg_batch* b)
{
    if (!b || !b->e.block) return 0;
    return qdtg::bcarve_bytes(b->e.capN, b->e.capS);
}

QDT_API int qdtg_batch_set_warp_nodes(qdtg_batch* b, int warp_nodes)
{
    if (!b || warp_nodes < 0) return 0;
    b->e.warp_nodes = warp_nodes;
    return 1;
}

QDT_API int qdtg_batch_set_persistent(qdtg_batch* b, int on)
{
    if (!b) return 0;
    if (on && b->e.persist_grid <= 0)
    {
        // as many blocks as are resident at once: the warps take their work
        // from a counter, so further blocks would only wait for a slot
        int dev = b->e.device, sms = 0, per = 0;
        if (cudaSetDevice(dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                cudaSuccess ||
            sms <= 0)
        {
            cudaGetLastError();
            return 0;
        }
        // resident blocks of both variants (a batch may run again with the
        // wide one)
        per = std::min(qdtg::narrow::persist_blocks_per_sm(), qdtg::wide::persist_blocks_per_sm());
        if (per <= 0) return 0;
        b->e.persist_grid = sms * per;
    }
    b->e.persistent = on != 0;
    return 1;
}

QDT_API int qdtg_batch_set_cell_points(qdtg_batch* b, int cell_points)
{
    if (!b) return 0;
    if (cell_points != 0 && (cell_points < 4 || cell_points > qdtg::kCellMax)) return 0;
    b->e.cell_points = cell_points;
    return 1;
}

namespace qdtg {
void fill_filter_stats(const RunInfo& r, qdtg_filter_stats* out);
}

// No counterpart in the reference (qdt_gpu.h).
QDT_API int qdtg_batch_get_filter_stats(const qdtg_batch* b, qdtg_filter_stats* stats)
{
    if (!b || !stats) return 0;
    qdtg::fill_filter_stats(b->e.info, stats);
    return 1;
}

QDT_API int qdtg_batch_get_run_info(const qdtg_batch* b, qdtg_run_info* info)
{
    if (!b || !info) return 0;
    const qdtg::RunInfo& r = b->e.info;
    *info = qdtg_run_info{};
    info->n = r.n;
    info->unique_points = r.unique_points;
    info->triangles = r.ntri;
    info->orient_exact = r.orient_exact;
    info->incircle_exact = r.incircle_exact;
    info->ms_sort = r.ms.keys_sort;
    info->ms_unique = r.ms.unique;
    info->ms_split = r.ms.split;
    info->ms_build = r.ms.build;
    info->ms_extract = r.ms.extract;
    info->ms_d2h = r.ms.d2h;
    info->ms_total = r.ms.total;
    info->device_flags = r.device_status;
    info->kernel_launches = r.launches;
    info->wide_exact = r.wide;
    return 1;
}

QDT_API void* qdtg_batch_stream(const qdtg_batch* b) { return b ? reinterpret_cast<void*>(b->e.stream) : nullptr; }

}  // extern "C"
