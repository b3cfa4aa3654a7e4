// Stages K3-K6 of the batch triangulation: leaves, level-by-level merges with
// the hull re-walk, and the extraction of triangles.
//
// The leaf construction, the merge (lower common tangent, then the rising
// bubble with its two candidate scans) and the hull walk follow the reference
// builder (builder.hxx:177-301) step for step, with the same queries on the
// same planar map, so that the same split tree gives the same topology, also
// on cocircular and collinear input. What is GB300-specific:
//
// * the map is stored as half-edges linked both ways around their origins
//   (see Rec): the reference's makeEdge/splice/connect/deleteEdge
//   (builder.hxx:131-166) become ring insertions and removals;
// * the tree is built bottom-up, one kernel launch per depth. At the deep
//   depths (hundreds of thousands of small merges) every node is one thread;
//   at the upper depths (few, long merges) every node is one warp, and the
//   warp evaluates the predicates of a bubble step together (warp_merge);
// * the records live in one pool of exactly 3 m records in HBM. Node [lo, hi)
//   owns records [3 lo, 3 hi) from its leaves; every node threads its dead
//   records onto a free list that it passes to its parent, and a merge takes
//   records from that list before anything else. A planar graph on s vertices
//   has at most 3 s - 6 edges, so the list never runs dry;
// * a record carries the coordinates of its two origins, so a record load
//   gives what the predicates need without a second, dependent load;
// * every record access is bounds-checked and every loop has an iteration
//   guard; a violation sets a device status bit and ends the thread, and the
//   host reports QDT_ERR_INTERNAL. No trap, no hang.
// This file is compiled twice: here with QDTG_WIDE_EXACT 0 (kernels in
// qdtg::narrow, without the widest exact tier, run on every call), and from
// k_build_wide.cu with it (qdtg::wide, run again on the rare call whose
// predicates needed that tier; see predicates.cuh).
#ifndef QDTG_BUILD_VARIANT
#define QDTG_WIDE_EXACT 0
#define QDTG_BUILD_VARIANT narrow
#endif

#include "builder.cuh"
#include "common.cuh"
#include "engine_kernels.hpp"
#include "predicates.cuh"
#include "scan.cuh"
#include "seam_split.cuh"

namespace qdtg {
namespace QDTG_BUILD_VARIANT {

__device__ __forceinline__ bool free_tail_ok(int t, int lo, int hi, int m, int nrec)
{
    return (t >= 3 * lo && t < 3 * hi) || (t >= 3 * m && t < nrec);
}

__device__ __forceinline__ double box_value(unsigned long long k)
{
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

// The range of node (d, k) along its seam (y for even d, x for odd d): the
// bounding box, narrowed by the cuts of its ancestors on that coordinate.
__device__ inline double2 seam_range(const double* __restrict__ seam, const unsigned long long* __restrict__ box,
    int d, long long k)
{
    double lo = (d & 1) ? box_value(box[0]) : box_value(box[1]);
    double hi = (d & 1) ? box_value(box[2]) : box_value(box[3]);
    for (int l = 0; l < d; ++l)
    {
        if (((l ^ d) & 1) == 0) continue;   // an ancestor cut on the other coordinate
        const long long kl = k >> (d - l);
        const double    c = seam[(1ll << l) + kl];
        if ((k >> (d - 1 - l)) & 1) lo = fmax(lo, c);
        else hi = fmin(hi, c);
    }
    return make_double2(lo, hi);
}

__device__ inline int seam_bin(double v, double2 range)
{
    const double w = range.y - range.x;
    if (!(w > 0.0)) return 0;
    const double t = (v - range.x) / w * kSeamBins;
    return t <= 0.0 ? 0 : (t >= kSeamBins - 1 ? kSeamBins - 1 : (int)t);
}

// One depth of the tree: leaves of that depth are built, internal nodes merge
// their children's results (written by the previous launch). WARP: one node
// per warp (with a window of WIN candidates), else one node per thread.
template <bool WARP, int WIN = kWinDefault>
__global__ void QDTG_BUILD_BOUNDS(WARP) k_build_level(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    const NodeOut* __restrict__ child, NodeOut* __restrict__ out, int m, int d, DevStatus* st, int count)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long k = WARP ? (g >> 5) : g;   // one node per warp: uniform inside the warp
    const int       lane = WARP ? (int)(threadIdx.x & 31) : 0;
    if (k >= (1ll << d)) return;
    unsigned flags = *(volatile unsigned*)&st->flags;
    if (WARP) flags = __shfl_sync(0xffffffffu, flags, 0);   // one decision for the whole warp
    if (flags & kFatal) return;
    int lo, hi;
    if (!node_range(m, d, k, lo, hi)) return;
    const int n = hi - lo;
    Builder   B{ R, nrec, st, pred_stage(st, n <= 3 ? kStageLeaf : (WARP ? kStageWarp : kStageThread), count), -1, -1,
        false };
    NodeOut   o;
    o.le2 = o.re2 = -1;
    o.pad0 = o.pad1 = 0;
    if (n <= 3)
    {
        if (lane != 0) return;
        B.leaf(lo, hi, V, o.le, o.re);
        if (d > 0 && !B.bad) extremes_by_walk(B, o.le, o.re, d & 1, 8, o.le2, o.re2);
    }
    else
    {
        const NodeOut L = child[2 * k], Rn = child[2 * k + 1];
        // the children's free lists lie inside their record ranges (or in
        // the spare records of split merges, after the pool's 3 m)
        if ((L.fhead >= 0 && !free_tail_ok(L.ftail, lo, hi, m, nrec)) ||
            (Rn.fhead >= 0 && !free_tail_ok(Rn.ftail, lo, hi, m, nrec)))
        {
            if (lane == 0) B.fail(ST_BAD_INDEX);
            return;
        }
        // concatenate the children's free lists
        if (L.fhead >= 0)
        {
            B.fhead = L.fhead;
            if (Rn.fhead >= 0)
            {
                if (lane == 0) R[L.ftail].link = Rn.fhead;
                B.ftail = Rn.ftail;
            }
            else
                B.ftail = L.ftail;
        }
        else
        {
            B.fhead = Rn.fhead;
            B.ftail = Rn.ftail;
        }
        const int lim = 8 * n + 64;
        const int g = (d - 1) & 1;   // the parent's frame
        int       rl = 0, rr = 0;
        volatile int* first = nullptr;
        if (d > 0 && lane == 0)
        {
            extremes_before_merge(R, nrec, st, &child[2 * k], &child[2 * k + 1], &out[k], g);
            first = lower_tangent_slot(&out[k]);
        }
        if (WARP) warp_merge<WIN>(B, L.le, L.re, Rn.le, Rn.re, lim, rl, rr, first);
        else B.merge(L.le, L.re, Rn.le, Rn.re, lim, rl, rr, first);
        if (lane != 0) return;
        // reference builder.hxx:340-346: the extremes in the parent's frame
        o.le2 = rl;
        o.re2 = rr;
        if (d > 0 && !B.bad)
        {
            const int2 x =
                extremes_after_merge(R, nrec, st, B.basel_last, &out[k], &child[2 * k], &child[2 * k + 1], g, n + 8);
            rl = x.x;
            rr = x.y;
        }
        o.le = rl;
        o.re = rr;
    }
    B.settle_tail();
    o.fhead = B.fhead;
    o.ftail = B.ftail;
    out[k] = o;
}

// The merges of one upper depth with two walkers each (seam_split.cuh): one
// block of three warps per node, the rising walker, the falling one and the
// ring inserter. The block's threads then remove the deleted edges
// together, and its first thread finds the node's extremes.
template <int WIN>
__global__ void __maxnreg__(232) k_build_split(Rec* __restrict__ R, int nrec, const NodeOut* __restrict__ child,
    NodeOut* __restrict__ out, int m, int d, DevStatus* st, int count, SplitPlan plan, const double* __restrict__ seam,
    const unsigned long long* __restrict__ hist, const unsigned long long* __restrict__ box)
{
    __shared__ SeamShared S;
    __shared__ int        go;
    const long long       k = blockIdx.x;
    const int             warp = threadIdx.x >> 5;
    int                   lo = 0, hi = 0;
    if (threadIdx.x == 0)
    {
        go = !(*(volatile unsigned*)&st->flags & kFatal) && k < (1ll << d) && node_range(m, d, k, lo, hi) &&
             hi - lo >= 4;
        S.tail[0] = S.tail[1] = 0;
        S.head[0] = S.head[1] = 0;
        S.state[0] = S.state[1] = 0;
        S.last_o = S.last_d = S.last_e = -1;
        S.first_dn = -1;
        S.ndel[0] = S.ndel[1] = 0;
        S.base0 = S.ldo = S.rdo = S.top = -1;
        S.fhead = S.ftail = -1;
        S.fail = 0;
    }
    __syncthreads();
    if (!go) return;
    node_range(m, d, k, lo, hi);
    const int     n = hi - lo;
    const NodeOut L = child[2 * k], Rn = child[2 * k + 1];
    const int     g = (d - 1) & 1;   // the parent's frame
    if (threadIdx.x == 0)
    {
        bool ok = !((L.fhead >= 0 && !free_tail_ok(L.ftail, lo, hi, m, nrec)) ||
                    (Rn.fhead >= 0 && !free_tail_ok(Rn.ftail, lo, hi, m, nrec)));
        if (ok)
        {
            // the children's free lists, concatenated
            if (L.fhead >= 0)
            {
                S.fhead = L.fhead;
                if (Rn.fhead >= 0)
                {
                    R[L.ftail].link = Rn.fhead;
                    S.ftail = Rn.ftail;
                }
                else
                    S.ftail = L.ftail;
            }
            else
            {
                S.fhead = Rn.fhead;
                S.ftail = Rn.ftail;
            }
            if (d > 0) extremes_before_merge(R, nrec, st, &child[2 * k], &child[2 * k + 1], &out[k], g);
        }
        else
        {
            atomicOr(&st->flags, ST_BAD_INDEX);
            S.fail = 1;
        }
    }
    __syncthreads();
    if (S.fail) return;
    // the meeting point: on the node's cut (x for even d), and along the seam
    // where half of the records near the seam lie (the histogram of the
    // seam prefetch), else the mean of the children's cuts
    const double cut = seam[(1ll << d) + k];
    double       along = 0.5 * (seam[(1ll << (d + 1)) + 2 * k] + seam[(1ll << (d + 1)) + 2 * k + 1]);
    if (hist)
    {
        const unsigned long long* h = hist + ((1ll << d) + k) * kSeamBins;
        unsigned long long        total = 0;
        for (int b = 0; b < kSeamBins; ++b) total += h[b];
        if (total > 0)
        {
            unsigned long long acc = 0;
            int                b = 0;
            while (b < kSeamBins - 1 && 2 * (acc + h[b]) < total) acc += h[b++];
            const double2 rg = seam_range(seam, box, d, k);
            along = rg.x + (b + 0.5) * ((rg.y - rg.x) / kSeamBins);
        }
    }
    SeamArgs     A;
    A.R = R;
    A.nrec = nrec;
    A.tag = 4u * (unsigned)((1ll << d) + k);
    A.q = (d & 1) ? make_double2(along, cut) : make_double2(cut, along);
    const long long off = plan.base[d] + 2ll * plan.per[d] * k;
    A.a0 = plan.spare0 + (int)(off + (long long)warp * plan.per[d]);
    A.a1 = A.a0 + plan.per[d];
    A.list[0] = plan.lists + off;
    A.list[1] = plan.lists + off + plan.per[d];
    A.cap = plan.per[d];
    A.lim = 8 * n + 64;
    A.frame = d & 1;
    A.st = st;
    Builder B{ R, nrec, st, pred_stage(st, kStageWarp, count), S.fhead, S.ftail, false };
    if (warp == 0) seam_walk<false, WIN>(B, S, A, L.le, L.re, Rn.le, Rn.re);
    else if (warp == 1) seam_walk<true, WIN>(B, S, A, L.le, L.re, Rn.le, Rn.re);
    else if ((threadIdx.x & 31) == 0)
    {
        bool bad = false;
        seam_inserter(S, R, nrec, A.tag, bad);
        if (bad)
        {
            atomicOr(&st->flags, ST_SPLIT);
            S.fail = 1;
        }
    }
    __syncthreads();
    if (S.fail) return;
    {
        bool bad = false;
        int  fh = S.fhead, ft = S.ftail;
        seam_apply(R, nrec, A.list[0], S.ndel[0], A.list[1], S.ndel[1], fh, ft, threadIdx.x, (int)blockDim.x,
            [] { __syncthreads(); }, bad);
        if (bad) atomicOr(&st->flags, ST_SPLIT);
        if (threadIdx.x == 0)
        {
            S.fhead = fh;
            S.ftail = ft;
        }
    }
    __syncthreads();
    if (threadIdx.x != 0 || (*(volatile unsigned*)&st->flags & kFatal)) return;
    NodeOut o;
    o.pad0 = o.pad1 = 0;
    int rl = S.ldo, rr = S.rdo;
    o.le2 = rl;
    o.re2 = rr;
    if (d > 0)
    {
        *lower_tangent_slot(&out[k]) = S.base0;
        const int top = S.first_dn >= 0 ? S.first_dn : S.top;
        const int2 x = extremes_after_merge(R, nrec, st, top, &out[k], &child[2 * k], &child[2 * k + 1], g, n + 8);
        rl = x.x;
        rr = x.y;
    }
    o.le = rl;
    o.re = rr;
    o.fhead = S.fhead;
    o.ftail = S.fhead >= 0 ? S.ftail : -1;
    out[k] = o;
}

// Before an upper depth merges, the records near its seams are fetched into
// L2 with the evict-last policy: the merges are chains of dependent loads,
// and their records were last touched by far deeper levels, so without this
// a bubble step waits on several DRAM round trips. A record lies near a seam
// when one of its origins is closer to the cut line than 3 times the edge's
// own length (long edges around the seam, at the local scale of the point
// set) or than a band of kSeamBand mean point spacings (the short edges at
// the vertices along the seam, which the candidate windows walk; seam[0]
// holds the band). Two kernels: the scan reads every record with streaming
// (evict-first) loads and lists the selected ones; then the list is
// prefetched, after the stream, so that the stream does not evict it.
constexpr double kSeamBand = 3.0;

// seam[0] = kSeamBand mean point spacings: sqrt(bounding-box area / m)
__global__ void k_seam_band(const unsigned long long* __restrict__ box, int m, double* __restrict__ seam)
{
    auto val = [](unsigned long long k) {
        return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
    };
    const double w = val(box[2]) - val(box[0]), h = val(box[3]) - val(box[1]);
    const double a = w * h;
    seam[0] = (m > 0 && a > 0.0 && isfinite(a)) ? kSeamBand * sqrt(a / m) : 0.0;
}

// hist (split depths, else nullptr): per node, the records within three of
// their own lengths of the node's cut, counted in kSeamBins bins along the
// seam. A merge makes about one step per point spacing along its seam, and
// a band as wide as the local spacing holds about as many records per unit
// of seam, in dense and sparse parts alike: the counts follow the steps, and
// the split merge meets at their median.
__global__ void k_prefetch_seams(const Rec* __restrict__ R, int nrec, int m, int d, const double* __restrict__ seam,
    uint32_t* __restrict__ list, uint32_t* __restrict__ count, uint32_t cap, unsigned long long* __restrict__ hist,
    const unsigned long long* __restrict__ box)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int4 org = __ldcs(reinterpret_cast<const int4*>(&R[r].org[0]));
    if (org.x < 0) return;
    const double2 p0 = __ldcs(&R[r].p[0]), p1 = __ldcs(&R[r].p[1]);
    // the node of depth d whose record range holds r
    const int i = r / 3;
    int       a = 0, b = m;
    long long k = 0;
    for (int l = 0; l < d; ++l)
    {
        if (b - a < 4) return;
        const int c = a + (b - a) / 2;
        if (i < c) b = c, k = 2 * k;
        else a = c, k = 2 * k + 1;
    }
    if (b - a < 4) return;
    const double s = seam[(1ll << d) + k];
    const double c0 = (d & 1) ? p0.y : p0.x, c1 = (d & 1) ? p1.y : p1.x;
    const double dist = fmin(fabs(c0 - s), fabs(c1 - s));
    const double len = fmax(fabs(p0.x - p1.x), fabs(p0.y - p1.y));
    if (dist <= 3.0 * len || dist <= seam[0])
    {
        const uint32_t i = atomicAdd(count, 1u);
        if (i < cap) list[i] = (uint32_t)r;
        if (hist && dist <= 3.0 * len)
        {
            const int bin = seam_bin((d & 1) ? p0.x : p0.y, seam_range(seam, box, d, k));
            atomicAdd(&hist[((1ll << d) + k) * kSeamBins + bin], 1ull);
        }
    }
}

__global__ void k_prefetch_list(const Rec* __restrict__ R, const uint32_t* __restrict__ list,
    const uint32_t* __restrict__ count, uint32_t cap)
{
    const uint32_t n = min(*count, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const char* base = reinterpret_cast<const char*>(&R[list[i]]);
        asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(base));
        asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(base + 32));
    }
}

// The cells of depth dc, one warp each (build_cell).
__global__ void __launch_bounds__(kCellBlockWarps * 32) k_build_cells(Rec* __restrict__ R,
    const double2* __restrict__ V, NodeOut* __restrict__ out, int m, int dc, int C, DevStatus* st, int count)
{
    extern __shared__ __align__(16) char cell_smem[];
    const int       w = threadIdx.x >> 5;
    const long long k = (long long)blockIdx.x * (blockDim.x >> 5) + w;
    if (k >= (1ll << dc)) return;
    const unsigned flags = __shfl_sync(0xffffffffu, *(volatile unsigned*)&st->flags, 0);
    if (flags & kFatal) return;
    int lo, hi;
    if (!node_range(m, dc, k, lo, hi) || hi - lo > C) return;
    build_cell(cell_smem + w * cell_smem_bytes(C), V, R, lo, hi, dc, st, pred_stage(st, kStageThread, count), out + k);
}

// Depths with at most b.warp_nodes nodes run one node per warp (few merges:
// the latency of each merge matters), the deeper ones one node per thread
// (many merges: throughput).
void launch_build(const BuildBuffers& b, int m, cudaStream_t s)
{
    const int nrec = 3 * m;
    // records in use: the pool, then the split merges' spare records, dead
    // until a walker takes one
    const int nall = b.split.depth >= 0 ? nrec + b.split.spare : nrec;
    if (nall > nrec) cudaMemsetAsync(b.recs + nrec, 0xFF, (size_t)(nall - nrec) * sizeof(Rec), s);
    int D = split_levels(m);
    const int C = b.cell_points;
    if (C >= 4 && C <= kCellMax)
    {
        // the bottom of the tree in shared-memory cells, then the levels above
        const int dc = cell_depth(m, C);
        const int warps = cell_block_warps(C);
        const int bytes = warps * cell_smem_bytes(C);
        cudaFuncSetAttribute(k_build_cells, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        const unsigned g = (unsigned)(((1ll << dc) + warps - 1) / warps);
        k_build_cells<<<g, warps * 32, bytes, s>>>(b.recs, b.V, b.node[dc & 1], m, dc, C, b.status, b.count_filter);
        ++launch_counter();
        D = dc - 1;
    }
    const bool prefetch = b.seam && b.box && m >= (1 << 16);
    if (prefetch)
    {
        k_seam_band<<<1, 1, 0, s>>>(b.box, m, const_cast<double*>(b.seam));
        ++launch_counter();
    }
    // the seam prefetch of depth pd on stream ps: the list lives in the
    // extraction's offsets (3 m words, unused until the extraction) and its
    // length in the triangle counter (written by the extraction's scan)
    auto prefetch_depth = [&](int pd, cudaStream_t ps) {
        uint32_t* const list = b.tri_off;
        uint32_t* const count = b.tri_count;
        cudaMemsetAsync(count, 0, sizeof(uint32_t), ps);
        unsigned long long* const hist = pd <= b.split.depth ? b.seam_hist : nullptr;
        if (hist)
            cudaMemsetAsync(hist + ((size_t)1 << pd) * kSeamBins, 0,
                ((size_t)1 << pd) * kSeamBins * sizeof(unsigned long long), ps);
        k_prefetch_seams<<<(unsigned)((nrec + 255) / 256), 256, 0, ps>>>(b.recs, nrec, m, pd, b.seam, list, count,
            (uint32_t)nrec, hist, b.box);
        k_prefetch_list<<<152 * 8, 256, 0, ps>>>(b.recs, list, count, (uint32_t)nrec);
        launch_counter() += 2;
    };
    // With a side stream, the prefetch of depth d - 1 runs beside the merges
    // of depth d (a few SMs), and depth d - 1 waits for it; it reads records
    // those merges may be editing, which only makes a hint less exact.
    const bool overlap = prefetch && b.side && b.fork && b.join;
    bool       pending = false;
    for (int d = D; d >= 0; --d)
    {
        const long long nodes = 1ll << d;
        if (d <= kSeamDepth && prefetch)
        {
            if (pending) cudaStreamWaitEvent(s, b.join, 0);
            else prefetch_depth(d, s);
            pending = false;
        }
        // (a split depth's prefetch also sums the seam histogram that places
        // its meeting points: it runs in line, when no merge edits records)
        if (overlap && d >= 1 && d - 1 <= kSeamDepth && d - 1 > b.split.depth)
        {
            cudaEventRecord(b.fork, s);
            cudaStreamWaitEvent(b.side, b.fork, 0);
            prefetch_depth(d - 1, b.side);
            cudaEventRecord(b.join, b.side);
            pending = true;
        }
        // a warp per merge at the depths with at most warp_nodes nodes, and
        // at those whose nodes hold at least kWarpMinPoints points (the 4 M
        // Gaussian mixture: depth 14, 244 points a node, 72.7 -> 70.2 ms;
        // at 160 points a node, 2.6 M uniform, either form takes the same)
        if (d <= b.split.depth)
        {
            // two walkers per merge, one block per node
            const unsigned long long* hist = prefetch && b.seam_hist ? b.seam_hist : nullptr;
            if (b.window == 1)
                k_build_split<1><<<(unsigned)nodes, 96, 0, s>>>(b.recs, nall, b.node[(d + 1) & 1], b.node[d & 1], m,
                    d, b.status, b.count_filter, b.split, b.seam, hist, b.box);
            else
                k_build_split<kWinDefault><<<(unsigned)nodes, 96, 0, s>>>(b.recs, nall, b.node[(d + 1) & 1],
                    b.node[d & 1], m, d, b.status, b.count_filter, b.split, b.seam, hist, b.box);
        }
        else if ((1ll << d) <= b.warp_nodes || (m >> d) >= kWarpMinPoints)
        {
            const unsigned g = (unsigned)((nodes * 32 + 127) / 128);
            if (b.window == 1)
                k_build_level<true, 1><<<g, 128, 0, s>>>(b.recs, nall, b.V, b.node[(d + 1) & 1], b.node[d & 1], m,
                    d, b.status, b.count_filter);
            else
                k_build_level<true><<<g, 128, 0, s>>>(b.recs, nall, b.V, b.node[(d + 1) & 1], b.node[d & 1], m, d,
                    b.status, b.count_filter);
        }
        else
        {
            const unsigned g = (unsigned)((nodes + 127) / 128);
            k_build_level<false><<<g, 128, 0, s>>>(b.recs, nall, b.V, b.node[(d + 1) & 1], b.node[d & 1], m, d,
                b.status, b.count_filter);
        }
        ++launch_counter();
    }
}

// ---------------------------------------------------------------------------
// Extraction (reference builder.hxx:98-116): a face is emitted once, by the
// smallest of its three half-edge ids, when it is a 3-cycle (lnext) oriented
// counter-clockwise.
// ---------------------------------------------------------------------------

__global__ void k_tri_mask(const Rec* __restrict__ R, int nrec, uint8_t* __restrict__ mask, DevStatus* st, int count)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrec) return;
    if (*(volatile unsigned*)&st->flags & kFatal)
    {
        mask[k] = 0;
        return;
    }
    Builder B{ const_cast<Rec*>(R), nrec, st, pred_stage(st, kStageExtract, count), -1, -1, false };
    uint8_t mk = 0;
    if (R[k].org[0] >= 0)
    {
        for (int s = 0; s < 2; ++s)
        {
            const int e = 2 * k + s;
            const int f = B.lnext(e), g = B.lnext(f);
            if (B.lnext(g) != e) continue;
            if (e > f || e > g) continue;
            if (ccw(B.porg(e), B.porg(f), B.porg(g), B.pc)) mk |= (uint8_t)(1 << s);
        }
    }
    mask[k] = B.bad ? 0 : mk;
}

struct MaskCount
{
    const uint8_t* m;
    __device__ __forceinline__ uint32_t operator()(size_t i) const { return __popc((unsigned)m[i]); }
};

__global__ void k_tri_write(const Rec* __restrict__ R, int nrec, const uint8_t* __restrict__ mask,
    const uint32_t* __restrict__ off, const uint32_t* __restrict__ vid, uint32_t* __restrict__ tris)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrec) return;
    const uint8_t mk = mask[k];
    if (!mk) return;
    uint32_t o = off[k];
    for (int s = 0; s < 2; ++s)
    {
        if (!(mk & (1 << s))) continue;
        const int e = 2 * k + s;
        const int f = R[sym(e) >> 1].prev[sym(e) & 1];   // lnext(e) = oprev(sym(e))
        const int g = R[sym(f) >> 1].prev[sym(f) & 1];
        tris[3 * (size_t)o + 0] = vid[R[e >> 1].org[e & 1]];
        tris[3 * (size_t)o + 1] = vid[R[f >> 1].org[f & 1]];
        tris[3 * (size_t)o + 2] = vid[R[g >> 1].org[g & 1]];
        ++o;
    }
}

void launch_extract(const BuildBuffers& b, int m, cudaStream_t s)
{
    const int      nrec = b.split.depth >= 0 ? 3 * m + b.split.spare : 3 * m;
    const unsigned g = (unsigned)((nrec + 255) / 256);
    k_tri_mask<<<g, 256, 0, s>>>(b.recs, nrec, b.tri_mask, b.status, b.count_filter);
    ++launch_counter();
    scan_exclusive(MaskCount{ b.tri_mask }, (size_t)nrec, b.tri_off, b.scratch, b.tri_count, s);
    k_tri_write<<<g, 256, 0, s>>>(b.recs, nrec, b.tri_mask, b.tri_off, b.vid, b.tris);
    ++launch_counter();
}

}  // namespace QDTG_BUILD_VARIANT
}  // namespace qdtg
