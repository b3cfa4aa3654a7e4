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

// The merges of one upper depth with split seams (seam_split.cuh): one block
// per node, two walker warps per seam segment (rising and falling) and the
// ring inserter in the last warp. Before the walkers start, the first warps
// look for the segment boundaries (one lane each) and thread 0 checks and
// links them; a node whose boundaries cannot all be found and checked runs
// as one segment. The block's threads then remove the deleted edges
// together, and its first thread finds the node's extremes.
constexpr int kSplitThreads = 32 * (kSeamWalkers + 1);

// the coordinate along the seam at which the histogram's cumulative count
// reaches the fraction f of its total, counted in the rising direction
// (increasing y for even depths, decreasing x for odd ones); bin: its bin
__device__ inline double seam_quantile(const unsigned long long* __restrict__ h, double2 rg, int frame, double f,
    int& bin)
{
    unsigned long long total = 0;
    for (int b = 0; b < kSeamBins; ++b) total += h[b];
    const double       target = (frame ? 1.0 - f : f) * (double)total;
    unsigned long long acc = 0;
    int                b = 0;
    while (b < kSeamBins - 1 && (double)(acc + h[b]) < target) acc += h[b++];
    bin = b;
    return rg.x + (b + 0.5) * ((rg.y - rg.x) / kSeamBins);
}

template <int WIN>
__global__ void __maxnreg__(168) k_build_split(Rec* __restrict__ R, int nrec, const NodeOut* __restrict__ child,
    NodeOut* __restrict__ out, int m, int d, DevStatus* st, int count, SplitPlan plan, const double* __restrict__ seam,
    const unsigned long long* __restrict__ hist, const unsigned long long* __restrict__ near,
    const unsigned long long* __restrict__ box)
{
    __shared__ SeamShared S;
    __shared__ int        go;
    __shared__ int        gl[kSeamSegs], gr[kSeamSegs];   // the boundary pairs found (half-edges, -1: none)
    const long long       k = blockIdx.x;
    const int             warp = threadIdx.x >> 5;
    const int             lane = threadIdx.x & 31;
    int                   lo = 0, hi = 0;
    if (threadIdx.x == 0)
    {
        go = !(*(volatile unsigned*)&st->flags & kFatal) && k < (1ll << d) && node_range(m, d, k, lo, hi) &&
             hi - lo >= 4;
        for (int v = 0; v < kSeamWalkers; ++v) S.tail[v] = S.head[v] = S.state[v] = S.ndel[v] = 0;
        S.ndel[kSeamWalkers] = 0;
        for (int j = 0; j < kSeamSegs; ++j)
        {
            S.last_o[j] = S.last_d[j] = S.last_e[j] = -1;
            S.rstop[j] = S.fdone[j] = S.fpub[j] = S.rdone[j] = 0;
            S.rlast_o[j] = S.rlast_d[j] = S.rlast_e[j] = -1;
            S.gate[j] = -1;
            gl[j] = gr[j] = -1;
        }
        S.nseg = 1;
        S.first_dn = -1;
        S.base0 = S.ldo = S.rdo = S.top = -1;
        S.fhead = S.ftail = -1;
        S.fail = 0;
    }
    __syncthreads();
    if (!go) return;
    node_range(m, d, k, lo, hi);
    const int     n = hi - lo;
    const int     mid = lo + n / 2;
    const NodeOut L = child[2 * k], Rn = child[2 * k + 1];
    const int     g = (d - 1) & 1;   // the parent's frame
    const int     frame = d & 1;
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
    // the meeting points: on the node's cut (x for even d), and along the
    // seam at quantiles of the records near the seam (the histogram of the
    // seam prefetch), else the mean of the children's cuts
    const double  cut = seam[(1ll << d) + k];
    const double2 rg = seam_range(seam, box, d, k);
    auto          at = [&](double along) { return frame ? make_double2(along, cut) : make_double2(cut, along); };
    const unsigned long long* h = hist ? hist + ((1ll << d) + k) * kSeamBins : nullptr;
    bool          counted = false;
    if (h)
        for (int b = 0; b < kSeamBins && !counted; ++b) counted = h[b] != 0;
    const int want = (counted && near) ? plan.segs[d] : 1;
    Builder   B{ R, nrec, st, pred_stage(st, kStageWarp, count), S.fhead, S.ftail, false };
    // ---- segment boundaries: one lane per boundary j = 1 .. want - 1 ----
    if (want > 1 && warp < want - 1 && lane == 0)
    {
        const int j = warp + 1;
        int       bin = 0;
        seam_quantile(h, rg, frame, (double)j / want, bin);
        // the vertices nearest to the cut in the nearest bins that have one
        int hs[2] = { -1, -1 };
        for (int side = 0; side < 2; ++side)
            for (int t = 0; t < 2 * kSeamBins && hs[side] < 0; ++t)
            {
                const int b = bin + ((t & 1) ? -((t + 1) >> 1) : (t >> 1));
                if (b < 0 || b >= kSeamBins) continue;
                const unsigned long long key = near[(((1ll << d) + k) * kSeamBins + b) * 2 + side];
                if (key == ~0ull) continue;
                const int e = (int)(unsigned)key;
                if ((unsigned)e >= 2u * (unsigned)nrec) continue;
                const int v = R[e >> 1].org[e & 1];
                if (side == 0 ? (v >= lo && v < mid) : (v >= mid && v < hi)) hs[side] = e;
            }
        if (hs[0] >= 0 && hs[1] >= 0 && seam_gabriel(R, nrec, hs[0], hs[1]))
        {
            const int vl = R[hs[0] >> 1].org[hs[0] & 1], vr = R[hs[1] >> 1].org[hs[1] & 1];
            if (vl >= lo && vl < mid && vr >= mid && vr < hi)
            {
                gl[j] = hs[0];
                gr[j] = hs[1];
            }
        }
    }
    __syncthreads();
    // ---- thread 0: check the boundaries and the meeting points, link them ----
    if (threadIdx.x == 0)
    {
        int nseg = want;
        for (int j = 1; j < nseg; ++j)
            if (gl[j] < 0) nseg = 1;
        // no two boundaries share a vertex (their ring slots are found apart)
        for (int a = 1; a < nseg; ++a)
            for (int c = a + 1; c < nseg; ++c)
            {
                const int la = R[gl[a] >> 1].org[gl[a] & 1], ra = R[gr[a] >> 1].org[gr[a] & 1];
                const int lc = R[gl[c] >> 1].org[gl[c] & 1], rc = R[gr[c] >> 1].org[gr[c] & 1];
                if (la == lc || ra == rc) nseg = 1;
            }
        double2 qs[kSeamSegs];
        int     sl[kSeamSegs], sr[kSeamSegs];
        if (nseg > 1)
        {
            // meeting points: below the first boundary and above the last at
            // the histogram's quantiles, between two boundaries halfway
            int bin = 0;
            qs[0] = at(seam_quantile(h, rg, frame, 0.5 / nseg, bin));
            qs[nseg - 1] = at(seam_quantile(h, rg, frame, (nseg - 0.5) / nseg, bin));
            for (int j = 1; j + 1 < nseg; ++j)
            {
                const double2 a0 = R[gl[j] >> 1].p[gl[j] & 1], a1 = R[gr[j] >> 1].p[gr[j] & 1];
                const double2 b0 = R[gl[j + 1] >> 1].p[gl[j + 1] & 1], b1 = R[gr[j + 1] >> 1].p[gr[j + 1] & 1];
                const double  ca = frame ? 0.5 * (a0.x + a1.x) : 0.5 * (a0.y + a1.y);
                const double  cb = frame ? 0.5 * (b0.x + b1.x) : 0.5 * (b0.y + b1.y);
                qs[j] = at(0.5 * (ca + cb));
            }
            // each meeting point strictly above its segment's lower boundary
            // and not above its upper one (boundary j: right end -> left end)
            for (int j = 0; j < nseg && nseg > 1; ++j)
            {
                const SeamKey kq = seam_keys(qs[j], frame);
                for (int t = j; t <= j + 1; ++t)
                {
                    if (t < 1 || t >= nseg) continue;
                    const double2 po = R[gr[t] >> 1].p[gr[t] & 1], pt = R[gl[t] >> 1].p[gl[t] & 1];
                    const bool    above =
                        seam_q_above(qs[j], kq, po, pt, seam_keys(po, frame), seam_keys(pt, frame), B.pc);
                    if (above != (t == j)) nseg = 1;
                }
            }
        }
        // the ring slots: right end counter-clockwise after sr, left end after sl
        for (int j = 1; j < nseg; ++j)
        {
            sr[j] = seam_slot(R, nrec, gr[j], R[gl[j] >> 1].p[gl[j] & 1], B.pc);
            sl[j] = seam_slot(R, nrec, gl[j], R[gr[j] >> 1].p[gr[j] & 1], B.pc);
            if (sr[j] < 0 || sl[j] < 0)
            {
                nseg = 1;
                break;
            }
            // the first candidates of the rising walker that starts here (the
            // next left edge counter-clockwise after the boundary, the next
            // right edge clockwise): a zero among their first tests (points
            // cocircular or collinear with the boundary) would fail that
            // walker, so such a boundary is not used
            const double2 pl = R[gl[j] >> 1].p[gl[j] & 1], pr = R[gr[j] >> 1].p[gr[j] & 1];
            const int     ya = R[sl[j] >> 1].next[sl[j] & 1];
            const double2 pa = R[ya >> 1].p[(ya & 1) ^ 1], pb = R[sr[j] >> 1].p[(sr[j] & 1) ^ 1];
            if (orient2d_sign(pa.x, pa.y, pl.x, pl.y, pr.x, pr.y, B.pc) == 0 ||
                orient2d_sign(pb.x, pb.y, pl.x, pl.y, pr.x, pr.y, B.pc) == 0 ||
                incircle_sign(pl.x, pl.y, pr.x, pr.y, pa.x, pa.y, pb.x, pb.y, B.pc) == 0)
            {
                nseg = 1;
                break;
            }
        }
        // the children's edges that cross a boundary, listed after the
        // walkers' lists (nseg == want here: the plan's last list)
        const int off = (int)(plan.base[d] + (long long)split_lists(plan.segs[d]) * plan.per[d] * k);
        int       npre = 0;
        int*      pre = plan.lists + off + 2 * want * plan.per[d];
        for (int j = 1; j < nseg; ++j)
            if (!seam_crossed(R, nrec, sl[j], R[gr[j] >> 1].p[gr[j] & 1], pre, npre, plan.per[d], B.pc) ||
                !seam_crossed(R, nrec, sr[j], R[gl[j] >> 1].p[gl[j] & 1], pre, npre, plan.per[d], B.pc))
                nseg = 1;
        if (nseg > 1)
        {
            for (int i = 0; i < npre; ++i) atomicOr(reinterpret_cast<unsigned*>(&R[pre[i]].pad), kSeamPre);
            S.ndel[2 * nseg] = npre;
            for (int j = 1; j < nseg; ++j)
            {
                // the boundary edge e from r to l: the first spare record of
                // segment j's rising walker
                const int     kk = plan.spare0 + off + 2 * j * plan.per[d];
                const int     e = 2 * kk;
                const int     vr = R[gr[j] >> 1].org[gr[j] & 1], vl = R[gl[j] >> 1].org[gl[j] & 1];
                const double2 pr = R[gr[j] >> 1].p[gr[j] & 1], pl = R[gl[j] >> 1].p[gl[j] & 1];
                const int     yr = R[sr[j] >> 1].next[sr[j] & 1], yl = R[sl[j] >> 1].next[sl[j] & 1];
                *reinterpret_cast<int4*>(&R[kk].org[0]) =
                    make_int4(vr, vl, -1, (int)(seam_gate_tag(kSeamTagStride * (unsigned)((1ll << d) + k), j) << 16));
                R[kk].p[0] = pr;
                R[kk].p[1] = pl;
                R[kk].next[0] = yr;
                R[kk].prev[0] = sr[j];
                R[kk].next[1] = yl;
                R[kk].prev[1] = sl[j];
                R[sr[j] >> 1].next[sr[j] & 1] = e;
                R[yr >> 1].prev[yr & 1] = e;
                R[sl[j] >> 1].next[sl[j] & 1] = e + 1;
                R[yl >> 1].prev[yl & 1] = e + 1;
                S.gate[j] = e;
            }
            for (int j = 0; j < nseg; ++j) S.q_seg[j] = qs[j];
        }
        else
        {
            // one segment: the meeting point at the median
            double along = 0.5 * (seam[(1ll << (d + 1)) + 2 * k] + seam[(1ll << (d + 1)) + 2 * k + 1]);
            if (counted)
            {
                int bin = 0;
                along = seam_quantile(h, rg, frame, 0.5, bin);
            }
            S.q_seg[0] = at(along);
        }
        S.nseg = nseg;
        __threadfence_block();
    }
    __syncthreads();
    const int nseg = S.nseg;
    SeamArgs  A;
    A.R = R;
    A.nrec = nrec;
    A.tag = kSeamTagStride * (unsigned)((1ll << d) + k);
    const long long off = plan.base[d] + (long long)split_lists(plan.segs[d]) * plan.per[d] * k;
    A.w = warp;
    A.seg = warp >> 1;
    A.nseg = nseg;
    A.q = S.q_seg[min(A.seg, kSeamSegs - 1)];
    A.start = -1;
    if (warp < 2 * nseg)
    {
        if (warp & 1) A.start = A.seg + 1 < nseg ? S.gate[A.seg + 1] : -1;
        else A.start = A.seg > 0 ? S.gate[A.seg] : -1;
    }
    A.a0 = plan.spare0 + (int)(off + (long long)warp * plan.per[d]) + ((warp & 1) == 0 && A.seg > 0 ? 1 : 0);
    A.a1 = plan.spare0 + (int)(off + (long long)(warp + 1) * plan.per[d]);
    A.lists = plan.lists + off;
    A.cap = plan.per[d];
    A.lim = 8 * n + 64;
    A.frame = frame;
    A.st = st;
    if (warp < 2 * nseg)
    {
        if (warp & 1) seam_walk<true, WIN>(B, S, A, L.le, L.re, Rn.le, Rn.re);
        else seam_walk<false, WIN>(B, S, A, L.le, L.re, Rn.le, Rn.re);
    }
    else if (warp == kSeamWalkers && lane == 0)
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
        seam_apply(R, nrec, plan.lists + off, plan.per[d], S.ndel, split_lists(nseg), fh, ft, threadIdx.x,
            (int)blockDim.x, [] { __syncthreads(); }, bad);
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
// the split merge places its segments and meeting points at their
// quantiles. near (with hist): per node, bin and side of the cut, the
// half-edge leaving the vertex nearest to the cut (the minimum of the
// distance's float bits above the half-edge id: the same whatever the
// order of the atomics), where the search for a segment boundary starts.
__global__ void k_prefetch_seams(const Rec* __restrict__ R, int nrec, int m, int d, const double* __restrict__ seam,
    uint32_t* __restrict__ list, uint32_t* __restrict__ count, uint32_t cap, unsigned long long* __restrict__ hist,
    unsigned long long* __restrict__ near, const unsigned long long* __restrict__ box)
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
        if (near)
        {
            // each end by its own vertex's node (a record of a split merge's
            // spare range lies outside every node's record range)
            for (int s = 0; s < 2; ++s)
            {
                const int v = s ? org.y : org.x;
                if (v < 0 || v >= m) continue;
                int       va = 0, vb = m;
                long long vk = 0;
                for (int l = 0; l < d && vb - va >= 4; ++l)
                {
                    const int c = va + (vb - va) / 2;
                    if (v < c) vb = c, vk = 2 * vk;
                    else va = c, vk = 2 * vk + 1;
                }
                if (vb - va < 4) continue;
                const double2 p = s ? p1 : p0;
                const double  sv = seam[(1ll << d) + vk];
                const float   dv = (float)fabs(((d & 1) ? p.y : p.x) - sv);
                const int     bin = seam_bin((d & 1) ? p.x : p.y, seam_range(seam, box, d, vk));
                const int     side = v >= va + (vb - va) / 2 ? 1 : 0;
                const unsigned long long key =
                    ((unsigned long long)__float_as_uint(dv) << 32) | (unsigned)(2 * r + s);
                atomicMin(&near[(((1ll << d) + vk) * kSeamBins + bin) * 2 + side], key);
            }
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
        unsigned long long* const near = hist && b.split.segs[pd] > 1 ? b.seam_near : nullptr;
        if (hist)
            cudaMemsetAsync(hist + ((size_t)1 << pd) * kSeamBins, 0,
                ((size_t)1 << pd) * kSeamBins * sizeof(unsigned long long), ps);
        if (near)
            cudaMemsetAsync(near + ((size_t)1 << pd) * kSeamBins * 2, 0xFF,
                ((size_t)1 << pd) * kSeamBins * 2 * sizeof(unsigned long long), ps);
        k_prefetch_seams<<<(unsigned)((nrec + 255) / 256), 256, 0, ps>>>(b.recs, nrec, m, pd, b.seam, list, count,
            (uint32_t)nrec, hist, near, b.box);
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
            // two walkers per seam segment, one block per node
            const unsigned long long* hist = prefetch && b.seam_hist ? b.seam_hist : nullptr;
            const unsigned long long* near = hist && b.split.segs[d] > 1 ? b.seam_near : nullptr;
            if (b.window == 1)
                k_build_split<1><<<(unsigned)nodes, kSplitThreads, 0, s>>>(b.recs, nall, b.node[(d + 1) & 1],
                    b.node[d & 1], m, d, b.status, b.count_filter, b.split, b.seam, hist, near, b.box);
            else
                k_build_split<kWinDefault><<<(unsigned)nodes, kSplitThreads, 0, s>>>(b.recs, nall,
                    b.node[(d + 1) & 1], b.node[d & 1], m, d, b.status, b.count_filter, b.split, b.seam, hist, near,
                    b.box);
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
