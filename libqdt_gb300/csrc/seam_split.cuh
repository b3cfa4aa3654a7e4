// Split merges: the seam of one top-level merge walked by several warps at
// once.
//
// The merge of the reference builder (builder.hxx:251-285) is one chain of
// bubble steps from the lower common tangent up to the upper one. At the top
// of the tree that chain is long (about 3,600 steps at the root of 2.6 M
// uniform points) and nothing else runs beside it. Here the seam is cut into
// up to kSeamSegs segments, each walked by two warps: a rising walker runs
// the reference's merge up from the segment's lower end while a falling
// walker runs its mirror image (the same merge with the rotations and the
// predicate signs reversed) down from its upper end. All are warp merges
// with the candidate window of warp_merge.
//
// Segment ends. The first segment starts at the lower tangent and the last
// ends at the upper one; the others meet at boundary edges found before the
// walkers start: pairs of mutually nearest vertices of the two halves, which
// are edges of every Delaunay triangulation of the merged points (see the
// segment boundaries below), linked into the rings first, with the
// children's edges that cross them deleted.
//
// The walkers never see each other's work:
// * each record carries a tag word (Rec::pad): one bit per walker marks the
//   edges it deleted (bit 12, kSeamPre, the ones deleted before the walkers), and
//   bits 16..31 name the walker that made the edge, or the boundary;
// * deletions only set the walker's bit: the edge stays in its rings until
//   the merge ends, and the walker that deleted it steps over it;
// * insertions are real ring insertions, but the other walkers step over
//   them; each one goes right next to one of the new edge's anchors (the
//   walker's own previous edge or the candidate edge it chose), never next
//   to an edge of another walker, so the walkers' insertions keep their
//   order in every ring they share.
// So each walker sees exactly the map its own sequential merge would have
// at that step: the bottom rising walker makes the reference's decisions,
// and every other walker those of a sequential merge (or its mirror)
// started at its segment's end.
//
// Where two walkers of a segment meet: q is a point on the seam (on the
// node's cut line, at a quantile of the records near the seam, or halfway
// between two boundaries). The rising walker keeps the edges that have q
// strictly above them, the falling walker the others; the test is one exact
// orientation, the same in both walkers. The rising walker's first edge
// without q above is the falling walker's last one: it stops there and
// takes that edge. A merge started anywhere but at the lower tangent
// decides like the reference only where no predicate it evaluates is zero
// (without zeros every decision holds for all small perturbations of the
// points; the edges made and deleted are then those of every Delaunay
// triangulation of the points, the reference's included). So a falling
// walker stops at its first zero (cocircular or collinear points), and the
// rising walker of its segment goes on past q up to the falling walker's
// last edge; a rising walker above the first segment that meets a zero
// fails the merge. A failed split merge (that, or a rising walker whose
// chain does not meet its falling walker's last edge) reports ST_SPLIT and
// the call runs again with one segment a merge, and then, if that fails
// too, without split merges.
//
// Spare records: a walker makes its edges before the deleted ones are
// freed, so each one has a range of spare records after the pool (the
// bottom rising one takes its node's free list first). When a falling
// walker's range or deletion list runs out it stops; when the bottom rising
// walker's runs out, it waits for every other walker to stop and then frees
// every deleted edge (seam_apply) before it goes on; another rising walker
// fails the merge.
//
// At the end the block removes the deleted edges from their rings and puts
// their records on the node's free list, the walkers' lists in order, then
// the edges deleted before the walkers: the record ids, and so the output,
// do not depend on how the warps were scheduled.
//
// Shared rings: one thread of the block (the inserter) makes every ring
// insertion, each walker's in its order, reading the anchors' neighbours
// as the rings are then.
//
// Every wait on another warp is bounded; a wait that runs out, like any
// other failure of a split merge, reports ST_SPLIT and ends the merge.
#pragma once

#include "builder.cuh"

#ifndef QDTG_SPLIT_DEBUG
#define QDTG_SPLIT_DEBUG 0
#endif
#if QDTG_SPLIT_DEBUG
#include <cstdio>
#endif

namespace qdtg {

// walkers of one merge at most: a rising and a falling one per segment of
// the seam (walker 2 j rises in segment j, walker 2 j + 1 falls)
constexpr int       kSeamSegs = kSplitMaxSegs;
constexpr int       kSeamWalkers = 2 * kSeamSegs;
static_assert(kSeamWalkers <= 12, "one deletion bit per walker below kSeamPre");
constexpr unsigned  kSeamPre = 1u << 12;   // deleted before the walkers start (crosses a segment boundary)
constexpr unsigned  kSeamDel = (1u << 13) - 1u;   // deletion flags of a record's tag word: one bit per walker, and kSeamPre
constexpr unsigned  kSeamTagStride = 32;  // creator values of one merge: tag .. tag + 31
// insertions a walker may have waiting (2: fewer registers held for the
// pending anchors at the 168-register cap, 2.6 M 22.83 -> 22.61 ms a call
// against 4)
constexpr int       kSeamQueue = 2;
constexpr long long kSeamSpin = 1ll << 24;

// A ring insertion a walker asks for: the new edge e = 2 k from vo to vt
// goes right before Q1 in the walker's rotation around vo, sym(e) right
// after P2 around vt.
struct SeamReq
{
    int     k, vo, vt, Q1, P2, pad;
    double2 po, pt;
};

struct SeamShared
{
    SeamReq q[kSeamWalkers][kSeamQueue];
    int     tail[kSeamWalkers];    // insertions each walker posted
    int     head[kSeamWalkers];    // of those, the ones the inserter made
    int     state[kSeamWalkers];   // 1 once the walker stopped
    int     ndel[kSeamWalkers + 1];   // deletion-list fills; [2 nseg]: the edges deleted before the walkers
    int     last_o[kSeamSegs], last_d[kSeamSegs], last_e[kSeamSegs];   // each falling walker's last edge (-1: none)
    // a rising walker above the first segment that ran out of records stops
    // early (rstop) at its last edge (rlast_*), and its falling walker goes
    // on down to that edge; fdone: the falling walker finished (set before
    // it reads rstop, as rstop is set before the rising walker reads fdone)
    int     rstop[kSeamSegs], fdone[kSeamSegs];
    // above the first segment a falling walker that reaches q publishes its
    // last edge (fpub) and waits until its rising walker is done (rdone) or
    // stopped early
    int     fpub[kSeamSegs], rdone[kSeamSegs];
    int     rlast_o[kSeamSegs], rlast_d[kSeamSegs], rlast_e[kSeamSegs];
    int     gate[kSeamSegs];       // the boundary edge where segment j begins (j >= 1)
    double2 q_seg[kSeamSegs];      // each segment's meeting point
    int     nseg;                  // segments of this merge
    int     first_dn;              // the top falling walker's first edge (the upper tangent), -1: none
    int     base0, ldo, rdo, top;  // the bottom rising walker's lower tangent and hull edges; the top one's last edge
    int     fhead, ftail;          // the node's free list
    int     fail;
};

struct SeamArgs
{
    Rec*       R;
    int        nrec;     // pool and spare records
    unsigned   tag;      // kSeamTagStride * node: creators tag + 1 + w, boundaries seam_gate_tag
    double2    q;        // the segment's meeting point on the seam
    int        w;        // this walker
    int        seg;      // its segment
    int        nseg;     // segments
    int        start;    // the boundary edge it starts from (-1: the tangent)
    int        a0, a1;   // this walker's spare records [a0, a1)
    int*       lists;    // deletion lists, cap entries a walker
    int        cap;
    int        lim;      // iteration guard
    int        frame;    // the merge's frame (depth & 1): the seam runs along y (0) or -x (1)
    DevStatus* st;
};

// order-preserving key of a double (+0 and -0 alike)
__device__ __forceinline__ unsigned long long seam_key(double v)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if ((b << 1) == 0ull) b = 0ull;
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// a point's keys along the seam (up: the direction the rising walker
// climbs) and across it (the coordinate the node's cut splits)
struct SeamKey
{
    unsigned long long up, across;
};

__device__ __forceinline__ SeamKey seam_keys(double2 p, int frame)
{
    return frame ? SeamKey{ ~seam_key(p.x), seam_key(p.y) } : SeamKey{ seam_key(p.y), seam_key(p.x) };
}

// Creators in a record's tag word (bits 16..31), per merge (tag =
// kSeamTagStride * node, nodes below 1,024): tag + 1 + w for walker w's
// edges, tag + 16 + j for the boundary edge where segment j begins (j >= 1,
// seen by the two walkers that start there).
__device__ __forceinline__ unsigned seam_gate_tag(unsigned tag, int j) { return tag + 16u + (unsigned)j; }

// a record walker w does not see: deleted by it (mydel: its flag, and
// kSeamPre for a walker that starts at a segment boundary), or made in the
// same merge by another walker, or a segment boundary other than the one it
// starts at
__device__ __forceinline__ bool seam_skip(unsigned pad, unsigned mydel, unsigned tag, unsigned mytag, unsigned mygate)
{
    const unsigned c = pad >> 16;
    return (pad & mydel) != 0u || ((c & ~(kSeamTagStride - 1u)) == tag && c != mytag && c != mygate);
}

// q strictly above the cross edge po -> pt (po on the right, pt on the left
// side) in the rising direction of the seam: the seam keys decide when both
// endpoints lie on one side of q along the seam, else one exact orientation.
__device__ __forceinline__ bool seam_q_above(double2 q, SeamKey kq, double2 po, double2 pt, SeamKey ko, SeamKey kt,
    PredCounters* pc)
{
    if (!(ko.across == kq.across && kt.across == kq.across))
    {
        if (ko.up < kq.up && kt.up < kq.up) return true;
        if (ko.up > kq.up && kt.up > kq.up) return false;
    }
    const double2 dqo = make_double2(sub_rn(po.x, q.x), sub_rn(po.y, q.y));
    const double2 dqt = make_double2(sub_rn(pt.x, q.x), sub_rn(pt.y, q.y));
    int sg = orient2d_f32(dqt.x, dqt.y, dqo.x, dqo.y);
    if (!sg) sg = orient2d_slow(pt.x, pt.y, po.x, po.y, q.x, q.y, pc);
    return sg > 0;
}

// ---- segment boundaries ----
//
// A seam is cut into segments at cross edges that are known to be edges of
// the merged triangulation before any walker runs: pairs (l, r), l a vertex
// of the left child and r of the right one, such that l is the unique
// left vertex nearest to r and r the unique right vertex nearest to l. A
// point p of the left side inside or on the circle with diameter lr would
// be nearer to r than l (the angle lpr is at least a right angle), and a
// point of the right side nearer to l than r: that circle holds no other
// point, so lr is an edge of every Delaunay triangulation of the merged
// points, the reference's included, and the sequential merge passes it.
//
// When the sequential merge makes lr its base edge, no edge of either child
// crosses lr any more (a new cross edge never crosses a remaining edge: the
// ones it would cross are the candidates its step deletes). The children's
// edges that cross lr are deleted before the walkers start (kSeamPre); from
// then on each walker keeps that invariant itself, so a walker that starts
// at lr sees, above (or, falling, below) it, the map the sequential merge
// sees there, up to edges at l and r that its own first steps delete.

// sign of |p - t|^2 - |s - t|^2, 0 when the double evaluation cannot tell.
// Each difference carries a relative error of at most u = 2^-53, each
// square and sum one more rounding: the computed value is within 5 u (A +
// B) of the exact one (A, B the two squared lengths); 8 u is the bound.
__device__ __forceinline__ int seam_farther(double2 p, double2 s, double2 t)
{
    const double ax = __dsub_rn(p.x, t.x), ay = __dsub_rn(p.y, t.y);
    const double bx = __dsub_rn(s.x, t.x), by = __dsub_rn(s.y, t.y);
    const double a = __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay));
    const double b = __dadd_rn(__dmul_rn(bx, bx), __dmul_rn(by, by));
    const double sum = a + b;
    if (!(sum > 1e-280) || !(sum < 1e280)) return 0;
    const double v = __dsub_rn(a, b);
    const double bound = 8.0 * 1.1102230246251565e-16 * sum;
    return v > bound ? 1 : (v < -bound ? -1 : 0);
}

// The vertex of one child nearest to t, by steepest descent along the
// child's edges from the origin of half-edge e (before the merge a ring
// holds only the child's own edges; in a Delaunay triangulation a vertex
// that is not the nearest has a strictly nearer neighbour). Returns a
// half-edge leaving that vertex, every neighbour of which is strictly
// farther from t; -1 when a comparison is too close to call, an index is
// out of range or the walk runs long.
static __device__ int seam_nearest(const Rec* __restrict__ R, int nrec, int e, double2 t, int steps)
{
    const unsigned lim2 = 2u * (unsigned)nrec;
    if ((unsigned)e >= lim2) return -1;
    for (int step = 0; step < steps; ++step)
    {
        const double2 pv = R[e >> 1].p[e & 1];
        int           best = -1;
        double2       pb = pv;
        int           x = e;
        for (int deg = 0;; ++deg)
        {
            if (deg > 64) return -1;
            const double2 pu = R[x >> 1].p[(x & 1) ^ 1];
            const int     c = seam_farther(pu, pv, t);
            if (c == 0) return -1;
            if (c < 0 && (best < 0 || seam_farther(pu, pb, t) < 0))
            {
                best = x;
                pb = pu;
            }
            x = R[x >> 1].next[x & 1];
            if ((unsigned)x >= lim2) return -1;
            if (x == e) break;
        }
        if (best < 0) return e;
        e = best ^ 1;   // leaves the nearer neighbour
    }
    return -1;
}

// A segment boundary near the start half-edges hl (leaving a vertex of the
// left child) and hr (of the right one): alternating nearest-vertex walks
// until the pair settles. On success hl and hr leave l and r.
static __device__ bool seam_gabriel(const Rec* __restrict__ R, int nrec, int& hl, int& hr)
{
    int l = hl, r = hr;
    for (int it = 0; it < 12; ++it)
    {
        l = seam_nearest(R, nrec, l, R[r >> 1].p[r & 1], 512);
        if (l < 0) return false;
        const int r2 = seam_nearest(R, nrec, r, R[l >> 1].p[l & 1], 512);
        if (r2 < 0) return false;
        if (R[r2 >> 1].org[r2 & 1] == R[r >> 1].org[r & 1])
        {
            hl = l;
            hr = r2;
            return true;
        }
        r = r2;
    }
    return false;
}

// lnext(e): the next edge of e's left face
__device__ __forceinline__ int seam_lnext(const Rec* __restrict__ R, int e)
{
    return R[(e ^ 1) >> 1].prev[(e ^ 1) & 1];
}

// The records of one child's edges that the segment from v (the origin of
// slot, whose counter-clockwise wedge up to next(slot) holds the direction
// to t, seam_slot) towards t crosses, in order, appended to out[cnt ..) and
// not already tagged kSeamPre (an edge two boundaries cross is listed
// once). The walk goes from face to face of the child's triangulation until
// it leaves the child's hull. False when a vertex lies on the segment's
// line, a face is not a triangle where one must be, an index is out of
// range or more than cap edges are listed.
static __device__ bool seam_crossed(const Rec* __restrict__ R, int nrec, int slot, double2 t, int* out, int& cnt,
    int cap, PredCounters* pc)
{
    const unsigned lim2 = 2u * (unsigned)nrec;
    auto           ok = [&](int e) { return (unsigned)e < lim2; };
    auto           dst = [&](int e) { return R[e >> 1].p[(e & 1) ^ 1]; };
    if (!ok(slot)) return false;
    const double2 v = R[slot >> 1].p[slot & 1];
    const int     y = R[slot >> 1].next[slot & 1];
    if (!ok(y)) return false;
    if (y == slot) return true;   // a single edge: the segment leaves at once
    const double2 pa0 = dst(slot), pb0 = dst(y);
    if (orient2d_sign(v.x, v.y, pa0.x, pa0.y, pb0.x, pb0.y, pc) <= 0) return true;   // the outer wedge
    // the left face of slot is the triangle (v, a, b); the segment leaves it
    // through f = a -> b
    int f = seam_lnext(R, slot);
    if (!ok(f) || !ok(seam_lnext(R, f)) || seam_lnext(R, seam_lnext(R, f)) != slot) return false;
    for (int it = 0; it < 256; ++it)
    {
        const int k = f >> 1;
        if (!((unsigned)R[k].pad & kSeamPre))
        {
            bool seen = false;
            for (int i = 0; i < cnt && !seen; ++i) seen = out[i] == k;
            if (!seen)
            {
                if (cnt >= cap) return false;
                out[cnt++] = k;
            }
        }
        // the face across f: (b, a, c)
        const int g = f ^ 1, h1 = seam_lnext(R, g);
        if (!ok(h1)) return false;
        const int h2 = seam_lnext(R, h1);
        if (!ok(h2)) return false;
        if (seam_lnext(R, h2) != g) return true;   // the outer face: the segment left the hull
        const double2 pb = R[g >> 1].p[g & 1], pa = R[g >> 1].p[(g & 1) ^ 1], pc2 = dst(h1);
        // (a hull of three edges is a 3-cycle too, turning clockwise)
        if (orient2d_sign(pb.x, pb.y, pa.x, pa.y, pc2.x, pc2.y, pc) <= 0) return true;
        const int     sa = orient2d_sign(v.x, v.y, t.x, t.y, pa.x, pa.y, pc);
        const int     sc = orient2d_sign(v.x, v.y, t.x, t.y, pc2.x, pc2.y, pc);
        if (sa == 0 || sc == 0) return false;
        f = sc == sa ? h2 : h1;   // c on a's side: out through c -> b, else through a -> c
    }
    return false;
}

// The ring slot of a new edge from the origin v of half-edge a towards t:
// the half-edge x of v's ring such that the direction to t lies strictly
// inside the counter-clockwise wedge from x to next(x). -1 when an
// orientation with an edge of the ring is zero or the ring runs long.
static __device__ int seam_slot(const Rec* __restrict__ R, int nrec, int a, double2 t, PredCounters* pc)
{
    const unsigned lim2 = 2u * (unsigned)nrec;
    if ((unsigned)a >= lim2) return -1;
    const double2 v = R[a >> 1].p[a & 1];
    int           x = a;
    for (int deg = 0; deg <= 64; ++deg)
    {
        const int y = R[x >> 1].next[x & 1];
        if ((unsigned)y >= lim2) return -1;
        const double2 px = R[x >> 1].p[(x & 1) ^ 1], py = R[y >> 1].p[(y & 1) ^ 1];
        const int     sxt = orient2d_sign(v.x, v.y, px.x, px.y, t.x, t.y, pc);
        if (sxt == 0) return -1;
        if (y == x) return x;   // one edge: every other direction
        const int sty = orient2d_sign(v.x, v.y, t.x, t.y, py.x, py.y, pc);
        if (sty == 0) return -1;
        const int  sxy = orient2d_sign(v.x, v.y, px.x, px.y, py.x, py.y, pc);
        const bool inside = sxy > 0 ? (sxt > 0 && sty > 0) : (sxt > 0 || sty > 0);
        if (inside) return x;
        x = y;
        if (x == a) return -1;
    }
    return -1;
}

// one window entry: half-edge e, its successor along the side's direction,
// its far end and that end's coordinates, the ring links of sym(e) in the
// walker's forward (sf) and backward (sb) rotation, and the tag word
struct SEnt
{
    int      e, nx, d, sf, sb;
    unsigned pad;
    double2  p;
};

// The walker's forward rotation is counter-clockwise (next) for the rising
// walker and clockwise (prev) for the falling one; the left side walks
// forward, the right side backward.
template <bool MIRROR>
__device__ __forceinline__ SEnt load_sent(const Rec* __restrict__ R, int e, int nrec, bool back)
{
    const int  k = (int)min((unsigned)(e >> 1), (unsigned)(nrec - 1));
    const int  s = e & 1;
    const int4 np = *reinterpret_cast<const int4*>(&R[k].next[0]);
    const int4 og = *reinterpret_cast<const int4*>(&R[k].org[0]);
    const int  nx_e = s ? np.y : np.x, pv_e = s ? np.w : np.z;
    const int  nx_s = s ? np.x : np.y, pv_s = s ? np.z : np.w;
    SEnt       x;
    x.e = e;
    x.nx = (back != MIRROR) ? pv_e : nx_e;
    x.d = s ? og.x : og.y;
    x.sf = MIRROR ? pv_s : nx_s;
    x.sb = MIRROR ? nx_s : pv_s;
    x.pad = (unsigned)og.w;
    x.p = R[k].p[s ^ 1];
    return x;
}

// ring link of half-edge e: forward (fwd) or backward in the walker's rotation
template <bool MIRROR>
__device__ __forceinline__ int& link_of(Rec* R, int e, bool fwd)
{
    return (fwd != MIRROR) ? R[e >> 1].next[e & 1] : R[e >> 1].prev[e & 1];
}

// ring link of half-edge e in walker w's rotation (w = 1: the mirror)
__device__ __forceinline__ int& link_w(Rec* R, int e, bool fwd, int w)
{
    return (fwd != (w != 0)) ? R[e >> 1].next[e & 1] : R[e >> 1].prev[e & 1];
}

// The inserter (one thread of the block's last warp): makes every ring
// insertion of every walker, each walker's in its order, reading the
// anchors' neighbours as the rings are then; being the only thread that
// writes ring links while the walkers run, it needs no lock. It returns
// once every walker stopped and their requests are done.
static __device__ void seam_inserter(SeamShared& S, Rec* R, int nrec, unsigned tag, bool& bad)
{
    const unsigned lim2 = 2u * (unsigned)nrec;
    const int      nw = 2 * S.nseg;
    long long      idle = 0;
    while (!bad)
    {
        bool did = false;
        for (int w = 0; w < nw; ++w)
        {
            const int h = S.head[w];
            if (h >= *(volatile int*)&S.tail[w]) continue;
            __threadfence_block();   // the request was written before the walker's tail
            const volatile SeamReq& r = S.q[w][h % kSeamQueue];
            const int     k = r.k, vo = r.vo, vt = r.vt, Q1 = r.Q1, P2 = r.P2;
            const double2 po = make_double2(r.po.x, r.po.y), pt = make_double2(r.pt.x, r.pt.y);
            const int     e = 2 * k;
            const int     m = w & 1;   // the falling walkers' rotation is the mirror
            if ((unsigned)k >= (unsigned)nrec || (unsigned)Q1 >= lim2 || (unsigned)P2 >= lim2)
            {
                bad = true;
                break;
            }
            const int P1 = link_w(R, Q1, false, m), Q2 = link_w(R, P2, true, m);
            if ((unsigned)P1 >= lim2 || (unsigned)Q2 >= lim2)
            {
                bad = true;
                break;
            }
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(vo, vt, -1, (int)((tag + 1u + (unsigned)w) << 16));
            R[k].p[0] = po;
            R[k].p[1] = pt;
            link_w(R, e, true, m) = Q1;
            link_w(R, e, false, m) = P1;
            link_w(R, e + 1, true, m) = Q2;
            link_w(R, e + 1, false, m) = P2;
            __threadfence_block();   // the new edge's own links before the links to it
            link_w(R, P1, true, m) = e;
            link_w(R, Q1, false, m) = e;
            link_w(R, P2, true, m) = e + 1;
            link_w(R, Q2, false, m) = e + 1;
            __threadfence_block();   // the links before the count that covers them
            *(volatile int*)&S.head[w] = h + 1;
            did = true;
        }
        if (did)
        {
            idle = 0;
            continue;
        }
        if (*(volatile int*)&S.fail) return;
        bool all = true;
        for (int w = 0; w < nw && all; ++w)
            all = *(volatile int*)&S.state[w] && S.head[w] == *(volatile int*)&S.tail[w];
        if (all) return;
        if (++idle > kSeamSpin) bad = true;
        __nanosleep(20);
    }
}

// The physical deletion of the tagged edges in the nl deletion lists (list
// v: lists + v * cap, n[v] entries; the walkers' lists, then with more than
// two lists the edges deleted before the walkers), by nt threads (tid), then
// their records onto the free list (fhead, ftail), the lists in order, each
// walker's without the records an earlier walker's list or the last list
// holds (an edge two walkers deleted). SYNC: barrier of the nt threads.
template <class SyncF>
__device__ void seam_apply(Rec* R, int nrec, int* lists, int cap, const int* n, int nl, int& fhead, int& ftail,
    int tid, int nt, SyncF sync, bool& bad)
{
    auto dead = [&](int e) { return ((unsigned)R[e >> 1].pad & kSeamDel) != 0u; };
    int total = 0;
    for (int v = 0; v < nl; ++v) total += n[v];
    // entry i of the concatenated lists
    auto at_ref = [&](int i) -> int& {
        int v = 0;
        while (v + 1 < nl && i >= n[v]) i -= n[v++];
        return lists[(size_t)v * cap + i];
    };
    auto list_of = [&](int i) {
        int v = 0;
        while (v + 1 < nl && i >= n[v]) i -= n[v++];
        return v;
    };
    // rings: the first half-edge of every run of deleted ones links its
    // predecessor to the run's successor
    for (int i = tid; i < 2 * total; i += nt)
    {
        const int k = at_ref(i >> 1);
        if ((unsigned)k >= (unsigned)nrec)
        {
            bad = true;
            continue;
        }
        const int h = 2 * k + (i & 1);
        const int p = R[k].prev[h & 1];
        if ((unsigned)p >= 2u * (unsigned)nrec)
        {
            bad = true;
            continue;
        }
        if (dead(p)) continue;
        int q = R[k].next[h & 1], g = 0;
        while ((unsigned)q < 2u * (unsigned)nrec && dead(q) && ++g < nrec) q = R[q >> 1].next[q & 1];
        if ((unsigned)q >= 2u * (unsigned)nrec || g >= nrec)
        {
            bad = true;
            continue;
        }
        R[p >> 1].next[p & 1] = q;
        R[q >> 1].prev[q & 1] = p;
    }
    sync();
    // each list without the records of the lists before it
    for (int i = tid; i < total; i += nt)
    {
        int&      k = at_ref(i);
        const int v = list_of(i);
        const bool walker = nl <= 2 || v + 1 < nl;
        if (walker && (v > 0 || nl > 2) &&
            ((unsigned)k >= (unsigned)nrec || ((unsigned)R[k].pad & (((1u << v) - 1u) | (nl > 2 ? kSeamPre : 0u)))))
            k = -1;
    }
    sync();
    // the free list: the lists in order, then the old list
    const int old = fhead;
    if (!bad)
        for (int i = tid; i < total; i += nt)
        {
            const int k = at_ref(i);
            if (k < 0) continue;
            int j = i + 1;
            while (j < total && at_ref(j) < 0) ++j;
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(-1, -1, j < total ? at_ref(j) : old, 0);
        }
    int first = -1, last = -1;
    for (int i = 0; i < total && first < 0; ++i) first = at_ref(i);
    for (int i = total - 1; i >= 0 && last < 0; --i) last = at_ref(i);
    if (first >= 0)
    {
        if (old < 0) ftail = last;
        fhead = first;
    }
    sync();
}

// One walker of a split merge: MIRROR false, the rising walker of its
// segment (walker 2 j), true the falling one (walker 2 j + 1). The bottom
// rising walker (walker 0) takes B's free list first; B.fhead/ftail come
// back through S. The bottom rising walker is the reference's merge from
// the lower tangent; every other walker starts at a segment boundary (or
// the upper tangent) and stops at the first predicate that is zero: the
// falling ones hand the rest of their segment to its rising walker, a
// rising one above the bottom fails the merge (ST_SPLIT).
template <bool MIRROR, int WIN>
__device__ void seam_walk(Builder& B, SeamShared& S, const SeamArgs& A, int ldo, int ldi, int rdi, int rdo)
{
    static_assert(WIN >= 1 && WIN <= 3, "window of 1 to 3 candidates");
    const unsigned FULL = 0xffffffffu;
    Rec* const     R = A.R;
    const int      nrec = A.nrec;
    const int      lane = threadIdx.x & 31;
    const bool     left = lane < 16;
    const int      j = lane & 15;
    const bool     slot = j < WIN;
    const int      qd = left ? (j - 4) : (j + 4);
    const int      ca = qd >> 2, rb = qd & 3;
    const bool     combo = j >= 4 && j < 12 && ca < WIN && rb < WIN;
    const int      jj = slot ? j : 0;
    const int      w = A.w, o = w ^ 1;   // o: the other walker of the segment
    const unsigned mydel = 1u << w;
    // the edges deleted before the walkers: gone for the walkers that start
    // at a segment boundary; the bottom rising and the top falling walker
    // see the children as the sequential merges do
    const unsigned myskip = mydel | (A.start >= 0 ? kSeamPre : 0u);
    const unsigned mytag = A.tag + 1u + (unsigned)w;
    const unsigned mygate = seam_gate_tag(A.tag, (w + 1) >> 1);   // the boundary it starts or ends at
    const bool     strict = MIRROR || A.seg > 0;   // stops at the first zero
    const bool     top_seg = A.seg == A.nseg - 1;
    int* const     list = A.lists + (size_t)w * A.cap;
    int            fill = 0;
    bool           bad = false;
    int            a_next = A.a0;
    int            flink = -1;   // link of the free list's head (rising walker, lane 0)
#if QDTG_SPLIT_DEBUG
    long long dbg_t0 = clock64(), dbg_wait = 0, dbg_lock = 0, dbg_win = 0, dbg_pred = 0, dbg_conn = 0, dbg_ins = 0;
    long long dbg_c = 0, dbg_snap = 0, dbg_post = 0, dbg_mid = 0;
    int       dbg_steps = 0, dbg_passes = 0, dbg_flush = 0, dbg_stop = 0, dbg_del = 0;
#endif
    int dbg_why = 0;   // the step that failed (the report of a failed split merge)
    auto fail_split = [&](unsigned bits) {
        if (lane == 0)
        {
            atomicOr(&A.st->flags, ST_SPLIT | bits);
            S.fail = 1;
        }
        bad = true;
    };
    // signs in the walker's frame
    auto orient = [&](double2 a, double2 b, double2 c) {
        const int s = orient2d_sign(a.x, a.y, b.x, b.y, c.x, c.y, B.pc);
        return MIRROR ? -s : s;
    };
    // the other warp has stopped (bounded wait)
    // the segment's falling walker has stopped or published its last edge
    auto other_done = [&]() { return *(volatile int*)&S.state[o] || *(volatile int*)&S.fpub[A.seg]; };
    auto wait_other = [&]() -> bool {
#if QDTG_SPLIT_DEBUG
        const long long c0 = clock64();
#endif
        for (long long i = 0; i < kSeamSpin; ++i)
        {
            if (other_done())
            {
#if QDTG_SPLIT_DEBUG
                dbg_wait += clock64() - c0;
#endif
                return true;
            }
            __nanosleep(64);
        }
        return false;
    };
    // single-lane helpers: the next edge this walker sees around org(e),
    // forward or backward in its rotation
    auto view_step = [&](int e, bool fwd) -> int {
        int x = e;
        for (int i = 0; i < A.lim; ++i)
        {
            if ((unsigned)x >= 2u * (unsigned)nrec) break;
            x = link_of<MIRROR>(R, x, fwd);
            if ((unsigned)x >= 2u * (unsigned)nrec) break;
            if (x == e || !seam_skip((unsigned)R[x >> 1].pad, myskip, A.tag, mytag, mygate)) return x;
        }
        bad = true;
        return e;
    };
    auto porg = [&](int e) { return R[min((unsigned)(e >> 1), (unsigned)(nrec - 1))].p[e & 1]; };
    auto vorg = [&](int e) { return R[min((unsigned)(e >> 1), (unsigned)(nrec - 1))].org[e & 1]; };
    // a record for a new edge: the free list (rising walker), then the spare range
    auto alloc = [&]() -> int {
        if (w == 0 && B.fhead >= 0 && B.fhead < nrec)
        {
            const int k = B.fhead;
            B.fhead = flink;
            return k;
        }
        if (a_next < A.a1) return a_next++;
        return -1;
    };
    // after an allocation: the next head's link, needed only at the next one
    auto refill_link = [&]() {
        if (w == 0) flink = (B.fhead >= 0 && B.fhead < nrec) ? R[B.fhead].link : -1;
    };
    auto have_record = [&]() { return (w == 0 && B.fhead >= 0) || a_next < A.a1; };
    // a ring insertion for the inserter (lane 0): e = 2 k from vo to vt right
    // before Q1 in this walker's rotation, sym(e) right after P2. Every lane
    // keeps the anchors of the requests not yet made: a window that reaches
    // one waits for them.
    int pend_q1[kSeamQueue], pend_p2[kSeamQueue];
#pragma unroll
    for (int i = 0; i < kSeamQueue; ++i) pend_q1[i] = pend_p2[i] = -1;
    int posted = 0;
    auto wait_queue = [&](int room) -> bool {   // lane 0: at most kSeamQueue - room waiting
        for (long long i = 0; i < kSeamSpin; ++i)
        {
            if (posted - *(volatile int*)&S.head[w] <= kSeamQueue - room) return true;
            if (*(volatile int*)&S.fail) return false;
            __nanosleep(20);
        }
        return false;
    };
    auto post = [&](int k, int vo, int vt, double2 po, double2 pt, int Q1, int P2) -> bool {
        if (!wait_queue(1)) return false;
        volatile SeamReq& r = S.q[w][posted % kSeamQueue];
        r.k = k;
        r.vo = vo;
        r.vt = vt;
        r.Q1 = Q1;
        r.P2 = P2;
        r.po.x = po.x;
        r.po.y = po.y;
        r.pt.x = pt.x;
        r.pt.y = pt.y;
        __threadfence_block();
        *(volatile int*)&S.tail[w] = posted + 1;
        return true;
    };
    auto remember = [&](int Q1, int P2) {   // every lane, after a post; [0] the newest
#pragma unroll
        for (int i = kSeamQueue - 1; i > 0; --i)
        {
            pend_q1[i] = pend_q1[i - 1];
            pend_p2[i] = pend_p2[i - 1];
        }
        pend_q1[0] = Q1;
        pend_p2[0] = P2;
        ++posted;
    };
    // the window entry x is the anchor of an insertion not made yet
    auto pending_anchor = [&](int x, int npend) {
        bool hit = false;
#pragma unroll
        for (int i = 0; i < kSeamQueue; ++i) hit = hit || (i < npend && (x == pend_q1[i] || x == pend_p2[i]));
        return hit;
    };
    // A cross edge meets the seam line between its endpoints, and q lies on
    // that line: with both endpoints strictly below q along the seam, q is
    // above the edge; with both strictly above, it is not. Only an edge with
    // an endpoint level with q, or lying on the seam line itself, needs the
    // orientation.
    const SeamKey kq = seam_keys(A.q, A.frame);
    auto q_above = [&](double2 po, double2 pt, SeamKey ko, SeamKey kt) {
        return seam_q_above(A.q, kq, po, pt, ko, kt, B.pc);
    };

    // (falling) going on past q down to the last edge of a rising walker that
    // stopped early; lane 0: the walker finished its part, did the rising one
    // stop early?
    bool down_more = false;
    auto fall_done_lane0 = [&]() -> bool {
        const int j = A.seg;
        *(volatile int*)&S.fdone[j] = 1;
        __threadfence_block();
        return *(volatile int*)&S.rstop[j] != 0;
    };

    // ---- the tangent and the first edge (lane 0) ----
    int     basel = -1, Fsb = 0, Bb = 0, tq1 = -1, tp2 = -1;
    int     t_o = 0, t_d = 0;                      // the first edge's endpoints (lane 0)
    double2 tp_o = make_double2(0, 0), tp_d = tp_o;
    SeamKey k_o = {}, k_d = {};   // the base edge's vertices' seam keys (lane 0)
    bool stop = false;   // the falling walker has nothing (more) to do
    const bool from_gate = A.start >= 0;   // starts at a segment boundary
    int        gate_o = -1, gate_d = -1;       // the boundary above this rising walker's segment
    if (lane == 0 && !MIRROR && !top_seg)
    {
        const int g = S.gate[A.seg + 1];
        gate_o = vorg(g);
        gate_d = vorg(sym(g));
    }
    if (lane == 0)
    {
        refill_link();
        int l = ldi, r = rdi;
        if (MIRROR && !from_gate)
        {
            // the upper tangent starts from the hull edges above the lower
            // ones at the inner extremes (builder.hxx:253-261 mirrored)
            l = view_step(ldi, false);   // the next edge counter-clockwise around org(ldi)
            r = view_step(rdi, true);    // the next edge clockwise around org(rdi)
            const double2 pl0 = porg(ldi), pr0 = porg(rdi);
            stop = l == ldi || r == rdi ||
                   orient2d_sign(porg(sym(ldi)).x, porg(sym(ldi)).y, pl0.x, pl0.y, porg(sym(l)).x, porg(sym(l)).y,
                       B.pc) <= 0 ||
                   orient2d_sign(porg(sym(r)).x, porg(sym(r)).y, pr0.x, pr0.y, porg(sym(rdi)).x, porg(sym(rdi)).y,
                       B.pc) <= 0;
        }
        // leftOf(org(r), l) ? l = lnext(l) : rightOf(org(l), r) ? r = rprev(r)
        for (int it = 0; !from_gate && !stop && !bad; ++it)
        {
            if (it > 2 * A.lim)
            {
                bad = true;
                break;
            }
            const double2 pr = porg(r), pl = porg(l);
            const int     s1 = orient(pr, pl, porg(sym(l)));
            if (MIRROR && s1 == 0)
            {
                stop = true;
                break;
            }
            if (s1 > 0)
            {
                l = view_step(sym(l), false);   // lnext
                continue;
            }
            const int s2 = orient(pl, porg(sym(r)), pr);
            if (MIRROR && s2 == 0)
            {
                stop = true;
                break;
            }
            if (s2 > 0)
            {
                r = view_step(sym(r), true);   // rprev
                continue;
            }
            break;
        }
        if (!bad && !stop)
        {
            // the tangent edge org(r) -> org(l), or the boundary edge
            const int     vo = from_gate ? vorg(A.start) : vorg(r), vt = from_gate ? vorg(sym(A.start)) : vorg(l);
            const double2 po = from_gate ? porg(A.start) : porg(r), pt = from_gate ? porg(sym(A.start)) : porg(l);
            t_o = vo, t_d = vt, tp_o = po, tp_d = pt;
            k_o = seam_keys(po, A.frame);
            k_d = seam_keys(pt, A.frame);
            const bool    above = q_above(po, pt, k_o, k_d);
            int           taken = -1;
            if (MIRROR)
                stop = above;
            else if (!above && !other_done())
            {
                if (!wait_other()) bad = true;
            }
            if (!MIRROR && !bad && other_done())
            {
                __threadfence_block();
                const int j = A.seg;
                if (S.last_e[j] >= 0 && S.last_o[j] == vo && S.last_d[j] == vt) taken = S.last_e[j];
            }
            if (!bad && !stop)
            {
                if (taken >= 0)
                    basel = taken;
                else if (from_gate)
                {
                    // the windows start at the boundary edge's raw neighbours
                    basel = A.start;
                    Bb = link_of<MIRROR>(R, basel, false);
                    Fsb = link_of<MIRROR>(R, sym(basel), true);
                }
                else
                {
                    const int k = alloc();
                    if (k < 0)
                        bad = true;
                    else
                    {
                        // e right before r, sym(e) right after l; the windows start
                        // at their raw neighbours (which the insertion keeps)
                        Bb = link_of<MIRROR>(R, r, false);
                        Fsb = link_of<MIRROR>(R, l, true);
                        if (!post(k, vo, vt, po, pt, r, l))
                        {
                            bad = true;
                            dbg_why = 1;
                        }
                        refill_link();
                        basel = 2 * k;
                        tq1 = r;
                        tp2 = l;
                    }
                }
                if (!MIRROR && !bad && !from_gate)
                {
                    S.base0 = basel;
                    if (vorg(l) == vorg(ldo)) ldo = sym(basel);
                    if (vorg(r) == vorg(rdo)) rdo = basel;
                    S.ldo = ldo;
                    S.rdo = rdo;
                }
                if (MIRROR && !bad && !from_gate) S.first_dn = basel;
                if (!MIRROR && taken >= 0) stop = true;   // the falling walker made the whole chain
            }
        }
    }
    __syncwarp();
    bad = __shfl_sync(FULL, (int)bad, 0) != 0;
    stop = __shfl_sync(FULL, (int)stop, 0) != 0;
    basel = __shfl_sync(FULL, basel, 0);
    Fsb = __shfl_sync(FULL, Fsb, 0);
    Bb = __shfl_sync(FULL, Bb, 0);
    tq1 = __shfl_sync(FULL, tq1, 0);
    tp2 = __shfl_sync(FULL, tp2, 0);
    if (tq1 >= 0) remember(tq1, tp2);
    a_next = __shfl_sync(FULL, a_next, 0);
    int fh = __shfl_sync(FULL, B.fhead, 0);
    B.fhead = fh;

    // the base edge's endpoints come from the tangent (its record is the
    // inserter's to write)
    int     bo = __shfl_sync(FULL, t_o, 0), bd = __shfl_sync(FULL, t_d, 0), lstart = 0, rstart = 0;
    double2 pbo = make_double2(__shfl_sync(FULL, tp_o.x, 0), __shfl_sync(FULL, tp_o.y, 0));
    double2 pbd = make_double2(__shfl_sync(FULL, tp_d.x, 0), __shfl_sync(FULL, tp_d.y, 0));
    if (!bad && !stop)
    {
        lstart = Fsb;   // the window loader steps over what this walker does not see
        rstart = Bb;
    }
    bool done_chain = false;   // the walker reached the end of the chain
    int  it = 0;
    while (!bad && !stop)
    {
        if (++it > A.lim)
        {
            bad = true;
            dbg_why = 8;
            break;
        }
        if (*(volatile int*)&S.fail) break;   // the other walker failed: the call runs again
        bool    cont_l = false, cont_r = false, lv = false, rv = false, choice = false;
        int     lcE = 0, lcD = 0, lcSf = 0, rcE = 0, rcD = 0, rcSb = 0;
        double2 lcP = pbo, rcP = pbo;
        bool    tie = false;
        for (int pass = 0;; ++pass)
        {
            if (pass > A.lim)
            {
                bad = true;
                break;
            }
#if QDTG_SPLIT_DEBUG
            ++dbg_passes;
#endif
            // room for this pass's deletions and, on the first pass, a record
            bool room = fill + 2 * WIN <= A.cap && (pass > 0 || __shfl_sync(FULL, (int)have_record(), 0) != 0);
            if (!room)
            {
                if (MIRROR)
                {
                    stop = true;
                    break;
                }
                if (w != 0)
                {
                    // a rising walker above the bottom one stops at its last
                    // edge and hands the rest of its segment to the falling
                    // walker, unless that one has finished
                    bool fail = false;
                    if (lane == 0)
                    {
                        const int j = A.seg;
                        S.rlast_e[j] = basel;
                        S.rlast_o[j] = bo;
                        S.rlast_d[j] = bd;
                        __threadfence_block();
                        *(volatile int*)&S.rstop[j] = 1;
                        __threadfence_block();
                        fail = *(volatile int*)&S.fdone[j] != 0;
                    }
                    if (__shfl_sync(FULL, (int)fail, 0))
                    {
                        bad = true;
                        dbg_why = 10;
                    }
                    else
                        stop = true;
                    break;
                }
#if QDTG_SPLIT_DEBUG
                ++dbg_flush;
#endif
                // the bottom rising walker frees every deleted edge, once every
                // other walker stopped and every insertion is made
                bool ok = true;
                if (lane == 0)
                {
                    ok = wait_queue(kSeamQueue);
                    for (int v = 1; ok && v < 2 * A.nseg; ++v)
                        for (long long i = 0;; ++i)
                        {
                            if (*(volatile int*)&S.state[v] && *(volatile int*)&S.head[v] == *(volatile int*)&S.tail[v])
                                break;
                            if (i + 1 >= kSeamSpin || *(volatile int*)&S.fail)
                            {
                                ok = false;
                                break;
                            }
                            __nanosleep(64);
                        }
                }
                ok = __shfl_sync(FULL, (int)ok, 0) != 0;
                if (!ok)
                {
                    bad = true;
                    break;
                }
                __threadfence_block();
                int  fh2 = __shfl_sync(FULL, B.fhead, 0), ft2 = __shfl_sync(FULL, B.ftail, 0);
                bool b2 = false;
                int  nd[kSeamWalkers + 1];
#pragma unroll
                for (int v = 0; v <= kSeamWalkers; ++v) nd[v] = v == 0 ? fill : *(volatile int*)&S.ndel[v];
                seam_apply(R, nrec, A.lists, A.cap, nd, split_lists(A.nseg), fh2, ft2, lane, 32, [] { __syncwarp(); },
                    b2);
                fh2 = __shfl_sync(FULL, fh2, 0);
                ft2 = __shfl_sync(FULL, ft2, 0);
                if (__any_sync(FULL, b2))
                {
                    bad = true;
                    break;
                }
                B.fhead = fh2;
                B.ftail = ft2;
                if (lane == 0) refill_link();
                fill = 0;
                if (lane == 0)
                    for (int v = 1; v < split_lists(A.nseg); ++v) S.ndel[v] = 0;
                // the raw ring links held lose the records just freed
                int f = 0, b = 0;
                if (lane == 0)
                {
                    f = link_of<MIRROR>(R, sym(basel), true);
                    b = link_of<MIRROR>(R, basel, false);
                }
                Fsb = __shfl_sync(FULL, f, 0);
                Bb = __shfl_sync(FULL, b, 0);
                lstart = Fsb;
                rstart = Bb;
                if (!(fill + 2 * WIN <= A.cap && (pass > 0 || __shfl_sync(FULL, (int)have_record(), 0) != 0)))
                {
                    bad = true;
                    break;
                }
            }

#if QDTG_SPLIT_DEBUG
            dbg_c = clock64();
#endif
            // --- the window: WIN + 1 records this walker sees along this side's ring
            SEnt mine = {}, succ = {};
            for (int retry = 0;; ++retry)
            {
            // the insertions not made yet, counted before the loads: one made
            // while the window loads may or may not be in it
            const int npend = posted - *(volatile int*)&S.head[w];
            __threadfence_block();
            bool skipped = false;
            {
                int cur = left ? lstart : rstart;
#pragma unroll
                for (int i = 0; i <= WIN; ++i)
                {
                    if ((unsigned)cur >= 2u * (unsigned)nrec)
                    {
                        skipped = true;
                        break;
                    }
                    const SEnt x = load_sent<MIRROR>(R, cur, nrec, !left);
                    skipped = skipped || seam_skip(x.pad, myskip, A.tag, mytag, mygate);
                    if (i == jj) mine = x;
                    if (i == jj + 1) succ = x;
                    cur = x.nx;
                }
            }
            if (skipped)
            {
                int cur = left ? lstart : rstart, found = 0, g = 0;
                while (found <= WIN)
                {
                    if ((unsigned)cur >= 2u * (unsigned)nrec) break;
                    const SEnt x = load_sent<MIRROR>(R, cur, nrec, !left);
                    if (!seam_skip(x.pad, myskip, A.tag, mytag, mygate))
                    {
                        if (found == jj) mine = x;
                        if (found == jj + 1) succ = x;
                        ++found;
                    }
                    cur = x.nx;
                    if (++g > A.lim) break;
                }
                if (found <= WIN)
                {
                    bad = true;
                    dbg_why = 4;
                }
            }
            // a window that reaches the anchor of an insertion of this walker
            // not made yet would miss that edge (a ring it wraps around): it
            // waits for the insertions and loads again
            const bool hit = npend > 0 && slot && (pending_anchor(mine.e, npend) || pending_anchor(succ.e, npend));
            if (!__any_sync(FULL, hit) || __any_sync(FULL, bad)) break;
            bool ok = true;
            if (lane == 0) ok = wait_queue(kSeamQueue);
            if (!__shfl_sync(FULL, (int)ok, 0) || retry > 2)
            {
                bad = true;
                dbg_why = 2 + (retry > 2 ? 1 : 0);
            }
            __threadfence_block();
            }
            if (__any_sync(FULL, bad))
            {
                bad = true;
                break;
            }
#if QDTG_SPLIT_DEBUG
            {
                const long long c1 = clock64();
                dbg_win += c1 - dbg_c;
                dbg_c = c1;
            }
#endif
            // --- one wave of predicates (signs in the walker's frame)
            const int     src_a = combo ? ca : 0, src_b = combo ? 16 + rb : 16;
            const int     ad = __shfl_sync(FULL, mine.d, src_a), bdst = __shfl_sync(FULL, mine.d, src_b);
            const double2 pa = make_double2(__shfl_sync(FULL, mine.p.x, src_a), __shfl_sync(FULL, mine.p.y, src_a));
            const double2 pb = make_double2(__shfl_sync(FULL, mine.p.x, src_b), __shfl_sync(FULL, mine.p.y, src_b));
            // a candidate that ends at bo or bd lies on the base edge: not
            // valid for the reference; a zero for the mirror
            const bool wrap = slot && (mine.d == bo || mine.d == bd);
            int        so = 0;
            if (slot && !wrap) so = orient(mine.p, pbd, pbo);
            const bool valid = so > 0;
            // (for a rising walker a wrap is the reference's own "not valid";
            // only a zero orientation is a tie)
            const bool vtie = slot && ((MIRROR && wrap) || (!wrap && so == 0));
            const int  ia = slot ? bd : ad, ib = slot ? bo : bd, ic = slot ? mine.d : bo, id = slot ? succ.d : bdst;
            const double2 qa = slot ? pbd : pa, qb = slot ? pbo : pbd, qc = slot ? mine.p : pbo,
                          qdp = slot ? succ.p : pb;
            int si = 0;
            bool rep = false;
            if (slot || combo)
            {
                rep = ia == id || ib == id || ic == id || ia == ib || ia == ic || ib == ic;
                if (!rep)
                {
                    si = incircle_sign(qa.x, qa.y, qb.x, qb.y, qc.x, qc.y, qdp.x, qdp.y, B.pc);
                    if (MIRROR) si = -si;
                }
            }
            const bool     inc = si > 0;
            const bool     itie = (slot || combo) && ((MIRROR && rep) || (!rep && si == 0));
            const unsigned vm = __ballot_sync(FULL, valid), im = __ballot_sync(FULL, inc);
            const unsigned vtm = __ballot_sync(FULL, vtie), itm = __ballot_sync(FULL, itie);
            const unsigned vl = vm & 0xFu, il = im & 0xFu, vr = (vm >> 16) & 0xFu, ir = (im >> 16) & 0xFu;
            const unsigned zl = ~il & 0xFu, zr = ~ir & 0xFu;
            const bool     runl = cont_l || (vl & 1u), runr = cont_r || (vr & 1u);
            const int      dl = runl ? (zl ? __ffs(zl) - 1 : WIN) : 0;
            const int      dr = runr ? (zr ? __ffs(zr) - 1 : WIN) : 0;
            const int      srcL = min(dl, WIN - 1), srcR = 16 + min(dr, WIN - 1);
            const bool     overL = dl == WIN, overR = dr == WIN;
            if (strict)
            {
                // the zeros the sequential merge would have evaluated
                unsigned used = 0;
                if (!cont_l) used |= vtm & 1u;
                if (!cont_r) used |= (vtm >> 16) & 1u;
                if (runl) used |= itm & ((2u << min(dl, WIN - 1)) - 1u);
                if (runr) used |= (itm >> 16) & ((2u << min(dr, WIN - 1)) - 1u);
                if (!overL && !overR)
                {
                    used |= (vtm >> dl) & 1u;
                    used |= (vtm >> (16 + dr)) & 1u;
                    const bool lvv = (vl >> dl) & 1u, rvv = (vr >> dr) & 1u;
                    const int  ql = dl * 4 + dr;
                    const int  qlane = ql < 8 ? 4 + ql : 20 + (ql - 8);
                    if (lvv && rvv) used |= (itm >> qlane) & 1u;
                }
                if (used)
                {
                    tie = true;
                    break;
                }
            }
#if QDTG_SPLIT_DEBUG
            {
                const long long c1 = clock64();
                dbg_pred += c1 - dbg_c;
                dbg_c = c1;
            }
#endif
            const int stopL = overL ? __shfl_sync(FULL, succ.e, srcL) : __shfl_sync(FULL, mine.e, srcL);
            const int stopR = overR ? __shfl_sync(FULL, succ.e, srcR) : __shfl_sync(FULL, mine.e, srcR);
            // --- deletions: tags and the list
            const bool del = slot && j < (left ? dl : dr);
            if (del)
            {
                atomicOr(reinterpret_cast<unsigned*>(&R[mine.e >> 1].pad), mydel);
                list[fill + (left ? j : dl + j)] = mine.e >> 1;
            }
            fill += dl + dr;
#if QDTG_SPLIT_DEBUG
            dbg_del += dl + dr;
#endif
            lstart = stopL;
            rstart = stopR;
            __syncwarp();
            if (overL || overR)
            {
                cont_l = cont_l || overL;
                cont_r = cont_r || overR;
                continue;
            }
            lv = (vl >> dl) & 1u;
            rv = (vr >> dr) & 1u;
            lcE = stopL;
            lcD = __shfl_sync(FULL, mine.d, srcL);
            lcP = make_double2(__shfl_sync(FULL, mine.p.x, srcL), __shfl_sync(FULL, mine.p.y, srcL));
            lcSf = __shfl_sync(FULL, mine.sf, srcL);
            rcE = stopR;
            rcD = __shfl_sync(FULL, mine.d, srcR);
            rcP = make_double2(__shfl_sync(FULL, mine.p.x, srcR), __shfl_sync(FULL, mine.p.y, srcR));
            rcSb = __shfl_sync(FULL, mine.sb, srcR);
            const int ql = dl * 4 + dr;
            const int qlane = ql < 8 ? 4 + ql : 20 + (ql - 8);
            choice = (im >> qlane) & 1u;
            break;
        }
#if QDTG_SPLIT_DEBUG
        const long long dbg_m0 = clock64();
#endif
        if (tie && !MIRROR)
        {
            bad = true;   // a zero for a rising walker above the bottom one
            dbg_why = 9;
        }
        if (bad || stop || tie) break;
        if (!lv && !rv)
        {
            // the end of the chain: for the falling walker, the whole chain
            // lies at or above q; the rising walker must have met the falling
            // one (and only the top segment's reaches the end)
            if (!MIRROR)
            {
                bool b2 = !top_seg;
                if (lane == 0 && !b2)
                {
                    if (!other_done() && !wait_other()) b2 = true;
                    __threadfence_block();
                    if (*(volatile int*)&S.last_e[A.seg] >= 0)
                    {
                        b2 = true;
                        dbg_why = 7;
                    }
                }
                bad = __shfl_sync(FULL, (int)b2, 0) != 0;
            }
            done_chain = true;
            break;
        }
        const bool    take_r = !lv || (rv && choice);
        const int     vo = take_r ? rcD : bo, vt = take_r ? bd : lcD;
        const double2 po = take_r ? rcP : pbo, pt = take_r ? pbd : lcP;
        // the meeting point
        int  taken = -1;
        bool halt = false;
        SeamKey k_new = {};
        if (lane == 0)
        {
            k_new = seam_keys(take_r ? rcP : lcP, A.frame);
            const bool above = take_r ? q_above(po, pt, k_new, k_d) : q_above(po, pt, k_o, k_new);
            if (MIRROR)
            {
                const int j = A.seg;
                if (!down_more && above)
                {
                    // q is passed: the falling walker's part ends here. Above
                    // the first segment it publishes its last edge and waits
                    // for its rising walker: done, or stopped early, when the
                    // falling walker goes on down to the rising one's last edge
                    if (j == 0)
                        halt = true;
                    else
                    {
                        S.last_e[j] = basel;
                        S.last_o[j] = bo;
                        S.last_d[j] = bd;
                        __threadfence_block();
                        *(volatile int*)&S.fpub[j] = 1;
                        __threadfence_block();
                        bool got = false;
                        for (long long i = 0; i < kSeamSpin && !got; ++i)
                        {
                            if (*(volatile int*)&S.rstop[j])
                                down_more = got = true;
                            else if (*(volatile int*)&S.rdone[j] || *(volatile int*)&S.fail)
                                halt = got = true;
                            else
                                __nanosleep(64);
                        }
                        if (!got) bad = true;
                        __threadfence_block();
                    }
                }
                if (down_more && *(volatile int*)&S.rlast_o[j] == vo && *(volatile int*)&S.rlast_d[j] == vt)
                    taken = *(volatile int*)&S.rlast_e[j];
            }
            else
            {
                if (!above && !other_done() && !wait_other()) bad = true;
                if (!bad && other_done())
                {
                    __threadfence_block();
                    const int j = A.seg;
                    if (S.last_e[j] >= 0 && S.last_o[j] == vo && S.last_d[j] == vt) taken = S.last_e[j];
                }
                // a rising walker never reaches the boundary above its segment
                // without taking its falling walker's last edge
                if (!bad && taken < 0 && !top_seg && vo == gate_o && vt == gate_d)
                {
                    bad = true;
                    dbg_why = 11;
                }
            }
        }
        bad = __shfl_sync(FULL, (int)bad, 0) != 0;
        halt = __shfl_sync(FULL, (int)halt, 0) != 0;
        taken = __shfl_sync(FULL, taken, 0);
        if (MIRROR) down_more = __shfl_sync(FULL, (int)down_more, 0) != 0;
        if (bad || halt) break;
        if (taken >= 0)
        {
            basel = taken;
            break;
        }
        // --- the new base edge: connect(rc, sym(basel)) or connect(sym(basel), sym(lc))
        int e = 0, nF = 0, nB = 0;
#if QDTG_SPLIT_DEBUG
        const long long dbg_cc = clock64();
        dbg_mid += dbg_cc - dbg_m0;
#endif
        // connect(rc, sym(basel)): e right before sym(rc), sym(e) right after
        // sym(basel); connect(sym(basel), sym(lc)): e right before basel,
        // sym(e) right after sym(lc). The next windows start at the raw
        // neighbours on the far side of the new edge.
        const int Q1 = take_r ? sym(rcE) : basel, P2 = take_r ? sym(basel) : sym(lcE);
        nF = take_r ? Fsb : lcSf;
        nB = take_r ? rcSb : Bb;
        if (lane == 0)
        {
            const int k = alloc();
            if (k < 0 || !post(k, vo, vt, po, pt, Q1, P2))
            {
                bad = true;
                dbg_why = k < 0 ? 5 : 6;
            }
            refill_link();
            e = 2 * k;
        }
        bad = __shfl_sync(FULL, (int)bad, 0) != 0;
#if QDTG_SPLIT_DEBUG
        const long long dbg_p0 = clock64();
        dbg_conn += dbg_p0 - dbg_cc;
#endif
        if (bad) break;
        e = __shfl_sync(FULL, e, 0);
        remember(Q1, P2);
        Fsb = nF;
        Bb = nB;
        basel = e;
        bo = vo, pbo = po, bd = vt, pbd = pt;
        if (take_r)
        {
            rstart = Bb;   // lstart: the left scan's stop
            k_o = k_new;
        }
        else
        {
            lstart = Fsb;
            k_d = k_new;
        }
#if QDTG_SPLIT_DEBUG
        ++dbg_steps;
        dbg_post += clock64() - dbg_p0;
#endif
        __syncwarp();
    }
    (void)done_chain;
#if QDTG_SPLIT_DEBUG
    {
        const int why = __shfl_sync(FULL, dbg_why, 0) | __reduce_or_sync(FULL, (unsigned)dbg_why);
        if (lane == 0 && bad)
            printf("split FAIL node=%u w=%d why=%d steps=%d posted=%d head=%d\n", A.tag / kSeamTagStride, w, why, dbg_steps, posted,
                *(volatile int*)&S.head[w]);
    }
#endif
#if QDTG_SPLIT_DEBUG
    if (lane == 0 && A.tag / kSeamTagStride < 16u)
        printf("split node=%u w=%d steps=%d passes=%d del=%d flush=%d stop=%d bad=%d chain=%d cyc=%lld wait=%lld "
               "lock=%lld win=%lld pred=%lld conn=%lld snap=%lld mid=%lld post=%lld spare=%d\n",
            A.tag / kSeamTagStride, w, dbg_steps, dbg_passes, dbg_del, dbg_flush, (int)stop, (int)bad, (int)done_chain,
            clock64() - dbg_t0, dbg_wait, dbg_lock, dbg_win, dbg_pred, dbg_conn, dbg_snap, dbg_mid, dbg_post,
            a_next - A.a0);
#endif
    if (lane == 0)
    {
        // a falling walker that ends anywhere but at the last edge of a
        // rising walker that stopped early leaves a gap
        if (MIRROR && !bad && fall_done_lane0() && !(basel >= 0 && basel == *(volatile int*)&S.rlast_e[A.seg]))
        {
            bad = true;
            dbg_why = 12;
        }
        if (bad && !S.fail) fail_split(0u);
        S.ndel[w] = fill;
        if (MIRROR)
        {
            if (basel >= 0 && !bad)
            {
                S.last_e[A.seg] = basel;
                S.last_o[A.seg] = bo;
                S.last_d[A.seg] = bd;
            }
        }
        else
        {
            *(volatile int*)&S.rdone[A.seg] = 1;
            if (top_seg) S.top = basel;
            if (w == 0)
            {
                S.fhead = B.fhead;
                S.ftail = B.ftail;
            }
        }
        __threadfence_block();
        *(volatile int*)&S.state[w] = 1;
    }
    __syncwarp();
}

}  // namespace qdtg
