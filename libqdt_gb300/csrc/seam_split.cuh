// Split merges: the seam of one top-level merge walked by two warps at once.
//
// The merge of the reference builder (builder.hxx:251-285) is one chain of
// bubble steps from the lower common tangent up to the upper one. At the top
// of the tree that chain is long (about 3,600 steps at the root of 2.6 M
// uniform points) and nothing else runs beside it. Here a rising walker runs
// the reference's merge from the lower tangent (warp 0 of the block) while a
// falling walker (warp 1) runs its mirror image (the same merge with the
// rotations and the predicate signs reversed) down from the upper tangent.
// Both are warp merges with the candidate window of warp_merge.
//
// The walkers never see each other's work:
// * each record carries a tag word (Rec::pad): one byte per walker marks the
//   edges it deleted, and bits 16..31 name the walker that made the edge;
// * deletions only set the walker's byte: the edge stays in its rings until
//   the merge ends, and the walker that deleted it steps over it;
// * insertions are real ring insertions, but the other walker steps over
//   them; each one goes right next to one of the new edge's anchors (the
//   walker's own previous edge or the candidate edge it chose), never next
//   to an edge of the other walker, so the two walkers' insertions keep
//   their order in every ring they share.
// So each walker sees exactly the map its own sequential merge would have
// at that step: the rising walker makes the reference's decisions, and the
// falling walker those of the mirror merge.
//
// Where they meet: q is a point on the seam (the node's cut coordinate,
// and the mean of its children's cuts along the seam). The rising walker
// keeps the edges that have q strictly above them, the falling walker the
// others; the test is one exact orientation, the same in both walkers. The
// rising walker's first edge without q above is the falling walker's last
// one: it stops there and takes that edge. The mirror merge decides like
// the reference only where no predicate it evaluates is zero, so the
// falling walker stops at its first zero (cocircular or collinear points),
// and then the rising walker goes on past q up to the falling walker's last
// edge. (Without zeros every decision holds for all small perturbations of
// the points; the edges made and deleted are then those of every Delaunay
// triangulation of the points, the reference's included.) A rising walker
// whose chain does not meet that edge reports ST_SPLIT and the call runs
// again without split merges.
//
// Spare records: a walker makes its edges before the deleted ones are
// freed, so each one has a range of spare records after the pool (the
// rising one takes its node's free list first). When the falling walker's
// range or deletion list runs out it stops; when the rising walker's runs
// out, it waits for the falling walker to stop and then frees every deleted
// edge (seam_apply) before it goes on.
//
// At the end the block removes the deleted edges from their rings and puts
// their records on the node's free list, the rising walker's in its order,
// then the falling walker's: the record ids, and so the output, do not
// depend on how the two warps were scheduled.
//
// Shared rings: a walker inserts under a block-wide lock, and keeps in
// shared memory the two origins of its last kSeamLog insertions. The ring
// neighbours a walker inserts next to were read earlier; they are read again
// only when the other walker has inserted at the same vertex since.
//
// Every wait on the other warp is bounded; a wait that runs out, like any
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

constexpr unsigned kDelRise = 0x000000FFu, kDelFall = 0x0000FF00u;
constexpr int      kSeamQueue = 4;   // insertions a walker may have waiting
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
    SeamReq q[2][kSeamQueue];
    int     tail[2];               // insertions each walker posted
    int     head[2];               // of those, the ones the inserter made
    int     state[2];              // 1 once the walker stopped
    int last_o, last_d, last_e;    // the falling walker's last edge (-1: none)
    int first_dn;                  // its first edge (the upper tangent), -1: none
    int ndel[2];                   // deletion-list fills
    int base0, ldo, rdo, top;      // the rising walker's lower tangent, hull edges, last edge
    int fhead, ftail;              // the node's free list
    int fail;
};

struct SeamArgs
{
    Rec*       R;
    int        nrec;     // pool and spare records
    unsigned   tag;      // 4 * node tag
    double2    q;        // the meeting point on the seam
    int        a0, a1;   // each walker's spare records [a0, a1)
    int*       list[2];  // deletion lists
    int        cap;      // entries in each
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

// a record this walker does not see: deleted by it, or made by the other
__device__ __forceinline__ bool seam_skip(unsigned pad, unsigned mydel, unsigned other)
{
    return (pad & mydel) != 0u || (pad >> 16) == other;
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

// The inserter (one thread of the block's third warp): makes every ring
// insertion of both walkers, each walker's in its order, reading the
// anchors' neighbours as the rings are then; being the only thread that
// writes ring links while the walkers run, it needs no lock. It returns
// once both walkers stopped and their requests are done.
static __device__ void seam_inserter(SeamShared& S, Rec* R, int nrec, unsigned tag, bool& bad)
{
    const unsigned lim2 = 2u * (unsigned)nrec;
    long long      idle = 0;
    while (!bad)
    {
        bool did = false;
        for (int w = 0; w < 2; ++w)
        {
            const int h = S.head[w];
            if (h >= *(volatile int*)&S.tail[w]) continue;
            __threadfence_block();   // the request was written before the walker's tail
            const volatile SeamReq& r = S.q[w][h % kSeamQueue];
            const int     k = r.k, vo = r.vo, vt = r.vt, Q1 = r.Q1, P2 = r.P2;
            const double2 po = make_double2(r.po.x, r.po.y), pt = make_double2(r.pt.x, r.pt.y);
            const int     e = 2 * k;
            if ((unsigned)k >= (unsigned)nrec || (unsigned)Q1 >= lim2 || (unsigned)P2 >= lim2)
            {
                bad = true;
                break;
            }
            const int P1 = link_w(R, Q1, false, w), Q2 = link_w(R, P2, true, w);
            if ((unsigned)P1 >= lim2 || (unsigned)Q2 >= lim2)
            {
                bad = true;
                break;
            }
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(vo, vt, -1, (int)((tag + 1u + (unsigned)w) << 16));
            R[k].p[0] = po;
            R[k].p[1] = pt;
            link_w(R, e, true, w) = Q1;
            link_w(R, e, false, w) = P1;
            link_w(R, e + 1, true, w) = Q2;
            link_w(R, e + 1, false, w) = P2;
            __threadfence_block();   // the new edge's own links before the links to it
            link_w(R, P1, true, w) = e;
            link_w(R, Q1, false, w) = e;
            link_w(R, P2, true, w) = e + 1;
            link_w(R, Q2, false, w) = e + 1;
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
        if (*(volatile int*)&S.state[0] && *(volatile int*)&S.state[1] &&
            S.head[0] == *(volatile int*)&S.tail[0] && S.head[1] == *(volatile int*)&S.tail[1])
            return;
        if (++idle > kSeamSpin) bad = true;
        __nanosleep(20);
    }
}

// The physical deletion of the tagged edges in lists[0][0, n0) and
// lists[1][0, n1), by nt threads (tid), then their records onto the free
// list (fhead, ftail), first list in order, then the second without the
// records the first holds. SYNC: barrier of the nt threads.
template <class SyncF>
__device__ void seam_apply(Rec* R, int nrec, const int* l0, int n0, int* l1, int n1, int& fhead, int& ftail, int tid,
    int nt, SyncF sync, bool& bad)
{
    auto dead = [&](int e) { return ((unsigned)R[e >> 1].pad & (kDelRise | kDelFall)) != 0u; };
    // rings: the first half-edge of every run of deleted ones links its
    // predecessor to the run's successor
    for (int i = tid; i < 2 * (n0 + n1); i += nt)
    {
        const int idx = i >> 1;
        const int k = idx < n0 ? l0[idx] : l1[idx - n0];
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
    // the second list without the records of the first
    for (int i = tid; i < n1; i += nt)
    {
        const int k = l1[i];
        if ((unsigned)k >= (unsigned)nrec || ((unsigned)R[k].pad & kDelRise)) l1[i] = -1;
    }
    sync();
    // the free list: the first list, the second, then the old list
    const int old = fhead;
    const int total = n0 + n1;
    auto at = [&](int i) { return i < n0 ? l0[i] : l1[i - n0]; };
    if (!bad)
        for (int i = tid; i < total; i += nt)
        {
            const int k = at(i);
            if (k < 0) continue;
            int j = i + 1;
            while (j < total && at(j) < 0) ++j;
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(-1, -1, j < total ? at(j) : old, 0);
        }
    int first = -1, last = -1;
    for (int i = 0; i < total && first < 0; ++i) first = at(i);
    for (int i = total - 1; i >= 0 && last < 0; --i) last = at(i);
    if (first >= 0)
    {
        if (old < 0) ftail = last;
        fhead = first;
    }
    sync();
}

// One walker of a split merge: MIRROR false, the rising walker (warp 0),
// true the falling one (warp 1). The rising walker takes B's free list
// first; B.fhead/ftail come back through S.
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
    const int      w = MIRROR ? 1 : 0, o = 1 - w;
    const unsigned mydel = MIRROR ? kDelFall : kDelRise;
    const unsigned mytag = A.tag + (MIRROR ? 2u : 1u), other = A.tag + (MIRROR ? 1u : 2u);
    int* const     list = A.list[w];
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
    auto wait_other = [&]() -> bool {
#if QDTG_SPLIT_DEBUG
        const long long c0 = clock64();
#endif
        for (long long i = 0; i < kSeamSpin; ++i)
        {
            if (*(volatile int*)&S.state[o])
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
            if (x == e || !seam_skip((unsigned)R[x >> 1].pad, mydel, other)) return x;
        }
        bad = true;
        return e;
    };
    auto porg = [&](int e) { return R[min((unsigned)(e >> 1), (unsigned)(nrec - 1))].p[e & 1]; };
    auto vorg = [&](int e) { return R[min((unsigned)(e >> 1), (unsigned)(nrec - 1))].org[e & 1]; };
    // a record for a new edge: the free list (rising walker), then the spare range
    auto alloc = [&]() -> int {
        if (!MIRROR && B.fhead >= 0 && B.fhead < nrec)
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
        if (!MIRROR) flink = (B.fhead >= 0 && B.fhead < nrec) ? R[B.fhead].link : -1;
    };
    auto have_record = [&]() { return (!MIRROR && B.fhead >= 0) || a_next < A.a1; };
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
        if (!(ko.across == kq.across && kt.across == kq.across))
        {
            if (ko.up < kq.up && kt.up < kq.up) return true;
            if (ko.up > kq.up && kt.up > kq.up) return false;
        }
        const double2 dqo = make_double2(sub_rn(po.x, A.q.x), sub_rn(po.y, A.q.y));
        const double2 dqt = make_double2(sub_rn(pt.x, A.q.x), sub_rn(pt.y, A.q.y));
        int sg = orient2d_f32(dqt.x, dqt.y, dqo.x, dqo.y);
        if (!sg) sg = orient2d_slow(pt.x, pt.y, po.x, po.y, A.q.x, A.q.y, B.pc);
        return sg > 0;
    };

    // ---- the tangent and the first edge (lane 0) ----
    int     basel = -1, Fsb = 0, Bb = 0, tq1 = -1, tp2 = -1;
    int     t_o = 0, t_d = 0;                      // the first edge's endpoints (lane 0)
    double2 tp_o = make_double2(0, 0), tp_d = tp_o;
    SeamKey k_o = {}, k_d = {};   // the base edge's vertices' seam keys (lane 0)
    bool stop = false;   // the falling walker has nothing (more) to do
    if (lane == 0)
    {
        refill_link();
        int l = ldi, r = rdi;
        if (MIRROR)
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
        for (int it = 0; !stop && !bad; ++it)
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
            // the tangent edge org(r) -> org(l)
            const int     vo = vorg(r), vt = vorg(l);
            const double2 po = porg(r), pt = porg(l);
            t_o = vo, t_d = vt, tp_o = po, tp_d = pt;
            k_o = seam_keys(po, A.frame);
            k_d = seam_keys(pt, A.frame);
            const bool    above = q_above(po, pt, k_o, k_d);
            int           taken = -1;
            if (MIRROR)
                stop = above;
            else if (!above && !*(volatile int*)&S.state[o])
            {
                if (!wait_other()) bad = true;
            }
            if (!MIRROR && !bad && *(volatile int*)&S.state[o])
            {
                __threadfence_block();
                if (S.last_e >= 0 && S.last_o == vo && S.last_d == vt) taken = S.last_e;
            }
            if (!bad && !stop)
            {
                if (taken >= 0)
                    basel = taken;
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
                if (!MIRROR && !bad)
                {
                    S.base0 = basel;
                    if (vorg(l) == vorg(ldo)) ldo = sym(basel);
                    if (vorg(r) == vorg(rdo)) rdo = basel;
                    S.ldo = ldo;
                    S.rdo = rdo;
                }
                if (MIRROR && !bad) S.first_dn = basel;
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
#if QDTG_SPLIT_DEBUG
                ++dbg_flush;
#endif
                // the rising walker frees every deleted edge, once the falling one
                // stopped and every insertion is made
                bool ok = true;
                if (lane == 0)
                {
                    ok = wait_other() && wait_queue(kSeamQueue);
                    for (long long i = 0; ok && i < kSeamSpin; ++i)
                    {
                        if (*(volatile int*)&S.head[o] == *(volatile int*)&S.tail[o]) break;
                        if (i + 1 == kSeamSpin) ok = false;
                        __nanosleep(20);
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
                seam_apply(R, nrec, list, fill, A.list[1], *(volatile int*)&S.ndel[1], fh2, ft2, lane, 32,
                    [] { __syncwarp(); }, b2);
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
                if (lane == 0) S.ndel[1] = 0;
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
                    skipped = skipped || seam_skip(x.pad, mydel, other);
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
                    if (!seam_skip(x.pad, mydel, other))
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
            const bool vtie = slot && (wrap || so == 0);
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
            const bool     itie = (slot || combo) && (rep || si == 0);
            const unsigned vm = __ballot_sync(FULL, valid), im = __ballot_sync(FULL, inc);
            const unsigned vtm = __ballot_sync(FULL, vtie), itm = __ballot_sync(FULL, itie);
            const unsigned vl = vm & 0xFu, il = im & 0xFu, vr = (vm >> 16) & 0xFu, ir = (im >> 16) & 0xFu;
            const unsigned zl = ~il & 0xFu, zr = ~ir & 0xFu;
            const bool     runl = cont_l || (vl & 1u), runr = cont_r || (vr & 1u);
            const int      dl = runl ? (zl ? __ffs(zl) - 1 : WIN) : 0;
            const int      dr = runr ? (zr ? __ffs(zr) - 1 : WIN) : 0;
            const int      srcL = min(dl, WIN - 1), srcR = 16 + min(dr, WIN - 1);
            const bool     overL = dl == WIN, overR = dr == WIN;
            if (MIRROR)
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
                reinterpret_cast<volatile unsigned char*>(&R[mine.e >> 1].pad)[w] = 1;
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
        if (bad || stop || tie) break;
        if (!lv && !rv)
        {
            // the end of the chain: for the falling walker, the whole chain
            // lies at or above q; the rising walker must have met the falling one
            if (!MIRROR)
            {
                bool b2 = false;
                if (lane == 0)
                {
                    if (!*(volatile int*)&S.state[o] && !wait_other()) b2 = true;
                    __threadfence_block();
                    if (*(volatile int*)&S.last_e >= 0)
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
                halt = above;
            else
            {
                if (!above && !*(volatile int*)&S.state[o] && !wait_other()) bad = true;
                if (!bad && *(volatile int*)&S.state[o])
                {
                    __threadfence_block();
                    if (S.last_e >= 0 && S.last_o == vo && S.last_d == vt) taken = S.last_e;
                }
            }
        }
        bad = __shfl_sync(FULL, (int)bad, 0) != 0;
        halt = __shfl_sync(FULL, (int)halt, 0) != 0;
        taken = __shfl_sync(FULL, taken, 0);
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
            printf("split FAIL node=%u w=%d why=%d steps=%d posted=%d head=%d\n", A.tag / 4u, w, why, dbg_steps, posted,
                *(volatile int*)&S.head[w]);
    }
#endif
#if QDTG_SPLIT_DEBUG
    if (lane == 0 && A.tag / 4u < 16u)
        printf("split node=%u w=%d steps=%d passes=%d del=%d flush=%d stop=%d bad=%d chain=%d cyc=%lld wait=%lld "
               "lock=%lld win=%lld pred=%lld conn=%lld snap=%lld mid=%lld post=%lld spare=%d\n",
            A.tag / 4u, w, dbg_steps, dbg_passes, dbg_del, dbg_flush, (int)stop, (int)bad, (int)done_chain,
            clock64() - dbg_t0, dbg_wait, dbg_lock, dbg_win, dbg_pred, dbg_conn, dbg_snap, dbg_mid, dbg_post,
            a_next - A.a0);
#endif
    if (lane == 0)
    {
        if (bad && !S.fail) fail_split(0u);
        S.ndel[w] = fill;
        if (MIRROR)
        {
            if (basel >= 0 && !bad)
            {
                S.last_e = basel;
                S.last_o = bo;
                S.last_d = bd;
            }
        }
        else
        {
            S.top = basel;
            S.fhead = B.fhead;
            S.ftail = B.ftail;
        }
        __threadfence_block();
        *(volatile int*)&S.state[w] = 1;
    }
    __syncwarp();
}

}  // namespace qdtg
