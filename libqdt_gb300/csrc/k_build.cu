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
#include "common.cuh"
#include "engine_kernels.hpp"
#include "predicates.cuh"
#include "scan.cuh"

namespace qdtg {

__device__ __forceinline__ int sym(int e) { return e ^ 1; }

// reference builder.hxx:71-76
__device__ __forceinline__ bool less_frame(double2 a, double2 b, int frame)
{
    if (frame == 0) return a.x < b.x || (a.x == b.x && a.y < b.y);
    return a.y < b.y || (a.y == b.y && a.x > b.x);
}

__device__ __forceinline__ bool ccw(double2 a, double2 b, double2 c, PredCounters* pc)
{
    return orient2d_sign(a.x, a.y, b.x, b.y, c.x, c.y, pc) > 0;
}

struct Builder
{
    Rec*          R;
    int           nrec;
    DevStatus*    st;
    PredCounters* pc;
    int           fhead, ftail;
    bool          bad;

    __device__ __forceinline__ void fail(unsigned bit)
    {
        if (!bad) atomicOr(&st->flags, bit);
        bad = true;
    }
    __device__ __forceinline__ int chk(int e)
    {
        // one unsigned compare: negative ids wrap to large values
        if ((unsigned)e >= 2u * (unsigned)nrec)
        {
            fail(ST_BAD_INDEX);
            return 0;
        }
        return e;
    }

    __device__ __forceinline__ int onext(int e)
    {
        e = chk(e);
        return R[e >> 1].next[e & 1];
    }
    __device__ __forceinline__ int oprev(int e)
    {
        e = chk(e);
        return R[e >> 1].prev[e & 1];
    }
    __device__ __forceinline__ int org(int e)
    {
        e = chk(e);
        return R[e >> 1].org[e & 1];
    }
    __device__ __forceinline__ double2 porg(int e)
    {
        e = chk(e);
        return R[e >> 1].p[e & 1];
    }
    __device__ __forceinline__ int     dest(int e) { return org(sym(e)); }
    __device__ __forceinline__ double2 pdest(int e) { return porg(sym(e)); }
    __device__ __forceinline__ int     lnext(int e) { return oprev(sym(e)); }
    __device__ __forceinline__ int     rprev(int e) { return onext(sym(e)); }

    // the ids written here were all read through onext/oprev just before,
    // which checked them
    __device__ __forceinline__ void set_next(int e, int v)
    {
        if (!bad) R[e >> 1].next[e & 1] = v;
    }
    __device__ __forceinline__ void set_prev(int e, int v)
    {
        if (!bad) R[e >> 1].prev[e & 1] = v;
    }

    // free list of the node (records of the subtree that are not in use)
    // The link of the popped record is needed only by the next alloc(), so
    // nothing waits for that load here; the tail is settled by
    // settle_tail() when the node is done (an emptied list has no tail).
    __device__ int alloc()
    {
        const int k = fhead;
        if (k < 0 || k >= nrec)
        {
            fail(ST_POOL_EMPTY);
            return -1;
        }
        fhead = R[k].link;
        return k;
    }
    __device__ void release(int k)
    {
        if (bad) return;
        R[k].org[0] = -1;
        R[k].link = fhead;
        if (fhead < 0) ftail = k;
        fhead = k;
    }
    __device__ void settle_tail()
    {
        if (fhead < 0) ftail = -1;
    }

    // reference builder.hxx:131-142: a new edge, alone in the rings of both
    // its origins, with both origins (and their coordinates) set at once
    __device__ int make_edge(int o0, int o1, double2 p0, double2 p1)
    {
        if (bad) return 0;
        const int k = alloc();
        if (k < 0) return 0;
        const int e = 2 * k;
        Rec&      r = R[k];
        *reinterpret_cast<int4*>(&r.next[0]) = make_int4(e, e + 1, e, e + 1);
        *reinterpret_cast<int4*>(&r.org[0]) = make_int4(o0, o1, -1, 0);
        r.p[0] = p0;
        r.p[1] = p1;
        return e;
    }

    // splice(e, x) of an edge e alone in its ring (builder.hxx:144-149):
    // e follows x counter-clockwise around their common origin
    __device__ void insert_after(int x, int e)
    {
        const int n = onext(x);
        set_next(e, n);
        set_prev(e, x);
        set_prev(n, e);
        set_next(x, e);
    }
    // splice(e, oprev(e)): e leaves the ring around its origin
    __device__ void remove(int e)
    {
        const int p = oprev(e), n = onext(e);
        set_next(p, n);
        set_prev(n, p);
    }

    // reference builder.hxx:151-159
    __device__ int connect(int a, int b)
    {
        const int e = make_edge(dest(a), org(b), pdest(a), porg(b));
        if (bad) return 0;
        insert_after(lnext(a), e);
        insert_after(b, sym(e));
        return e;
    }

    // reference builder.hxx:161-166
    __device__ void delete_edge(int e)
    {
        e = chk(e);
        remove(e);
        remove(sym(e));
        release(e >> 1);
    }

    // reference builder.hxx:171-175: false when two of the vertices coincide
    __device__ bool in_circle(int a, double2 pa, int b, double2 pb, int c, double2 pc_, int d, double2 pd)
    {
        if (a == d || b == d || c == d || a == b || a == c || b == c) return false;
        return incircle_sign(pa.x, pa.y, pb.x, pb.y, pc_.x, pc_.y, pd.x, pd.y, pc) > 0;
    }

    // reference builder.hxx:177-201. The leaf's points are V[lo, hi), already
    // in the order of the frame; its records are [3 lo, 3 hi).
    __device__ void leaf(int lo, int hi, const double2* __restrict__ V, int& le, int& re)
    {
        const int r0 = 3 * lo, r1 = 3 * hi;
        for (int k = r0; k < r1; ++k)
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(-1, -1, k + 1 < r1 ? k + 1 : -1, 0);
        fhead = r0;
        ftail = r1 - 1;
        const int     n = hi - lo, s1 = lo, s2 = lo + 1;
        const double2 p1 = V[s1], p2 = V[s2];
        if (n == 2)
        {
            const int a = make_edge(s1, s2, p1, p2);
            le = a;
            re = sym(a);
            return;
        }
        const int     s3 = lo + 2;
        const double2 p3 = V[s3];
        const int     a = make_edge(s1, s2, p1, p2), b = make_edge(s2, s3, p2, p3);
        insert_after(sym(a), b);
        const int o = orient2d_sign(p1.x, p1.y, p2.x, p2.y, p3.x, p3.y, pc);
        if (o > 0)
        {
            connect(b, a);
            le = a;
            re = sym(b);
            return;
        }
        if (o < 0)
        {
            const int c = connect(b, a);
            le = sym(c);
            re = c;
            return;
        }
        le = a;
        re = sym(b);
    }

    // lower common tangent (builder.hxx:253-261)
    __device__ int tangent(int& ldo, int& ldi, int& rdi, int& rdo, int lim)
    {
        int it = 0;
        for (;;)
        {
            if (bad) return 0;
            if (++it > lim)
            {
                fail(ST_GUARD);
                return 0;
            }
            // leftOf(org(rdi), ldi), then rightOf(org(ldi), rdi)
            const double2 prdi = porg(rdi), pldi = porg(ldi);
            if (ccw(prdi, pldi, pdest(ldi), pc)) ldi = lnext(ldi);
            else if (ccw(pldi, pdest(rdi), prdi, pc)) rdi = rprev(rdi);
            else break;
        }
        const int basel = connect(sym(rdi), ldi);
        if (org(ldi) == org(ldo)) ldo = sym(basel);
        if (org(rdi) == org(rdo)) rdo = basel;
        return basel;
    }

    // reference builder.hxx:251-285 (with the scans :205-249 in line)
    __device__ void merge(int ldo, int ldi, int rdi, int rdo, int lim, int& out_l, int& out_r)
    {
        int basel = tangent(ldo, ldi, rdi, rdo, lim);
        int it = 0;
        for (;;)
        {
            if (bad) return;
            if (++it > lim)
            {
                fail(ST_GUARD);
                return;
            }
            const int     bo = org(basel), bd = dest(basel);
            const double2 pbo = porg(basel), pbd = pdest(basel);
            // left candidate (builder.hxx:205-226)
            int     lc = onext(sym(basel));
            int     lcd = dest(lc);
            double2 plcd = pdest(lc);
            bool    lv = ccw(plcd, pbd, pbo, pc);
            if (lv)
            {
                bool deleted = false;
                int  j = 0;
                for (;;)
                {
                    const int     t = onext(lc);
                    const int     td = dest(t);
                    const double2 ptd = pdest(t);
                    if (!in_circle(bd, pbd, bo, pbo, lcd, plcd, td, ptd)) break;
                    if (bad || ++j > lim)
                    {
                        fail(ST_GUARD);
                        return;
                    }
                    delete_edge(lc);
                    lc = t;
                    lcd = td;
                    plcd = ptd;
                    deleted = true;
                }
                if (deleted) lv = ccw(plcd, pbd, pbo, pc);
            }
            // right candidate (builder.hxx:228-249)
            int     rc = oprev(basel);
            int     rcd = dest(rc);
            double2 prcd = pdest(rc);
            bool    rv = ccw(prcd, pbd, pbo, pc);
            if (rv)
            {
                bool deleted = false;
                int  j = 0;
                for (;;)
                {
                    const int     t = oprev(rc);
                    const int     td = dest(t);
                    const double2 ptd = pdest(t);
                    if (!in_circle(bd, pbd, bo, pbo, rcd, prcd, td, ptd)) break;
                    if (bad || ++j > lim)
                    {
                        fail(ST_GUARD);
                        return;
                    }
                    delete_edge(rc);
                    rc = t;
                    rcd = td;
                    prcd = ptd;
                    deleted = true;
                }
                if (deleted) rv = ccw(prcd, pbd, pbo, pc);
            }
            if (!lv && !rv) break;
            if (!lv || (rv && in_circle(lcd, plcd, bd, pbd, bo, pbo, rcd, prcd)))
                basel = connect(rc, sym(basel));
            else
                basel = connect(sym(basel), sym(lc));
        }
        out_l = ldo;
        out_r = rdo;
    }

    // reference builder.hxx:287-301
    __device__ int hull_walk(int e, int frame, bool want_max, int lim)
    {
        for (int it = 0;; ++it)
        {
            if (bad) return e;
            if (it > lim)
            {
                fail(ST_GUARD);
                return e;
            }
            const int     nx = rprev(e);
            const int     pv = sym(oprev(e));
            const double2 pe = porg(e);
            const double2 pn = porg(nx);
            if (want_max ? less_frame(pe, pn, frame) : less_frame(pn, pe, frame))
            {
                e = nx;
                continue;
            }
            const double2 pp = porg(pv);
            if (want_max ? less_frame(pe, pp, frame) : less_frame(pp, pe, frame))
            {
                e = pv;
                continue;
            }
            return e;
        }
    }
};

// ---------------------------------------------------------------------------
// Warp-cooperative merge (the upper levels)
// ---------------------------------------------------------------------------
//
// The same merge as Builder::merge, organised around a window of candidates
// that the warp loads once per bubble step:
//
// * left lanes 0..15 walk the ring of bd counter-clockwise from
//   c_0 = onext(sym(basel)), right lanes 16..31 the ring of bo clockwise from
//   r_0 = oprev(basel), loading kWin+1 records (c_0..c_4); every lane of a
//   side loads the same records, so each load is one broadcast transaction;
// * lanes 0..3 and 16..19 evaluate validE(c_j) and inCircle(bd, bo,
//   dest(c_j), dest(c_j+1)); lanes 4..11 and 20..27 evaluate the final choice
//   inCircle(dest(c_a), bd, bo, dest(r_b)) for all 16 (a, b): one wave of
//   predicates, one warp instruction stream for all of them;
// * ballots give what the reference's sequential loop (builder.hxx:205-283)
//   computes one test after the other: how many candidates each scan
//   deletes (up to the first failing in-circle test), lv, rv and the choice.
//   The two scans touch disjoint edges (builder.hxx:203-204), so evaluating
//   them together decides the same;
// * the map edits need no further loads: the deleted candidates c_0..c_dl-1
//   are a run of consecutive edges in bd's ring (one link update), and each
//   one's far end leaves the ring of its other origin using the prev/next of
//   its own record, already in the window -- one lane per deleted edge; the
//   new base edge is inserted between neighbours that the window also holds.
//   The free list takes the deleted records in the reference's order.
// A scan that deletes its whole window goes on in another pass, without
// re-testing validity (builder.hxx:216-222). Record indices are clamped to
// the pool, so no access leaves it; the loops are bounded by guards.
constexpr int kWin = 4;

struct Ent
{
    int     e;    // half-edge
    int     nx;   // its successor along the scan (onext for the left side, oprev for the right)
    int     d;    // dest(e)
    int     fp;   // oprev(sym(e)): neighbours of the far end in the ring of dest(e)
    int     fn;   // onext(sym(e))
    double2 p;    // coordinates of dest(e)
};

__device__ __forceinline__ Ent load_ent(const Rec* __restrict__ R, int e, int nrec, bool left)
{
    const int  k = (int)min((unsigned)(e >> 1), (unsigned)(nrec - 1));
    const int  s = e & 1;
    const int4 np = *reinterpret_cast<const int4*>(&R[k].next[0]);   // next0 next1 prev0 prev1
    const int2 og = *reinterpret_cast<const int2*>(&R[k].org[0]);
    Ent        x;
    x.e = e;
    x.nx = left ? (s ? np.y : np.x) : (s ? np.w : np.z);
    x.d = s ? og.x : og.y;
    x.fp = s ? np.z : np.w;
    x.fn = s ? np.x : np.y;
    x.p = R[k].p[s ^ 1];
    return x;
}

__device__ __forceinline__ Rec& recof(Rec* R, int e, int nrec)
{
    return R[min((unsigned)(e >> 1), (unsigned)(nrec - 1))];
}
__device__ __forceinline__ void st_next(Rec* R, int e, int v, int nrec) { recof(R, e, nrec).next[e & 1] = v; }
__device__ __forceinline__ void st_prev(Rec* R, int e, int v, int nrec) { recof(R, e, nrec).prev[e & 1] = v; }

__device__ __forceinline__ double2 shfl_d2(double2 v, int src)
{
    return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

__device__ void warp_merge(Builder& B, int ldo, int ldi, int rdi, int rdo, int lim, int& out_l, int& out_r)
{
    const unsigned FULL = 0xffffffffu;
    Rec* const     R = B.R;
    const int      nrec = B.nrec;
    const int      lane = threadIdx.x & 31;
    const bool     left = lane < 16;
    const int      j = lane & 15;
    const bool     slot = j < kWin;
    const bool     combo = j >= 4 && j < 12;
    const int      q = left ? (j - 4) : (j + 4);   // combo index 0..15 = 4 a + b
    const int      ca = q >> 2, rb = q & 3;
    const int      jj = slot ? j : 0;               // window slot this lane keeps

    int basel = 0;
    if (lane == 0) basel = B.tangent(ldo, ldi, rdi, rdo, lim);
    __syncwarp();
    basel = __shfl_sync(FULL, basel, 0);
    bool bad = __shfl_sync(FULL, (int)B.bad, 0) != 0;
    // free list: head and the link of the head
    int fhead = __shfl_sync(FULL, B.fhead, 0), ftail = __shfl_sync(FULL, B.ftail, 0);
    int flink = (fhead >= 0 && !bad) ? recof(R, 2 * fhead, nrec).link : -1;
    // the base edge, its endpoints and the starts of both windows
    int     bo = 0, bd = 0, lstart = 0, rstart = 0;
    double2 pbo = make_double2(0, 0), pbd = pbo;
    if (!bad)
    {
        bo = B.org(basel);
        bd = B.dest(basel);
        pbo = B.porg(basel);
        pbd = B.pdest(basel);
        lstart = B.onext(sym(basel));
        rstart = B.oprev(basel);
    }
    int it = 0;
    while (!bad)
    {
        if (++it > lim)
        {
            if (lane == 0) B.fail(ST_GUARD);
            break;
        }
        bool cont_l = false, cont_r = false, lv = false, rv = false, choice = false;
        int  lcE = 0, lcD = 0, lcFn = 0, rcE = 0, rcD = 0, rcFp = 0;
        double2 lcP = pbo, rcP = pbo;
        for (int pass = 0;; ++pass)
        {
            if (pass > lim)
            {
                if (lane == 0) B.fail(ST_GUARD);
                bad = true;
                break;
            }
            // --- the window: kWin + 1 records along this side's ring
            Ent cur = load_ent(R, left ? lstart : rstart, nrec, left);
            Ent mine = cur, succ = cur;
#pragma unroll
            for (int i = 1; i <= kWin; ++i)
            {
                const Ent nx = load_ent(R, cur.nx, nrec, left);
                if (i == jj) mine = nx;
                if (i == jj + 1) succ = nx;
                cur = nx;
            }
            // --- one wave of predicates
            const int     src_a = combo ? ca : 0, src_b = combo ? 16 + rb : 16;
            const int     ad = __shfl_sync(FULL, mine.d, src_a), bdst = __shfl_sync(FULL, mine.d, src_b);
            const double2 pa = shfl_d2(mine.p, src_a), pb = shfl_d2(mine.p, src_b);
            const bool valid = slot && ccw(mine.p, pbd, pbo, B.pc);
            // one in-circle call for both roles, so the lanes share one
            // instruction stream: slot (bd, bo, dest c_j, dest c_j+1),
            // choice (dest c_a, bd, bo, dest r_b)
            const int     ia = slot ? bd : ad, ib = slot ? bo : bd, ic = slot ? mine.d : bo, id = slot ? succ.d : bdst;
            const double2 qa = slot ? pbd : pa, qb = slot ? pbo : pbd, qc = slot ? mine.p : pbo,
                          qd = slot ? succ.p : pb;
            const bool inc = (slot || combo) && B.in_circle(ia, qa, ib, qb, ic, qc, id, qd);
            const unsigned vm = __ballot_sync(FULL, valid), im = __ballot_sync(FULL, inc);
            const unsigned vl = vm & 0xFu, il = im & 0xFu, vr = (vm >> 16) & 0xFu, ir = (im >> 16) & 0xFu;
            const unsigned zl = ~il & 0xFu, zr = ~ir & 0xFu;
            const int      dl = (cont_l || (vl & 1u)) ? (zl ? __ffs(zl) - 1 : kWin) : 0;
            const int      dr = (cont_r || (vr & 1u)) ? (zr ? __ffs(zr) - 1 : kWin) : 0;
            // the candidate each scan stops at: slot dl (slot kWin is the
            // successor of slot kWin - 1)
            const int  srcL = min(dl, kWin - 1), srcR = 16 + min(dr, kWin - 1);
            const bool overL = dl == kWin, overR = dr == kWin;
            const int  stopL = overL ? __shfl_sync(FULL, succ.e, srcL) : __shfl_sync(FULL, mine.e, srcL);
            const int  stopR = overR ? __shfl_sync(FULL, succ.e, srcR) : __shfl_sync(FULL, mine.e, srcR);
            // --- deletions: far ends (one lane per deleted edge), the
            // near-end rings, and the free list in the reference's order
            const int prevrec = __shfl_up_sync(FULL, mine.e >> 1, 1);
            const int lastL = dl > 0 ? __shfl_sync(FULL, mine.e >> 1, dl - 1) : -1;
            const int lastR = dr > 0 ? __shfl_sync(FULL, mine.e >> 1, 16 + dr - 1) : -1;
            const int firstL = __shfl_sync(FULL, mine.e >> 1, 0), firstR = __shfl_sync(FULL, mine.e >> 1, 16);
            const bool del = slot && j < (left ? dl : dr);
            if (del)
            {
                st_next(R, mine.fp, mine.fn, nrec);
                st_prev(R, mine.fn, mine.fp, nrec);
                Rec&      r = recof(R, mine.e, nrec);
                const int below = (j > 0) ? prevrec : (left ? fhead : (dl > 0 ? lastL : fhead));
                r.org[0] = -1;
                r.link = below;
            }
            if (lane == 0 && dl > 0)
            {
                st_next(R, sym(basel), stopL, nrec);
                st_prev(R, stopL, sym(basel), nrec);
            }
            if (lane == 16 && dr > 0)
            {
                st_prev(R, basel, stopR, nrec);
                st_next(R, stopR, basel, nrec);
            }
            if (dl + dr > 0)
            {
                const int old = fhead;
                const int newhead = dr > 0 ? lastR : lastL;
                if (old < 0) ftail = dl > 0 ? firstL : firstR;
                flink = dr > 1 ? __shfl_sync(FULL, mine.e >> 1, 16 + dr - 2)
                               : (dr == 1 ? (dl > 0 ? lastL : old) : (dl > 1 ? __shfl_sync(FULL, mine.e >> 1, dl - 2) : old));
                fhead = newhead;
            }
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
            lcP = shfl_d2(mine.p, srcL);
            lcFn = __shfl_sync(FULL, mine.fn, srcL);
            rcE = stopR;
            rcD = __shfl_sync(FULL, mine.d, srcR);
            rcP = shfl_d2(mine.p, srcR);
            rcFp = __shfl_sync(FULL, mine.fp, srcR);
            const int ql = dl * 4 + dr;
            const int qlane = ql < 8 ? 4 + ql : 20 + (ql - 8);
            choice = (im >> qlane) & 1u;
            break;
        }
        if (bad || (!lv && !rv)) break;
        // --- the new base edge (builder.hxx:279-282), from window values only
        const bool take_r = !lv || (rv && choice);
        const int  k = fhead;
        if (k < 0 || k >= nrec)
        {
            if (lane == 0) B.fail(ST_POOL_EMPTY);
            break;
        }
        fhead = flink;
        const int e = 2 * k;
        int       o0, o1, x0, n0, x1, n1;   // e after x0 (before n0); sym(e) after x1 (before n1)
        double2   p0, p1;
        if (take_r)
        {
            // connect(rc, sym(basel)): from dest(rc) to bd
            o0 = rcD, p0 = rcP, o1 = bd, p1 = pbd;
            x0 = rcFp, n0 = sym(rcE);
            x1 = sym(basel), n1 = lstart;
        }
        else
        {
            // connect(sym(basel), sym(lc)): from bo to dest(lc)
            o0 = bo, p0 = pbo, o1 = lcD, p1 = lcP;
            x0 = rstart, n0 = basel;
            x1 = sym(lcE), n1 = lcFn;
        }
        if (lane == 0)
        {
            Rec& r = R[k];
            *reinterpret_cast<int4*>(&r.next[0]) = make_int4(n0, n1, x0, x1);
            *reinterpret_cast<int4*>(&r.org[0]) = make_int4(o0, o1, -1, 0);
            r.p[0] = p0;
            r.p[1] = p1;
            st_next(R, x0, e, nrec);
            st_prev(R, n0, e, nrec);
            st_next(R, x1, e + 1, nrec);
            st_prev(R, n1, e + 1, nrec);
        }
        // the next step's base edge and window starts
        basel = e;
        bo = o0, pbo = p0, bd = o1, pbd = p1;
        lstart = n1;   // onext(sym(e))
        rstart = x0;   // oprev(e)
        if (fhead >= 0) flink = recof(R, 2 * fhead, nrec).link;
        __syncwarp();
    }
    if (lane == 0)
    {
        B.fhead = fhead;
        B.ftail = ftail;
    }
    out_l = __shfl_sync(FULL, ldo, 0);
    out_r = __shfl_sync(FULL, rdo, 0);
}

constexpr unsigned kFatal = ST_POOL_EMPTY | ST_GUARD | ST_BAD_INDEX;

// One depth of the tree: leaves of that depth are built, internal nodes merge
// their children's results (written by the previous launch). WARP: one node
// per warp, else one node per thread.
template <bool WARP>
__global__ void __launch_bounds__(128) k_build_level(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
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
    Builder B{ R, nrec, st, count ? &st->pc : nullptr, -1, -1, false };
    const int n = hi - lo;
    NodeOut   o;
    if (n <= 3)
    {
        if (lane != 0) return;
        B.leaf(lo, hi, V, o.le, o.re);
    }
    else
    {
        const NodeOut L = child[2 * k], Rn = child[2 * k + 1];
        // the children's free lists lie inside their record ranges
        if ((L.fhead >= 0 && (L.ftail < 3 * lo || L.ftail >= 3 * hi)) ||
            (Rn.fhead >= 0 && (Rn.ftail < 3 * lo || Rn.ftail >= 3 * hi)))
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
        int       rl = 0, rr = 0;
        if (WARP) warp_merge(B, L.le, L.re, Rn.le, Rn.re, lim, rl, rr);
        else B.merge(L.le, L.re, Rn.le, Rn.re, lim, rl, rr);
        if (lane != 0) return;
        if (d > 0 && !B.bad)
        {
            // reference builder.hxx:340-346: re-pick the extremes in the
            // parent's frame
            const int frame = (d - 1) & 1;
            const int le2 = B.hull_walk(rl, frame, false, n + 8);
            const int reccw = B.hull_walk(B.onext(rr), frame, true, n + 8);
            rl = le2;
            rr = B.oprev(reccw);
        }
        o.le = rl;
        o.re = rr;
    }
    B.settle_tail();
    o.fhead = B.fhead;
    o.ftail = B.ftail;
    out[k] = o;
}

// Before an upper depth merges, the records near its seams are fetched into
// L2 with the evict-last policy: the merges are chains of dependent loads,
// and their records were last touched by far deeper levels, so without this
// a bubble step waits on several DRAM round trips. A record lies near a seam
// when one of its origins is closer to the cut line than 3 times the edge's
// own length -- the edges a merge walks or deletes around the seam, at the
// local scale of the point set. The scan reads the records with streaming
// (evict-first) loads so that it does not displace what it prefetches.
__global__ void k_prefetch_seams(const Rec* __restrict__ R, int nrec, int m, int d, const double* __restrict__ seam)
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
    if (dist <= 3.0 * len)
    {
        const char* base = reinterpret_cast<const char*>(&R[r]);
        asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(base));
        asm volatile("prefetch.global.L2::evict_last [%0];" ::"l"(base + 32));
    }
}

// Depths with at most this many nodes run one node per warp.
constexpr long long kWarpNodes = 1 << 12;

void launch_build(const BuildBuffers& b, int m, cudaStream_t s)
{
    const int D = split_levels(m);
    const int nrec = 3 * m;
    for (int d = D; d >= 0; --d)
    {
        const long long nodes = 1ll << d;
        if (d <= kSeamDepth && b.seam && m >= (1 << 16))
        {
            k_prefetch_seams<<<(unsigned)((nrec + 255) / 256), 256, 0, s>>>(b.recs, nrec, m, d, b.seam);
            ++launch_counter();
        }
        if (nodes <= kWarpNodes)
        {
            const unsigned g = (unsigned)((nodes * 32 + 127) / 128);
            k_build_level<true><<<g, 128, 0, s>>>(b.recs, nrec, b.V, b.node[(d + 1) & 1], b.node[d & 1], m, d,
                b.status, b.count_filter);
        }
        else
        {
            const unsigned g = (unsigned)((nodes + 127) / 128);
            k_build_level<false><<<g, 128, 0, s>>>(b.recs, nrec, b.V, b.node[(d + 1) & 1], b.node[d & 1], m, d,
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
    Builder B{ const_cast<Rec*>(R), nrec, st, count ? &st->pc : nullptr, -1, -1, false };
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
    const int      nrec = 3 * m;
    const unsigned g = (unsigned)((nrec + 255) / 256);
    k_tri_mask<<<g, 256, 0, s>>>(b.recs, nrec, b.tri_mask, b.status, b.count_filter);
    ++launch_counter();
    scan_exclusive(MaskCount{ b.tri_mask }, (size_t)nrec, b.tri_off, b.scratch, b.tri_count, s);
    k_tri_write<<<g, 256, 0, s>>>(b.recs, nrec, b.tri_mask, b.tri_off, b.vid, b.tris);
    ++launch_counter();
}

}  // namespace qdtg
