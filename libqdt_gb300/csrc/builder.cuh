// The device-side builder shared by the single-set engine (k_build.cu) and
// the many-set engine (batch.cu): half-edge records, the reference's leaf,
// tangent, merge and hull walk on them (Builder), and the warp-cooperative
// merge of the upper levels (warp_merge).
#pragma once

#include "common.cuh"
#include "predicates.cuh"

#ifndef QDTG_SPLIT_DEBUG
#define QDTG_SPLIT_DEBUG 0
#endif
#if QDTG_SPLIT_DEBUG
#include <cstdio>
#endif

// Register cap of the level kernels (launched with 128 threads): 168, no
// spills in any form. Without a cap ptxas gave the warp forms 128 registers
// and 48-76 bytes of spills in the merge loop, which made the many-set
// build's warp heights markedly slower. (A lower cap for more resident
// blocks measured no faster: the thread-per-node levels are chains of
// dependent loads and predicates that run in about one wave.)
#define QDTG_BUILD_BOUNDS(WARP) __maxnreg__(168)

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

// The planar map lives in one of two stores, which give the builder the same
// primitives: the ring links of a half-edge, its origin and the origin's
// coordinates, record allocation from the node's free list, and status bits.
//
// GlobalMap: the map in HBM, 64-byte records (Rec) that carry the coordinates
// of both origins, ids global to the pool.
struct GlobalMap
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
    // onext (dir 0) or oprev (dir 1) with one load: next[2] and prev[2] are
    // adjacent in the record
    __device__ __forceinline__ int ring(int e, int dir)
    {
        e = chk(e);
        return (&R[e >> 1].next[0])[2 * dir + (e & 1)];
    }

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
    // records [r0, r1) of a leaf: free, chained in order
    __device__ void init_free(int r0, int r1)
    {
        for (int k = r0; k < r1; ++k)
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(-1, -1, k + 1 < r1 ? k + 1 : -1, 0);
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
};

// CellMap: the map of one cell (a subtree of at most kCellMax points) in
// shared memory, 16-byte records with 16-bit ids local to the cell; the
// coordinates are looked up in the cell's copy of its points.
struct SRec
{
    short next[2];
    short prev[2];
    short org[2];
    short link;
    short pad;
};

struct CellMap
{
    SRec*          R;
    int            nrec;
    DevStatus*     st;
    PredCounters*  pc;
    int            fhead, ftail;
    bool           bad;
    const double2* V;    // the cell's points
    int            nv;

    __device__ __forceinline__ void fail(unsigned bit)
    {
        if (!bad) atomicOr(&st->flags, bit);
        bad = true;
    }
    __device__ __forceinline__ int chk(int e)
    {
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
        // a dead record's origin is -1: the clamp keeps the read in the cell
        return V[min((unsigned)org(e), (unsigned)(nv - 1))];
    }
    __device__ __forceinline__ int ring(int e, int dir)
    {
        e = chk(e);
        return (&R[e >> 1].next[0])[2 * dir + (e & 1)];
    }
    __device__ __forceinline__ void set_next(int e, int v)
    {
        if (!bad) R[e >> 1].next[e & 1] = (short)v;
    }
    __device__ __forceinline__ void set_prev(int e, int v)
    {
        if (!bad) R[e >> 1].prev[e & 1] = (short)v;
    }
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
        R[k].link = (short)fhead;
        if (fhead < 0) ftail = k;
        fhead = k;
    }
    __device__ void settle_tail()
    {
        if (fhead < 0) ftail = -1;
    }
    __device__ void init_free(int r0, int r1)
    {
        for (int k = r0; k < r1; ++k)
            *reinterpret_cast<uint2*>(&R[k].org[0]) =
                make_uint2(0xFFFFFFFFu, (unsigned)(unsigned short)(k + 1 < r1 ? k + 1 : -1));
    }
    __device__ int make_edge(int o0, int o1, double2, double2)
    {
        if (bad) return 0;
        const int k = alloc();
        if (k < 0) return 0;
        const int      e = 2 * k;
        const unsigned ring = (unsigned)(e & 0xFFFF) | ((unsigned)(e + 1) << 16);
        *reinterpret_cast<uint4*>(&R[k]) =
            make_uint4(ring, ring, (unsigned)(o0 & 0xFFFF) | ((unsigned)o1 << 16), 0x0000FFFFu);
        return e;
    }
};

// The reference's map operations and the divide-and-conquer steps on either
// store.
template <class Map>
struct MapBuilder : Map
{
    using Map::R;
    using Map::nrec;
    using Map::pc;
    using Map::fhead;
    using Map::ftail;
    using Map::bad;
    using Map::fail;
    using Map::chk;
    using Map::onext;
    using Map::oprev;
    using Map::org;
    using Map::porg;
    using Map::set_next;
    using Map::set_prev;
    using Map::alloc;
    using Map::release;
    using Map::settle_tail;
    using Map::make_edge;

    // the last merge's upper tangent (its last base edge, from the right
    // part's vertex to the left part's); the lower one goes to memory (the
    // merge's first_out), so that no register holds it through the merge
    int basel_last = -1;

    __device__ __forceinline__ int     dest(int e) { return org(sym(e)); }
    __device__ __forceinline__ double2 pdest(int e) { return porg(sym(e)); }
    __device__ __forceinline__ int     lnext(int e) { return oprev(sym(e)); }
    __device__ __forceinline__ int     rprev(int e) { return onext(sym(e)); }

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
        this->init_free(r0, r1);
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

    // The same walk with one orient2d call site for both tests: shorter code
    // for the warp merge, whose first lane walks the tangent alone (measured
    // faster there, slower in the thread-per-node merges, which prefer the
    // form above with one load fewer per test).
    __device__ int tangent_one_site(int& ldo, int& ldi, int& rdi, int& rdo, int lim)
    {
        // leftOf(org(rdi), ldi) = ccw(org(rdi), org(ldi), dest(ldi)); when it
        // fails, rightOf(org(ldi), rdi) = ccw(org(ldi), dest(rdi), org(rdi))
        // (second: the rightOf test is next)
        int  it = 0;
        bool second = false;
        for (;;)
        {
            if (bad) return 0;
            if (++it > 2 * lim)
            {
                fail(ST_GUARD);
                return 0;
            }
            const double2 prdi = porg(rdi), pldi = porg(ldi);
            const double2 b = porg(second ? sym(rdi) : ldi);
            const double2 c = porg(second ? rdi : sym(ldi));
            if (ccw(second ? pldi : prdi, b, c, pc))
            {
                if (second)
                {
                    rdi = rprev(rdi);
                    second = false;
                }
                else
                    ldi = lnext(ldi);
            }
            else if (second)
                break;
            else
                second = true;
        }
        const int basel = connect(sym(rdi), ldi);
        if (org(ldi) == org(ldo)) ldo = sym(basel);
        if (org(rdi) == org(rdo)) rdo = basel;
        return basel;
    }

    // reference builder.hxx:251-285 (with the scans :205-249 in line)
    __device__ void merge(int ldo, int ldi, int rdi, int rdo, int lim, int& out_l, int& out_r,
        volatile int* first_out = nullptr)
    {
        int basel = tangent(ldo, ldi, rdi, rdo, lim);
        if (first_out) *first_out = basel;
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
            int           lc = 0, lcd = 0, rc = 0, rcd = 0;
            double2       plcd = pbo, prcd = pbo;
            bool          lv = false, rv = false;
            // the two candidate scans, left then right, as one loop over the
            // sides so that their predicate calls share code: side 0 walks
            // the ring of bd counter-clockwise from onext(sym(basel))
            // (builder.hxx:205-226), side 1 the ring of bo clockwise from
            // oprev(basel) (:228-249)
#pragma unroll 1
            for (int side = 0; side < 2; ++side)
            {
                int     c = side ? oprev(basel) : onext(sym(basel));
                int     cd = dest(c);
                double2 pcd = pdest(c);
                bool    v = false;
                // validE(c); if valid, the delete loop, and validE again after
                // deletions (one call site for both validity tests)
                for (int pass = 0;; ++pass)
                {
                    // a candidate ending at bo or bd is collinear: not valid
                    v = cd != bo && cd != bd && ccw(pcd, pbd, pbo, pc);
                    if (!v || pass) break;
                    bool deleted = false;
                    int  j = 0;
                    for (;;)
                    {
                        const int     t = this->ring(c, side);
                        const int     td = dest(t);
                        const double2 ptd = pdest(t);
                        if (!in_circle(bd, pbd, bo, pbo, cd, pcd, td, ptd)) break;
                        if (bad || ++j > lim)
                        {
                            fail(ST_GUARD);
                            return;
                        }
                        delete_edge(c);
                        c = t;
                        cd = td;
                        pcd = ptd;
                        deleted = true;
                    }
                    if (!deleted) break;
                }
                if (side)
                    rc = c, rcd = cd, prcd = pcd, rv = v;
                else
                    lc = c, lcd = cd, plcd = pcd, lv = v;
            }
            if (!lv && !rv) break;
            if (!lv || (rv && in_circle(lcd, plcd, bd, pbd, bo, pbo, rcd, prcd)))
                basel = connect(rc, sym(basel));
            else
                basel = connect(sym(basel), sym(lc));
        }
        basel_last = basel;
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

using Builder = MapBuilder<GlobalMap>;
using CellBuilder = MapBuilder<CellMap>;

// The extremes of a merged node in the frame g of its parent (the reference
// walks the merged hull to them, builder.hxx:340-346, which takes as many
// steps as the hull has vertices between the old and the new extremes: all
// of them for points in convex position). The union's extreme vertex is one
// of the children's extremes in g, and its hull edge is that child's
// unless the vertex is a tangent point: with the lower tangent b -> a and
// the upper tangent d -> c (a, c in the left part), the counter-clockwise
// hull edge out of a becomes a -> b and out of d becomes d -> c; the
// clockwise one out of c becomes c -> d and out of b becomes b -> a. Every
// other hull edge of the children at an extreme vertex lies on the merged
// hull untouched. The hull walk from that prediction then returns at once
// with the reference's edge (it walks on if the prediction is off).
//
// Both steps are out of line and take plain pointers: the merge loop between
// them keeps its registers. Across the merge the node's own output slot
// holds the choice (pad0, pad1: the union's extreme vertices in g, bit 31
// set when the right child holds it) and the lower tangent (le2, written by
// the merge through its first_out); the slot's final value comes after.
//
// Before the merge (it may delete hull edges of the part that does not hold
// an extreme): the choice, from the children's slots.
static __device__ __noinline__ void extremes_before_merge(Rec* R, int nrec, DevStatus* st, const NodeOut* Lc,
    const NodeOut* Rc, NodeOut* self, int g)
{
    Builder   B{ R, nrec, st, nullptr, -1, -1, false };
    const int l0 = Lc->le2, l1 = Lc->re2, r0 = Rc->le2, r1 = Rc->re2;
    const bool min_right = less_frame(B.porg(r0), B.porg(l0), g);
    const bool max_right = less_frame(B.porg(l1), B.porg(r1), g);
    const int  vmin = B.org(min_right ? r0 : l0), vmax = B.org(max_right ? r1 : l1);
    volatile int* p = &self->pad0;
    p[0] = (int)((unsigned)vmin | (min_right ? 0x80000000u : 0u));
    p[1] = (int)((unsigned)vmax | (max_right ? 0x80000000u : 0u));
}

__device__ __forceinline__ volatile int* lower_tangent_slot(NodeOut* slot) { return &slot->le2; }

// After the merge, with its upper tangent b1: (le, re) in frame g, as the
// reference's hull walks give them.
static __device__ __noinline__ int2 extremes_after_merge(Rec* R, int nrec, DevStatus* st, int b1,
    const NodeOut* self, const NodeOut* Lc, const NodeOut* Rc, int g, int lim)
{
    Builder             B{ R, nrec, st, nullptr, -1, -1, false };
    const volatile int* sp = &self->le2;
    const int           b0 = sp[0];   // b -> a; b1 is d -> c
    const int           xmin = sp[2], xmax = sp[3];
    const bool          min_right = xmin < 0, max_right = xmax < 0;
    const int           vmin = xmin & 0x7FFFFFFF, vmax = xmax & 0x7FFFFFFF;
    int                 e;
    if (!min_right) e = vmin == B.dest(b0) ? sym(b0) : Lc->le2;
    else e = vmin == B.org(b1) ? b1 : Rc->le2;
    const int le = B.hull_walk(e, g, false, lim);
    if (!max_right) e = vmax == B.dest(b1) ? sym(b1) : Lc->re2;
    else e = vmax == B.org(b0) ? b0 : Rc->re2;
    const int re = B.oprev(B.hull_walk(B.onext(e), g, true, lim));
    return make_int2(le, re);
}

// A node's extremes in frame g by walking its hull from le, re (a leaf: at
// most three vertices; a cell root: at most the cell's).
template <class BuilderT>
__device__ inline void extremes_by_walk(BuilderT& B, int le, int re, int g, int lim, int& le2, int& re2)
{
    le2 = B.hull_walk(le, g, false, lim);
    re2 = B.oprev(B.hull_walk(B.onext(re), g, true, lim));
}

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
//
// The window width kWin (1..3, a template parameter: any width gives the
// same decisions) trades passes against speculative predicate lanes: on
// points in general position 2 is fastest; on integer lattices and snapped
// grids, where most speculative in-circle tests are cocircular and go to
// the exact evaluation side by side in the lanes, 1 is (1024² lattice build
// 40.5 -> 29.2 ms, 256² grid 11.0 -> 9.4 ms; uniform and circle inputs are
// 10-25 % slower with 1). The build picks 1 when most distinct points share
// their x with another (kTieWindow).
constexpr int kWinDefault = 2;

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

template <int kWin = kWinDefault>
static __device__ void warp_merge(Builder& B, int ldo, int ldi, int rdi, int rdo, int lim, int& out_l, int& out_r,
    volatile int* first_out = nullptr)
{
    static_assert(kWin >= 1 && kWin <= 3, "window of 1 to 3 candidates");
    const unsigned FULL = 0xffffffffu;
    Rec* const     R = B.R;
    const int      nrec = B.nrec;
    const int      lane = threadIdx.x & 31;
    const bool     left = lane < 16;
    const int      j = lane & 15;
    const bool     slot = j < kWin;
    const int      q = left ? (j - 4) : (j + 4);   // combo index 0..15 = 4 a + b
    const int      ca = q >> 2, rb = q & 3;
    // lanes 4..11 and 20..27 hold the choice tests of the pairs (a, b) inside
    // the window (dl, dr < kWin when a pass ends with a choice)
    const bool     combo = j >= 4 && j < 12 && ca < kWin && rb < kWin;
    const int      jj = slot ? j : 0;               // window slot this lane keeps

    int basel = 0;
    if (lane == 0)
    {
        basel = B.tangent_one_site(ldo, ldi, rdi, rdo, lim);
        if (first_out) *first_out = basel;
    }
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
#if QDTG_SPLIT_DEBUG
    long long dbg_t0 = clock64(), dbg_win = 0, dbg_pred = 0, dbg_conn = 0, dbg_c = 0;
    int       dbg_steps = 0, dbg_passes = 0;
#endif
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
#if QDTG_SPLIT_DEBUG
            ++dbg_passes;
            dbg_c = clock64();
#endif
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
#if QDTG_SPLIT_DEBUG
            {
                const int sink = __shfl_sync(FULL, cur.e ^ mine.e ^ succ.e, 0);
                const long long c1 = clock64() + (sink & 0);
                dbg_win += c1 - dbg_c;
                dbg_c = c1;
            }
#endif
            // --- one wave of predicates
            const int     src_a = combo ? ca : 0, src_b = combo ? 16 + rb : 16;
            const int     ad = __shfl_sync(FULL, mine.d, src_a), bdst = __shfl_sync(FULL, mine.d, src_b);
            const double2 pa = shfl_d2(mine.p, src_a), pb = shfl_d2(mine.p, src_b);
            // a candidate that ends at bo or bd (a window that wrapped around a
            // short ring) is collinear with the base edge: not valid, decided by
            // its id without a predicate (distinct ids have distinct points)
            const bool valid = slot && mine.d != bo && mine.d != bd && ccw(mine.p, pbd, pbo, B.pc);
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
#if QDTG_SPLIT_DEBUG
            {
                const long long c1 = clock64();
                dbg_pred += c1 - dbg_c;
                dbg_c = c1;
            }
#endif
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
#if QDTG_SPLIT_DEBUG
        const long long dbg_cc = clock64();
        ++dbg_steps;
#endif
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
#if QDTG_SPLIT_DEBUG
        dbg_conn += clock64() - dbg_cc;
#endif
    }
#if QDTG_SPLIT_DEBUG
    if (lane == 0 && B.nrec > 0 && first_out && dbg_steps > 300)
        printf("warp merge steps=%d passes=%d cyc=%lld win=%lld pred=%lld conn=%lld\n", dbg_steps, dbg_passes,
            clock64() - dbg_t0, dbg_win, dbg_pred, dbg_conn);
#endif
    if (lane == 0)
    {
        B.fhead = fhead;
        B.ftail = ftail;
    }
    B.basel_last = basel;
    out_l = __shfl_sync(FULL, ldo, 0);
    out_r = __shfl_sync(FULL, rdo, 0);
}

constexpr unsigned kFatal = ST_POOL_EMPTY | ST_GUARD | ST_BAD_INDEX | ST_SPLIT;

// ---------------------------------------------------------------------------
// Cells: the bottom of the tree in shared memory
// ---------------------------------------------------------------------------
//
// Most of the merge work of a large set is in the deep levels: millions of
// merges of a few points each, every one a chain of dependent record reads.
// Out of HBM each read waits a DRAM round trip. A cell is the subtree under a
// node of at most C points (C <= kCellMax): one warp copies the cell's points
// into shared memory, builds every level of the subtree there with the same
// builder on 16-byte records (one lane per node, the lanes synchronised
// between depths), and writes the cell's records to the pool once, in the
// pool's format and ids. The records, free lists and decisions are those of
// the level-by-level build, so the result is the same.

// levels below a node of c points (the depth of its deepest leaves)
__host__ __device__ inline int subtree_levels(int c)
{
    int d = 0;
    while ((((long long)c + (1ll << d) - 1) >> d) >= 4) ++d;
    return d;
}

// depth of the cells of a set of m points: the first depth whose nodes have
// at most C points
__host__ __device__ inline int cell_depth(int m, int C)
{
    int d = 0;
    while ((((long long)m + (1ll << d) - 1) >> d) > C) ++d;
    return d;
}

struct CellNode
{
    short le, re, fh, ft;
};

// shared memory of one warp's cell: records, points, node results
__host__ __device__ inline int cell_smem_bytes(int C)
{
    return 3 * C * (int)sizeof(SRec) + C * (int)sizeof(double2) + (2 << subtree_levels(C)) * (int)sizeof(CellNode);
}

// warps (cells) per block: up to 4, within the 227 KB a block may have
constexpr int kCellBlockWarps = 4;
__host__ __device__ inline int cell_block_warps(int C)
{
    const int w = (227 * 1024) / cell_smem_bytes(C);
    return w < 1 ? 1 : (w > kCellBlockWarps ? kCellBlockWarps : w);
}

// Builds the cell [clo, chi) (positions of V), whose root is at depth dc, in
// the shared memory at smem (cell_smem_bytes(C) bytes, 16-byte aligned), and
// writes its records [3 clo, 3 chi) to the pool R and its root's result to
// *out. Called by all 32 lanes of a warp.
__device__ inline void build_cell(char* smem, const double2* __restrict__ V, Rec* __restrict__ R, int clo, int chi,
    int dc, DevStatus* st, PredCounters* pc, NodeOut* out)
{
    const int lane = threadIdx.x & 31;
    const int c = chi - clo;
    const int Lmax = subtree_levels(c);
    SRec*     sR = reinterpret_cast<SRec*>(smem);
    double2*  sV = reinterpret_cast<double2*>(smem + 3 * c * sizeof(SRec));
    CellNode* sN = reinterpret_cast<CellNode*>(smem + 3 * c * sizeof(SRec) + c * sizeof(double2));
    for (int i = lane; i < c; i += 32) sV[i] = V[clo + i];
    __syncwarp();
    bool bad = false;
    for (int L = Lmax; L >= 0; --L)
    {
        for (int kk = lane; kk < (1 << L); kk += 32)
        {
            int lo, hi;
            if (!node_range(c, L, kk, lo, hi)) continue;
            CellBuilder B{ sR, 3 * c, st, pc, -1, -1, false, sV, c };
            const int   n = hi - lo;
            int         le = 0, re = 0;
            if (n <= 3)
                B.leaf(lo, hi, sV, le, re);
            else
            {
                const CellNode a = sN[(2 << L) + 2 * kk], b = sN[(2 << L) + 2 * kk + 1];
                if ((a.fh >= 0 && (a.ft < 3 * lo || a.ft >= 3 * hi)) || (b.fh >= 0 && (b.ft < 3 * lo || b.ft >= 3 * hi)))
                {
                    B.fail(ST_BAD_INDEX);
                    bad = true;
                    continue;
                }
                if (a.fh >= 0)
                {
                    B.fhead = a.fh;
                    if (b.fh >= 0)
                    {
                        sR[a.ft].link = b.fh;
                        B.ftail = b.ft;
                    }
                    else
                        B.ftail = a.ft;
                }
                else
                {
                    B.fhead = b.fh;
                    B.ftail = b.ft;
                }
                B.merge(a.le, a.re, b.le, b.re, 8 * n + 64, le, re);
                const int d = dc + L;
                if (d > 0 && !B.bad)
                {
                    const int frame = (d - 1) & 1;
                    const int le2 = B.hull_walk(le, frame, false, n + 8);
                    const int reccw = B.hull_walk(B.onext(re), frame, true, n + 8);
                    le = le2;
                    re = B.oprev(reccw);
                }
            }
            B.settle_tail();
            bad |= B.bad;
            sN[(1 << L) + kk] = CellNode{ (short)le, (short)re, (short)B.fhead, (short)B.ftail };
        }
        __syncwarp();
    }
    if (__any_sync(0xffffffffu, bad)) return;
    // the cell's records in the pool's format: ids shifted to the pool's,
    // coordinates of both origins attached
    const int ebase = 6 * clo, rbase = 3 * clo;
    for (int k = lane; k < 3 * c; k += 32)
    {
        const uint4 w = *reinterpret_cast<const uint4*>(&sR[k]);
        const SRec& s = sR[k];
        int4        a, b;
        double2     p0 = make_double2(0, 0), p1 = p0;
        if (s.org[0] < 0)
        {
            a = make_int4(0, 0, 0, 0);
            b = make_int4(-1, -1, s.link < 0 ? -1 : rbase + s.link, 0);
        }
        else
        {
            a = make_int4(ebase + (short)(w.x & 0xFFFF), ebase + (short)(w.x >> 16), ebase + (short)(w.y & 0xFFFF),
                ebase + (short)(w.y >> 16));
            b = make_int4(clo + s.org[0], clo + s.org[1], -1, 0);
            p0 = sV[min((unsigned)s.org[0], (unsigned)(c - 1))];
            p1 = sV[min((unsigned)s.org[1], (unsigned)(c - 1))];
        }
        Rec& r = R[rbase + k];
        *reinterpret_cast<int4*>(&r.next[0]) = a;
        *reinterpret_cast<int4*>(&r.org[0]) = b;
        r.p[0] = p0;
        r.p[1] = p1;
    }
    if (lane == 0)
    {
        const CellNode o = sN[1];
        NodeOut        no;
        no.le = ebase + o.le;
        no.re = ebase + o.re;
        no.fhead = o.fh < 0 ? -1 : rbase + o.fh;
        no.ftail = o.ft < 0 ? -1 : rbase + o.ft;
        no.le2 = no.re2 = -1;
        no.pad0 = no.pad1 = 0;
        if (dc > 0)
        {
            // the root's extremes in its own merge frame, walked in shared memory
            CellBuilder B{ sR, 3 * c, st, pc, -1, -1, false, sV, c };
            int         le2 = 0, re2 = 0;
            extremes_by_walk(B, o.le, o.re, dc & 1, c + 8, le2, re2);
            no.le2 = ebase + le2;
            no.re2 = ebase + re2;
        }
        *out = no;
    }
}

}  // namespace qdtg
