// Stages K3-K6 of the batch triangulation: leaves, level-by-level merges with
// the hull re-walk, and the extraction of triangles.
//
// The quad-edge algebra, the leaf construction, the merge (lower common
// tangent, then the rising bubble with its two candidate scans) and the hull
// walk follow the reference builder (builder.hxx:123-301) step for step, so
// that the same split tree gives the same topology, also on cocircular and
// collinear input. What is GB300-specific is the schedule and the memory:
//
// * the tree is built bottom-up, one kernel launch per depth. At the deep
//   depths (hundreds of thousands of small merges) every node is one thread;
//   at the upper depths (few, long merges) every node is one warp, so that the
//   merges of a depth never share a warp and their load latencies overlap
//   across warps and SMs instead of serialising on divergence;
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

__device__ __forceinline__ int rot(int e) { return (e & ~3) | ((e + 1) & 3); }
__device__ __forceinline__ int invrot(int e) { return (e & ~3) | ((e + 3) & 3); }
__device__ __forceinline__ int sym(int e) { return e ^ 2; }

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
        if ((unsigned)e >= 4u * (unsigned)nrec)
        {
            fail(ST_BAD_INDEX);
            return 0;
        }
        return e;
    }

    // reference builder.hxx:123-129
    __device__ __forceinline__ int onext(int e)
    {
        e = chk(e);
        return R[e >> 2].nx[e & 3];
    }
    // e is always an id this thread has just read through onext(), which
    // checked it
    __device__ __forceinline__ void set_onext(int e, int v)
    {
        if (bad) return;   // after a failure, write nothing (other threads own other records)
        R[e >> 2].nx[e & 3] = v;
    }
    __device__ __forceinline__ int org(int e)
    {
        e = chk(e);
        return R[e >> 2].org[(e >> 1) & 1];
    }
    __device__ __forceinline__ double2 porg(int e)
    {
        e = chk(e);
        return R[e >> 2].p[(e >> 1) & 1];
    }
    __device__ __forceinline__ int     dest(int e) { return org(sym(e)); }
    __device__ __forceinline__ double2 pdest(int e) { return porg(sym(e)); }
    __device__ __forceinline__ int     oprev(int e) { return rot(onext(rot(e))); }
    __device__ __forceinline__ int     lnext(int e) { return rot(onext(invrot(e))); }
    __device__ __forceinline__ int     rprev(int e) { return onext(sym(e)); }

    // free list of the node (records of the subtree that are not in use)
    __device__ int alloc()
    {
        const int k = fhead;
        if (k < 0 || k >= nrec)
        {
            fail(ST_POOL_EMPTY);
            return -1;
        }
        fhead = R[k].link;
        if (fhead < 0) ftail = -1;
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

    // reference builder.hxx:131-142, with both origins (and their
    // coordinates) set at once
    __device__ int make_edge(int o0, int o1, double2 p0, double2 p1)
    {
        if (bad) return 0;
        const int k = alloc();
        if (k < 0) return 0;
        const int e = 4 * k;
        Rec&      r = R[k];
        *reinterpret_cast<int4*>(&r.nx[0]) = make_int4(e, e + 3, e + 2, e + 1);
        *reinterpret_cast<int4*>(&r.org[0]) = make_int4(o0, o1, -1, 0);
        r.p[0] = p0;
        r.p[1] = p1;
        return e;
    }

    // reference builder.hxx:144-149
    __device__ void splice(int a, int b)
    {
        const int ta = onext(a), tb = onext(b);
        const int alpha = rot(ta), beta = rot(tb);
        set_onext(a, tb);
        set_onext(b, ta);
        const int tal = onext(alpha), tbe = onext(beta);
        set_onext(alpha, tbe);
        set_onext(beta, tal);
    }

    // reference builder.hxx:151-159
    __device__ int connect(int a, int b)
    {
        const int e = make_edge(dest(a), org(b), pdest(a), porg(b));
        if (bad) return 0;
        splice(e, lnext(a));
        splice(sym(e), b);
        return e;
    }

    // reference builder.hxx:161-166
    __device__ void delete_edge(int e)
    {
        splice(e, oprev(e));
        splice(sym(e), oprev(sym(e)));
        release(chk(e) >> 2);
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
        {
            *reinterpret_cast<int4*>(&R[k].nx[0]) = make_int4(0, 0, 0, 0);
            *reinterpret_cast<int4*>(&R[k].org[0]) = make_int4(-1, -1, k + 1 < r1 ? k + 1 : -1, 0);
        }
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
        splice(sym(a), b);
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

    // reference builder.hxx:251-285 (with the scans :205-249 in line)
    __device__ void merge(int ldo, int ldi, int rdi, int rdo, int lim, int& out_l, int& out_r)
    {
        int it = 0;
        for (;;)
        {
            if (bad) return;
            if (++it > lim)
            {
                fail(ST_GUARD);
                return;
            }
            // leftOf(org(rdi), ldi), then rightOf(org(ldi), rdi)
            const double2 prdi = porg(rdi), pldi = porg(ldi);
            if (ccw(prdi, pldi, pdest(ldi), pc)) ldi = lnext(ldi);
            else if (ccw(pldi, pdest(rdi), prdi, pc)) rdi = rprev(rdi);
            else break;
        }
        int basel = connect(sym(rdi), ldi);
        if (org(ldi) == org(ldo)) ldo = sym(basel);
        if (org(rdi) == org(rdo)) rdo = basel;

        it = 0;
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
                    const int t = onext(lc);
                    const int td = dest(t);
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
                    const int t = oprev(rc);
                    const int td = dest(t);
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

constexpr unsigned kFatal = ST_POOL_EMPTY | ST_GUARD | ST_BAD_INDEX;

// One depth of the tree: leaves of that depth are built, internal nodes merge
// their children's results (written by the previous launch). WARP: one node
// per warp (lane 0 works), else one node per thread.
template <bool WARP>
__global__ void __launch_bounds__(128) k_build_level(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    const NodeOut* __restrict__ child, NodeOut* __restrict__ out, int m, int d, DevStatus* st, int count)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long k = WARP ? (g >> 5) : g;
    if (WARP && (threadIdx.x & 31)) return;
    if (k >= (1ll << d)) return;
    if (*(volatile unsigned*)&st->flags & kFatal) return;
    int lo, hi;
    if (!node_range(m, d, k, lo, hi)) return;
    Builder B{ R, nrec, st, count ? &st->pc : nullptr, -1, -1, false };
    const int n = hi - lo;
    NodeOut   o;
    if (n <= 3)
    {
        B.leaf(lo, hi, V, o.le, o.re);
    }
    else
    {
        const NodeOut L = child[2 * k], Rn = child[2 * k + 1];
        // the children's free lists lie inside their record ranges
        if ((L.fhead >= 0 && (L.ftail < 3 * lo || L.ftail >= 3 * hi)) ||
            (Rn.fhead >= 0 && (Rn.ftail < 3 * lo || Rn.ftail >= 3 * hi)))
        {
            B.fail(ST_BAD_INDEX);
            return;
        }
        // concatenate the children's free lists
        if (L.fhead >= 0)
        {
            B.fhead = L.fhead;
            if (Rn.fhead >= 0)
            {
                R[L.ftail].link = Rn.fhead;
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
        B.merge(L.le, L.re, Rn.le, Rn.re, lim, rl, rr);
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
    o.fhead = B.fhead;
    o.ftail = B.ftail;
    out[k] = o;
}

// Depths with at most this many nodes run one node per warp.
constexpr long long kWarpNodes = 1 << 14;

void launch_build(const BuildBuffers& b, int m, cudaStream_t s)
{
    const int D = split_levels(m);
    const int nrec = 3 * m;
    for (int d = D; d >= 0; --d)
    {
        const long long nodes = 1ll << d;
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
// smallest of its three edge ids, when it is a 3-cycle oriented
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
        for (int r = 0; r < 4; r += 2)
        {
            const int e = 4 * k + r;
            const int f = B.lnext(e), g = B.lnext(f);
            if (B.lnext(g) != e) continue;
            if (e > f || e > g) continue;
            if (ccw(B.porg(e), B.porg(f), B.porg(g), B.pc)) mk |= (uint8_t)(1 << (r >> 1));
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
    for (int r = 0; r < 4; r += 2)
    {
        if (!(mk & (1 << (r >> 1)))) continue;
        const int e = 4 * k + r;
        const int f = rot(R[invrot(e) >> 2].nx[invrot(e) & 3]);
        const int g = rot(R[invrot(f) >> 2].nx[invrot(f) & 3]);
        const int a = R[e >> 2].org[(e >> 1) & 1];
        const int b = R[f >> 2].org[(f >> 1) & 1];
        const int c = R[g >> 2].org[(g >> 1) & 1];
        tris[3 * (size_t)o + 0] = vid[a];
        tris[3 * (size_t)o + 1] = vid[b];
        tris[3 * (size_t)o + 2] = vid[c];
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
