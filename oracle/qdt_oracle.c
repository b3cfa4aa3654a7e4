/*
 * CPU oracle for the batch Delaunay path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's batch triangulation, written from
 * the reference's behaviour (libqdt, MIT). Each function names the reference
 * file:line it follows. Used by the tests as the checker of the CUDA path and
 * by the benchmark as the timed CPU baseline ("port"); the product library
 * never links or calls it.
 *
 * Build: -O2 -ffp-contract=off (never -ffast-math): the filters' error bounds
 * assume separately rounded products, as the reference's CMakeLists.txt:52-58
 * demands.
 */
#define _GNU_SOURCE
#include "qdt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

enum
{
    ST_OK = 0,
    ST_NULL_ARG = -2,
    ST_TOO_MANY = -3,
    ST_NOT_FINITE = -4,
    ST_OOM = -10,
    ST_INTERNAL = -11
};

/* wrapper.hxx:15 */
#define MAX_POINTS ((size_t)100000000)

/* builder.hxx:66-69: a distinct input point and its lowest input index. */
typedef struct ovtx
{
    double   x, y;
    uint32_t id;
    uint32_t pad;
} ovtx;

/* builder.hxx:82-86: one quad-edge record; edge id = 4 * record + rotation. */
typedef struct oqe
{
    int32_t nx[4];
    int32_t org[2];
} oqe;

/* ------------------------------------------------------------------------ */
/* Robust predicates (robust.hxx)                                           */
/* ------------------------------------------------------------------------ */

/* robust.hxx:281-289 */
#define R_EPS 1.1102230246251565e-16
#define R_ERR_ORIENT ((3.0 + 16.0 * R_EPS) * R_EPS)
#define R_ERR_INCIRCLE ((10.0 + 96.0 * R_EPS) * R_EPS)
#define R_FILTER_FLOOR 1e-250

/* Error-free transformations (robust.hxx:166-178). */
static inline void two_sum(double a, double b, double* x, double* y)
{
    const double s = a + b;
    const double bv = s - a;
    const double av = s - bv;
    *y = (a - av) + (b - bv);
    *x = s;
}

static inline void two_prod(double a, double b, double* x, double* y)
{
    const double p = a * b;
    *y = fma(a, b, -p);
    *x = p;
}

/* Expansion arithmetic with zero elimination; components are kept in order
   of increasing magnitude, so the last one carries the sign. Each routine
   returns the length of its result. */

/* robust.hxx:180-189 */
static int x_diff(double a, double b, double* r)
{
    double x, y;
    int    n = 0;
    two_sum(a, -b, &x, &y);
    if (y != 0.0) r[n++] = y;
    if (x != 0.0) r[n++] = x;
    return n;
}

/* robust.hxx:191-206: r = e + b. */
static int x_grow(const double* e, int ne, double b, double* r)
{
    double q = b;
    int    n = 0;
    for (int i = 0; i < ne; ++i)
    {
        double qn, h;
        two_sum(q, e[i], &qn, &h);
        q = qn;
        if (h != 0.0) r[n++] = h;
    }
    if (q != 0.0) r[n++] = q;
    return n;
}

/* robust.hxx:208-217: r = a + b, one component of b at a time. r and tmp must
   hold na + nb entries; r may not alias a or b. */
static int x_add(const double* a, int na, const double* b, int nb, double* r, double* tmp)
{
    memcpy(r, a, (size_t)na * sizeof(double));
    int n = na;
    for (int i = 0; i < nb; ++i)
    {
        const int m = x_grow(r, n, b[i], tmp);
        memcpy(r, tmp, (size_t)m * sizeof(double));
        n = m;
    }
    return n;
}

/* robust.hxx:233-255: r = e * b. r holds 2 * ne entries. */
static int x_scale(const double* e, int ne, double b, double* r)
{
    if (ne == 0 || b == 0.0) return 0;
    int    n = 0;
    double q, hh;
    two_prod(e[0], b, &q, &hh);
    if (hh != 0.0) r[n++] = hh;
    for (int i = 1; i < ne; ++i)
    {
        double p1, p0, s;
        two_prod(e[i], b, &p1, &p0);
        two_sum(q, p0, &s, &hh);
        if (hh != 0.0) r[n++] = hh;
        two_sum(p1, s, &q, &hh);
        if (hh != 0.0) r[n++] = hh;
    }
    if (q != 0.0) r[n++] = q;
    return n;
}

/* robust.hxx:257-271: r = a * b as a sum of scaled copies of the longer
   operand. r holds 2 * na * nb entries. */
static int x_mul(const double* a, int na, const double* b, int nb, double* r)
{
    if (na == 0 || nb == 0) return 0;
    const double* big = na >= nb ? a : b;
    const double* sml = na >= nb ? b : a;
    const int     nbig = na >= nb ? na : nb;
    const int     nsml = na >= nb ? nb : na;
    /* every operand here has at most 16 components, so 2 * 16 * 16 bounds
       the product */
    double sc[40], acc[520], tmp[520];
    int    n = 0;
    for (int i = 0; i < nsml; ++i)
    {
        const int ns = x_scale(big, nbig, sml[i], sc);
        const int m = x_add(r, n, sc, ns, acc, tmp);
        memcpy(r, acc, (size_t)m * sizeof(double));
        n = m;
    }
    return n;
}

/* r = a - b for operands of at most 16 components. */
static int x_sub(const double* a, int na, const double* b, int nb, double* r)
{
    double nb_[16], tmp[40];
    for (int i = 0; i < nb; ++i) nb_[i] = -b[i];
    return x_add(a, na, nb_, nb, r, tmp);
}

/* robust.hxx:273-278 */
static int x_sign(const double* e, int n)
{
    if (n == 0) return 0;
    return e[n - 1] > 0 ? 1 : -1;
}

/* robust.hxx:297-306: the power of two that brings the largest magnitude
   near 1, only when it is far from 1. */
static int normalizing_exponent(const double* v, int n)
{
    double m = 0.0;
    for (int i = 0; i < n; ++i)
    {
        const double a = fabs(v[i]);
        if (a > m) m = a;
    }
    if (m == 0.0 || !isfinite(m)) return 0;
    const int e = ilogb(m);
    return (e >= -64 && e <= 64) ? 0 : e;
}

/* robust.hxx:321-336 */
int qdo_orient2d_exact(const double* a0, const double* b0, const double* c0)
{
    double    v[6] = { a0[0], a0[1], b0[0], b0[1], c0[0], c0[1] };
    const int e = normalizing_exponent(v, 6);
    if (e)
        for (int i = 0; i < 6; ++i) v[i] = ldexp(v[i], -e);
    double acx[2], acy[2], bcx[2], bcy[2], m1[8], m2[8], s[16];
    const int nacx = x_diff(v[0], v[4], acx), nacy = x_diff(v[1], v[5], acy);
    const int nbcx = x_diff(v[2], v[4], bcx), nbcy = x_diff(v[3], v[5], bcy);
    const int n1 = x_mul(acx, nacx, bcy, nbcy, m1);
    const int n2 = x_mul(acy, nacy, bcx, nbcx, m2);
    const int ns = x_sub(m1, n1, m2, n2, s);
    return x_sign(s, ns);
}

/* robust.hxx:348-376 */
int qdo_incircle_exact(const double* a0, const double* b0, const double* c0, const double* d0)
{
    double    v[8] = { a0[0], a0[1], b0[0], b0[1], c0[0], c0[1], d0[0], d0[1] };
    const int e = normalizing_exponent(v, 8);
    if (e)
        for (int i = 0; i < 8; ++i) v[i] = ldexp(v[i], -e);
    double adx[2], ady[2], bdx[2], bdy[2], cdx[2], cdy[2];
    const int nadx = x_diff(v[0], v[6], adx), nady = x_diff(v[1], v[7], ady);
    const int nbdx = x_diff(v[2], v[6], bdx), nbdy = x_diff(v[3], v[7], bdy);
    const int ncdx = x_diff(v[4], v[6], cdx), ncdy = x_diff(v[5], v[7], cdy);

    double m1[8], m2[8], tmp[1600];
    double ea[16], eb[16], ec[16];
    int    n1, n2;
    n1 = x_mul(adx, nadx, adx, nadx, m1);
    n2 = x_mul(ady, nady, ady, nady, m2);
    const int nea = x_add(m1, n1, m2, n2, ea, tmp);
    n1 = x_mul(bdx, nbdx, bdx, nbdx, m1);
    n2 = x_mul(bdy, nbdy, bdy, nbdy, m2);
    const int neb = x_add(m1, n1, m2, n2, eb, tmp);
    n1 = x_mul(cdx, ncdx, cdx, ncdx, m1);
    n2 = x_mul(cdy, ncdy, cdy, ncdy, m2);
    const int nec = x_add(m1, n1, m2, n2, ec, tmp);

    double s1[16], s2[16], s3[16];
    double p1[520], p2[520], p3[520], a1[1040], tot[1600];
    n1 = x_mul(bdx, nbdx, cdy, ncdy, m1);
    n2 = x_mul(cdx, ncdx, bdy, nbdy, m2);
    const int ns1 = x_sub(m1, n1, m2, n2, s1);
    const int np1 = x_mul(ea, nea, s1, ns1, p1);
    n1 = x_mul(cdx, ncdx, ady, nady, m1);
    n2 = x_mul(adx, nadx, cdy, ncdy, m2);
    const int ns2 = x_sub(m1, n1, m2, n2, s2);
    const int np2 = x_mul(eb, neb, s2, ns2, p2);
    n1 = x_mul(adx, nadx, bdy, nbdy, m1);
    n2 = x_mul(bdx, nbdx, ady, nady, m2);
    const int ns3 = x_sub(m1, n1, m2, n2, s3);
    const int np3 = x_mul(ec, nec, s3, ns3, p3);
    const int na1 = x_add(p1, np1, p2, np2, a1, tmp);
    const int nt = x_add(a1, na1, p3, np3, tot, tmp);
    return x_sign(tot, nt);
}

/* robust.hxx:337-347: the filter, then the exact sign. */
static inline int orient_sign(const double* a, const double* b, const double* c, qdo_stats* st)
{
    st->orient_calls++;
    const double detleft = (a[0] - c[0]) * (b[1] - c[1]);
    const double detright = (a[1] - c[1]) * (b[0] - c[0]);
    const double det = detleft - detright;
    const double mag = fabs(detleft) + fabs(detright);
    const double bound = R_ERR_ORIENT * mag;
    if ((det > bound || -det > bound) && mag > R_FILTER_FLOOR) return det > 0 ? 1 : -1;
    st->orient_exact++;
    return qdo_orient2d_exact(a, b, c);
}

/* robust.hxx:377-396 */
static inline int incircle_sign(const double* a, const double* b, const double* c, const double* d, qdo_stats* st)
{
    st->incircle_calls++;
    const double adx = a[0] - d[0], ady = a[1] - d[1];
    const double bdx = b[0] - d[0], bdy = b[1] - d[1];
    const double cdx = c[0] - d[0], cdy = c[1] - d[1];
    const double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    const double cdxady = cdx * ady, adxcdy = adx * cdy;
    const double adxbdy = adx * bdy, bdxady = bdx * ady;
    const double alift = adx * adx + ady * ady;
    const double blift = bdx * bdx + bdy * bdy;
    const double clift = cdx * cdx + cdy * cdy;
    const double det = alift * (bdxcdy - cdxbdy) + blift * (cdxady - adxcdy) + clift * (adxbdy - bdxady);
    const double perm = (fabs(bdxcdy) + fabs(cdxbdy)) * alift + (fabs(cdxady) + fabs(adxcdy)) * blift +
        (fabs(adxbdy) + fabs(bdxady)) * clift;
    const double bound = R_ERR_INCIRCLE * perm;
    if ((det > bound || -det > bound) && perm > R_FILTER_FLOOR) return det > 0 ? 1 : -1;
    st->incircle_exact++;
    return qdo_incircle_exact(a, b, c, d);
}

int qdo_orient2d(const double* a, const double* b, const double* c)
{
    qdo_stats st;
    memset(&st, 0, sizeof st);
    return orient_sign(a, b, c, &st);
}

int qdo_incircle(const double* a, const double* b, const double* c, const double* d)
{
    qdo_stats st;
    memset(&st, 0, sizeof st);
    return incircle_sign(a, b, c, d, &st);
}

/* ------------------------------------------------------------------------ */
/* Divide-and-conquer builder (builder.hxx:88-349)                          */
/* ------------------------------------------------------------------------ */

/* Threads.cpp:164-169, :31, :284 */
#define CHUNK_SIZE 65536
#define MAX_PARALLEL_DEPTH 3
#define PARALLEL_MIN_SIZE 524288
#define MERGE_PARALLEL_DEPTH 1
#define MAX_WORKERS 64
#define PARALLEL_MIN_POINTS 200000

/* Per-thread edge allocator (Wrapper.cpp:29-52 serial; Threads.cpp:182-213
   threaded: blocks of CHUNK_SIZE records and a private free list). */
typedef struct oalloc
{
    int32_t   free_head;
    int32_t   next_slot;
    int32_t   block_end;
    qdo_stats st;
} oalloc;

typedef struct obuild
{
    ovtx*       V;
    oqe*        qe;
    int64_t     cap;
    int         threaded;   /* pre-allocated pool handed out in chunks */
    int         use_pool;   /* threads may run (Threads.cpp:220-228) */
    int32_t     serial_next;
    atomic_int  g_next;
    atomic_int  bail;       /* the pool ran out: abandon the attempt */
    int         oom;
} obuild;

static inline int rot_(int e) { return (e & ~3) | ((e + 1) & 3); }
static inline int invrot_(int e) { return (e & ~3) | ((e + 3) & 3); }
static inline int sym_(int e) { return e ^ 2; }

#define ONEXT(B, e) ((B)->qe[(e) >> 2].nx[(e)&3])
#define ORG(B, e) ((B)->qe[(e) >> 2].org[((e) >> 1) & 1])

static inline int dest_(obuild* B, int e) { return ORG(B, sym_(e)); }
static inline int oprev_(obuild* B, int e) { return rot_(ONEXT(B, rot_(e))); }
static inline int lnext_(obuild* B, int e) { return rot_(ONEXT(B, invrot_(e))); }
static inline int rprev_(obuild* B, int e) { return ONEXT(B, sym_(e)); }

static int alloc_rec(obuild* B, oalloc* A)
{
    if (A->free_head >= 0)
    {
        const int k = A->free_head;
        A->free_head = B->qe[k].nx[0];
        return k;
    }
    if (!B->threaded)
    {
        if (B->serial_next >= B->cap)
        {
            const int64_t ncap = B->cap * 2 + 16;
            oqe*          q = (oqe*)realloc(B->qe, sizeof(oqe) * (size_t)ncap);
            if (!q)
            {
                B->oom = 1;
                atomic_store(&B->bail, 1);
                return 0;
            }
            B->qe = q;
            B->cap = ncap;
        }
        return B->serial_next++;
    }
    if (A->next_slot >= A->block_end)
    {
        const int s = atomic_fetch_add(&B->g_next, CHUNK_SIZE);
        if ((int64_t)s + CHUNK_SIZE > B->cap)
        {
            atomic_store(&B->bail, 1);
            return 0;
        }
        for (int i = 0; i < CHUNK_SIZE; ++i)
        {
            B->qe[s + i].org[0] = -1;
            B->qe[s + i].org[1] = -1;
        }
        A->next_slot = s;
        A->block_end = s + CHUNK_SIZE;
    }
    return A->next_slot++;
}

static void release_rec(obuild* B, oalloc* A, int k)
{
    B->qe[k].org[0] = -1;
    B->qe[k].nx[0] = A->free_head;
    A->free_head = k;
}

/* builder.hxx:131-142 */
static int make_edge(obuild* B, oalloc* A)
{
    const int k = alloc_rec(B, A);
    oqe*      q = &B->qe[k];
    const int e = 4 * k;
    q->nx[0] = e;
    q->nx[1] = e + 3;
    q->nx[2] = e + 2;
    q->nx[3] = e + 1;
    q->org[0] = q->org[1] = -1;
    return e;
}

/* builder.hxx:144-149 */
static void splice(obuild* B, int a, int b)
{
    const int alpha = rot_(ONEXT(B, a)), beta = rot_(ONEXT(B, b));
    int       t = ONEXT(B, a);
    ONEXT(B, a) = ONEXT(B, b);
    ONEXT(B, b) = t;
    t = ONEXT(B, alpha);
    ONEXT(B, alpha) = ONEXT(B, beta);
    ONEXT(B, beta) = t;
}

/* builder.hxx:151-159 */
static int connect_(obuild* B, oalloc* A, int a, int b)
{
    const int e = make_edge(B, A);
    ORG(B, e) = dest_(B, a);
    ORG(B, sym_(e)) = ORG(B, b);
    splice(B, e, lnext_(B, a));
    splice(B, sym_(e), b);
    return e;
}

/* builder.hxx:161-166 */
static void delete_edge(obuild* B, oalloc* A, int e)
{
    splice(B, e, oprev_(B, e));
    splice(B, sym_(e), oprev_(B, sym_(e)));
    release_rec(B, A, e >> 2);
}

static inline const double* P_(obuild* B, int v) { return &B->V[v].x; }

/* builder.hxx:168-175 */
static inline int ccw_(obuild* B, oalloc* A, int a, int b, int c)
{
    return orient_sign(P_(B, a), P_(B, b), P_(B, c), &A->st) > 0;
}
static inline int right_of(obuild* B, oalloc* A, int x, int e) { return ccw_(B, A, x, dest_(B, e), ORG(B, e)); }
static inline int left_of(obuild* B, oalloc* A, int x, int e) { return ccw_(B, A, x, ORG(B, e), dest_(B, e)); }
static inline int in_circle(obuild* B, oalloc* A, int a, int b, int c, int d)
{
    if (a == d || b == d || c == d || a == b || a == c || b == c) return 0;
    return incircle_sign(P_(B, a), P_(B, b), P_(B, c), P_(B, d), &A->st) > 0;
}

/* builder.hxx:71-76: the strict orders of the two frames. */
static inline int less_frame(const ovtx* a, const ovtx* b, int frame)
{
    if (frame == 0) return a->x < b->x || (a->x == b->x && a->y < b->y);
    return a->y < b->y || (a->y == b->y && a->x > b->x);
}

/* builder.hxx:177-201 */
static void leaf(obuild* B, oalloc* A, int lo, int hi, int frame, int* le, int* re)
{
    ovtx* V = B->V;
    /* sort the 2-3 points in the frame order */
    for (int i = lo + 1; i < hi; ++i)
        for (int j = i; j > lo && less_frame(&V[j], &V[j - 1], frame); --j)
        {
            ovtx t = V[j];
            V[j] = V[j - 1];
            V[j - 1] = t;
        }
    const int n = hi - lo, s1 = lo, s2 = lo + 1;
    if (n == 2)
    {
        const int a = make_edge(B, A);
        ORG(B, a) = s1;
        ORG(B, sym_(a)) = s2;
        *le = a;
        *re = sym_(a);
        return;
    }
    const int s3 = lo + 2;
    const int a = make_edge(B, A), b = make_edge(B, A);
    splice(B, sym_(a), b);
    ORG(B, a) = s1;
    ORG(B, sym_(a)) = s2;
    ORG(B, b) = s2;
    ORG(B, sym_(b)) = s3;
    const int o = orient_sign(P_(B, s1), P_(B, s2), P_(B, s3), &A->st);
    if (o > 0)
    {
        connect_(B, A, b, a);
        *le = a;
        *re = sym_(b);
        return;
    }
    if (o < 0)
    {
        const int c = connect_(B, A, b, a);
        *le = sym_(c);
        *re = c;
        return;
    }
    *le = a;
    *re = sym_(b);
}

/* builder.hxx:205-226 */
static void scan_left(obuild* B, oalloc* A, int basel, int* lc_out, int* lv_out)
{
    const int bo = ORG(B, basel), bd = dest_(B, basel);
    int       lc = ONEXT(B, sym_(basel));
    int       lv = ccw_(B, A, dest_(B, lc), bd, bo);
    if (lv)
    {
        int deleted = 0;
        while (!atomic_load_explicit(&B->bail, memory_order_relaxed) &&
            in_circle(B, A, bd, bo, dest_(B, lc), dest_(B, ONEXT(B, lc))))
        {
            const int t = ONEXT(B, lc);
            delete_edge(B, A, lc);
            lc = t;
            deleted = 1;
        }
        if (deleted) lv = ccw_(B, A, dest_(B, lc), bd, bo);
    }
    *lc_out = lc;
    *lv_out = lv;
}

/* builder.hxx:228-249 */
static void scan_right(obuild* B, oalloc* A, int basel, int* rc_out, int* rv_out)
{
    const int bo = ORG(B, basel), bd = dest_(B, basel);
    int       rc = oprev_(B, basel);
    int       rv = ccw_(B, A, dest_(B, rc), bd, bo);
    if (rv)
    {
        int deleted = 0;
        while (!atomic_load_explicit(&B->bail, memory_order_relaxed) &&
            in_circle(B, A, bd, bo, dest_(B, rc), dest_(B, oprev_(B, rc))))
        {
            const int t = oprev_(B, rc);
            delete_edge(B, A, rc);
            rc = t;
            deleted = 1;
        }
        if (deleted) rv = ccw_(B, A, dest_(B, rc), bd, bo);
    }
    *rc_out = rc;
    *rv_out = rv;
}

/* The concurrent left scan of the root merge (builder.hxx:263-269 with
   Threads.cpp:225-228): a helper thread takes the left scan of every step. */
typedef struct scan_helper
{
    obuild*    B;
    oalloc     A;
    atomic_int state; /* 0 idle, 1 work posted, 2 done, 3 quit */
    int        basel, lc, lv;
} scan_helper;

static void* scan_helper_main(void* p)
{
    scan_helper* h = (scan_helper*)p;
    for (;;)
    {
        int s;
        unsigned spins = 0;
        while ((s = atomic_load_explicit(&h->state, memory_order_acquire)) == 0 || s == 2)
        {
            if (++spins > 4096) sched_yield();
        }
        if (s == 3) return NULL;
        scan_left(h->B, &h->A, h->basel, &h->lc, &h->lv);
        atomic_store_explicit(&h->state, 2, memory_order_release);
    }
}

/* builder.hxx:251-285 */
static void merge(obuild* B, oalloc* A, int ldo, int ldi, int rdi, int rdo, int depth, int* ro, int* rr)
{
    for (;;)
    {
        if (atomic_load_explicit(&B->bail, memory_order_relaxed)) break;
        if (left_of(B, A, ORG(B, rdi), ldi)) ldi = lnext_(B, ldi);
        else if (right_of(B, A, ORG(B, ldi), rdi)) rdi = rprev_(B, rdi);
        else break;
    }
    int basel = connect_(B, A, sym_(rdi), ldi);
    if (ORG(B, ldi) == ORG(B, ldo)) ldo = sym_(basel);
    if (ORG(B, rdi) == ORG(B, rdo)) rdo = basel;

    const int    concurrent = B->use_pool && depth < MERGE_PARALLEL_DEPTH;
    scan_helper* hp = NULL;
    pthread_t    th;
    if (concurrent)
    {
        hp = (scan_helper*)calloc(1, sizeof(scan_helper));
        if (hp)
        {
            hp->B = B;
            hp->A.free_head = -1;
            atomic_store(&hp->state, 0);
            if (pthread_create(&th, NULL, scan_helper_main, hp) != 0)
            {
                free(hp);
                hp = NULL;
            }
        }
    }

    for (;;)
    {
        if (atomic_load_explicit(&B->bail, memory_order_relaxed)) break;
        int lc, lv, rc, rv;
        if (hp)
        {
            hp->basel = basel;
            atomic_store_explicit(&hp->state, 1, memory_order_release);
            scan_right(B, A, basel, &rc, &rv);
            unsigned spins = 0;
            while (atomic_load_explicit(&hp->state, memory_order_acquire) != 2)
            {
                if (++spins > 4096) sched_yield();
            }
            atomic_store_explicit(&hp->state, 0, memory_order_relaxed);
            lc = hp->lc;
            lv = hp->lv;
        }
        else
        {
            scan_left(B, A, basel, &lc, &lv);
            scan_right(B, A, basel, &rc, &rv);
        }
        if (!lv && !rv) break;
        const int bo = ORG(B, basel), bd = dest_(B, basel);
        if (!lv || (rv && in_circle(B, A, dest_(B, lc), bd, bo, dest_(B, rc))))
            basel = connect_(B, A, rc, sym_(basel));
        else
            basel = connect_(B, A, sym_(basel), sym_(lc));
    }
    if (hp)
    {
        atomic_store_explicit(&hp->state, 3, memory_order_release);
        pthread_join(th, NULL);
        A->st.orient_calls += hp->A.st.orient_calls;
        A->st.orient_exact += hp->A.st.orient_exact;
        A->st.incircle_calls += hp->A.st.incircle_calls;
        A->st.incircle_exact += hp->A.st.incircle_exact;
        free(hp);
    }
    *ro = ldo;
    *rr = rdo;
}

/* builder.hxx:287-301 */
static int hull_walk(obuild* B, int e, int frame, int want_max)
{
    for (;;)
    {
        if (atomic_load_explicit(&B->bail, memory_order_relaxed)) return e;
        const int nx = rprev_(B, e);
        const int pv = sym_(oprev_(B, e));
        const ovtx* ve = &B->V[ORG(B, e)];
        const ovtx* vn = &B->V[ORG(B, nx)];
        const ovtx* vp = &B->V[ORG(B, pv)];
        const int better_n = want_max ? less_frame(ve, vn, frame) : less_frame(vn, ve, frame);
        if (better_n)
        {
            e = nx;
            continue;
        }
        const int better_p = want_max ? less_frame(ve, vp, frame) : less_frame(vp, ve, frame);
        if (better_p)
        {
            e = pv;
            continue;
        }
        return e;
    }
}

/* Quickselect: puts the k-th smallest point (frame order) at a[k], smaller
   ones before it and larger ones after it (std::nth_element semantics, used
   by builder.hxx:308-325). */
static void select_nth(ovtx* a, int n, int k, int frame)
{
    int lo = 0, hi = n - 1;
    while (hi - lo > 16)
    {
        const int mid = lo + (hi - lo) / 2;
        /* median of three to a[lo] */
        if (less_frame(&a[mid], &a[lo], frame)) { ovtx t = a[mid]; a[mid] = a[lo]; a[lo] = t; }
        if (less_frame(&a[hi], &a[lo], frame)) { ovtx t = a[hi]; a[hi] = a[lo]; a[lo] = t; }
        if (less_frame(&a[hi], &a[mid], frame)) { ovtx t = a[hi]; a[hi] = a[mid]; a[mid] = t; }
        /* now a[lo] <= a[mid] <= a[hi]; use a[mid] as pivot */
        const ovtx pv = a[mid];
        int        i = lo, j = hi;
        while (i <= j)
        {
            while (less_frame(&a[i], &pv, frame)) ++i;
            while (less_frame(&pv, &a[j], frame)) --j;
            if (i <= j)
            {
                ovtx t = a[i];
                a[i] = a[j];
                a[j] = t;
                ++i;
                --j;
            }
        }
        if (k <= j) hi = j;
        else if (k >= i) lo = i;
        else return;
    }
    for (int i = lo + 1; i <= hi; ++i)
        for (int j = i; j > lo && less_frame(&a[j], &a[j - 1], frame); --j)
        {
            ovtx t = a[j];
            a[j] = a[j - 1];
            a[j - 1] = t;
        }
}

typedef struct build_task
{
    obuild* B;
    int     lo, hi, axis, out_axis, presorted, depth;
    int     le, re;
} build_task;

static void build(obuild* B, oalloc* A, int lo, int hi, int axis, int out_axis, int presorted, int depth, int* le,
    int* re);

static void* build_task_main(void* p)
{
    build_task* t = (build_task*)p;
    oalloc      A;
    memset(&A, 0, sizeof A);
    A.free_head = -1;
    build(t->B, &A, t->lo, t->hi, t->axis, t->out_axis, t->presorted, t->depth, &t->le, &t->re);
    /* the task's counters are folded in by the joiner */
    {
        qdo_stats* s = (qdo_stats*)malloc(sizeof(qdo_stats));
        if (s) *s = A.st;
        return s;
    }
}

/* builder.hxx:303-348 */
static void build(obuild* B, oalloc* A, int lo, int hi, int axis, int out_axis, int presorted, int depth, int* le,
    int* re)
{
    const int n = hi - lo;
    if (atomic_load_explicit(&B->bail, memory_order_relaxed))
    {
        *le = *re = 0;
        return;
    }
    if (n <= 3)
    {
        leaf(B, A, lo, hi, out_axis, le, re);
        return;
    }
    const int mid = lo + n / 2;
    if (!presorted) select_nth(B->V + lo, n, mid - lo, axis);
    const int child = 1 - axis;
    int       L0, L1, R0, R1;
    int       forked = 0;
    if (B->use_pool && depth < MAX_PARALLEL_DEPTH && n >= PARALLEL_MIN_SIZE)
    {
        build_task t = { B, lo, mid, child, axis, 0, depth + 1, 0, 0 };
        pthread_t  th;
        if (pthread_create(&th, NULL, build_task_main, &t) == 0)
        {
            forked = 1;
            build(B, A, mid, hi, child, axis, 0, depth + 1, &R0, &R1);
            void* ret = NULL;
            pthread_join(th, &ret);
            if (ret)
            {
                const qdo_stats* s = (const qdo_stats*)ret;
                A->st.orient_calls += s->orient_calls;
                A->st.orient_exact += s->orient_exact;
                A->st.incircle_calls += s->incircle_calls;
                A->st.incircle_exact += s->incircle_exact;
                free(ret);
            }
            L0 = t.le;
            L1 = t.re;
        }
    }
    if (!forked)
    {
        build(B, A, lo, mid, child, axis, 0, depth + 1, &L0, &L1);
        build(B, A, mid, hi, child, axis, 0, depth + 1, &R0, &R1);
    }
    if (atomic_load_explicit(&B->bail, memory_order_relaxed))
    {
        *le = *re = 0;
        return;
    }
    int r0, r1;
    merge(B, A, L0, L1, R0, R1, depth, &r0, &r1);
    if (out_axis != axis)
    {
        const int le2 = hull_walk(B, r0, out_axis, 0);
        const int reccw = hull_walk(B, ONEXT(B, r1), out_axis, 1);
        r0 = le2;
        r1 = oprev_(B, reccw);
    }
    *le = r0;
    *re = r1;
}

/* ------------------------------------------------------------------------ */
/* Unique-point loading (builder.hxx:356-390)                               */
/* ------------------------------------------------------------------------ */

static inline int vtx_less_xyid(const ovtx* a, const ovtx* b)
{
    if (a->x != b->x) return a->x < b->x;
    if (a->y != b->y) return a->y < b->y;
    return a->id < b->id;
}

/* introsort-style quicksort on (x, y, id) with insertion sort for short runs */
static void sort_xyid(ovtx* a, int n)
{
    typedef struct { int lo, hi; } rng;
    rng stack[128];
    int sp = 0;
    stack[sp++] = (rng){ 0, n - 1 };
    while (sp)
    {
        rng r = stack[--sp];
        int lo = r.lo, hi = r.hi;
        while (hi - lo > 24)
        {
            const int mid = lo + (hi - lo) / 2;
            if (vtx_less_xyid(&a[mid], &a[lo])) { ovtx t = a[mid]; a[mid] = a[lo]; a[lo] = t; }
            if (vtx_less_xyid(&a[hi], &a[lo])) { ovtx t = a[hi]; a[hi] = a[lo]; a[lo] = t; }
            if (vtx_less_xyid(&a[hi], &a[mid])) { ovtx t = a[hi]; a[hi] = a[mid]; a[mid] = t; }
            const ovtx pv = a[mid];
            int        i = lo, j = hi;
            while (i <= j)
            {
                while (vtx_less_xyid(&a[i], &pv)) ++i;
                while (vtx_less_xyid(&pv, &a[j])) --j;
                if (i <= j)
                {
                    ovtx t = a[i];
                    a[i] = a[j];
                    a[j] = t;
                    ++i;
                    --j;
                }
            }
            /* recurse into the smaller part first (bounded stack) */
            if (j - lo < hi - i)
            {
                if (i < hi) stack[sp++] = (rng){ i, hi };
                hi = j;
            }
            else
            {
                if (lo < j) stack[sp++] = (rng){ lo, j };
                lo = i;
            }
        }
        for (int i = lo + 1; i <= hi; ++i)
            for (int j = i; j > lo && vtx_less_xyid(&a[j], &a[j - 1]); --j)
            {
                ovtx t = a[j];
                a[j] = a[j - 1];
                a[j - 1] = t;
            }
    }
}

/* qdt.cpp:29-43: TOO_MANY, then NULL, then NOT_FINITE. */
int qdo_check_input(const double* xy, size_t n)
{
    if (n > MAX_POINTS) return ST_TOO_MANY;
    if (n == 0) return ST_OK;
    if (!xy) return ST_NULL_ARG;
    for (size_t i = 0; i < 2 * n; ++i)
        if (!isfinite(xy[i])) return ST_NOT_FINITE;
    return ST_OK;
}

/* builder.hxx:98-116 */
static int extract(obuild* B, int count, qdo_result* out, qdo_stats* st)
{
    size_t    cap = 2 * (size_t)(count / 3 + 4);
    uint32_t* tris = (uint32_t*)malloc(sizeof(uint32_t) * 3 * cap);
    size_t    nt = 0;
    if (!tris) return ST_OOM;
    for (int k = 0; k < count; ++k)
    {
        if (B->qe[k].org[0] < 0) continue;
        for (int r = 0; r < 4; r += 2)
        {
            const int e = 4 * k + r;
            const int f = lnext_(B, e), g = lnext_(B, f);
            if (lnext_(B, g) != e) continue;
            if (e > f || e > g) continue;
            const int a = ORG(B, e), b = ORG(B, f), c = ORG(B, g);
            if (orient_sign(P_(B, a), P_(B, b), P_(B, c), st) > 0)
            {
                if (nt == cap)
                {
                    cap *= 2;
                    uint32_t* t2 = (uint32_t*)realloc(tris, sizeof(uint32_t) * 3 * cap);
                    if (!t2)
                    {
                        free(tris);
                        return ST_OOM;
                    }
                    tris = t2;
                }
                tris[3 * nt + 0] = B->V[a].id;
                tris[3 * nt + 1] = B->V[b].id;
                tris[3 * nt + 2] = B->V[c].id;
                ++nt;
            }
        }
    }
    out->tris = tris;
    out->ntri = nt;
    return ST_OK;
}

static int run_builder(ovtx* V, int m, int threaded, int use_pool, qdo_result* out, int* bailed)
{
    obuild B;
    memset(&B, 0, sizeof B);
    B.V = V;
    B.threaded = threaded;
    B.use_pool = use_pool;
    /* Wrapper.cpp:32 reserves 3n + 16; Threads.cpp:179 allocates 5n + 64 Ki */
    B.cap = threaded ? 5 * (int64_t)m + 64 * 1024 : 3 * (int64_t)m + 16;
    B.qe = (oqe*)malloc(sizeof(oqe) * (size_t)B.cap);
    if (!B.qe) return ST_OOM;
    atomic_store(&B.g_next, 0);
    atomic_store(&B.bail, 0);
    oalloc A;
    memset(&A, 0, sizeof A);
    A.free_head = -1;
    int le, re;
    build(&B, &A, 0, m, 0, 0, 1, 0, &le, &re);
    *bailed = atomic_load(&B.bail);
    if (B.oom)
    {
        free(B.qe);
        return ST_OOM;
    }
    if (*bailed)
    {
        free(B.qe);
        return ST_OK;
    }
    const int count = threaded ? atomic_load(&B.g_next) : B.serial_next;
    const int rc = extract(&B, count, out, &A.st);
    A.st.records_used = (uint64_t)count;
    out->stats = A.st;
    free(B.qe);
    return rc;
}

static int hw_threads(void)
{
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    if (n < 1) n = 1;
    if (n > MAX_WORKERS) n = MAX_WORKERS;
    return (int)n;
}

/* Wrapper.cpp:1287-1305 (serial) and Threads.cpp:270-320 (threaded). The
   input_points copy of the handle is the caller's business. */
int qdo_triangulate(const double* xy, size_t n, int threaded, int nthreads, qdo_result* out)
{
    memset(out, 0, sizeof *out);
    const int st = qdo_check_input(xy, n);
    if (st != ST_OK) return st;
    out->n = n;
    if (n == 0) return ST_OK;

    out->rep = (uint32_t*)malloc(sizeof(uint32_t) * n);
    ovtx* V = (ovtx*)malloc(sizeof(ovtx) * n);
    if (!out->rep || !V)
    {
        free(V);
        qdo_result_free(out);
        return ST_OOM;
    }
    for (size_t i = 0; i < n; ++i)
    {
        V[i].x = xy[2 * i];
        V[i].y = xy[2 * i + 1];
        V[i].id = (uint32_t)i;
        V[i].pad = 0;
        out->rep[i] = (uint32_t)i;
    }
    sort_xyid(V, (int)n);
    size_t m = 0;
    for (size_t i = 0; i < n; ++i)
    {
        if (m > 0 && V[m - 1].x == V[i].x && V[m - 1].y == V[i].y)
        {
            out->rep[V[i].id] = V[m - 1].id;
            continue;
        }
        if (m != i) V[m] = V[i];
        ++m;
    }
    out->unique_points = m;

    int rc = ST_OK;
    if (m >= 3)
    {
        if (!threaded)
        {
            int bailed = 0;
            rc = run_builder(V, (int)m, 0, 0, out, &bailed);
        }
        else
        {
            int nt = nthreads > 0 ? nthreads : hw_threads();
            if (nt > MAX_WORKERS) nt = MAX_WORKERS;
            const int use_pool = nt > 1 && m >= PARALLEL_MIN_POINTS;
            int       bailed = 0;
            /* the attempt may reorder V; keep a copy for the serial fallback */
            ovtx* Vsave = NULL;
            if (use_pool)
            {
                Vsave = (ovtx*)malloc(sizeof(ovtx) * m);
                if (Vsave) memcpy(Vsave, V, sizeof(ovtx) * m);
            }
            rc = run_builder(V, (int)m, 1, use_pool, out, &bailed);
            if (rc == ST_OK && bailed)
            {
                /* Threads.cpp:298-305: fall back to the serial builder */
                if (Vsave) memcpy(V, Vsave, sizeof(ovtx) * m);
                rc = run_builder(V, (int)m, 0, 0, out, &bailed);
                out->stats.fell_back = 1;
            }
            else
                out->stats.threaded_used = use_pool;
            free(Vsave);
        }
    }
    free(V);
    if (rc != ST_OK)
    {
        qdo_result_free(out);
        return rc;
    }
    return ST_OK;
}

void qdo_result_free(qdo_result* r)
{
    if (!r) return;
    free(r->tris);
    free(r->rep);
    r->tris = NULL;
    r->rep = NULL;
    r->ntri = 0;
}

/* Batched exact signs for the Delaunay checker: out[i] = sign of the
   predicate on the points whose indices are idx[3 i .. 3 i + 2] (orient) or
   idx[4 i .. 4 i + 3] (in-circle). */
void qdo_orient_batch(const double* xy, const int64_t* idx, size_t k, int8_t* out)
{
    qdo_stats st;
    memset(&st, 0, sizeof st);
    for (size_t i = 0; i < k; ++i)
        out[i] = (int8_t)orient_sign(xy + 2 * idx[3 * i], xy + 2 * idx[3 * i + 1], xy + 2 * idx[3 * i + 2], &st);
}

void qdo_incircle_batch(const double* xy, const int64_t* idx, size_t k, int8_t* out)
{
    qdo_stats st;
    memset(&st, 0, sizeof st);
    for (size_t i = 0; i < k; ++i)
        out[i] = (int8_t)incircle_sign(xy + 2 * idx[4 * i], xy + 2 * idx[4 * i + 1], xy + 2 * idx[4 * i + 2],
            xy + 2 * idx[4 * i + 3], &st);
}
