// Robust orient2d / in-circle predicates for the GPU.
//
// Decisions are exact signs. Each predicate first evaluates the reference's
// floating-point filter (reference robust.hxx:337-347 and :377-396, with the
// same error bounds :281-289); when the filter cannot decide, the determinant
// is evaluated exactly in integer arithmetic:
//
//   every double v is (-1)^s * m * 2^e with m odd; with E the smallest e over
//   the predicate's coordinates, every coordinate is an integer N * 2^E, and
//   the determinant is a polynomial with integer coefficients in the N, so
//   its sign is that of an integer computation -- no rounding, no underflow,
//   no overflow, for every finite input including subnormals.
//
// The integer evaluation picks the narrowest form that holds the result:
// int64/int128 when the coordinates span few bits (integer lattices), and
// little-endian 32-bit-limb arithmetic of the needed length otherwise. The
// reference evaluates its exact fallback with floating-point expansions
// instead (robust.hxx:31-278); both give the exact sign, so the decisions
// are the same wherever the reference's arithmetic is exact.
//
// Products in the filter use dmul / dadd / dsub, so the
// compiler cannot contract them into FMAs: the filter's error bounds assume
// separately rounded operations.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "common.cuh"

// The predicates are compiled for the device (the engine) and for the host
// (the incremental insertion and constraint code).
#define QDT_HD __host__ __device__

namespace qdtg {

QDT_HD __forceinline__ uint64_t dbits(double v)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
#endif
}
QDT_HD __forceinline__ int ctz64(uint64_t x)   // x != 0
{
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}
QDT_HD __forceinline__ int clz64(uint64_t x)   // x != 0
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}
// separately rounded operations (no contraction into FMA)
QDT_HD __forceinline__ double mul_rn(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
QDT_HD __forceinline__ double add_rn(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
QDT_HD __forceinline__ double sub_rn(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}

constexpr double kEps = 1.1102230246251565e-16;
constexpr double kErrOrient = (3.0 + 16.0 * kEps) * kEps;
constexpr double kErrIncircle = (10.0 + 96.0 * kEps) * kEps;
constexpr double kFilterFloor = 1e-250;

// ---------------------------------------------------------------------------
// Exact integer evaluation
// ---------------------------------------------------------------------------

struct Dec
{
    uint64_t m;   // odd mantissa (0 for a zero coordinate)
    int      e;   // exponent of the lowest set bit
    int      neg;
};

QDT_HD __forceinline__ Dec decompose(double v)
{
    const uint64_t b = dbits(v);
    Dec            d;
    d.neg = (int)(b >> 63);
    const int      ex = (int)((b >> 52) & 0x7FF);
    uint64_t       man = b & ((1ull << 52) - 1);
    if (ex == 0)
    {
        if (man == 0)
        {
            d.m = 0;
            d.e = 0;
            d.neg = 0;
            return d;
        }
        d.e = -1074;
    }
    else
    {
        man |= 1ull << 52;
        d.e = ex - 1075;
    }
    const int tz = ctz64(man);
    d.m = man >> tz;
    d.e += tz;
    return d;
}

QDT_HD __forceinline__ int bitlen64(uint64_t x) { return x ? 64 - clz64(x) : 0; }

// Signed-magnitude big integers on caller-provided limb storage.
struct BigRef
{
    uint32_t* d;
    int       n;    // limbs in use (no leading zero limbs)
    int       neg;
};

QDT_HD __forceinline__ void big_trim(BigRef& a)
{
    while (a.n > 0 && a.d[a.n - 1] == 0) --a.n;
    if (a.n == 0) a.neg = 0;
}

// a = m << sh (m < 2^53), with sign
QDT_HD inline void big_set_shifted(BigRef& a, uint64_t m, int sh, int neg)
{
    const int limb = sh >> 5, bit = sh & 31;
    for (int i = 0; i < limb; ++i) a.d[i] = 0;
    // m << bit spans at most 53 + 31 = 84 bits: three limbs
    const uint64_t lo = m << bit;
    const uint64_t hi = bit ? (m >> (64 - bit)) : 0;
    a.d[limb + 0] = (uint32_t)lo;
    a.d[limb + 1] = (uint32_t)(lo >> 32);
    a.d[limb + 2] = (uint32_t)hi;
    a.n = limb + 3;
    a.neg = neg;
    big_trim(a);
}

QDT_HD inline int mag_cmp(const uint32_t* a, int na, const uint32_t* b, int nb)
{
    if (na != nb) return na < nb ? -1 : 1;
    for (int i = na - 1; i >= 0; --i)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

// r = |a| + |b|; r may alias a or b
QDT_HD inline int mag_add(uint32_t* r, const uint32_t* a, int na, const uint32_t* b, int nb)
{
    if (na < nb)
    {
        const uint32_t* t = a;
        a = b;
        b = t;
        const int tn = na;
        na = nb;
        nb = tn;
    }
    uint64_t c = 0;
    for (int i = 0; i < na; ++i)
    {
        c += (uint64_t)a[i] + (i < nb ? b[i] : 0u);
        r[i] = (uint32_t)c;
        c >>= 32;
    }
    int n = na;
    if (c) r[n++] = (uint32_t)c;
    return n;
}

// r = |a| - |b| with |a| >= |b|; r may alias a or b
QDT_HD inline int mag_sub(uint32_t* r, const uint32_t* a, int na, const uint32_t* b, int nb)
{
    int64_t c = 0;
    for (int i = 0; i < na; ++i)
    {
        c += (int64_t)a[i] - (int64_t)(i < nb ? b[i] : 0u);
        r[i] = (uint32_t)c;
        c >>= 32;   // arithmetic: 0 or -1
    }
    int n = na;
    while (n > 0 && r[n - 1] == 0) --n;
    return n;
}

// r = a + (sb ? -b : b); r may alias a or b
QDT_HD inline void big_addsub(BigRef& r, const BigRef& a, const BigRef& b, int negate_b)
{
    const int bneg = b.neg ^ (negate_b && b.n ? 1 : 0);
    if (a.neg == bneg)
    {
        const int neg = a.neg;
        r.n = mag_add(r.d, a.d, a.n, b.d, b.n);
        r.neg = neg;
    }
    else
    {
        const int c = mag_cmp(a.d, a.n, b.d, b.n);
        if (c >= 0)
        {
            const int neg = a.neg;
            r.n = mag_sub(r.d, a.d, a.n, b.d, b.n);
            r.neg = neg;
        }
        else
        {
            r.n = mag_sub(r.d, b.d, b.n, a.d, a.n);
            r.neg = bneg;
        }
    }
    big_trim(r);
}

// r = a * b; r must not alias a or b
QDT_HD inline void big_mul(BigRef& r, const BigRef& a, const BigRef& b)
{
    if (a.n == 0 || b.n == 0)
    {
        r.n = 0;
        r.neg = 0;
        return;
    }
    const int n = a.n + b.n;
    for (int i = 0; i < n; ++i) r.d[i] = 0;
    for (int i = 0; i < a.n; ++i)
    {
        uint64_t  c = 0;
        const uint64_t ai = a.d[i];
        for (int j = 0; j < b.n; ++j)
        {
            c += ai * b.d[j] + r.d[i + j];
            r.d[i + j] = (uint32_t)c;
            c >>= 32;
        }
        r.d[i + b.n] = (uint32_t)c;
    }
    r.n = n;
    r.neg = a.neg ^ b.neg;
    big_trim(r);
}

QDT_HD __forceinline__ int big_sign(const BigRef& a) { return a.n == 0 ? 0 : (a.neg ? -1 : 1); }

// Coordinates of one predicate as integers N_i * 2^E.
template <int K>
struct IntCoords
{
    Dec d[K];
    int emin;
    int width;   // max bit length of |N_i|
};

template <int K>
QDT_HD inline void int_coords(const double* v, IntCoords<K>& c)
{
    c.emin = 1 << 20;
    for (int i = 0; i < K; ++i)
    {
        c.d[i] = decompose(v[i]);
        if (c.d[i].m && c.d[i].e < c.emin) c.emin = c.d[i].e;
    }
    c.width = 0;
    for (int i = 0; i < K; ++i)
    {
        if (!c.d[i].m) continue;
        const int w = bitlen64(c.d[i].m) + (c.d[i].e - c.emin);
        if (w > c.width) c.width = w;
    }
}

template <int K>
QDT_HD __forceinline__ int64_t int_small(const IntCoords<K>& c, int i)
{
    if (!c.d[i].m) return 0;
    const int64_t x = (int64_t)(c.d[i].m << (c.d[i].e - c.emin));
    return c.d[i].neg ? -x : x;
}

// The widest coordinate span a predicate can have: from the top bit of the
// largest double (2^1023 * (2 - 2^-52)) to the lowest bit of the smallest
// subnormal (2^-1074): 2098 bits, 66 limbs.
constexpr int kCoordLimbs = 68;               // a coordinate difference
constexpr int kProdLimbs = 2 * kCoordLimbs + 1;
constexpr int kDetLimbs = 2 * kProdLimbs + 2;

template <int K>
QDT_HD inline void big_coord(BigRef& r, const IntCoords<K>& c, int i)
{
    if (!c.d[i].m)
    {
        r.n = 0;
        r.neg = 0;
        return;
    }
    big_set_shifted(r, c.d[i].m, c.d[i].e - c.emin, c.d[i].neg);
}

// exact sign of (ax-cx)(by-cy) - (ay-cy)(bx-cx); v = {ax, ay, bx, by, cx, cy}
static QDT_HD __noinline__ int orient2d_exact(const double* v)
{
    IntCoords<6> c;
    int_coords<6>(v, c);
    if (c.width <= 62)
    {
        const int64_t ax = int_small(c, 0), ay = int_small(c, 1), bx = int_small(c, 2), by = int_small(c, 3),
                      cx = int_small(c, 4), cy = int_small(c, 5);
        const __int128 l = (__int128)(ax - cx) * (__int128)(by - cy);
        const __int128 r = (__int128)(ay - cy) * (__int128)(bx - cx);
        return l > r ? 1 : (l < r ? -1 : 0);
    }
    uint32_t s0[kCoordLimbs], s1[kCoordLimbs], s2[kCoordLimbs], s3[kCoordLimbs];
    uint32_t p0[kProdLimbs], p1[kProdLimbs];
    BigRef   acx{ s0, 0, 0 }, acy{ s1, 0, 0 }, bcx{ s2, 0, 0 }, bcy{ s3, 0, 0 };
    BigRef   t{ p0, 0, 0 };
    big_coord(acx, c, 0);
    big_coord(t, c, 4);
    big_addsub(acx, acx, t, 1);
    big_coord(acy, c, 1);
    big_coord(t, c, 5);
    big_addsub(acy, acy, t, 1);
    big_coord(bcx, c, 2);
    big_coord(t, c, 4);
    big_addsub(bcx, bcx, t, 1);
    big_coord(bcy, c, 3);
    big_coord(t, c, 5);
    big_addsub(bcy, bcy, t, 1);
    BigRef l{ p0, 0, 0 }, r{ p1, 0, 0 };
    big_mul(l, acx, bcy);
    big_mul(r, acy, bcx);
    big_addsub(l, l, r, 1);
    return big_sign(l);
}

// exact sign of the in-circle determinant; v = {ax, ay, bx, by, cx, cy, dx, dy}
static QDT_HD __noinline__ int incircle_exact(const double* v)
{
    IntCoords<8> c;
    int_coords<8>(v, c);
    if (c.width <= 29)
    {
        // |N| < 2^29: differences < 2^30, lifts < 2^61, cross terms < 2^61,
        // terms < 2^122, sum < 2^124
        const int64_t dx = int_small(c, 6), dy = int_small(c, 7);
        const int64_t adx = int_small(c, 0) - dx, ady = int_small(c, 1) - dy;
        const int64_t bdx = int_small(c, 2) - dx, bdy = int_small(c, 3) - dy;
        const int64_t cdx = int_small(c, 4) - dx, cdy = int_small(c, 5) - dy;
        const int64_t al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
        const int64_t ca = bdx * cdy - cdx * bdy, cb = cdx * ady - adx * cdy, cc = adx * bdy - bdx * ady;
        const __int128 det = (__int128)al * ca + (__int128)bl * cb + (__int128)cl * cc;
        return det > 0 ? 1 : (det < 0 ? -1 : 0);
    }
    uint32_t dxs[6][kCoordLimbs];
    BigRef   D[6];
    uint32_t tl[kCoordLimbs];
    BigRef   t{ tl, 0, 0 };
    for (int i = 0; i < 6; ++i)
    {
        D[i] = BigRef{ dxs[i], 0, 0 };
        big_coord(D[i], c, i);
        big_coord(t, c, 6 + (i & 1));
        big_addsub(D[i], D[i], t, 1);
    }
    // D = {adx, ady, bdx, bdy, cdx, cdy}
    uint32_t lift_l[kProdLimbs + 1], cr_l[kProdLimbs + 1], q0_l[kProdLimbs], q1_l[kProdLimbs];
    uint32_t term_l[kDetLimbs], acc_l[kDetLimbs + 2];
    BigRef   acc{ acc_l, 0, 0 };
    // term k: lift(k) * cross(k), with (k, i, j) in {(a,b,c), (b,c,a), (c,a,b)}
    for (int k = 0; k < 3; ++k)
    {
        const int i = (k + 1) % 3, j = (k + 2) % 3;
        BigRef    lift{ lift_l, 0, 0 }, q0{ q0_l, 0, 0 }, q1{ q1_l, 0, 0 }, cr{ cr_l, 0, 0 }, term{ term_l, 0, 0 };
        big_mul(q0, D[2 * k], D[2 * k]);
        big_mul(q1, D[2 * k + 1], D[2 * k + 1]);
        big_addsub(lift, q0, q1, 0);
        big_mul(q0, D[2 * i], D[2 * j + 1]);
        big_mul(q1, D[2 * j], D[2 * i + 1]);
        big_addsub(cr, q0, q1, 1);
        big_mul(term, lift, cr);
        big_addsub(acc, acc, term, 0);
    }
    return big_sign(acc);
}

// ---------------------------------------------------------------------------
// Single-precision pre-filter
// ---------------------------------------------------------------------------
//
// The FP64 pipe of this GPU issues 2 lanes per cycle per SM (FP32: 128), and
// the merges are chains of dependent predicate evaluations. So every
// predicate first tries a float evaluation with a rigorous error bound; only
// when that cannot decide does it run the reference's double filter, and
// then the exact evaluation. The decision is always the exact sign.
//
// Derivation (forward error analysis, u = 2^-24). The coordinate differences
// X are computed in double (relative error <= 2^-53) and truncated to float
// by integer operations (relative error < 2^-23), so every float difference
// is x = X (1 + t) with |t| <= 2u (1 + 2^-29). Each float product of two
// differences then has relative error <= 5u + O(u^2), a lift (sum of two
// squares) <= 6u, a cross term |C~ - C| <= 5u P + u |C~| with P the sum of
// the two products' magnitudes, a term L C <= 12u L P, and the two final
// additions add <= 2u sum(L P). Hence
//   orient2d: |D~ - D| <= 5u M + u |D~|,   M = |p| + |q|
//   incircle: |D~ - D| <= 15u perm,        perm = sum_k L_k P_k
// (the same permanent as the reference's filter). The filter accepts when
// |D~| > 8u M (orient2d) or |D~| > 24u perm (incircle). Differences outside
// [2^-60, 2^60) (orient2d) or [2^-30, 2^30) (incircle), zero excepted, are
// refused, so no float product overflows and none underflows below the
// normal range by more than the bounds' margin absorbs.

QDT_HD __forceinline__ float f32_bits(uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
#endif
}

// Truncates a double to float with integer operations; clears ok when |v|
// is nonzero and outside [2^emin, 2^(emax+1)).
QDT_HD __forceinline__ float trunc_f32(double v, int emin, int emax, bool& ok)
{
    const uint64_t b = dbits(v);
    const uint64_t mag = b & 0x7FFFFFFFFFFFFFFFull;
    if (mag == 0) return 0.0f;
    const int e = (int)(mag >> 52) - 1023;
    if (e < emin || e > emax) ok = false;
    const uint32_t fb = ((uint32_t)(b >> 63) << 31) | ((uint32_t)(e + 127) << 23) | (uint32_t)((mag >> 29) & 0x7FFFFF);
    return f32_bits(fb);
}

QDT_HD __forceinline__ float fmul_(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
QDT_HD __forceinline__ float fadd_(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
QDT_HD __forceinline__ float fsub_(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

constexpr float kF32Orient = 8.0f * 5.9604644775390625e-08f;     // 8u
constexpr float kF32Incircle = 24.0f * 5.9604644775390625e-08f;  // 24u

// +1 / -1 when decided, 0 otherwise. acx..bcy are the double differences.
QDT_HD __forceinline__ int orient2d_f32(double acx, double acy, double bcx, double bcy)
{
    bool        ok = true;
    const float x1 = trunc_f32(acx, -60, 59, ok), x2 = trunc_f32(acy, -60, 59, ok);
    const float x3 = trunc_f32(bcx, -60, 59, ok), x4 = trunc_f32(bcy, -60, 59, ok);
    const float p = fmul_(x1, x4), q = fmul_(x2, x3);
    const float d = fsub_(p, q);
    const float mag = fadd_(fabsf(p), fabsf(q));
    const float bound = fmul_(kF32Orient, mag);
    if (!ok || !(fabsf(d) > bound)) return 0;
    return d > 0.0f ? 1 : -1;
}

QDT_HD __forceinline__ int incircle_f32(double adx_, double ady_, double bdx_, double bdy_, double cdx_, double cdy_)
{
    bool        ok = true;
    const float adx = trunc_f32(adx_, -30, 29, ok), ady = trunc_f32(ady_, -30, 29, ok);
    const float bdx = trunc_f32(bdx_, -30, 29, ok), bdy = trunc_f32(bdy_, -30, 29, ok);
    const float cdx = trunc_f32(cdx_, -30, 29, ok), cdy = trunc_f32(cdy_, -30, 29, ok);
    const float bc = fmul_(bdx, cdy), cb = fmul_(cdx, bdy);
    const float ca = fmul_(cdx, ady), ac = fmul_(adx, cdy);
    const float ab = fmul_(adx, bdy), ba = fmul_(bdx, ady);
    const float al = fadd_(fmul_(adx, adx), fmul_(ady, ady));
    const float bl = fadd_(fmul_(bdx, bdx), fmul_(bdy, bdy));
    const float cl = fadd_(fmul_(cdx, cdx), fmul_(cdy, cdy));
    const float det = fadd_(fadd_(fmul_(al, fsub_(bc, cb)), fmul_(bl, fsub_(ca, ac))), fmul_(cl, fsub_(ab, ba)));
    const float perm = fadd_(fadd_(fmul_(fadd_(fabsf(bc), fabsf(cb)), al), fmul_(fadd_(fabsf(ca), fabsf(ac)), bl)),
        fmul_(fadd_(fabsf(ab), fabsf(ba)), cl));
    const float bound = fmul_(kF32Incircle, perm);
    if (!ok || !(fabsf(det) > bound)) return 0;
    return det > 0.0f ? 1 : -1;
}

// ---------------------------------------------------------------------------
// Filtered predicates (reference robust.hxx:337-347, :377-396)
// ---------------------------------------------------------------------------

// The double filter and the exact evaluation run only when the single-
// precision filter cannot decide: they are out of line (one copy each), so
// that the code of a merge loop, which calls the predicates from many
// places, stays small enough for the instruction cache.
static QDT_HD __noinline__ int orient2d_slow(double ax, double ay, double bx, double by, double cx, double cy,
    PredCounters* ctr)
{
    const double detleft = mul_rn(sub_rn(ax, cx), sub_rn(by, cy));
    const double detright = mul_rn(sub_rn(ay, cy), sub_rn(bx, cx));
    const double det = sub_rn(detleft, detright);
    const double mag = add_rn(fabs(detleft), fabs(detright));
    const double bound = mul_rn(kErrOrient, mag);
    if ((det > bound || -det > bound) && mag > kFilterFloor) return det > 0 ? 1 : -1;
#ifdef __CUDA_ARCH__
    if (ctr) atomicAdd(&ctr->orient_exact, 1ull);
#else
    if (ctr) ++ctr->orient_exact;
#endif
    const double v[6] = { ax, ay, bx, by, cx, cy };
    return orient2d_exact(v);
}

static QDT_HD __noinline__ int incircle_slow(double ax, double ay, double bx, double by, double cx, double cy,
    double dx, double dy, PredCounters* ctr)
{
    const double adx = sub_rn(ax, dx), ady = sub_rn(ay, dy);
    const double bdx = sub_rn(bx, dx), bdy = sub_rn(by, dy);
    const double cdx = sub_rn(cx, dx), cdy = sub_rn(cy, dy);
    const double bdxcdy = mul_rn(bdx, cdy), cdxbdy = mul_rn(cdx, bdy);
    const double cdxady = mul_rn(cdx, ady), adxcdy = mul_rn(adx, cdy);
    const double adxbdy = mul_rn(adx, bdy), bdxady = mul_rn(bdx, ady);
    const double alift = add_rn(mul_rn(adx, adx), mul_rn(ady, ady));
    const double blift = add_rn(mul_rn(bdx, bdx), mul_rn(bdy, bdy));
    const double clift = add_rn(mul_rn(cdx, cdx), mul_rn(cdy, cdy));
    const double det = add_rn(add_rn(mul_rn(alift, sub_rn(bdxcdy, cdxbdy)),
                                     mul_rn(blift, sub_rn(cdxady, adxcdy))),
        mul_rn(clift, sub_rn(adxbdy, bdxady)));
    const double perm = add_rn(add_rn(mul_rn(add_rn(fabs(bdxcdy), fabs(cdxbdy)), alift),
                                      mul_rn(add_rn(fabs(cdxady), fabs(adxcdy)), blift)),
        mul_rn(add_rn(fabs(adxbdy), fabs(bdxady)), clift));
    const double bound = mul_rn(kErrIncircle, perm);
    if ((det > bound || -det > bound) && perm > kFilterFloor) return det > 0 ? 1 : -1;
#ifdef __CUDA_ARCH__
    if (ctr) atomicAdd(&ctr->incircle_exact, 1ull);
#else
    if (ctr) ++ctr->incircle_exact;
#endif
    const double v[8] = { ax, ay, bx, by, cx, cy, dx, dy };
    return incircle_exact(v);
}

QDT_HD __forceinline__ int orient2d_sign(double ax, double ay, double bx, double by, double cx, double cy,
    PredCounters* ctr = nullptr)
{
    const int s = orient2d_f32(sub_rn(ax, cx), sub_rn(ay, cy), sub_rn(bx, cx), sub_rn(by, cy));
    return s ? s : orient2d_slow(ax, ay, bx, by, cx, cy, ctr);
}

QDT_HD __forceinline__ int incircle_sign(double ax, double ay, double bx, double by, double cx, double cy,
    double dx, double dy, PredCounters* ctr = nullptr)
{
    const int s = incircle_f32(sub_rn(ax, dx), sub_rn(ay, dy), sub_rn(bx, dx), sub_rn(by, dy), sub_rn(cx, dx),
        sub_rn(cy, dy));
    return s ? s : incircle_slow(ax, ay, bx, by, cx, cy, dx, dy, ctr);
}

}  // namespace qdtg
