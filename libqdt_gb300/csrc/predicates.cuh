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

// Counters passed to the predicates: a tagged pointer (bit 0: count calls)
QDT_HD __forceinline__ PredCounters* pc_of(PredCounters* t)
{
    return reinterpret_cast<PredCounters*>(reinterpret_cast<uintptr_t>(t) & ~(uintptr_t)1);
}
QDT_HD __forceinline__ bool pc_counts(const PredCounters* t) { return (reinterpret_cast<uintptr_t>(t) & 1u) != 0; }
// one event per calling lane; on the device one atomic per warp
QDT_HD __forceinline__ void pc_add(unsigned long long* c)
{
#ifdef __CUDA_ARCH__
    const unsigned mask = __activemask();
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) atomicAdd(c, (unsigned long long)__popc(mask));
#else
    ++*c;
#endif
}

// Counting every call takes code at every call site of the merges: only
// kernels built with QDTG_COUNT_CALLS 1 (the single-set build's wide
// variant, which the engine runs when a call counts) have it; elsewhere
// `calls` stays 0 and only the slow paths are counted.
#ifndef QDTG_COUNT_CALLS
#define QDTG_COUNT_CALLS 0
#endif

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

// a = m << sh (m < 2^53), with sign, in at most cap limbs (the limbs past
// cap are zero: the caller sized cap for the value)
QDT_HD inline void big_set_shifted(BigRef& a, uint64_t m, int sh, int neg, int cap)
{
    const int limb = sh >> 5, bit = sh & 31;
    for (int i = 0; i < limb; ++i) a.d[i] = 0;
    // m << bit spans at most 53 + 31 = 84 bits: three limbs
    const uint64_t lo = m << bit;
    const uint64_t hi = bit ? (m >> (64 - bit)) : 0;
    const uint32_t w[3] = { (uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi };
    int            n = limb;
    for (int i = 0; i < 3 && limb + i < cap; ++i) a.d[n++] = w[i];
    a.n = n;
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

// Coordinates of one predicate as integers N_i * 2^E: E (emin) and the
// largest bit length of |N_i| (width); each N_i is formed from its double
// when it is needed (the loops over the coordinates are unrolled, so the
// doubles stay in registers and no per-coordinate table takes stack space).
template <int K>
struct IntCoords
{
    double v[K];
    int    emin;
    int    width;
};

template <int K>
QDT_HD __forceinline__ void int_coords(IntCoords<K>& c)
{
    c.emin = 1 << 20;
#pragma unroll
    for (int i = 0; i < K; ++i)
    {
        const Dec d = decompose(c.v[i]);
        if (d.m && d.e < c.emin) c.emin = d.e;
    }
    c.width = 0;
#pragma unroll
    for (int i = 0; i < K; ++i)
    {
        const Dec d = decompose(c.v[i]);
        if (!d.m) continue;
        const int w = bitlen64(d.m) + (d.e - c.emin);
        if (w > c.width) c.width = w;
    }
}

template <int K>
QDT_HD __forceinline__ int64_t int_small(const IntCoords<K>& c, int i)
{
    const Dec d = decompose(c.v[i]);
    if (!d.m) return 0;
    const int64_t x = (int64_t)(d.m << (d.e - c.emin));
    return d.neg ? -x : x;
}

// The widest coordinate span a predicate can have: from the top bit of the
// largest double (2^1023 * (2 - 2^-52)) to the lowest bit of the smallest
// subnormal (2^-1074): 2098 bits, 66 limbs. Limb counts of the two
// multi-limb tiers: CL limbs hold a coordinate.
template <int CL>
struct Limbs
{
    static constexpr int coord = CL + 1;          // a difference of two CL-limb coordinates
    static constexpr int prod = 2 * coord + 1;    // a product of two differences, a sum of two
    static constexpr int det = 2 * prod + 2;      // a product of two such sums, a sum of three
};
constexpr int kMidLimbs = 3;    // spans of up to 95 bits: circles, clustered and snapped points
constexpr int kWideLimbs = 67;  // any span
constexpr int kMidWidth = 32 * kMidLimbs - 1;

template <int K>
QDT_HD inline void big_coord(BigRef& r, const IntCoords<K>& c, int i, int cap)
{
    const Dec d = decompose(c.v[i]);
    if (!d.m)
    {
        r.n = 0;
        r.neg = 0;
        return;
    }
    big_set_shifted(r, d.m, d.e - c.emin, d.neg, cap);
}

// sign of (ax-cx)(by-cy) - (ay-cy)(bx-cx) in CL-limb arithmetic
template <int CL>
QDT_HD inline int orient2d_limbs(const IntCoords<6>& c)
{
    using L = Limbs<CL>;
    uint32_t s0[L::coord], s1[L::coord], s2[L::coord], s3[L::coord];
    uint32_t p0[L::prod], p1[L::prod];
    BigRef   acx{ s0, 0, 0 }, acy{ s1, 0, 0 }, bcx{ s2, 0, 0 }, bcy{ s3, 0, 0 };
    BigRef   t{ p0, 0, 0 };
    big_coord(acx, c, 0, CL);
    big_coord(t, c, 4, CL);
    big_addsub(acx, acx, t, 1);
    big_coord(acy, c, 1, CL);
    big_coord(t, c, 5, CL);
    big_addsub(acy, acy, t, 1);
    big_coord(bcx, c, 2, CL);
    big_coord(t, c, 4, CL);
    big_addsub(bcx, bcx, t, 1);
    big_coord(bcy, c, 3, CL);
    big_coord(t, c, 5, CL);
    big_addsub(bcy, bcy, t, 1);
    BigRef l{ p0, 0, 0 }, r{ p1, 0, 0 };
    big_mul(l, acx, bcy);
    big_mul(r, acy, bcx);
    big_addsub(l, l, r, 1);
    return big_sign(l);
}

// sign of the in-circle determinant in CL-limb arithmetic
template <int CL>
QDT_HD inline int incircle_limbs(const IntCoords<8>& c)
{
    using L = Limbs<CL>;
    // term_l serves as the scratch of the differences and of the partial
    // products before it holds each term
    uint32_t dxs[6][L::coord];
    uint32_t lift_l[L::prod], cr_l[L::prod];
    uint32_t term_l[L::det], acc_l[L::det + 2];
    BigRef   D[6];
    BigRef   t{ term_l, 0, 0 };
#pragma unroll
    for (int i = 0; i < 6; ++i)
    {
        D[i] = BigRef{ dxs[i], 0, 0 };
        big_coord(D[i], c, i, CL);
        big_coord(t, c, 6 + (i & 1), CL);
        big_addsub(D[i], D[i], t, 1);
    }
    // D = {adx, ady, bdx, bdy, cdx, cdy}; term k: lift(k) * cross(k), with
    // (k, i, j) in {(a,b,c), (b,c,a), (c,a,b)}
    BigRef acc{ acc_l, 0, 0 };
    for (int k = 0; k < 3; ++k)
    {
        const int i = (k + 1) % 3, j = (k + 2) % 3;
        BigRef    lift{ lift_l, 0, 0 }, q{ term_l, 0, 0 }, cr{ cr_l, 0, 0 }, term{ term_l, 0, 0 };
        big_mul(lift, D[2 * k], D[2 * k]);
        big_mul(q, D[2 * k + 1], D[2 * k + 1]);
        big_addsub(lift, lift, q, 0);
        big_mul(cr, D[2 * i], D[2 * j + 1]);
        big_mul(q, D[2 * j], D[2 * i + 1]);
        big_addsub(cr, cr, q, 1);
        big_mul(term, lift, cr);
        big_addsub(acc, acc, term, 0);
    }
    return big_sign(acc);
}

// Device code compiled with QDTG_WIDE_EXACT 0 (the single-set build's
// default kernels) has no room for the widest tier: a predicate whose
// coordinates span more than kMidWidth bits sets `wide` in its counters and
// answers 0, and the engine runs the call again with the kernels built with
// QDTG_WIDE_EXACT 1. That keeps the 67-limb arrays, and the local memory the
// driver reserves for them on every resident thread, out of the kernels that
// run every call.
#ifndef QDTG_WIDE_EXACT
#define QDTG_WIDE_EXACT 1
#endif
#if defined(__CUDA_ARCH__) && !QDTG_WIDE_EXACT
#define QDTG_WIDE_TIER(call)                          \
    do                                                \
    {                                                 \
        if (ctr) atomicOr(&pc_of(ctr)->wide, 1u);     \
        return 0;                                     \
    } while (0)
#else
#define QDTG_WIDE_TIER(call) return call
#endif

// exact sign of (ax-cx)(by-cy) - (ay-cy)(bx-cx); out of line, like the
// filter that calls it, so the merge loops stay small
static QDT_HD __noinline__ int orient2d_exact_sign(double ax, double ay, double bx, double by, double cx, double cy,
    PredCounters* ctr)
{
    IntCoords<6> c{ { ax, ay, bx, by, cx, cy }, 0, 0 };
    int_coords<6>(c);
    if (c.width <= 62)
    {
        const int64_t ax_ = int_small(c, 0), ay_ = int_small(c, 1), bx_ = int_small(c, 2), by_ = int_small(c, 3),
                      cx_ = int_small(c, 4), cy_ = int_small(c, 5);
        const __int128 l = (__int128)(ax_ - cx_) * (__int128)(by_ - cy_);
        const __int128 r = (__int128)(ay_ - cy_) * (__int128)(bx_ - cx_);
        return l > r ? 1 : (l < r ? -1 : 0);
    }
    if (c.width <= kMidWidth) return orient2d_limbs<kMidLimbs>(c);
    QDTG_WIDE_TIER(orient2d_limbs<kWideLimbs>(c));
}

// exact sign of the in-circle determinant of a, b, c, d
static QDT_HD __noinline__ int incircle_exact_sign(double ax, double ay, double bx, double by, double cx, double cy,
    double dx, double dy, PredCounters* ctr)
{
    IntCoords<8> c{ { ax, ay, bx, by, cx, cy, dx, dy }, 0, 0 };
    int_coords<8>(c);
    if (c.width <= 29)
    {
        // |N| < 2^29: differences < 2^30, lifts < 2^61, cross terms < 2^61,
        // terms < 2^122, sum < 2^124
        const int64_t dx_ = int_small(c, 6), dy_ = int_small(c, 7);
        const int64_t adx = int_small(c, 0) - dx_, ady = int_small(c, 1) - dy_;
        const int64_t bdx = int_small(c, 2) - dx_, bdy = int_small(c, 3) - dy_;
        const int64_t cdx = int_small(c, 4) - dx_, cdy = int_small(c, 5) - dy_;
        const int64_t al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
        const int64_t ca = bdx * cdy - cdx * bdy, cb = cdx * ady - adx * cdy, cc = adx * bdy - bdx * ady;
        const __int128 det = (__int128)al * ca + (__int128)bl * cb + (__int128)cl * cc;
        return det > 0 ? 1 : (det < 0 ? -1 : 0);
    }
    if (c.width <= kMidWidth) return incircle_limbs<kMidLimbs>(c);
    QDTG_WIDE_TIER(incircle_limbs<kWideLimbs>(c));
}

// the same on arrays v = {ax, ay, bx, by, cx, cy} / {ax, ..., dy}
QDT_HD inline int orient2d_exact(const double* v, PredCounters* ctr = nullptr)
{
    return orient2d_exact_sign(v[0], v[1], v[2], v[3], v[4], v[5], ctr);
}
QDT_HD inline int incircle_exact(const double* v, PredCounters* ctr = nullptr)
{
    return incircle_exact_sign(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], ctr);
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
    if (pc_counts(ctr)) pc_add(&pc_of(ctr)->f32_undecided[0]);
    const double detleft = mul_rn(sub_rn(ax, cx), sub_rn(by, cy));
    const double detright = mul_rn(sub_rn(ay, cy), sub_rn(bx, cx));
    const double det = sub_rn(detleft, detright);
    const double mag = add_rn(fabs(detleft), fabs(detright));
    const double bound = mul_rn(kErrOrient, mag);
    if ((det > bound || -det > bound) && mag > kFilterFloor) return det > 0 ? 1 : -1;
    if (pc_counts(ctr)) pc_add(&pc_of(ctr)->exact[0]);
    return orient2d_exact_sign(ax, ay, bx, by, cx, cy, ctr);
}

static QDT_HD __noinline__ int incircle_slow(double ax, double ay, double bx, double by, double cx, double cy,
    double dx, double dy, PredCounters* ctr)
{
    if (pc_counts(ctr)) pc_add(&pc_of(ctr)->f32_undecided[1]);
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
    if (pc_counts(ctr)) pc_add(&pc_of(ctr)->exact[1]);
    return incircle_exact_sign(ax, ay, bx, by, cx, cy, dx, dy, ctr);
}

QDT_HD __forceinline__ int orient2d_sign(double ax, double ay, double bx, double by, double cx, double cy,
    PredCounters* ctr = nullptr)
{
    const int s = orient2d_f32(sub_rn(ax, cx), sub_rn(ay, cy), sub_rn(bx, cx), sub_rn(by, cy));
#if QDTG_COUNT_CALLS
    if (pc_counts(ctr)) pc_add(&pc_of(ctr)->calls[0]);
#endif
    return s ? s : orient2d_slow(ax, ay, bx, by, cx, cy, ctr);
}

QDT_HD __forceinline__ int incircle_sign(double ax, double ay, double bx, double by, double cx, double cy,
    double dx, double dy, PredCounters* ctr = nullptr)
{
    const int s = incircle_f32(sub_rn(ax, dx), sub_rn(ay, dy), sub_rn(bx, dx), sub_rn(by, dy), sub_rn(cx, dx),
        sub_rn(cy, dy));
#if QDTG_COUNT_CALLS
    if (pc_counts(ctr)) pc_add(&pc_of(ctr)->calls[1]);
#endif
    return s ? s : incircle_slow(ax, ay, bx, by, cx, cy, dx, dy, ctr);
}

}  // namespace qdtg
