// cr_quant.h -- the loaders' double quantisation of an int32 coordinate,
// evaluated exactly in 64-bit integer arithmetic.
//
// Both GPU builders quantise a LAS integer coordinate X through a chain of
// rounded double operations:
//   p  = RN(X * s)            (s: the header scale)
//   v1 = RN(p + o)            (o: the header offset)
//   v2 = RN(v1 - m1)          (m1: the file's boxMin, or the header min)
//   d  = RN(v2 - m2)          (m2: the batch's AABB min; absent for Morton keys)
//   t  = RN(d / size) * 2^K   (size: the batch extent, or the header cube)
//   q  = clamp(floor(t), 0, qmax)
// LasLoaderSparse.cpp:93-105,146-148 with K = 30 (the 30-bit batch
// coordinates) and Sort_Frugal/src/main.cpp:82-105 with K = 21 (the Morton
// key's cells).  On this GPU every double operation issues at a small
// fraction of the integer rate, which makes both builders FP64-bound.
//
// t is within a small bound E of the real value t* = (X s + o - m1 - m2) 2^K /
// size, which is affine in X: t* = C + dx * A with dx = |X - Xc| for a
// reference coordinate Xc at one end of the X range.  C and A are computed
// once (double-double arithmetic, converted exactly to fixed point with 64
// fraction bits), and per point t* is evaluated with two 32 x 64-bit integer
// products.  When floor(t* - E') and floor(t* + E') clamp to the same integer
// (E' = E plus the fixed-point error) that integer is q; otherwise -- a point
// within about 2^-30 units of a cell boundary, or a setup the bound does not
// cover -- the caller evaluates the double chain itself.
//
// Bound used for E: each RN step errs by at most 2^-53 of its result's
// magnitude, and every intermediate is a monotone function of X, so its
// largest magnitude over [xlo, xhi] is at an end of the range:
//   |t - t*| <= 2^K (2^-52 (P + V1 + V2 + D) / size + 2^-52 D / size)
// with P, V1, V2, D the largest magnitudes of p, v1, v2, d (a factor 2 over
// the 2^-53 rounding bound covers the bound's own evaluation in double).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define CR_QHD __host__ __device__ __forceinline__
#else
#define CR_QHD inline
#endif

namespace cr {

// A signed fixed-point number i + f * 2^-64 (f in [0, 2^64)).
struct Fx {
    int64_t i;
    uint64_t f;
};

CR_QHD Fx fx_add(Fx a, Fx b) {
    Fx r;
    r.f = a.f + b.f;
    r.i = a.i + b.i + (r.f < a.f ? 1 : 0);
    return r;
}

CR_QHD uint64_t double_bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
#endif
}

// x as a fixed-point number, truncated toward zero to a multiple of 2^-64.
// Requires a finite |x| < 2^62.
CR_QHD Fx fx_of(double x) {
    const uint64_t bits = double_bits(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    uint64_t m = bits & ((1ull << 52) - 1);
    int e2 = -1074;  // subnormal: x = m 2^-1074
    if (ex != 0) {
        m |= 1ull << 52;
        e2 = ex - 1075;
    }
    uint64_t ip = 0, fp = 0;
    if (m != 0) {
        if (e2 >= 0) {
            ip = m << e2;  // |x| < 2^62 keeps e2 <= 9
        } else {
            const int sh = -e2;
            if (sh < 64) {
                ip = m >> sh;
                fp = m << (64 - sh);
            } else if (sh < 128) {
                fp = m >> (sh - 64);
            }
        }
    }
    Fx r;
    if (bits >> 63) {
        r.i = fp ? -(int64_t)ip - 1 : -(int64_t)ip;
        r.f = 0 - fp;
    } else {
        r.i = (int64_t)ip;
        r.f = fp;
    }
    return r;
}

// Error-free transformations (Knuth's TwoSum; the product's error by fma).
CR_QHD void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
CR_QHD void two_prod(double a, double b, double& p, double& e) {
    p = a * b;
    e = fma(a, b, -p);
}

struct QuantFx {
    Fx c;              // t* at X = xc
    uint64_t a_i, a_f; // A = |s| 2^K / size >= 0, integer part and fraction
    uint64_t e;        // E', in 2^-64 units
    int32_t xc;
    int32_t neg;       // dx = neg ? xc - X : X - xc, in [0, 2^32) over the range
    int32_t ok;        // 0: the bound does not cover this setup; use the double chain
    int32_t pad;
};

// The double chain itself (the reference's arithmetic, no contraction).
CR_QHD double quant_chain_d(int32_t X, double s, double o, double m1, double m2, bool has_m2) {
    const double p = (double)X * s;
    const double v1 = p + o;
    const double v2 = v1 - m1;
    return has_m2 ? v2 - m2 : v2;
}

CR_QHD double fabs_q(double x) { return x < 0.0 ? -x : x; }
CR_QHD bool finite_q(double x) { return x - x == 0.0; }

// Setup for X in [xlo, xhi].  ok = 0 where the fast path would not be exact
// by the bound above (size zero, subnormal or not finite, a result range
// beyond the fixed-point format, or E' >= 2^-6).
CR_QHD QuantFx quant_setup(double s, double o, double m1, double m2, bool has_m2, double size, int K,
                           int32_t xlo, int32_t xhi) {
    QuantFx q;
    q.c.i = 0;
    q.c.f = 0;
    q.a_i = q.a_f = 0;
    q.e = 0;
    q.xc = s < 0.0 ? xhi : xlo;
    q.neg = s < 0.0 ? 1 : 0;
    q.ok = 0;
    q.pad = 0;
    if (!(size >= 0x1p-1000) || !finite_q(size) || !finite_q(s) || !finite_q(o) || !finite_q(m1) ||
        (has_m2 && !finite_q(m2)) || xlo > xhi)
        return q;
    const double scaleK = (double)(1ll << K);
    // Largest magnitudes of the intermediates, at the ends of the range.
    double P = 0.0, V1 = 0.0, V2 = 0.0, D = 0.0;
    const int32_t ends[2] = {xlo, xhi};
    for (int k = 0; k < 2; k++) {
        const double p = (double)ends[k] * s;
        const double v1 = p + o;
        const double v2 = v1 - m1;
        const double d = has_m2 ? v2 - m2 : v2;
        P = fmax(P, fabs_q(p));
        V1 = fmax(V1, fabs_q(v1));
        V2 = fmax(V2, fabs_q(v2));
        D = fmax(D, fabs_q(d));
    }
    const double u2 = 0x1p-52;
    double E = scaleK * (u2 * (P + V1 + V2 + (has_m2 ? D : 0.0)) / size + u2 * D / size);
    // C = (xc s + o - m1 - m2) 2^K / size in double-double.
    double S, lo, e1, e2, e3 = 0.0;
    two_prod((double)q.xc, s, S, lo);
    two_sum(S, o, S, e1);
    two_sum(S, -m1, S, e2);
    if (has_m2) two_sum(S, -m2, S, e3);
    lo = lo + e1 + e2 + e3;
    const double c1 = S / size;
    const double c2 = (fma(-c1, size, S) + lo) / size;
    // A = |s| 2^K / size in double-double.
    const double as = fabs_q(s);
    const double a1 = as / size;
    const double a2 = fma(-a1, size, as) / size;
    const double C1 = c1 * scaleK, C2 = c2 * scaleK, A1 = a1 * scaleK, A2 = a2 * scaleK;
    if (!finite_q(C1) || !finite_q(A1) || !(fabs_q(C1) < 0x1p60) || !(A1 < 0x1p30)) return q;
    // The double-double results and their conversions: the neglected terms
    // (lo's rounding, c2 / a2 rounding) are below 2^-100 of the terms'
    // magnitudes; each conversion truncates by less than 2^-64, times the
    // largest dx (< 2^32) for A.
    const double terms = fabs_q((double)q.xc * s) + fabs_q(o) + fabs_q(m1) + (has_m2 ? fabs_q(m2) : 0.0);
    E += scaleK * 0x1p-100 * terms / size + 0x1p-100 * (fabs_q(C1) + A1 * 0x1p32) + 0x1p-30;
    E = E * 1.25;
    if (!(E < 0x1p-6)) return q;
    q.c = fx_add(fx_of(C1), fx_of(C2));
    Fx a = fx_add(fx_of(A1), fx_of(A2));
    if (a.i < 0) a.i = 0, a.f = 0;  // A is within 2^-63 of zero
    // Every t* of the range: |C| + 2^32 (A + 1) must stay inside int64.
    if (a.i >= (1ll << 30)) return q;
    q.a_i = (uint64_t)a.i;
    q.a_f = a.f;
    q.e = (uint64_t)ldexp(E, 64) + 1;
    q.ok = 1;
    return q;
}

// The quantised value for X in the setup's range: true and *out when the
// bound decides it, false when the caller must evaluate the double chain.
CR_QHD bool quant_fast(const QuantFx& q, int32_t X, uint32_t qmax, uint32_t* out) {
    const uint32_t dx = q.neg ? (uint32_t)((int64_t)q.xc - X) : (uint32_t)((int64_t)X - q.xc);
    // dx * a_f as a 96-bit value: hi:lo
    const uint64_t p0 = (uint64_t)dx * (uint32_t)q.a_f;
    const uint64_t p1 = (uint64_t)dx * (q.a_f >> 32);
    const uint64_t mid = p1 + (p0 >> 32);
    const uint64_t lo = (mid << 32) | (uint32_t)p0;
    const uint64_t hi = mid >> 32;
    const uint64_t f = q.c.f + lo;
    const int64_t i = q.c.i + (int64_t)((uint64_t)dx * q.a_i + hi) + (f < lo ? 1 : 0);
    const int64_t il = i - (f < q.e ? 1 : 0);
    const uint64_t fu = f + q.e;
    const int64_t iu = i + (fu < f ? 1 : 0);
    const int64_t cl = il < 0 ? 0 : (il > (int64_t)qmax ? (int64_t)qmax : il);
    const int64_t cu = iu < 0 ? 0 : (iu > (int64_t)qmax ? (int64_t)qmax : iu);
    *out = (uint32_t)cl;
    return q.ok && cl == cu;
}

}  // namespace cr
