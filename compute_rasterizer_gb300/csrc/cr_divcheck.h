// Quotients for the self-check of the literal pair body's division
// (f2_neg_div_rn in cr_device.cuh): the numerators that cr_check_reciprocal
// divides by every float x with |x| in [2^-64, 2^64), and the rule that a
// result must meet.  Shared by the device check and its host test
// (tests/cpp/div_check.cpp), so that both draw the same quotients.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define CR_DC __host__ __device__ __forceinline__
#else
#define CR_DC inline
#endif

namespace cr {

CR_DC uint64_t divcheck_hash(uint32_t i) {  // splitmix64's finaliser
    uint64_t z = (uint64_t)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

CR_DC float divcheck_bits(uint32_t u) {
    union { uint32_t u; float f; } v;
    v.u = u;
    return v.f;
}

// The product of two floats, rounded once (a single multiply: no contraction
// can apply, and the callers' products are exact or rounded alike anywhere).
CR_DC float divcheck_mul(float a, float b) { return a * b; }

// A numerator for the divisor with bit pattern xb (|x| in [2^-64, 2^64)).
// hard, when x's significand X (24 bits) is odd: a = A 2^s with
// A 2^25 = X M + t, where M = -t X^-1 mod 2^25 and t is odd with |t| < 32, so
// that a / |x| = (M + t / X) 2^(k-24) lies within |t| / (2X) < 2^-18 ulp of
// M 2^(k-24), a rounding midpoint (M odd, 25 bits) or a float (M < 2^24), for
// k drawn in [-27, 1].  Otherwise a = RN(|x| r) with r random, exponent in
// [-30, 3], so a / x covers both sides of every test the raster makes.
CR_DC float divcheck_numerator(uint32_t xb, bool hard) {
    const uint64_t h = divcheck_hash(xb);
    const uint32_t X = (xb & 0x7FFFFFu) | 0x800000u;
    const int ex = (int)((xb >> 23) & 0xFFu) - 127;
    if (hard && (X & 1u)) {
        uint32_t inv = X;  // X^-1 mod 2^32: each Newton step doubles the correct low bits
        for (int s = 0; s < 5; s++) inv *= 2u - X * inv;
        const int32_t t = 2 * (int32_t)(h & 31u) - 31;
        const uint32_t M = ((uint32_t)(-t) * inv) & 0x1FFFFFFu;
        const uint64_t A = (uint64_t)((int64_t)((uint64_t)X * M) + t) >> 25;
        const int k = -27 + (int)((h >> 40) % 29u);
        // a = A 2^(ex + k - 22): A < 2^24 is exact, the power of two is normal
        return divcheck_mul((float)(uint32_t)A, divcheck_bits((uint32_t)(127 + ex + k - 22) << 23));
    }
    const int er = -30 + (int)((h >> 40) % 34u);
    const float r = divcheck_bits(((uint32_t)(127 + er) << 23) | ((uint32_t)(h >> 9) & 0x7FFFFFu));
    return divcheck_mul(divcheck_bits(xb & 0x7FFFFFFFu), r);
}

// Whether nq (a negated quotient from f2_neg_div_rn) meets q = RN(a / x): the
// same bits (negated) where |q| is in [2^-27, 2]; above 2, outside [-1, 1]
// (a NaN counts as outside); below 2^-27, under 2^-25 in magnitude.
CR_DC bool divcheck_quotient_ok(float q, float nq) {
    union { float f; uint32_t u; } a, b;
    a.f = q;
    b.f = nq;
    const float aq = q < 0.0f ? -q : q, anq = nq < 0.0f ? -nq : nq;
    if (aq >= 0x1p-27f && aq <= 2.0f) return b.u == (a.u ^ 0x80000000u);
    if (aq > 2.0f) return !(anq <= 1.0f);
    return anq < 0x1p-25f;
}

}  // namespace cr
