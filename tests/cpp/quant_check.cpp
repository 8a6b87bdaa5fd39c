// Checks the integer evaluation of the loaders' double quantisation
// (compute_rasterizer_gb300/csrc/cr_quant.h) against the double chain it
// stands for, on the setups the two GPU builders make: per-batch encoder
// boxes (K = 30, LasLoaderSparse.cpp:93-105,146-148) and the Morton cube over
// the whole int32 range (K = 21, Sort_Frugal/src/main.cpp:82-105).  Points
// are drawn uniformly and next to the cell boundaries (where the fast path
// must defer to the chain).  Built with contraction off; exits 1 on the first
// disagreement.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "../../compute_rasterizer_gb300/csrc/cr_quant.h"

namespace {

uint64_t g_state = 0x9E3779B97F4A7C15ull;
uint64_t next_u64() {
    uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uni() { return (double)(next_u64() >> 11) * 0x1p-53; }
int64_t irange(int64_t a, int64_t b) { return a + (int64_t)(next_u64() % (uint64_t)(b - a + 1)); }

// the reference's truncation: encoder (NaN -> 0, then min) and Morton forms
uint32_t trunc_encode(double t, uint32_t qmax) {
    const uint32_t u = (t != t) ? 0u : (t < 0.0 ? 0u : (t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t));
    return u < qmax ? u : qmax;
}

struct Counts {
    long long checked = 0, fast = 0;
};

bool check_point(const cr::QuantFx& q, int32_t X, double s, double o, double m1, double m2, bool has_m2,
                 double size, int K, Counts& c) {
    const uint32_t qmax = (uint32_t)((1ll << K) - 1);
    const double d = cr::quant_chain_d(X, s, o, m1, m2, has_m2);
    const double t = (d / size) * (double)(1ll << K);
    const uint32_t want = trunc_encode(t, qmax);
    uint32_t got = 0;
    c.checked++;
    if (cr::quant_fast(q, X, qmax, &got)) {
        c.fast++;
        if (got != want) {
            std::printf("MISMATCH K=%d X=%d s=%.17g o=%.17g m1=%.17g m2=%.17g size=%.17g t=%.17g want=%u got=%u\n",
                        K, X, s, o, m1, m2, size, t, want, got);
            return false;
        }
    }
    return true;
}

// X values with t* near the boundary of cell j (and a few neighbours)
template <typename F>
bool near_boundaries(const cr::QuantFx& q, int32_t xlo, int32_t xhi, double s, double o, double m1, double m2,
                     bool has_m2, double size, int K, int tries, Counts& c, F&& pick_cell) {
    const double A = std::fabs(s) * std::ldexp(1.0, K) / size;
    const double C = (double)q.c.i + std::ldexp((double)q.c.f, -64);
    for (int r = 0; r < tries; r++) {
        const double j = pick_cell();
        if (!(A > 0.0)) break;
        const double dxr = (j - C) / A;
        if (!(dxr > -4.0 && dxr < 4294967300.0)) continue;
        const int64_t dx0 = (int64_t)std::floor(dxr);
        for (int64_t dd = -2; dd <= 2; dd++) {
            const int64_t dx = dx0 + dd;
            const int64_t X = q.neg ? (int64_t)q.xc - dx : (int64_t)q.xc + dx;
            if (X < xlo || X > xhi) continue;
            if (!check_point(q, (int32_t)X, s, o, m1, m2, has_m2, size, K, c)) return false;
        }
    }
    return true;
}

double pick_scale() {
    static const double scales[] = {0.001, 0.01, 0.0001, 0.00025, 0.1, 1.0, 1e-7, 0.5, 0.003};
    double s = scales[next_u64() % 9];
    if (next_u64() % 4 == 0) s = std::ldexp(uni() + 0.5, -(int)(next_u64() % 30));
    if (next_u64() % 6 == 0) s = -s;
    return s;
}
double pick_offset() {
    switch (next_u64() % 5) {
        case 0: return 0.0;
        case 1: return std::floor(uni() * 1e6);            // UTM easting
        case 2: return std::floor(uni() * 1e7);            // UTM northing
        case 3: return (uni() - 0.5) * 2e5;
        default: return (uni() - 0.5) * 10.0;
    }
}

// encoder: one batch box per setup, the box and size as k_encode computes them
bool encode_cases(int setups, Counts& c) {
    for (int n = 0; n < setups; n++) {
        const double s = pick_scale(), o = pick_offset();
        const int64_t span = (int64_t)1 << (next_u64() % 32);
        int64_t lo = irange(INT32_MIN, (int64_t)INT32_MAX - span);
        int64_t hi = lo + irange(0, span);
        if (next_u64() % 8 == 0) hi = lo;  // a flat batch: size 0 on this axis
        // boxMin: the file's, at or below the smallest coordinate (a whole-file value)
        const double vlo_raw = (double)lo * s + o, vhi_raw = (double)hi * s + o;
        const double bm = std::fmin(vlo_raw, vhi_raw) - (next_u64() % 3 == 0 ? 0.0 : uni() * 1e3);
        const double vlo = (double)lo * s + o - bm, vhi = (double)hi * s + o - bm;
        const double b0 = s < 0.0 ? vhi : vlo, b1 = s < 0.0 ? vlo : vhi;
        const double size = b1 - b0;
        const cr::QuantFx q = cr::quant_setup(s, o, bm, b0, true, size, 30, (int32_t)lo, (int32_t)hi);
        for (int r = 0; r < 64; r++)
            if (!check_point(q, (int32_t)irange(lo, hi), s, o, bm, b0, true, size, 30, c)) return false;
        if (!check_point(q, (int32_t)lo, s, o, bm, b0, true, size, 30, c)) return false;
        if (!check_point(q, (int32_t)hi, s, o, bm, b0, true, size, 30, c)) return false;
        if (!near_boundaries(q, (int32_t)lo, (int32_t)hi, s, o, bm, b0, true, size, 30, 64, c,
                             [] { return (double)irange(0, (1ll << 30)); }))
            return false;
    }
    return true;
}

// Morton: the header min and the largest extent, the whole int32 range
bool morton_cases(int setups, Counts& c) {
    for (int n = 0; n < setups; n++) {
        const double s = pick_scale(), o = pick_offset();
        const int64_t span = (int64_t)1 << (1 + next_u64() % 31);
        const int64_t lo = irange(INT32_MIN, (int64_t)INT32_MAX - span), hi = lo + span;
        const double a = (double)lo * s + o, b = (double)hi * s + o;
        double mn = std::fmin(a, b), mx = std::fmax(a, b);
        if (next_u64() % 3 == 0) mn -= uni() * (mx - mn) * 0.1;  // a header box wider than the points
        double cube = mx - mn;
        if (next_u64() % 4 == 0) cube *= 1.0 + 3.0 * uni();      // another axis is the largest
        const cr::QuantFx q = cr::quant_setup(s, o, mn, 0.0, false, cube, 21, INT32_MIN, INT32_MAX);
        for (int r = 0; r < 64; r++)
            if (!check_point(q, (int32_t)irange(lo, hi), s, o, mn, 0.0, false, cube, 21, c)) return false;
        for (int r = 0; r < 8; r++)  // outside the header box too
            if (!check_point(q, (int32_t)irange(INT32_MIN, INT32_MAX), s, o, mn, 0.0, false, cube, 21, c))
                return false;
        if (!check_point(q, INT32_MIN, s, o, mn, 0.0, false, cube, 21, c)) return false;
        if (!check_point(q, INT32_MAX, s, o, mn, 0.0, false, cube, 21, c)) return false;
        if (!near_boundaries(q, INT32_MIN, INT32_MAX, s, o, mn, 0.0, false, cube, 21, 64, c,
                             [] { return (double)irange(0, (1ll << 21)); }))
            return false;
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    const int setups = argc > 1 ? std::atoi(argv[1]) : 20000;
    Counts ce, cm;
    if (!encode_cases(setups, ce) || !morton_cases(setups, cm)) return 1;
    std::printf("encode checked %lld fast %lld; morton checked %lld fast %lld\n", ce.checked, ce.fast,
                cm.checked, cm.fast);
    return 0;
}
