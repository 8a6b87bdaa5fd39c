// cr_device.cuh -- device helpers shared by the kernel files: the float
// helpers of the arithmetic contract, the per-batch cull and precision-level
// math (render.cs:130-231), the per-CTA z-cache and the per-point projection.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "cr_internal.h"

namespace cr {
namespace {

// Launches `k` and returns 0 when the launch itself was accepted.  The launch's
// own status is checked, so an error left behind by other work in the
// process is neither reported nor cleared here.
template <typename... KArgs, typename... Args>
int launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = s;
    return cudaLaunchKernelEx(&cfg, k, static_cast<Args&&>(args)...) == cudaSuccess ? 0 : -1;
}

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kNoPixel = 0xFFFFFFFFu;

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// float(x) for the 10-bit coordinates, exact.  The hardware conversion runs
// on the conversion pipe, which the raster leaves mostly idle; it measured
// faster than the two-instruction float trick on the issue-bound raster.
__device__ __forceinline__ float small_u2f(uint32_t x) { return __uint2float_rn(x); }
// int(f) by truncation, for the pixel coordinate (f >= 0 for every point
// inside the view; the value of an outside point is never used).
__device__ __forceinline__ int32_t small_f2i(float f) { return __float2int_rz(f); }

__device__ __forceinline__ uint4 ld_stream(const uint4* p) {
    uint4 r;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p));
    return r;
}

__device__ __forceinline__ uint32_t lane_id() {
    uint32_t l;
    asm("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

__device__ __forceinline__ uint32_t u4get(const uint4& v, int j) {
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// 1 / x, correctly rounded to nearest: the value __frcp_rn(x) returns, for
// every x.  For |x| in [2^-126, 2^126) (reciprocal and every intermediate
// normal) it takes one Newton-Raphson step from the hardware approximation
// rcp.approx (at most 1 ulp off): the residual e = 1 - x*y is exact as one
// FMA, and y + e*y rounds to the correctly rounded reciprocal (Markstein,
// "Computation of elementary functions on the IBM RISC System/6000 processor",
// IBM J. Res. Dev. 34(1), 1990).  Every other x (zero, subnormal, huge, inf,
// NaN) goes to __frcp_rn.  cr_check_reciprocal compares the two over all 2^32
// inputs.  Measured 1.6 % faster than __frcp_rn alone on the raster.
// rcp_rn_normal: the Newton step alone, for callers that guarantee |x| in
// [2^-126, 2^126) (the paired path: batches whose every w is proven to lie in
// [2^-120, 2^120], see w_safe); without the range test and the __frcp_rn
// call the raster measured 3-11 % faster.
__device__ __forceinline__ float rcp_rn_normal(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    const float e = __fmaf_rn(-x, y, 1.0f);
    return __fmaf_rn(e, y, y);
}
__device__ __forceinline__ float rcp_rn(float x) {
    float r = rcp_rn_normal(x);
    if (((__float_as_uint(x) & 0x7FFFFFFFu) - 0x00800000u) >= 0x7E000000u) r = __frcp_rn(x);
    return r;
}

// Whether the clip w = fma(T11, z, fma(T7, y, fma(T3, x, T15))) of every point
// decoded from a batch lies in [lo_bound, hi_bound] (by default [2^-120, 2^120];
// T column-major, the w row is T[3], T[7], T[11], T[15]).  w is linear, so over
// the AABB its extremes are at corners; decoded points stay within a few ulps of
// the AABB and each operation rounds once (the FMAs here, or the shaders' own
// products and sums), so a computed w differs from the corner range by far less
// than 2^-16 of the largest term sum, the margin taken here.  The extents must be
// finite: with an infinite one the decode step is infinite and a decoded
// coordinate (so w) can be infinite although every corner is finite.  A NaN
// or infinite corner value fails the test.
__device__ __forceinline__ bool w_safe(const float* T, float mnx, float mny, float mnz, float mxx,
                                       float mxy, float mxz, float lo_bound = 0x1p-120f,
                                       float hi_bound = 0x1p120f) {
    if (!isfinite(fsub(mxx, mnx)) || !isfinite(fsub(mxy, mny)) || !isfinite(fsub(mxz, mnz)))
        return false;
    float lo = 0.0f, hi = 0.0f, mag = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float x = (k & 1) ? mxx : mnx, y = (k & 2) ? mxy : mny, z = (k & 4) ? mxz : mnz;
        const float w = __fmaf_rn(T[11], z, __fmaf_rn(T[7], y, __fmaf_rn(T[3], x, T[15])));
        const float m = fadd(fadd(fadd(fabsf(fmul(T[3], x)), fabsf(fmul(T[7], y))),
                                  fabsf(fmul(T[11], z))), fabsf(T[15]));
        lo = k == 0 ? w : fminf(lo, w);
        hi = k == 0 ? w : fmaxf(hi, w);
        mag = fmaxf(mag, m);
    }
    const float err = fmul(mag, 0x1p-16f);
    return fsub(lo, err) >= lo_bound && fadd(hi, err) <= hi_bound;
}

// ---- per-batch math (render.cs:130-231), no contraction --------------------

__device__ bool intersects_frustum(const float* pl, float mnx, float mny, float mnz, float mxx,
                                   float mxy, float mxz) {
#pragma unroll 1
    for (int i = 0; i < 6; i++) {
        float nx = pl[4 * i + 0], ny = pl[4 * i + 1], nz = pl[4 * i + 2], c = pl[4 * i + 3];
        float vx = nx > 0.0f ? mxx : mnx;
        float vy = ny > 0.0f ? mxy : mny;
        float vz = nz > 0.0f ? mxz : mnz;
        float d = fadd(fadd(fadd(fmul(nx, vx), fmul(ny, vy)), fmul(nz, vz)), c);
        if (d < 0.0f) return false;
    }
    return true;
}

// literal (CR_QUIRK_LITERAL_ARITH): glm's association, (m0 x + m1 y) + (m2 z + m3 w)
__device__ void mat4_vec4(const float* m, const float v[4], float o[4], bool literal = false) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
        if (literal) {
            o[r] = fadd(fadd(fmul(m[r], v[0]), fmul(m[4 + r], v[1])),
                        fadd(fmul(m[8 + r], v[2]), fmul(m[12 + r], v[3])));
            continue;
        }
        float s = fmul(m[r], v[0]);
        s = fadd(s, fmul(m[4 + r], v[1]));
        s = fadd(s, fmul(m[8 + r], v[2]));
        s = fadd(s, fmul(m[12 + r], v[3]));
        o[r] = s;
    }
}

// lvl4_px: the pixel size below which a batch is level 4 (render.cs:217 100,
// compute_loop_nodes/render.cs:199 80)
__device__ int precision_level(const float* P, const float* VW, int32_t W, int32_t H, float mnx,
                               float mny, float mnz, float mxx, float mxy, float mxz,
                               float lvl4_px = 100.0f, bool literal = false) {
    float c[4] = {__fdiv_rn(fadd(mnx, mxx), 2.0f), __fdiv_rn(fadd(mny, mxy), 2.0f),
                  __fdiv_rn(fadd(mnz, mxz), 2.0f), 1.0f};
    float dx = fsub(mnx, mxx), dy = fsub(mny, mxy), dz = fsub(mnz, mxz);
    float radius = __fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
    float vc[4], ve[4], pc[4], pe[4];
    mat4_vec4(VW, c, vc, literal);
    ve[0] = fadd(vc[0], radius);
    ve[1] = fadd(vc[1], 0.0f);
    ve[2] = fadd(vc[2], 0.0f);
    ve[3] = fadd(vc[3], 0.0f);
    mat4_vec4(P, vc, pc, literal);
    mat4_vec4(P, ve, pe, literal);
    // render.cs:210-211 `xy / w`: one correctly rounded reciprocal per vector
    // (literal: a division per component)
    float pcx, pcy, pex, pey;
    if (literal) {
        pcx = __fdiv_rn(pc[0], pc[3]); pcy = __fdiv_rn(pc[1], pc[3]);
        pex = __fdiv_rn(pe[0], pe[3]); pey = __fdiv_rn(pe[1], pe[3]);
    } else {
        const float rc = rcp_rn(pc[3]), re = rcp_rn(pe[3]);
        pcx = fmul(pc[0], rc); pcy = fmul(pc[1], rc);
        pex = fmul(pe[0], re); pey = fmul(pe[1], re);
    }
    float Wf = (float)W, Hf = (float)H;
    float scx = __fdiv_rn(fmul(Wf, fadd(pcx, 1.0f)), 2.0f);
    float scy = __fdiv_rn(fmul(Hf, fadd(pcy, 1.0f)), 2.0f);
    float sex = __fdiv_rn(fmul(Wf, fadd(pex, 1.0f)), 2.0f);
    float sey = __fdiv_rn(fmul(Hf, fadd(pey, 1.0f)), 2.0f);
    float ex = fsub(sex, scx), ey = fsub(sey, scy);
    float px = __fsqrt_rn(fadd(fmul(ex, ex), fmul(ey, ey)));
    if (px < lvl4_px) return 4;
    if (px < 200.0f) return 3;
    if (px < 500.0f) return 2;
    if (px < 10000.0f) return 1;
    return 0;
}

// Points a batch's loop visits, from its first point: num_points (+1 with the
// inclusive end), at most 10,240; with CR_QUIRK_NODE_LOOP the loop of
// compute_loop_nodes/render.cs:296-300 (min(ceil(n/128), 500) + 4 iterations
// of uvec4 per thread, 4 at a time: nodes of up to 64,512 points).
__device__ __forceinline__ int64_t points_in_batch(int32_t num_points, int32_t first_point,
                                                   int32_t quirks) {
    int64_t n = num_points;
    if (quirks & CR_QUIRK_NODE_LOOP) {
        if (n < 0) return 0;
        const int64_t loop = min((n + 127) / 128, (int64_t)500);
        const int64_t reach = 512 * ((loop + 4) / 4) - (first_point & 3);
        return min(n, reach);
    }
    if (quirks & CR_QUIRK_INCLUSIVE_END) n += 1;
    if (n > kPointsPerBatch) n = kPointsPerBatch;
    return n < 0 ? 0 : n;
}

struct BatchCtx {
    float mnx, mny, mnz;
    float sx, sy, sz;
    float T0, T1, T3, T4, T5, T7, T8, T9, T11, T12, T13, T15;
    float Wf, Hf;
    int32_t W;
};

// Per-CTA early-z cache in shared memory: a direct-mapped table (slot: the
// tag's low bits for one view, a Fibonacci hash of the tag for several) of
// words `depth << 32 | tag`, where the tag names one
// framebuffer word (the pixel id; with several views, the view's word offset
// plus the pixel id).  Every depth stored is one this CTA submitted to the
// framebuffer during the frame, so it is never below the word's final minimum
// depth: a point deeper than the cached depth cannot win and is dropped
// without touching global memory.  Entries are single 64-bit words, so a racing
// writer replaces an entry but never tears one; the table starts empty (tag
// 0xFFFFFFFF).
constexpr int kZCacheBits = 11;
constexpr int kZCacheSlots = 1 << kZCacheBits;

__device__ __forceinline__ uint32_t zslot(uint32_t tag) {
    return (tag * 2654435761u) >> (32 - kZCacheBits);
}
// Single-view slots: a CTA's batch covers a compact screen region, whose pixel
// ids already differ in their low bits (measured faster than the hash there;
// the multi-view tags, offset per view, keep the hash).
__device__ __forceinline__ uint32_t zslot_pixel(uint32_t pix) { return pix & (kZCacheSlots - 1); }

// Writes one point's contribution.  All 32 lanes of the warp call run()
// together (inactive lanes with ok = false).
template <int MODE>
struct Emit;

// Submits `key` for the framebuffer word `g` (cache tag `tag`) and records
// the key's depth as the word's upper bound in the cache: after the atomic the
// word holds at most `key`.  A cache miss goes straight to the atomic (a
// fire-and-forget RED): reading the word first to skip the atomic for a point
// behind it measured 4 % slower on the single-view raster and 9 % on the
// multi-view one, the read's latency costing more than the extra REDs.
template <typename T>
__device__ __forceinline__ void submit_min(T* g, unsigned long long* zc, uint32_t slot,
                                           uint32_t tag, T key, uint32_t depth_of_key) {
    atomicMin(g, key);
    zc[slot] = ((unsigned long long)depth_of_key << 32) | tag;
}

__device__ __forceinline__ bool zcache_rejects(const unsigned long long* zc, uint32_t slot,
                                               uint32_t tag, uint32_t wbits) {
    const unsigned long long e = zc[slot];
    return (uint32_t)e == tag && wbits > (uint32_t)(e >> 32);
}

// Clip-space position of a decoded point (render.cs:399-401).  LIT
// (CR_QUIRK_LITERAL_ARITH): `transform * vec4(p, 1.0)` with glm's
// association, (T0 x + T4 y) + (T8 z + T12 * 1), each operation rounded.
template <bool LIT = false>
__device__ __forceinline__ void project_clip(const BatchCtx& c, float x, float y, float z,
                                             float& px, float& py, float& pw) {
    if (LIT) {
        px = fadd(fadd(fmul(c.T0, x), fmul(c.T4, y)), fadd(fmul(c.T8, z), fmul(c.T12, 1.0f)));
        py = fadd(fadd(fmul(c.T1, x), fmul(c.T5, y)), fadd(fmul(c.T9, z), fmul(c.T13, 1.0f)));
        pw = fadd(fadd(fmul(c.T3, x), fmul(c.T7, y)), fadd(fmul(c.T11, z), fmul(c.T15, 1.0f)));
        return;
    }
    px = __fmaf_rn(c.T8, z, __fmaf_rn(c.T4, y, __fmaf_rn(c.T0, x, c.T12)));
    py = __fmaf_rn(c.T9, z, __fmaf_rn(c.T5, y, __fmaf_rn(c.T1, x, c.T13)));
    pw = __fmaf_rn(c.T11, z, __fmaf_rn(c.T7, y, __fmaf_rn(c.T3, x, c.T15)));
}

// Divide, inside test and pixel (render.cs:402-409).  SAFE: the caller
// guarantees w in [2^-120, 2^120] (w_safe), so the reciprocal needs no range
// test.
template <bool SAFE = false, bool LIT = false>
__device__ __forceinline__ bool project_finish(const BatchCtx& c, float px, float py, float pw,
                                               int32_t& pix, uint32_t& wbits) {
    // render.cs:402 `pos.xyz / pos.w`: one correctly rounded reciprocal of w
    // (LIT: a division per component)
    float qx, qy;
    if (LIT) {
        qx = __fdiv_rn(px, pw);
        qy = __fdiv_rn(py, pw);
    } else {
        const float rw = SAFE ? rcp_rn_normal(pw) : rcp_rn(pw);
        qx = fmul(px, rw);
        qy = fmul(py, rw);
    }
    // render.cs:404 written positively, so a NaN position is outside (the
    // negated form would keep it and index the framebuffer with garbage); in
    // w-safe batches w >= 2^-120 at every point, so w > 0 needs no test
    bool in = (SAFE || pw > 0.0f) && qx >= -1.0f && qx <= 1.0f && qy >= -1.0f && qy <= 1.0f;
    // qx * 0.5 is exact (or, below 2^-125, far under half an ulp of 0.5), so
    // the fused form rounds as render.cs:406's product then sum does
    int32_t ix = small_f2i(fmul(__fmaf_rn(qx, 0.5f, 0.5f), c.Wf));
    int32_t iy = small_f2i(fmul(__fmaf_rn(qy, 0.5f, 0.5f), c.Hf));
    pix = ix + iy * c.W;
    wbits = __float_as_uint(pw);
    return in;
}

// Project a decoded point (render.cs:399-409 under the arithmetic contract,
// or as written with LIT).
template <bool SAFE = false, bool LIT = false>
__device__ __forceinline__ bool project(const BatchCtx& c, float x, float y, float z, int32_t& pix,
                                        uint32_t& wbits) {
    float px, py, pw;
    project_clip<LIT>(c, x, y, z, px, py, pw);
    return project_finish<SAFE, LIT>(c, px, py, pw, pix, wbits);
}

// ---- packed fp32 pairs ------------------------------------------------------
//
// fma.rn.f32x2 / mul.rn.f32x2 (sm_100 family) do two IEEE single-precision
// operations, each rounded on its own exactly like __fmaf_rn / __fmul_rn, in
// one instruction.  Two points of a lane go through the decode and the
// projection side by side, which halves those float instructions on the
// issue-bound raster without changing a bit of any result.  The uniforms the
// pairs need are (u, u) for each uniform u.  A file's transform is proj * view
// * translate(boxMin): its columns 0-2 are proj * view's, computed by the same
// operations on the same operands for every file, so the nine pairs of those
// columns are the same for all files and sit in the kernel parameters
// (constant-bank operands, no registers); only column 3 (T12, T13, T15)
// belongs to the batch's file and is held in registers per batch.
struct PairParams {
    uint64_t T[9];          // (T[k], T[k]) for T0, T1, T3, T4, T5, T7, T8, T9, T11
    uint64_t half, Wf, Hf;  // (0.5, 0.5), (W, W), (H, H)
    uint64_t bias;          // (-2^23, -2^23)
    uint64_t one, nhalf;    // (1, 1), (-0.5, -0.5)
};
struct PairCol3 {
    uint64_t T12, T13, T15;  // the batch's file's translation column, as pairs
};

__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
    uint64_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// -RN(1/w) for both elements of a pair, |w| in [2^-126, 2^126): the Newton
// step of rcp_rn_normal done once for the pair.  NY holds the approximations
// of -1/w (rcp.approx of -w); E = fma(w, NY, 1) = 1 - w*y is exact, and
// fma(E, NY, NY) = -(y + E*y) rounds to -RN(1/w), rounding to nearest being
// symmetric.  The negated result spares negating a pair (the callers fold the
// sign into their next operation); cr_check_reciprocal runs this form against
// __frcp_rn over every float in the range.  On the raster (1B points):
// index payload 1.408 -> 1.353 ms, HQS 3.425 -> 3.334 ms, color 1.562 -> 1.554 ms.
__device__ __forceinline__ uint64_t f2_neg_rcp_rn_normal(uint64_t W, uint64_t one) {
    float w0, w1, n0, n1;
    f2_unpack(W, w0, w1);
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(n0) : "f"(-w0));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(n1) : "f"(-w1));
    const uint64_t NY = f2_pack(n0, n1);
    return f2_fma(f2_fma(W, NY, one), NY, NY);
}

// -RN(a / w) for both elements of a pair, from NR = -RN(1/w), by Markstein's
// method (IBM J. Res. Dev. 34(1), 1990, cited at rcp_rn_normal).  The product
// q0 = a * y (y = RN(1/w)) lies within 1.5 ulp of a/w; one correction
// q1 = q0 + (a - q0 w) y brings it within 1 ulp (the residual's own rounding
// is far below that), and Markstein's theorem makes the second,
// q2 = RN(q1 + (a - q1 w) y), equal to RN(a/w): y is within half an ulp of
// 1/w, q1 within 1 ulp of a/w, and the residual a - q1 w is exact.  Each
// residual is one FMA.  Holds for w in [2^-64, 2^64] wherever RN(a/w) lies in
// [2^-27, 2] in magnitude: every value is then normal and the residual's
// exact value sits on a grid of at least 2^-137.  Outside that interval the
// callers' tests come out the same way: |q2| > 1 (or NaN, when a * y
// overflows) where |a/w| > 2, and |q2| < 2^-25 where |a/w| < 2^-27, so that
// q * 0.5 + 0.5 rounds to 0.5 for both.  Negated like NR: NQ = -q at every
// step, E = fma(NQ, w, a) = a - q w, fma(E, NR, NQ) = -(q + E y).
// cr_check_reciprocal compares it with __fdiv_rn on 2^32 quotients, a
// quarter of them within 2^-18 ulp of a rounding midpoint or of a float
// (cr_divcheck.h).
__device__ __forceinline__ uint64_t f2_neg_div_rn(uint64_t A, uint64_t W, uint64_t NR) {
    const uint64_t NQ0 = f2_mul(A, NR);
    const uint64_t NQ1 = f2_fma(f2_fma(NQ0, W, A), NR, NQ0);
    return f2_fma(f2_fma(NQ1, W, A), NR, NQ1);
}

// a + b element by element as two scalar single-precision sums (see
// project_pair10's literal body).
__device__ __forceinline__ uint64_t f2_add_scalar(uint64_t a, uint64_t b) {
    float a0, a1, b0, b1;
    f2_unpack(a, a0, a1);
    f2_unpack(b, b0, b1);
    return f2_pack(fadd(a0, b0), fadd(a1, b1));
}

// A batch's 10-bit decode uniforms as pairs (per batch, in registers): the
// steps sx, sy * 2^-10, sz * 2^-20 and the minimum corner (see project_pair10).
struct PairBatch {
    uint64_t sx, sy, sz, mnx, mny, mnz;
};
__device__ __forceinline__ PairBatch pair_batch(const BatchCtx& c) {
    const float sy = fmul(c.sy, 0x1p-10f), sz = fmul(c.sz, 0x1p-20f);
    return PairBatch{f2_pack(c.sx, c.sx), f2_pack(sy, sy), f2_pack(sz, sz),
                     f2_pack(c.mnx, c.mnx), f2_pack(c.mny, c.mny), f2_pack(c.mnz, c.mnz)};
}
// Whether sy * 2^-10 and sz * 2^-20 are exact (no underflow: steps of at least
// 2^-106, or zero, or infinite); batches where they are not take the scalar body.
__device__ __forceinline__ bool pair_batch_exact(const BatchCtx& c) {
    return fmul(fmul(c.sy, 0x1p-10f), 0x1p10f) == c.sy &&
           fmul(fmul(c.sz, 0x1p-20f), 0x1p20f) == c.sz;
}

// project_finish() for two points: clip positions (PX, PY, PW) as pairs.  The
// pair quotients come out negated (NQ = -q, from -RN(1/w)): the inside test is
// symmetric, and q * 0.5 + 0.5 is the same real value as NQ * -0.5 + 0.5, so
// every result is the scalar path's.  LIT: a correctly rounded division per
// component (f2_neg_div_rn) for the one reciprocal.
template <bool LIT = false>
__device__ __forceinline__ void project_pair_finish(uint64_t PX, uint64_t PY, uint64_t PW,
                                                    const PairParams& pp, int32_t W, bool ok[2],
                                                    int32_t pix[2], uint32_t wbits[2]) {
    // callers: w-safe batches only (every w in [2^-120, 2^120]; with LIT in
    // [2^-64, 2^64])
    const uint64_t NR = f2_neg_rcp_rn_normal(PW, pp.one);
    const uint64_t NQX = LIT ? f2_neg_div_rn(PX, PW, NR) : f2_mul(PX, NR);
    const uint64_t NQY = LIT ? f2_neg_div_rn(PY, PW, NR) : f2_mul(PY, NR);
    const uint64_t FX = f2_mul(f2_fma(NQX, pp.nhalf, pp.half), pp.Wf);
    const uint64_t FY = f2_mul(f2_fma(NQY, pp.nhalf, pp.half), pp.Hf);
    float pw[2], nqx[2], nqy[2], fx[2], fy[2];
    f2_unpack(PW, pw[0], pw[1]);
    f2_unpack(NQX, nqx[0], nqx[1]);
    f2_unpack(NQY, nqy[0], nqy[1]);
    f2_unpack(FX, fx[0], fx[1]);
    f2_unpack(FY, fy[0], fy[1]);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        // w >= 2^-120 for every point of a w-safe batch: render.cs:404's w > 0
        // holds, so only the x and y bounds are tested (HQS 3.334 -> 3.281 ms)
        ok[k] = nqx[k] >= -1.0f && nqx[k] <= 1.0f && nqy[k] >= -1.0f && nqy[k] <= 1.0f;
        pix[k] = small_f2i(fx[k]) + small_f2i(fy[k]) * W;
        wbits[k] = __float_as_uint(pw[k]);
    }
}

// Two 10-bit points (words a0, a1) through decode_point<2> and project(), as
// pairs: the same operations in the same order, element by element.  The
// integer fields reach the decode FMA as floats without shifts: x as the
// float 2^23 + x (x in the mantissa's low bits) minus 2^23, y as 2^23 + y*2^10
// minus 2^23, z as float(word & 0x3FF00000) = z*2^20, every value exact.  y
// and z then meet the steps sy*2^-10 and sz*2^-20, whose products with them
// are the same real numbers y*sy and z*sz, so each FMA rounds exactly as
// fma(float(y), sy, min_y) does (measured 1.6 % faster on the color raster,
// 3.9 % on the index one, than shift, mask and convert per field).
// LIT (CR_QUIRK_LITERAL_ARITH): the operations the shaders write, element by
// element as project<true, true> does them: the decode as product then sum,
// transform * vec4(p, 1) as (T0 x + T4 y) + (T8 z + T12), and a division per
// component.  The products run as pairs and the sums that take a product as
// scalars: the toolchain contracts a packed product into the packed sum that
// consumes it (the results came out 1 ulp off), while it leaves scalar sums
// of a packed product's halves alone.  The outer sum of a row adds two sums
// and runs as a pair.
template <bool LIT = false>
__device__ __forceinline__ void project_pair10(const PairParams& pp, const PairCol3& f,
                                               const PairBatch& b, int32_t W, uint32_t a0,
                                               uint32_t a1, bool ok[2], int32_t pix[2],
                                               uint32_t wbits[2]) {
    const uint64_t XF = f2_add(f2_pack(__uint_as_float((a0 & 0x3FFu) | 0x4B000000u),
                                       __uint_as_float((a1 & 0x3FFu) | 0x4B000000u)), pp.bias);
    const uint64_t YF = f2_add(f2_pack(__uint_as_float((a0 & 0xFFC00u) | 0x4B000000u),
                                       __uint_as_float((a1 & 0xFFC00u) | 0x4B000000u)), pp.bias);
    const uint64_t ZF =
        f2_pack(__uint2float_rn(a0 & 0x3FF00000u), __uint2float_rn(a1 & 0x3FF00000u));
    // project_clip: T0 T1 T3 T4 T5 T7 T8 T9 T11 are pp.T[0..8]
    if (LIT) {
        const uint64_t X = f2_add_scalar(f2_mul(XF, b.sx), b.mnx);
        const uint64_t Y = f2_add_scalar(f2_mul(YF, b.sy), b.mny);
        const uint64_t Z = f2_add_scalar(f2_mul(ZF, b.sz), b.mnz);
        const uint64_t PX = f2_add(f2_add_scalar(f2_mul(pp.T[0], X), f2_mul(pp.T[3], Y)),
                                   f2_add_scalar(f2_mul(pp.T[6], Z), f.T12));
        const uint64_t PY = f2_add(f2_add_scalar(f2_mul(pp.T[1], X), f2_mul(pp.T[4], Y)),
                                   f2_add_scalar(f2_mul(pp.T[7], Z), f.T13));
        const uint64_t PW = f2_add(f2_add_scalar(f2_mul(pp.T[2], X), f2_mul(pp.T[5], Y)),
                                   f2_add_scalar(f2_mul(pp.T[8], Z), f.T15));
        project_pair_finish<true>(PX, PY, PW, pp, W, ok, pix, wbits);
        return;
    }
    const uint64_t X = f2_fma(XF, b.sx, b.mnx);
    const uint64_t Y = f2_fma(YF, b.sy, b.mny);
    const uint64_t Z = f2_fma(ZF, b.sz, b.mnz);
    const uint64_t PX = f2_fma(pp.T[6], Z, f2_fma(pp.T[3], Y, f2_fma(pp.T[0], X, f.T12)));
    const uint64_t PY = f2_fma(pp.T[7], Z, f2_fma(pp.T[4], Y, f2_fma(pp.T[1], X, f.T13)));
    const uint64_t PW = f2_fma(pp.T[8], Z, f2_fma(pp.T[5], Y, f2_fma(pp.T[2], X, f.T15)));
    project_pair_finish(PX, PY, PW, pp, W, ok, pix, wbits);
}

// Host side: the pair uniforms of a view (file 0's columns 0-2, which every
// file shares).
inline void fill_pair_params(const ViewParams& vp, PairParams* pp) {
    auto dup = [](float f) {
        uint32_t u;
        __builtin_memcpy(&u, &f, 4);
        return ((uint64_t)u << 32) | u;
    };
    static const int kIdx[9] = {0, 1, 3, 4, 5, 7, 8, 9, 11};
    for (int k = 0; k < 9; k++) pp->T[k] = dup(vp.files[0].T[kIdx[k]]);
    pp->half = dup(0.5f);
    pp->bias = dup(-8388608.0f);
    pp->Wf = dup((float)vp.W);
    pp->Hf = dup((float)vp.H);
    pp->one = dup(1.0f);
    pp->nhalf = dup(-0.5f);
}

}  // namespace
}  // namespace cr
