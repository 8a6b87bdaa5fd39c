// cr_kernels.cu -- sm_103a kernels of the point-rasterizer hot path.
//
// Compiled with -fmad=false: every fused multiply-add below is an explicit
// __fmaf_rn, every other float operation rounds on its own, scalar / and sqrt
// are IEEE (__fdiv_rn, __fsqrt_rn), and a vector divided by a scalar is a
// multiplication by the scalar's correctly rounded reciprocal (__frcp_rn), the
// one reciprocal a shader compiler emits for it.  The operation order follows
// the arithmetic contract the oracle states, which is what makes the
// framebuffers bit-exact.
//
// Kernels
//   k_cull      one thread per batch record: validation, frustum cull
//               (render.cs:176-197), precision level (render.cs:199-231);
//               appends (batch | level << 29) to a work list.
//   k_batched   persistent CTAs pull work items; per batch the points are read
//               with 128-bit streaming loads (4 consecutive points per lane,
//               the loop_las2 `uvec4` scheme), decoded at 10/20/30 bit,
//               projected, tested against a per-CTA shared-memory z-cache,
//               and the survivors issue 64-bit atomicMin (render.cs:399-432).
//               The same body runs the HQS depth pass (u32 atomicMin,
//               hqs/depth.cs) and color pass (__match_any_sync partitioned
//               sums + two 64-bit atomicAdd per pixel, hqs/color.cs:388-444).
//   k_plain     16 B/point path (compute_2021_earlyz/render.cs:35-74).
//   k_resolve_* per-pixel resolves (resolve.cs files), optionally re-clearing.
#include <cuda_runtime.h>

#include <cstdint>

#include "cr_internal.h"

namespace cr {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kNoPixel = 0xFFFFFFFFu;

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// float(x) for x < 2^23, exact: the bit pattern 2^23 + x minus 2^23.
__device__ __forceinline__ float small_u2f(uint32_t x) {
    return __fsub_rn(__uint_as_float(x | 0x4B000000u), 8388608.0f);
}
// int(f) for 0 <= f < 2^22 (truncation): add 2^23 rounding toward zero.
__device__ __forceinline__ int32_t small_f2i(float f) {
    return __float_as_int(__fadd_rz(f, 8388608.0f)) - 0x4B000000;
}

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

__device__ void mat4_vec4(const float* m, const float v[4], float o[4]) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
        float s = fmul(m[r], v[0]);
        s = fadd(s, fmul(m[4 + r], v[1]));
        s = fadd(s, fmul(m[8 + r], v[2]));
        s = fadd(s, fmul(m[12 + r], v[3]));
        o[r] = s;
    }
}

__device__ int precision_level(const float* P, const float* VW, int32_t W, int32_t H, float mnx,
                               float mny, float mnz, float mxx, float mxy, float mxz) {
    float c[4] = {__fdiv_rn(fadd(mnx, mxx), 2.0f), __fdiv_rn(fadd(mny, mxy), 2.0f),
                  __fdiv_rn(fadd(mnz, mxz), 2.0f), 1.0f};
    float dx = fsub(mnx, mxx), dy = fsub(mny, mxy), dz = fsub(mnz, mxz);
    float radius = __fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
    float vc[4], ve[4], pc[4], pe[4];
    mat4_vec4(VW, c, vc);
    ve[0] = fadd(vc[0], radius);
    ve[1] = fadd(vc[1], 0.0f);
    ve[2] = fadd(vc[2], 0.0f);
    ve[3] = fadd(vc[3], 0.0f);
    mat4_vec4(P, vc, pc);
    mat4_vec4(P, ve, pe);
    // render.cs:210-211 `xy / w`: one correctly rounded reciprocal per vector
    const float rc = __frcp_rn(pc[3]), re = __frcp_rn(pe[3]);
    float pcx = fmul(pc[0], rc), pcy = fmul(pc[1], rc);
    float pex = fmul(pe[0], re), pey = fmul(pe[1], re);
    float Wf = (float)W, Hf = (float)H;
    float scx = __fdiv_rn(fmul(Wf, fadd(pcx, 1.0f)), 2.0f);
    float scy = __fdiv_rn(fmul(Hf, fadd(pcy, 1.0f)), 2.0f);
    float sex = __fdiv_rn(fmul(Wf, fadd(pex, 1.0f)), 2.0f);
    float sey = __fdiv_rn(fmul(Hf, fadd(pey, 1.0f)), 2.0f);
    float ex = fsub(sex, scx), ey = fsub(sey, scy);
    float px = __fsqrt_rn(fadd(fmul(ex, ex), fmul(ey, ey)));
    if (px < 100.0f) return 4;
    if (px < 200.0f) return 3;
    if (px < 500.0f) return 2;
    if (px < 10000.0f) return 1;
    return 0;
}

__device__ __forceinline__ int64_t points_in_batch(int32_t num_points, int32_t quirks) {
    int64_t n = num_points;
    if (quirks & CR_QUIRK_INCLUSIVE_END) n += 1;
    if (n > kPointsPerBatch) n = kPointsPerBatch;
    return n < 0 ? 0 : n;
}

// ---- cull + level: one thread per batch record -----------------------------

__global__ void __launch_bounds__(256) k_cull(ViewParams vp, const cr_batch* __restrict__ batches,
                                              int64_t nb, int64_t capacity, int32_t quirks,
                                              uint32_t* __restrict__ scratch) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    uint32_t item = 0;
    if (b < nb) {
        const int4* r4 = reinterpret_cast<const int4*>(batches + b);
        int4 a = __ldg(r4), c = __ldg(r4 + 1), d = __ldg(r4 + 2);
        float mnx = __int_as_float(a.y), mny = __int_as_float(a.z), mnz = __int_as_float(a.w);
        float mxx = __int_as_float(c.x), mxy = __int_as_float(c.y), mxz = __int_as_float(c.z);
        int32_t np = c.w, fp = d.x, fi = d.y;
        int64_t count = points_in_batch(np, quirks);
        bool ok = np >= 0 && np <= kPointsPerBatch && fp >= 0 &&
                  (int64_t)fp + count + 4 <= capacity && fi >= 0 && fi < vp.nfiles;
        if (!ok) {
            atomicOr(&scratch[kErrWord], kErrBadBatch);
        } else if (count > 0) {
            const FileRec& f = vp.files[fi];
            bool vis = !vp.culling || intersects_frustum(f.planes, mnx, mny, mnz, mxx, mxy, mxz);
            if (vis) {
                int level = precision_level(vp.P, f.VW, vp.W, vp.H, mnx, mny, mnz, mxx, mxy, mxz);
                keep = true;
                item = (uint32_t)b | ((uint32_t)level << 29);
            }
        }
    }
    uint32_t m = __ballot_sync(kFull, keep);
    if (m) {
        uint32_t lane = lane_id();
        uint32_t leader = __ffs(m) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&scratch[kItemCount], __popc(m));
        base = __shfl_sync(kFull, base, leader);
        if (keep) scratch[kScratchHead + base + __popc(m & ((1u << lane) - 1u))] = item;
    }
}

// ---- batched raster / HQS body ---------------------------------------------

struct BatchCtx {
    float mnx, mny, mnz;
    float sx, sy, sz;
    float T0, T1, T3, T4, T5, T7, T8, T9, T11, T12, T13, T15;
    float Wf, Hf;
    int32_t W;
};

// Early-z reads of the framebuffer go through L1 and may return a stale copy
// of a word; within a frame every word only decreases, so a stale value is
// never below the current one: a point it rejects is rejected by the current
// value too, and a point it passes goes on to the atomic, which decides.
__device__ __forceinline__ unsigned long long ld_cached_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.global.ca.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ld_cached_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.global.ca.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// Per-CTA early-z cache in shared memory: a direct-mapped table (Fibonacci
// hash of the pixel id) of words `depth << 32 | pixel`.  Every depth stored is
// one this CTA submitted to, or read from, the framebuffer during the frame, so
// it is never below the pixel's final minimum depth: a point deeper than the
// cached depth of its pixel cannot win and is dropped without touching global
// memory.  Entries are single 64-bit words, so a racing writer replaces an
// entry but never tears one; the table starts empty (pixel 0xFFFFFFFF).
constexpr int kZCacheBits = 11;
constexpr int kZCacheSlots = 1 << kZCacheBits;

__device__ __forceinline__ uint32_t zslot(int32_t pix) {
    return ((uint32_t)pix * 2654435761u) >> (32 - kZCacheBits);
}

// Writes one point's contribution.  All 32 lanes of the warp call run()
// together (inactive lanes with ok = false).  Points that survive the early-z
// test are merged per pixel inside the warp (__match_any_sync, then a min or
// sum reduction over the peers), and one leader per pixel issues the atomic.
template <int MODE>
struct Emit;

// Leader side of the raster / depth passes: submit `key` for `pix` and record
// the pixel's new upper bound in the cache.  On a cache miss the framebuffer
// word is read first (a possibly stale L1 copy, which is still an upper bound)
// so that a point behind the stored minimum issues no atomic.
template <typename T>
__device__ __forceinline__ void submit_min(T* gslot, unsigned long long* zc, uint32_t slot,
                                           int32_t pix, T key, uint32_t depth_of_key);

template <>
__device__ __forceinline__ void submit_min<unsigned long long>(unsigned long long* g,
                                                               unsigned long long* zc,
                                                               uint32_t slot, int32_t pix,
                                                               unsigned long long key,
                                                               uint32_t kd) {
    const unsigned long long e = zc[slot];
    uint32_t bound = kd;
    if ((uint32_t)e == (uint32_t)pix) {
        atomicMin(g, key);
    } else {
        const unsigned long long cur = ld_cached_u64(g);
        if (key < cur) atomicMin(g, key);
        else bound = (uint32_t)(cur >> 32);
    }
    zc[slot] = ((unsigned long long)bound << 32) | (uint32_t)pix;
}

template <>
__device__ __forceinline__ void submit_min<uint32_t>(uint32_t* g, unsigned long long* zc,
                                                     uint32_t slot, int32_t pix, uint32_t key,
                                                     uint32_t kd) {
    const unsigned long long e = zc[slot];
    uint32_t bound = kd;
    if ((uint32_t)e == (uint32_t)pix) {
        atomicMin(g, key);
    } else {
        const uint32_t cur = ld_cached_u32(g);
        if (key < cur) atomicMin(g, key);
        else bound = cur;
    }
    zc[slot] = ((unsigned long long)bound << 32) | (uint32_t)pix;
}

__device__ __forceinline__ bool zcache_rejects(const unsigned long long* zc, uint32_t slot,
                                               int32_t pix, uint32_t wbits) {
    const unsigned long long e = zc[slot];
    return (uint32_t)e == (uint32_t)pix && wbits > (uint32_t)(e >> 32);
}

// The raster and depth passes merge same-pixel candidates through the CTA's
// z-cache rather than with __match_any_sync: a warp vote skips the atomic path
// when no lane survives the cache test, and each surviving lane submits its
// own 64-bit (or 32-bit) atomic min.  Measured on 1B points, a match-and-reduce
// merge in front of the atomics made the frame 6-11% slower at every
// threshold tried.
template <>
struct Emit<kModeRaster> {
    static __device__ __forceinline__ void run(const BatchedLaunch& bl, unsigned long long* zc,
                                               bool ok, int32_t pix, uint32_t wbits,
                                               uint32_t payload, uint32_t) {
        const uint32_t slot = zslot(pix);
        // render.cs:423-424 early depth test, against the CTA's cache
        const bool cand = ok && !zcache_rejects(zc, slot, pix, wbits);
        if (__any_sync(kFull, cand) && cand)
            submit_min<unsigned long long>(reinterpret_cast<unsigned long long*>(bl.fb) + pix, zc,
                                           slot, pix, ((unsigned long long)wbits << 32) | payload,
                                           wbits);
    }
};

template <>
struct Emit<kModeHqsDepth> {
    static __device__ __forceinline__ void run(const BatchedLaunch& bl, unsigned long long* zc,
                                               bool ok, int32_t pix, uint32_t wbits, uint32_t,
                                               uint32_t) {
        const uint32_t slot = zslot(pix);
        // hqs/depth.cs:375-379
        const bool cand = ok && !zcache_rejects(zc, slot, pix, wbits);
        if (__any_sync(kFull, cand) && cand)
            submit_min<uint32_t>(bl.depth + pix, zc, slot, pix, wbits, wbits);
    }
};

template <>
struct Emit<kModeHqsColor> {
    static __device__ __forceinline__ void run(const BatchedLaunch& bl, unsigned long long*,
                                               bool ok, int32_t pix, uint32_t wbits, uint32_t,
                                               uint32_t color) {
        bool vis = false;
        if (ok) {
            // the depth buffer is read-only during this pass
            const uint32_t d = __ldg(bl.depth + pix);
            // color.cs:399-403: depth <= bufferDepth * 1.01
            vis = __uint_as_float(wbits) <= fmul(__uint_as_float(d), 1.01f);
        }
        if (__any_sync(kFull, vis)) {
            // color.cs:408-441: partitioned sums of (R, G, B, 1), leader adds
            const uint32_t peers = __match_any_sync(kFull, vis ? (uint32_t)pix : kNoPixel);
            if (vis) {
                const uint32_t rg = (color & 0xFFu) | (((color >> 8) & 0xFFu) << 16);
                const uint32_t bc = ((color >> 16) & 0xFFu) | (1u << 16);
                const uint32_t srg = __reduce_add_sync(peers, rg);
                const uint32_t sbc = __reduce_add_sync(peers, bc);
                if (lane_id() == (uint32_t)(__ffs(peers) - 1)) {
                    unsigned long long* a =
                        reinterpret_cast<unsigned long long*>(bl.accum) + 2 * (int64_t)pix;
                    atomicAdd(a, (unsigned long long)(srg & 0xFFFFu) |
                                     ((unsigned long long)(srg >> 16) << 32));
                    atomicAdd(a + 1, (unsigned long long)(sbc & 0xFFFFu) |
                                         ((unsigned long long)(sbc >> 16) << 32));
                }
            }
        }
    }
};

// Project a decoded point (render.cs:399-409 under the arithmetic contract).
__device__ __forceinline__ bool project(const BatchCtx& c, float x, float y, float z, int32_t& pix,
                                        uint32_t& wbits) {
    float px = __fmaf_rn(c.T8, z, __fmaf_rn(c.T4, y, __fmaf_rn(c.T0, x, c.T12)));
    float py = __fmaf_rn(c.T9, z, __fmaf_rn(c.T5, y, __fmaf_rn(c.T1, x, c.T13)));
    float pw = __fmaf_rn(c.T11, z, __fmaf_rn(c.T7, y, __fmaf_rn(c.T3, x, c.T15)));
    // render.cs:402 `pos.xyz / pos.w`: one correctly rounded reciprocal of w
    const float rw = __frcp_rn(pw);
    float qx = fmul(px, rw), qy = fmul(py, rw);
    // render.cs:404 written positively, so a NaN position is outside (the
    // negated form would keep it and index the framebuffer with garbage)
    bool in = pw > 0.0f && qx >= -1.0f && qx <= 1.0f && qy >= -1.0f && qy <= 1.0f;
    int32_t ix = small_f2i(fmul(__fmaf_rn(qx, 0.5f, 0.5f), c.Wf));
    int32_t iy = small_f2i(fmul(__fmaf_rn(qy, 0.5f, 0.5f), c.Hf));
    pix = ix + iy * c.W;
    wbits = __float_as_uint(pw);
    return in;
}

// LC: 2 = 10 bit (levels 2-4), 1 = 20 bit (level 1), 0 = 30 bit (level 0).
// Points [first, first + count) are read as 128-bit vectors starting at the
// aligned word below `first`; lanes mask the words outside the range.  The
// next vector is loaded before the current one is processed.
template <int MODE, int PAYLOAD, int BLOCK, int LC>
__device__ __forceinline__ void run_points(const BatchedLaunch& bl, unsigned long long* zc,
                                           const BatchCtx& c, int64_t first, int32_t count,
                                           bool l0_x12) {
    constexpr bool kNeedColor = (MODE == kModeHqsColor) || (MODE == kModeRaster && PAYLOAD == CR_PAYLOAD_COLOR);
    const int64_t v0 = first >> 2;
    const int32_t head = (int32_t)(first & 3);
    const int nv = (head + count + 3) >> 2;
    const uint32_t index0 = (uint32_t)(first - head);  // global index of word 0 of vector v0
    const uint4* lo4 = reinterpret_cast<const uint4*>(bl.lo) + v0;
    const uint4* md4 = reinterpret_cast<const uint4*>(bl.md) + v0;
    const uint4* hi4 = reinterpret_cast<const uint4*>(bl.hi) + v0;
    const uint4* co4 = reinterpret_cast<const uint4*>(bl.rgba) + v0;
    const uint4 zero = make_uint4(0, 0, 0, 0);
    uint4 n4 = zero, n8 = zero, n12 = zero, ncol = zero;
    if ((int)threadIdx.x < nv) {
        n4 = ld_stream(lo4 + threadIdx.x);
        if (LC <= 1) n8 = ld_stream(md4 + threadIdx.x);
        if (LC == 0) n12 = ld_stream(hi4 + threadIdx.x);
        if (kNeedColor) ncol = ld_stream(co4 + threadIdx.x);
    }
    for (int base = 0; base < nv; base += BLOCK) {
        const int v = base + (int)threadIdx.x;
        const uint4 w4 = n4, w8 = n8, w12 = n12, col = ncol;
        const int vn = v + BLOCK;
        if (vn < nv) {
            n4 = ld_stream(lo4 + vn);
            if (LC <= 1) n8 = ld_stream(md4 + vn);
            if (LC == 0) n12 = ld_stream(hi4 + vn);
            if (kNeedColor) ncol = ld_stream(co4 + vn);
        }
        const int32_t rel0 = 4 * v - head;  // batch-local index of word 0
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const bool valid = (uint32_t)(rel0 + j) < (uint32_t)count;
            const uint32_t idx = index0 + 4u * (uint32_t)v + (uint32_t)j;
            const uint32_t a = u4get(w4, j);
            float x, y, z;
            if (LC == 2) {
                x = __fmaf_rn(small_u2f(a & 1023u), c.sx, c.mnx);
                y = __fmaf_rn(small_u2f((a >> 10) & 1023u), c.sy, c.mny);
                z = __fmaf_rn(small_u2f((a >> 20) & 1023u), c.sz, c.mnz);
            } else {
                const uint32_t b = u4get(w8, j);
                uint32_t X = ((a & 1023u) << 20) | ((b & 1023u) << 10);
                uint32_t Y = (((a >> 10) & 1023u) << 20) | (((b >> 10) & 1023u) << 10);
                uint32_t Z = (((a >> 20) & 1023u) << 20) | (((b >> 20) & 1023u) << 10);
                if (LC == 0) {
                    const uint32_t h = u4get(w12, j);
                    uint32_t x12 = h & 1023u, y12 = (h >> 10) & 1023u, z12 = (h >> 20) & 1023u;
                    if (l0_x12) { y12 = x12; z12 = x12; }
                    X |= x12; Y |= y12; Z |= z12;
                }
                x = __fmaf_rn(__uint2float_rn(X), c.sx, c.mnx);
                y = __fmaf_rn(__uint2float_rn(Y), c.sy, c.mny);
                z = __fmaf_rn(__uint2float_rn(Z), c.sz, c.mnz);
            }
            int32_t pix;
            uint32_t wbits;
            const bool ok = project(c, x, y, z, pix, wbits) && valid;
            const uint32_t color = kNeedColor ? u4get(col, j) : 0u;
            const uint32_t payload = (PAYLOAD == CR_PAYLOAD_COLOR) ? color : (uint32_t)idx;
            Emit<MODE>::run(bl, zc, ok, pix, wbits, payload, color);
        }
    }
}

template <int MODE, int PAYLOAD, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_batched(ViewParams vp, BatchedLaunch bl) {
    __shared__ uint32_t s_item[2];
    __shared__ unsigned long long s_zc[MODE == kModeHqsColor ? 1 : kZCacheSlots];
    uint32_t* cursor = bl.scratch + (MODE == kModeHqsColor ? kCursor1 : kCursor0);
    const uint32_t nitems = *reinterpret_cast<volatile uint32_t*>(bl.scratch + kItemCount);
    if (MODE != kModeHqsColor)
        for (int i = threadIdx.x; i < kZCacheSlots; i += BLOCK) s_zc[i] = 0xFFFFFFFFull;
    if (threadIdx.x == 0) s_item[0] = atomicAdd(cursor, 1u);
    __syncthreads();
    int buf = 0;
    while (true) {
        const uint32_t wi = s_item[buf];
        if (wi >= nitems) break;
        if (threadIdx.x == 0) s_item[buf ^ 1] = atomicAdd(cursor, 1u);
        const uint32_t item = bl.scratch[kScratchHead + wi];
        const uint32_t b = item & 0x1FFFFFFFu;
        const int level = (int)(item >> 29);

        const int4* r4 = reinterpret_cast<const int4*>(bl.batches + b);
        const int4 ra = __ldg(r4), rc = __ldg(r4 + 1), rd = __ldg(r4 + 2);
        const float mnx = __int_as_float(ra.y), mny = __int_as_float(ra.z), mnz = __int_as_float(ra.w);
        const float mxx = __int_as_float(rc.x), mxy = __int_as_float(rc.y), mxz = __int_as_float(rc.z);
        const int64_t first = rd.x;
        const int32_t count = (int32_t)points_in_batch(rc.w, bl.quirks);
        const FileRec& f = vp.files[rd.y];

        BatchCtx c;
        const float steps = level >= 2 ? 1024.0f : 1073741824.0f;
        c.mnx = mnx; c.mny = mny; c.mnz = mnz;
        c.sx = __fdiv_rn(fsub(mxx, mnx), steps);
        c.sy = __fdiv_rn(fsub(mxy, mny), steps);
        c.sz = __fdiv_rn(fsub(mxz, mnz), steps);
        c.T0 = f.T[0]; c.T1 = f.T[1]; c.T3 = f.T[3];
        c.T4 = f.T[4]; c.T5 = f.T[5]; c.T7 = f.T[7];
        c.T8 = f.T[8]; c.T9 = f.T[9]; c.T11 = f.T[11];
        c.T12 = f.T[12]; c.T13 = f.T[13]; c.T15 = f.T[15];
        c.Wf = (float)vp.W; c.Hf = (float)vp.H; c.W = vp.W;
        const bool l0_x12 = (bl.quirks & CR_QUIRK_L0_X12) != 0;
        if (level >= 2) run_points<MODE, PAYLOAD, BLOCK, 2>(bl, s_zc, c, first, count, l0_x12);
        else if (level == 1) run_points<MODE, PAYLOAD, BLOCK, 1>(bl, s_zc, c, first, count, l0_x12);
        else run_points<MODE, PAYLOAD, BLOCK, 0>(bl, s_zc, c, first, count, l0_x12);
        __syncthreads();
        buf ^= 1;
    }
}

// ---- plain 16 B/point path --------------------------------------------------

struct PlainParams {
    float T[16];
    int32_t W, H;
};

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_plain(PlainParams pp, const uint4* __restrict__ v,
                                                 int64_t n, uint64_t* __restrict__ fb) {
    BatchCtx c;
    c.T0 = pp.T[0]; c.T1 = pp.T[1]; c.T3 = pp.T[3];
    c.T4 = pp.T[4]; c.T5 = pp.T[5]; c.T7 = pp.T[7];
    c.T8 = pp.T[8]; c.T9 = pp.T[9]; c.T11 = pp.T[11];
    c.T12 = pp.T[12]; c.T13 = pp.T[13]; c.T15 = pp.T[15];
    c.Wf = (float)pp.W; c.Hf = (float)pp.H; c.W = pp.W;
    BatchedLaunch bl{};
    bl.fb = fb;
    __shared__ unsigned long long s_zc[kZCacheSlots];
    for (int i = threadIdx.x; i < kZCacheSlots; i += BLOCK) s_zc[i] = 0xFFFFFFFFull;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    for (int64_t base = (int64_t)blockIdx.x * BLOCK; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool act = i < n;
        uint4 p = make_uint4(0, 0, 0, 0);
        if (act) p = ld_stream(v + i);
        int32_t pix;
        uint32_t wbits;
        const bool ok = project(c, __uint_as_float(p.x), __uint_as_float(p.y), __uint_as_float(p.z),
                                pix, wbits) && act;
        Emit<kModeRaster>::run(bl, s_zc, ok, pix, wbits, p.w, 0u);
    }
}

// ---- resolves ----------------------------------------------------------------

__device__ __forceinline__ bool depth_valid(uint64_t v) {
    float d = __uint_as_float((uint32_t)(v >> 32));
    return d > 0.0f && d < 1000000.0f;
}

// resolve.cs:100-146 (index payload) -- 2 pixels per thread.
__global__ void k_resolve_index(int64_t P, int64_t tail, uint64_t* __restrict__ fb,
                                const uint32_t* __restrict__ rgba, int64_t rgba_words,
                                uint32_t* __restrict__ image, int clear_after, uint64_t clear) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t p = 2 * t;
    if (p < P) {
        if (p + 1 < P) {
            ulonglong2 v = reinterpret_cast<const ulonglong2*>(fb)[t];
            uint32_t i0 = depth_valid(v.x) ? (uint32_t)v.x : 0u;
            uint32_t i1 = depth_valid(v.y) ? (uint32_t)v.y : 0u;
            uint2 o;
            o.x = (i0 == 0u || i0 >= rgba_words) ? kBackground : __ldg(rgba + i0);
            o.y = (i1 == 0u || i1 >= rgba_words) ? kBackground : __ldg(rgba + i1);
            reinterpret_cast<uint2*>(image)[t] = o;
            if (clear_after) reinterpret_cast<ulonglong2*>(fb)[t] = make_ulonglong2(clear, clear);
        } else {
            uint64_t v = fb[p];
            uint32_t i0 = depth_valid(v) ? (uint32_t)v : 0u;
            image[p] = (i0 == 0u || i0 >= rgba_words) ? kBackground : __ldg(rgba + i0);
            if (clear_after) fb[p] = clear;
        }
    }
    if (clear_after && t < tail) fb[P + t] = clear;
}

__global__ void k_resolve_color(int64_t P, int64_t tail, uint64_t* __restrict__ fb,
                                uint32_t* __restrict__ image, int clear_after, uint64_t clear) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t p = 2 * t;
    if (p < P) {
        if (p + 1 < P) {
            ulonglong2 v = reinterpret_cast<const ulonglong2*>(fb)[t];
            uint2 o;
            o.x = depth_valid(v.x) ? (uint32_t)v.x : kBackground;
            o.y = depth_valid(v.y) ? (uint32_t)v.y : kBackground;
            reinterpret_cast<uint2*>(image)[t] = o;
            if (clear_after) reinterpret_cast<ulonglong2*>(fb)[t] = make_ulonglong2(clear, clear);
        } else {
            uint64_t v = fb[p];
            image[p] = depth_valid(v) ? (uint32_t)v : kBackground;
            if (clear_after) fb[p] = clear;
        }
    }
    if (clear_after && t < tail) fb[P + t] = clear;
}

// compute_2021_earlyz/resolve.cs:41-77
__device__ __forceinline__ uint32_t plain_rgba8(uint64_t v) {
    uint32_t ucol = (uint32_t)(v & 0x00FFFFFFull);
    if (ucol == 0u) return 0xFF000000u;
    uint32_t o = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float cf = small_u2f((ucol >> (8 * k)) & 0xFFu);
        float f = fmul(255.0f, __fdiv_rn(cf, 255.0f));
        o |= ((uint32_t)small_f2i(f) & 0xFFu) << (8 * k);
    }
    return o;
}

__global__ void k_resolve_plain(int64_t P, int64_t tail, uint64_t* __restrict__ fb,
                                uint32_t* __restrict__ image, int clear_after, uint64_t clear) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P) {
        image[t] = plain_rgba8(fb[t]);
        if (clear_after) fb[t] = clear;
    }
    if (clear_after && t < tail) fb[P + t] = clear;
}

// compute_loop_las_hqs/resolve.cs:62-130
__global__ void k_resolve_hqs(int64_t P, int64_t tail, uint32_t* __restrict__ depth,
                              uint64_t* __restrict__ accum, uint32_t* __restrict__ image,
                              int clear_after) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P) {
        ulonglong2 a = reinterpret_cast<const ulonglong2*>(accum)[t];
        uint32_t R = (uint32_t)a.x, G = (uint32_t)(a.x >> 32);
        uint32_t B = (uint32_t)a.y, cnt = (uint32_t)(a.y >> 32);
        uint32_t out = kBackground;
        if (cnt != 0u) out = (R / cnt) | ((G / cnt) << 8) | ((B / cnt) << 16);
        image[t] = out;
        if (clear_after) {
            reinterpret_cast<ulonglong2*>(accum)[t] = make_ulonglong2(0ull, 0ull);
            depth[t] = kHqsDepthClear;
        }
    }
    if (clear_after && t < tail) {
        reinterpret_cast<ulonglong2*>(accum)[P + t] = make_ulonglong2(0ull, 0ull);
        depth[P + t] = kHqsDepthClear;
    }
}

__global__ void k_fill_u64(uint64_t* p, int64_t n, uint64_t v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}
__global__ void k_fill_u32(uint32_t* p, int64_t n, uint32_t v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

inline int blocks_for(int64_t n, int per) { return (int)((n + per - 1) / per); }

int launch_status() { return cudaGetLastError() == cudaSuccess ? 0 : -1; }

}  // namespace

int launch_cull(const ViewParams& vp, const cr_batch* batches, int64_t nb, int64_t capacity,
                int32_t quirks, uint32_t* scratch, void* stream) {
    if (nb <= 0) return 0;
    k_cull<<<blocks_for(nb, 256), 256, 0, (cudaStream_t)stream>>>(vp, batches, nb, capacity,
                                                                   quirks, scratch);
    return launch_status();
}

template <int MODE, int PAYLOAD>
static void launch_batched_t(const ViewParams& vp, const BatchedLaunch& bl, int block, int grid,
                             cudaStream_t s) {
    switch (block) {
        case 128: k_batched<MODE, PAYLOAD, 128><<<grid, 128, 0, s>>>(vp, bl); break;
        case 512: k_batched<MODE, PAYLOAD, 512><<<grid, 512, 0, s>>>(vp, bl); break;
        default: k_batched<MODE, PAYLOAD, 256><<<grid, 256, 0, s>>>(vp, bl); break;
    }
}

int launch_batched(const ViewParams& vp, const BatchedLaunch& bl, int block, int grid, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (bl.mode == kModeRaster) {
        if (bl.payload == CR_PAYLOAD_COLOR) launch_batched_t<kModeRaster, CR_PAYLOAD_COLOR>(vp, bl, block, grid, s);
        else launch_batched_t<kModeRaster, CR_PAYLOAD_INDEX>(vp, bl, block, grid, s);
    } else if (bl.mode == kModeHqsDepth) {
        launch_batched_t<kModeHqsDepth, CR_PAYLOAD_INDEX>(vp, bl, block, grid, s);
    } else {
        launch_batched_t<kModeHqsColor, CR_PAYLOAD_INDEX>(vp, bl, block, grid, s);
    }
    return launch_status();
}

template <int MODE, int PAYLOAD>
static int occupancy_t(int block) {
    int n = 0;
    cudaError_t e;
    switch (block) {
        case 128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 128>, 128, 0); break;
        case 512: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 512>, 512, 0); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 256>, 256, 0); break;
    }
    return e == cudaSuccess ? n : 1;
}

int batched_blocks_per_sm(int mode, int payload, int block) {
    if (mode == kModeRaster)
        return payload == CR_PAYLOAD_COLOR ? occupancy_t<kModeRaster, CR_PAYLOAD_COLOR>(block)
                                           : occupancy_t<kModeRaster, CR_PAYLOAD_INDEX>(block);
    if (mode == kModeHqsDepth) return occupancy_t<kModeHqsDepth, CR_PAYLOAD_INDEX>(block);
    return occupancy_t<kModeHqsColor, CR_PAYLOAD_INDEX>(block);
}

int launch_plain(const float T[16], int32_t W, int32_t H, const cr_vertex* v, int64_t n,
                 uint64_t* fb, int grid, void* stream) {
    if (n <= 0) return 0;
    PlainParams pp;
    for (int i = 0; i < 16; i++) pp.T[i] = T[i];
    pp.W = W;
    pp.H = H;
    int64_t need = (n + 255) / 256;
    if (need < grid) grid = (int)need;
    k_plain<256><<<grid, 256, 0, (cudaStream_t)stream>>>(pp, reinterpret_cast<const uint4*>(v), n, fb);
    return launch_status();
}

int launch_resolve_index(int32_t W, int32_t H, uint64_t* fb, const uint32_t* rgba,
                         int64_t rgba_words, uint32_t* image, int clear_after, uint64_t clear,
                         void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = (P + 1) / 2 > tail ? (P + 1) / 2 : tail;
    k_resolve_index<<<blocks_for(threads, 256), 256, 0, (cudaStream_t)stream>>>(
        P, tail, fb, rgba, rgba_words, image, clear_after, clear);
    return launch_status();
}

int launch_resolve_color(int32_t W, int32_t H, uint64_t* fb, uint32_t* image, int clear_after,
                         uint64_t clear, void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = (P + 1) / 2 > tail ? (P + 1) / 2 : tail;
    k_resolve_color<<<blocks_for(threads, 256), 256, 0, (cudaStream_t)stream>>>(
        P, tail, fb, image, clear_after, clear);
    return launch_status();
}

int launch_resolve_plain(int32_t W, int32_t H, uint64_t* fb, uint32_t* image, int clear_after,
                         uint64_t clear, void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = P > tail ? P : tail;
    k_resolve_plain<<<blocks_for(threads, 256), 256, 0, (cudaStream_t)stream>>>(P, tail, fb, image,
                                                                                 clear_after, clear);
    return launch_status();
}

int launch_resolve_hqs(int32_t W, int32_t H, uint32_t* depth, uint64_t* accum, uint32_t* image,
                       int clear_after, void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = P > tail ? P : tail;
    k_resolve_hqs<<<blocks_for(threads, 256), 256, 0, (cudaStream_t)stream>>>(P, tail, depth, accum,
                                                                               image, clear_after);
    return launch_status();
}

int launch_fill_u64(uint64_t* p, int64_t n, uint64_t v, void* stream) {
    if (n <= 0) return 0;
    int grid = blocks_for(n, 256);
    if (grid > 65535) grid = 65535;
    k_fill_u64<<<grid, 256, 0, (cudaStream_t)stream>>>(p, n, v);
    return launch_status();
}

int launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, void* stream) {
    if (n <= 0) return 0;
    int grid = blocks_for(n, 256);
    if (grid > 65535) grid = 65535;
    k_fill_u32<<<grid, 256, 0, (cudaStream_t)stream>>>(p, n, v);
    return launch_status();
}

}  // namespace cr
