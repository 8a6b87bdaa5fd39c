// cr_kernels.cu -- sm_103a kernels of the point-rasterizer hot path.
//
// Compiled with -fmad=false: every fused multiply-add below is an explicit
// __fmaf_rn, every other float operation rounds on its own, scalar / and sqrt
// are IEEE (__fdiv_rn, __fsqrt_rn), and a vector divided by a scalar is a
// multiplication by the scalar's correctly rounded reciprocal (rcp_rn, equal
// to __frcp_rn for every input), the one reciprocal a shader compiler emits
// for it.  The operation order follows the arithmetic contract the oracle
// states, which is what makes the framebuffers bit-exact; the packed-pair
// forms (fma.rn.f32x2, mul.rn.f32x2) round each element as the scalar
// instructions do.
//
// Kernels
//   k_cull      one thread per batch record: validation, frustum cull
//               (render.cs:176-197), precision level (render.cs:199-231);
//               w-safe flag (w_safe); appends (batch | flag | level << 29)
//               to a work list.
//   k_batched   persistent CTAs pull work items; per batch the points are read
//               with 128-bit streaming loads (4 consecutive points per lane,
//               the loop_las2 `uvec4` scheme), decoded at 10/20/30 bit,
//               projected (full 10-bit batches two points per packed
//               instruction), tested against a per-CTA shared-memory z-cache,
//               and the survivors issue 64-bit atomicMin (render.cs:399-432).
//               The same body runs the HQS depth pass (u32 atomicMin,
//               hqs/depth.cs) and color pass (per-lane run sums; a lane's
//               last run through __match_any_sync partitioned sums; two
//               64-bit atomicAdd per pixel, hqs/color.cs:388-444).
//   k_plain     16 B/point path (compute_2021_earlyz/render.cs:35-74).
//   k_resolve_* per-pixel resolves (resolve.cs files), optionally re-clearing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "cr_internal.h"
#include "cr_device.cuh"
#include "cr_divcheck.h"
#include "cr_filerec.h"

namespace cr {

namespace {

// ---- per-file records of one view (clouds with more than kInlineFiles files)

constexpr int kFilesPerLaunch = 1024;
struct FileChunk {
    double view[16], proj[16];
    int32_t first, count, float_uniforms, literal;
    double box_min[3 * kFilesPerLaunch];
};
static_assert(sizeof(FileChunk) < 32000, "kernel parameters are limited to 32 KB");

__global__ void __launch_bounds__(128) k_file_records(const __grid_constant__ FileChunk c,
                                                      FileRec* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.count) return;
    FileRec r;
    if (c.float_uniforms) file_record_float(c.view, c.proj, &c.box_min[3 * i], &r, c.literal != 0);
    else file_record(c.view, c.proj, &c.box_min[3 * i], &r, c.literal != 0);
    out[c.first + i] = r;
}

// The record of file `fi`: kernel parameters for the first kInlineFiles files,
// the device array beyond (filled by k_file_records for this view).
__device__ __forceinline__ const FileRec* file_rec(const ViewParams& vp, int fi) {
    return fi < kInlineFiles ? &vp.files[fi] : vp.dfiles + fi;
}

// The 12 transform entries the projection uses (render.cs:399-401).
__device__ __forceinline__ void load_transform(const float* T, BatchCtx& c) {
    c.T0 = T[0]; c.T1 = T[1]; c.T3 = T[3];
    c.T4 = T[4]; c.T5 = T[5]; c.T7 = T[7];
    c.T8 = T[8]; c.T9 = T[9]; c.T11 = T[11];
    c.T12 = T[12]; c.T13 = T[13]; c.T15 = T[15];
}

// ---- cull + level: one thread per batch record -----------------------------

__global__ void __launch_bounds__(256) k_cull(const __grid_constant__ ViewParams vp,
                                              const cr_batch* __restrict__ batches, int64_t nb,
                                              int64_t capacity, int32_t quirks,
                                              uint32_t* __restrict__ scratch, int64_t list_cap,
                                              int32_t node_slices) {
    int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    uint32_t item = 0, slices = 1;
    if (b < nb) {
        const int4* r4 = reinterpret_cast<const int4*>(batches + b);
        int4 a = __ldg(r4), c = __ldg(r4 + 1), d = __ldg(r4 + 2);
        float mnx = __int_as_float(a.y), mny = __int_as_float(a.z), mnz = __int_as_float(a.w);
        float mxx = __int_as_float(c.x), mxy = __int_as_float(c.y), mxz = __int_as_float(c.z);
        int32_t np = c.w, fp = d.x, fi = vp.one_world ? 0 : d.y;
        int64_t count = points_in_batch(np, fp, quirks);
        bool ok = np >= 0 && (np <= kPointsPerBatch || (quirks & CR_QUIRK_NODE_LOOP)) && fp >= 0 &&
                  (int64_t)fp + count + 4 <= capacity && fi >= 0 && fi < vp.nfiles;
        if (!ok) {
            atomicOr(&scratch[kErrWord], kErrBadBatch);
        } else if (count > 0) {
            const FileRec& f = *file_rec(vp, fi);
            bool vis = !vp.culling || intersects_frustum(f.planes, mnx, mny, mnz, mxx, mxy, mxz);
            if (vis) {
                int level = precision_level(vp.P, f.VW, vp.W, vp.H, mnx, mny, mnz, mxx, mxy, mxz,
                                            vp.level4_px, vp.literal != 0);
                // compute_loop_nodes/render.cs:273-276: the level-of-detail cut
                keep = vp.lod_skip_level <= 0 || level < vp.lod_skip_level;
                // the literal pair body's division wants w in [2^-64, 2^64]
                // (the quirk that selects the literal k_batched instance)
                const bool lit = (quirks & CR_QUIRK_LITERAL_ARITH) != 0;
                const float wlo = lit ? 0x1p-64f : 0x1p-120f;
                const float whi = lit ? 0x1p64f : 0x1p120f;
                item = (uint32_t)b | ((uint32_t)level << 29) |
                       (w_safe(f.T, mnx, mny, mnz, mxx, mxy, mxz, wlo, whi) ? kItemWSafe : 0u);
                if (node_slices) slices = (uint32_t)cr::node_slices(fp, count);
            }
        }
    }
    // 10-bit items to the front of the list region, 20/30-bit items to the back
    const bool front = keep && (item >> 29) >= 2u;
    const bool back = keep && !front;
    const uint32_t lane = lane_id();
    if (node_slices) {
        // a node's slices side by side: warp-wide prefix sums of the slice counts
        uint32_t sf = front ? slices : 0u, sb = back ? slices : 0u;
        uint32_t incf = sf, incb = sb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t uf = __shfl_up_sync(kFull, incf, o), ub = __shfl_up_sync(kFull, incb, o);
            if (lane >= (uint32_t)o) {
                incf += uf;
                incb += ub;
            }
        }
        const uint32_t totf = __shfl_sync(kFull, incf, 31), totb = __shfl_sync(kFull, incb, 31);
        uint32_t basef = 0, baseb = 0;
        if (lane == 0) {
            if (totf) basef = atomicAdd(&scratch[kItemCount], totf);
            if (totb) baseb = atomicAdd(&scratch[kItemCount2], totb);
        }
        basef = __shfl_sync(kFull, basef, 0) + incf - sf;
        baseb = __shfl_sync(kFull, baseb, 0) + incb - sb;
        for (uint32_t k = 0; k < sf; k++)
            scratch[kScratchHead + basef + k] = item | (k << kItemSliceShift);
        for (uint32_t k = 0; k < sb; k++)
            scratch[kScratchHead + list_cap - 1 - (int64_t)(baseb + k)] = item | (k << kItemSliceShift);
        return;
    }
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t mf = __ballot_sync(kFull, front);
    if (mf) {
        const uint32_t leader = __ffs(mf) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&scratch[kItemCount], __popc(mf));
        base = __shfl_sync(kFull, base, leader);
        if (front) scratch[kScratchHead + base + __popc(mf & below)] = item;
    }
    const uint32_t mb = __ballot_sync(kFull, back);
    if (mb) {
        const uint32_t leader = __ffs(mb) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&scratch[kItemCount2], __popc(mb));
        base = __shfl_sync(kFull, base, leader);
        if (back) scratch[kScratchHead + list_cap - 1 - (int64_t)(base + __popc(mb & below))] = item;
    }
}

// ---- batched raster / HQS body ---------------------------------------------

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
        const uint32_t slot = zslot_pixel((uint32_t)pix);
        // render.cs:423-424 early depth test, against the CTA's cache
        const bool cand = ok && !zcache_rejects(zc, slot, (uint32_t)pix, wbits);
        if (__any_sync(kFull, cand) && cand)
            submit_min<unsigned long long>(reinterpret_cast<unsigned long long*>(bl.fb) + pix, zc,
                                           slot, (uint32_t)pix,
                                           ((unsigned long long)wbits << 32) | payload, wbits);
    }
};

template <>
struct Emit<kModeHqsDepth> {
    static __device__ __forceinline__ void run(const BatchedLaunch& bl, unsigned long long* zc,
                                               bool ok, int32_t pix, uint32_t wbits, uint32_t,
                                               uint32_t) {
        const uint32_t slot = zslot_pixel((uint32_t)pix);
        // hqs/depth.cs:375-379
        const bool cand = ok && !zcache_rejects(zc, slot, (uint32_t)pix, wbits);
        if (__any_sync(kFull, cand) && cand)
            submit_min<uint32_t>(bl.depth + pix, zc, slot, (uint32_t)pix, wbits, wbits);
    }
};

// HQS color pass (color.cs:399-441): the sums of (R, G, B, 1) over the points
// of a lane's run (consecutive in-view points on one pixel, see run_points)
// are added to the pixel's two 64-bit accumulators.  All sums are integer
// adds, so the accumulators equal one add per point in any order.  Per lane a
// run has at most 4 points, so the 16-bit fields hold a warp's sums
// (32 x 4 x 255).
//
// hqs_color_add: one lane's run, added directly.
__device__ __forceinline__ void hqs_color_add(const BatchedLaunch& bl, uint32_t pix, uint32_t rg,
                                              uint32_t bc) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(bl.accum) + 2 * (int64_t)pix;
    atomicAdd(a, (unsigned long long)(rg & 0xFFFFu) | ((unsigned long long)(rg >> 16) << 32));
    atomicAdd(a + 1, (unsigned long long)(bc & 0xFFFFu) | ((unsigned long long)(bc >> 16) << 32));
}

// hqs_color_flush: every lane's last run of the vector joins the warp's
// partitioned sum over lanes on the same pixel, and the leader adds it.  Most
// lanes' last runs share pixels with their neighbours' (Morton order), so the
// merge saves contended atomics there; runs that end inside a vector are few
// per lane but some lane of almost every warp has one, and sending those
// through the merge too (a merge at every point position) measured 24 %
// slower on the whole HQS frame than adding them directly, and a segmented
// suffix sum over neighbouring lanes on one pixel (shuffles, no match) in
// place of the partition 4 % slower.
__device__ __forceinline__ void hqs_color_flush(const BatchedLaunch& bl, bool active, uint32_t pix,
                                                uint32_t rg, uint32_t bc) {
    if (!__any_sync(kFull, active)) return;
    const uint32_t peers = __match_any_sync(kFull, active ? pix : kNoPixel);
    if (active) {
        const uint32_t srg = __reduce_add_sync(peers, rg);
        const uint32_t sbc = __reduce_add_sync(peers, bc);
        if (lane_id() == (uint32_t)(__ffs(peers) - 1)) hqs_color_add(bl, pix, srg, sbc);
    }
}

// float(X) * step + min: one FMA, or (LIT, CR_QUIRK_LITERAL_ARITH) the
// product then the sum as render.cs:355-357 writes it.
template <bool LIT>
__device__ __forceinline__ float decode_axis(float X, float step, float mn) {
    return LIT ? fadd(fmul(X, step), mn) : __fmaf_rn(X, step, mn);
}

// Decodes point j of the lane's vector at level class LC (render.cs:333-397).
template <int LC, bool LIT = false>
__device__ __forceinline__ void decode_point(const uint4& w4, const uint4& w8, const uint4& w12, int j,
                                             const BatchCtx& c, bool l0_x12, float& x, float& y,
                                             float& z) {
    const uint32_t a = u4get(w4, j);
    if (LC == 2) {
        x = decode_axis<LIT>(small_u2f(a & 1023u), c.sx, c.mnx);
        y = decode_axis<LIT>(small_u2f((a >> 10) & 1023u), c.sy, c.mny);
        z = decode_axis<LIT>(small_u2f((a >> 20) & 1023u), c.sz, c.mnz);
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
        x = decode_axis<LIT>(__uint2float_rn(X), c.sx, c.mnx);
        y = decode_axis<LIT>(__uint2float_rn(Y), c.sy, c.mny);
        z = decode_axis<LIT>(__uint2float_rn(Z), c.sz, c.mnz);
    }
}

// LC: 2 = 10 bit (levels 2-4), 1 = 20 bit (level 1), 0 = 30 bit (level 0).
// Points [first, first + count) are read as 128-bit vectors starting at the
// aligned word below `first`; lanes mask the words outside the range.  The
// next vector is loaded before the current one is processed.  PAIRS (full
// 10-bit batches that the cull flagged w-safe): points are decoded and
// projected two at a time with the unchecked reciprocal (project_pair10).
template <int MODE, int PAYLOAD, int BLOCK, int LC, bool FULL = false, bool PAIRS = false,
          bool LIT = false>
__device__ __forceinline__ void run_points(const BatchedLaunch& bl, unsigned long long* zc,
                                           const BatchCtx& c, const PairParams& pp, int64_t first,
                                           int32_t count, bool l0_x12) {
    static_assert(!PAIRS || (FULL && LC == 2), "pairs decode full 10-bit batches");
    PairCol3 pf{};
    if constexpr (PAIRS) pf = PairCol3{f2_pack(c.T12, c.T12), f2_pack(c.T13, c.T13), f2_pack(c.T15, c.T15)};
    constexpr bool kNeedColor = (MODE == kModeHqsColor) || (MODE == kModeRaster && PAYLOAD == CR_PAYLOAD_COLOR);
    const int64_t v0 = first >> 2;
    const int32_t head = (int32_t)(first & 3);
    // las2/render.cs:319-341 (CR_QUIRK_UVEC4_BASE, batches with firstPoint % 4 != 0):
    // the reference's 128 threads read vectors 0..2559 from firstPoint / 4, so
    // vector v's word j is batch point 4v + j - head; thread 0 (vectors v with
    // v % 128 == 0) underflows its first localIndex and returns, and vectors past
    // 2559 are never read.  Full batches start aligned (head == 0), where the
    // addressing is the same as here.  Only the raster reads this way (HQS
    // passes walk their batches with stride 128, hqs/depth.cs:270-276).
    const bool uvec4 = MODE == kModeRaster && !FULL && head != 0 && (bl.quirks & CR_QUIRK_UVEC4_BASE) != 0;
    const int nv = uvec4 ? min((head + count + 3) >> 2, kPointsPerBatch / 4) : (head + count + 3) >> 2;
    const uint32_t index0 = (uint32_t)(first - head);  // global index of word 0 of vector v0
    const uint4* lo4 = reinterpret_cast<const uint4*>(bl.lo) + v0;
    const uint4* md4 = reinterpret_cast<const uint4*>(bl.md) + v0;
    const uint4* hi4 = reinterpret_cast<const uint4*>(bl.hi) + v0;
    const uint4* co4 = reinterpret_cast<const uint4*>(bl.rgba) + v0;
    const uint4 zero = make_uint4(0, 0, 0, 0);
    uint4 n4 = zero, n8 = zero, n12 = zero, ncol = zero;
    PairBatch pb{};
    if constexpr (PAIRS) pb = pair_batch(c);
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
        // the reference's thread 0 returns before any point when head != 0
        const bool lane_live = !uvec4 || (v & 127) != 0;
        if constexpr (MODE == kModeHqsColor) {
            // The lane's 4 consecutive points, in runs of in-view points on one
            // pixel (Morton order puts most of them on the same pixel): project
            // all 4, read the depth of every run start at once (the reads
            // overlap; the depth buffer is read-only in this pass), then sum
            // each run's visible colors and flush it once.
            int32_t pix[4];
            uint32_t wb[4];
            bool ok[4];
            if constexpr (PAIRS) {
                project_pair10<LIT>(pp, pf, pb, c.W, w4.x, w4.y, ok, pix, wb);
                project_pair10<LIT>(pp, pf, pb, c.W, w4.z, w4.w, ok + 2, pix + 2, wb + 2);
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const bool valid = FULL || ((uint32_t)(rel0 + j) < (uint32_t)count && lane_live);
                    float x, y, z;
                    decode_point<LC, LIT>(w4, w8, w12, j, c, l0_x12, x, y, z);
                    ok[j] = project<false, LIT>(c, x, y, z, pix[j], wb[j]) && valid;
                }
            }
            bool cont[4];
            float lim[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int jp = j > 0 ? j - 1 : 0;
                cont[j] = j > 0 && ok[jp] && ok[j] && pix[j] == pix[jp];
                // color.cs:399-403: visible if depth <= bufferDepth * 1.01
                lim[j] = ok[j] && !cont[j] ? fmul(__uint_as_float(__ldg(bl.depth + pix[j])), 1.01f) : 0.0f;
            }
            uint32_t rg = 0u, bc = 0u;
            float run_lim = 0.0f;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int jp = j > 0 ? j - 1 : 0;
                // a run that ends inside the vector goes straight to the
                // accumulators; only the lane's last run joins the warp merge
                if (j > 0 && ok[jp] && !cont[j] && bc != 0u) hqs_color_add(bl, pix[jp], rg, bc);
                if (!cont[j]) {
                    rg = bc = 0u;
                    run_lim = lim[j];
                }
                if (ok[j] && __uint_as_float(wb[j]) <= run_lim) {
                    // R | G << 16 and B | 1 << 16, one byte permute each
                    const uint32_t color = u4get(col, j);
                    rg += __byte_perm(color, 0u, 0x4140);
                    bc += __byte_perm(color, 0x00010000u, 0x7642);
                }
            }
            hqs_color_flush(bl, ok[3] && bc != 0u, pix[3], rg, bc);
        } else if constexpr (PAIRS) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                int32_t pix[2];
                uint32_t wb[2];
                bool ok[2];
                project_pair10<LIT>(pp, pf, pb, c.W, h ? w4.z : w4.x, h ? w4.w : w4.y, ok, pix, wb);
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    const int j = 2 * h + k;
                    const uint32_t idx = index0 + 4u * (uint32_t)v + (uint32_t)j;
                    const uint32_t color = kNeedColor ? u4get(col, j) : 0u;
                    const uint32_t payload = (PAYLOAD == CR_PAYLOAD_COLOR) ? color : idx;
                    Emit<MODE>::run(bl, zc, ok[k], pix[k], wb[k], payload, color);
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const bool valid = FULL || ((uint32_t)(rel0 + j) < (uint32_t)count && lane_live);
                const uint32_t idx = index0 + 4u * (uint32_t)v + (uint32_t)j;
                float x, y, z;
                decode_point<LC, LIT>(w4, w8, w12, j, c, l0_x12, x, y, z);
                int32_t pix;
                uint32_t wbits;
                const bool ok = project<false, LIT>(c, x, y, z, pix, wbits) && valid;
                const uint32_t color = kNeedColor ? u4get(col, j) : 0u;
                const uint32_t payload = (PAYLOAD == CR_PAYLOAD_COLOR) ? color : (uint32_t)idx;
                Emit<MODE>::run(bl, zc, ok, pix, wbits, payload, color);
            }
        }
    }
}

// The HQS color pass's 10-bit instance is held to 48 registers, at which 10
// CTAs of 128 threads stay resident per SM (its uncapped 51 leave 9 CTAs per
// SM; measured 1 % slower).  UNCAPPED: the many-file literal instance, which
// spills under the cap.
template <int MODE, int BLOCK, int LIST, bool UNCAPPED = false>
constexpr int kMinBlocks = MODE == kModeHqsColor && LIST == 0 && !UNCAPPED ? 1280 / BLOCK : 0;

// LIST 0: the 10-bit items (front of the list region), LIST 1: the 20/30-bit
// items (back of the region).  Each list runs in its own instance, so the
// common 10-bit instance carries no wider decode state (fewer registers).
// List 1 is launched first and lets the list-0 grid start at once
// (programmatic dependent launch); every list-0 CTA waits for the list-1 grid
// before it exits, so work that follows on the stream sees both lists' writes.
// MANY: the cloud has more than kInlineFiles files, whose records are read
// from vp.dfiles (a separate instance, so the common case's code is untouched).
// LIT: CR_QUIRK_LITERAL_ARITH, the decode and projection as the shaders write
// them (the pairs with project_pair10's literal body, on batches whose w lies
// in [2^-64, 2^64]).
template <int MODE, int PAYLOAD, int BLOCK, int LIST, bool MANY, bool LIT = false>
__global__ void __launch_bounds__(BLOCK, (kMinBlocks<MODE, BLOCK, LIST, MANY && LIT>))
    k_batched(ViewParams vp, BatchedLaunch bl, PairParams pp) {
    if (LIST == 1) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ uint32_t s_item[2];
    __shared__ unsigned long long s_zc[MODE == kModeHqsColor ? 1 : kZCacheSlots];
    uint32_t* cursor = bl.scratch + (LIST == 0 ? (MODE == kModeHqsColor ? kCursor1 : kCursor0)
                                               : (MODE == kModeHqsColor ? kCursor3 : kCursor2));
    const uint32_t nitems =
        *reinterpret_cast<volatile uint32_t*>(bl.scratch + (LIST == 0 ? kItemCount : kItemCount2));
    if (nitems != 0) {
        if (MODE != kModeHqsColor)
            for (int i = threadIdx.x; i < kZCacheSlots; i += BLOCK) s_zc[i] = 0xFFFFFFFFull;
        if (threadIdx.x == 0) s_item[0] = atomicAdd(cursor, 1u);
        __syncthreads();
        int buf = 0;
        while (true) {
            const uint32_t wi = s_item[buf];
            if (wi >= nitems) break;
            if (threadIdx.x == 0) s_item[buf ^ 1] = atomicAdd(cursor, 1u);
            const uint32_t item =
                bl.scratch[kScratchHead + (LIST == 0 ? (int64_t)wi : bl.list_cap - 1 - (int64_t)wi)];
            const uint32_t b = item & (bl.node_slices ? kItemNodeMask : kItemBatchMask);
            const int level = (int)(item >> 29);

            const int4* r4 = reinterpret_cast<const int4*>(bl.batches + b);
            const int4 ra = __ldg(r4), rc = __ldg(r4 + 1), rd = __ldg(r4 + 2);
            const float mnx = __int_as_float(ra.y), mny = __int_as_float(ra.z), mnz = __int_as_float(ra.w);
            const float mxx = __int_as_float(rc.x), mxy = __int_as_float(rc.y), mxz = __int_as_float(rc.z);
            int64_t first = rd.x;
            int32_t count = (int32_t)points_in_batch(rc.w, rd.x, bl.quirks);
            if (bl.node_slices) {  // this item's slice of the node
                int64_t sf, sc;
                node_slice(first, count, (item >> kItemSliceShift) & 31u, &sf, &sc);
                first = sf;
                count = (int32_t)sc;
            }
            const int fi = vp.one_world ? 0 : rd.y;
            BatchCtx c;
            // render.cs:355-357, 392-394 boxSize / STEPS: a division by a power
            // of two is the same real value as the product with its exact
            // reciprocal, so both round alike for every input
            const float inv = level >= 2 ? 0x1p-10f : 0x1p-30f;
            c.mnx = mnx; c.mny = mny; c.mnz = mnz;
            c.sx = fmul(fsub(mxx, mnx), inv);
            c.sy = fmul(fsub(mxy, mny), inv);
            c.sz = fmul(fsub(mxz, mnz), inv);
            if constexpr (MANY) {
                load_transform(vp.dfiles[fi].T, c);
            } else {
                const FileRec& f = vp.files[fi];
                load_transform(f.T, c);
            }
            c.Wf = (float)vp.W; c.Hf = (float)vp.H; c.W = vp.W;
            const bool l0_x12 = (bl.quirks & CR_QUIRK_L0_X12) != 0;
            // full, vector-aligned batches whose w range is proven safe (nearly
            // all) skip the per-point range test and decode in pairs; the rest
            // take the general body
            // (node slices of kNodeSlice points qualify too: whole vectors for
            // every thread, as the full path needs)
            if (LIST == 0 && (item & kItemWSafe) &&
                (count == kPointsPerBatch ||
                 (kNodeSlice % (4 * BLOCK) == 0 && bl.node_slices && count == kNodeSlice)) &&
                (first & 3) == 0 && pair_batch_exact(c))
                run_points<MODE, PAYLOAD, BLOCK, 2, true, true, LIT>(bl, s_zc, c, pp, first, count, l0_x12);
            else if (LIST == 0)
                run_points<MODE, PAYLOAD, BLOCK, 2, false, false, LIT>(bl, s_zc, c, pp, first, count, l0_x12);
            else if (level == 1)
                run_points<MODE, PAYLOAD, BLOCK, 1, false, false, LIT>(bl, s_zc, c, pp, first, count, l0_x12);
            else
                run_points<MODE, PAYLOAD, BLOCK, 0, false, false, LIT>(bl, s_zc, c, pp, first, count, l0_x12);
            __syncthreads();
            buf ^= 1;
        }
    }
    if (LIST == 0) asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ---- plain 16 B/point path --------------------------------------------------

struct PlainParams {
    float T[16];
    int32_t W, H;
};

// VARIANT 0: compute_2021_earlyz/render.cs:35-74, key depth << 32 | color
//   through the CTA z-cache.
// VARIANT 1, 2: compute_2021_dedup/render.cs:33-69 and
//   compute_2021_earlyz_reduce/render.cs:44-82.  A warp is 32 consecutive
//   points (the grid stride is a multiple of 32), the reference's subgroup;
//   lanes whose point is outside the view are not part of the reduction.
//   key = depth << 24 | color, the color's top byte overlapping the low depth
//   byte as in the reference, so the reduction decides which keys reach the
//   framebuffer.  Writers submit an atomicMin.
template <int BLOCK, int VARIANT, bool LIT = false>
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
    __shared__ unsigned long long s_zc[VARIANT == 0 ? kZCacheSlots : 1];
    // VARIANT 1: per warp a 4096-bit map of the pixels its in-view lanes hit
    __shared__ uint32_t s_bits[VARIANT == 1 ? BLOCK / 32 * 128 : 1];
    if (VARIANT == 0) {
        for (int i = threadIdx.x; i < kZCacheSlots; i += BLOCK) s_zc[i] = 0xFFFFFFFFull;
        __syncthreads();
    }
    if (VARIANT == 1) {
        for (int i = threadIdx.x; i < BLOCK / 32 * 128; i += BLOCK) s_bits[i] = 0u;
        __syncthreads();
    }
    uint32_t* warp_bits = s_bits + (VARIANT == 1 ? (threadIdx.x >> 5) * 128 : 0);
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    for (int64_t base = (int64_t)blockIdx.x * BLOCK; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool act = i < n;
        uint4 p = make_uint4(0, 0, 0, 0);
        if (act) p = ld_stream(v + i);
        int32_t pix;
        uint32_t wbits;
        const bool ok = project<false, LIT>(c, __uint_as_float(p.x), __uint_as_float(p.y),
                                            __uint_as_float(p.z), pix, wbits) && act;
        if (VARIANT == 0) {
            Emit<kModeRaster>::run(bl, s_zc, ok, pix, wbits, p.w, 0u);
            continue;
        }
        // wbits = floatBitsToInt(pos.w), positive for every point in view
        bool write;
        if (VARIANT == 1) {
            // subgroupPartitionNV(pixelID) + subgroupPartitionedMinNV(depth).
            // Each in-view lane first sets bit (pixelID mod 4096) of the warp's
            // map: when no lane finds its bit already set, the lanes' pixels
            // are distinct, every lane is its partition's minimum and writes.
            // A warp with a repeated bit (a shared pixel, or two pixels equal
            // mod 4096) takes the exact partition.  For the uniformly random
            // points of the 4M-point frame 87.0 -> 46.0 us.
            const uint32_t h = (uint32_t)pix & 4095u, m = 1u << (h & 31u);
            bool seen = false;
            if (ok) seen = (atomicOr(&warp_bits[h >> 5], m) & m) != 0u;
            if (__any_sync(kFull, seen)) {
                const uint32_t peers = __match_any_sync(kFull, ok ? (uint32_t)pix : kNoPixel);
                const uint32_t mind = __reduce_min_sync(peers, ok ? wbits : 0xFFFFFFFFu);
                write = ok && wbits == mind;
            } else {
                write = ok;
            }
            __syncwarp();
            if (ok) warp_bits[h >> 5] = 0u;  // every set bit's word, cleared for the next step
            __syncwarp();
        } else {
            const uint32_t active = __ballot_sync(kFull, ok);
            const int first = active ? __ffs(active) - 1 : 0;
            const int32_t first_pix = __shfl_sync(kFull, pix, first);
            // subgroupAllEqual(pixelID) over the active lanes
            const bool same = __all_sync(kFull, !ok || pix == first_pix);
            const uint32_t mind = __reduce_min_sync(kFull, ok ? wbits : 0xFFFFFFFFu);
            // pair partner (lane ^ 1): subgroupClusteredXor / ClusteredMin over 2
            const int32_t q_pix = __shfl_xor_sync(kFull, pix, 1);
            const uint32_t q_depth = __shfl_xor_sync(kFull, wbits, 1);
            const bool q_ok = (active >> (lane_id() ^ 1u)) & 1u;
            write = ok && (same ? wbits == mind : (!q_ok || q_pix != pix || wbits <= q_depth));
        }
        if (write) {
            // dedup/render.cs:66-69 reads the word and submits only a smaller
            // key; atomicMin leaves a word that is already smaller unchanged,
            // so the direct atomic gives the same words without exposing the
            // read's latency (early-z & reduce 48.3 -> 39.6 us, dedup 91.2 ->
            // 87.2 us per 4M-point frame)
            const unsigned long long key = ((unsigned long long)wbits << 24) | p.w;
            atomicMin(reinterpret_cast<unsigned long long*>(fb) + pix, key);
        }
    }
}

// ---- resolves ----------------------------------------------------------------

__device__ __forceinline__ bool depth_valid(uint64_t v) {
    float d = __uint_as_float((uint32_t)(v >> 32));
    return d > 0.0f && d < 1000000.0f;
}

// Whether pixel p lies in the floor(W/16) x floor(H/16) tiles a resolve of
// 16x16 groups covers (CR_QUIRK_RESOLVE_TILES).
__device__ __forceinline__ bool in_tiles(int64_t p, int32_t W, int32_t H) {
    const int64_t y = p / W, x = p - y * W;
    return x < (W & ~15) && y < (H & ~15);
}

// resolve.cs:100-146 (index payload) -- 2 pixels per thread.  tiles: only the
// pixels of full 16x16 tiles are resolved (compute_loop_nodes.h:199-201); the
// re-clear covers every pixel (loop_nodes clears separately,
// compute_loop_nodes.h:239-251).
__global__ void k_resolve_index(int64_t P, int64_t tail, uint64_t* __restrict__ fb,
                                const uint32_t* __restrict__ rgba, int64_t rgba_words,
                                uint32_t* __restrict__ image, int clear_after, uint64_t clear,
                                int32_t W, int32_t H, int tiles) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t p = 2 * t;
    if (p < P) {
        if (tiles) {
            for (int64_t q = p; q < p + 2 && q < P; q++) {
                if (in_tiles(q, W, H)) {
                    const uint64_t v = fb[q];
                    const uint32_t i0 = depth_valid(v) ? (uint32_t)v : 0u;
                    image[q] = (i0 == 0u || i0 >= rgba_words) ? kBackground : __ldg(rgba + i0);
                }
                if (clear_after) fb[q] = clear;
            }
        } else if (p + 1 < P) {
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
// uvec4(255.0 * unpackUnorm4x8(ucol)) per byte is trunc(255 * RN(c / 255)),
// which is c again for every byte c (checked over all 256 values, the CPU
// test test_plain_byte_round_trip), so the image word is ucol itself.
// early-z and early-z & reduce map ucol == 0 to opaque black (resolve.cs:44-46);
// the dedup resolve has no such rule (compute_2021_dedup/resolve.cs:15-21).
__device__ __forceinline__ uint32_t plain_rgba8(uint64_t v, int zero_rule) {
    const uint32_t ucol = (uint32_t)(v & 0x00FFFFFFull);
    return ucol == 0u && zero_rule ? 0xFF000000u : ucol;
}

// tiles != 0 (CR_QUIRK_RESOLVE_TILES): only the pixels of the floor(W/16) x
// floor(H/16) tiles of 16x16 that the reference dispatches
// (compute_2021_earlyz.h:161-163) are resolved and re-cleared; every other
// image and framebuffer word, the guard tail included, keeps its value.
__global__ void k_resolve_plain(int64_t P, int64_t tail, int32_t W, int32_t H, int tiles,
                                int zero_rule, uint64_t* __restrict__ fb,
                                uint32_t* __restrict__ image, int clear_after, uint64_t clear) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < P) {
        bool covered = true;
        if (tiles) {
            const int64_t y = t / W, x = t - y * W;
            covered = x < (W & ~15) && y < (H & ~15);
        }
        if (covered) {
            image[t] = plain_rgba8(fb[t], zero_rule);
            if (clear_after) fb[t] = clear;
        }
    }
    if (clear_after && !tiles && t < tail) fb[P + t] = clear;
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

// Every float bit pattern: rcp_rn(x) against __frcp_rn(x), bit for bit (a NaN
// matches any NaN), the pair reciprocal, and the pair division against
// __fdiv_rn.
__global__ void __launch_bounds__(256) k_check_reciprocal(unsigned long long* bad, uint32_t* first) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long mine = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (1ull << 32); i += stride) {
        const float x = __uint_as_float((uint32_t)i);
        const float a = rcp_rn(x), b = __frcp_rn(x);
        bool bad_x = __float_as_uint(a) != __float_as_uint(b) && !(a != a && b != b);
        // the pair form of the w-safe batches, on (x, -x): (-RN(1/x), RN(1/x))
        if ((((uint32_t)i & 0x7FFFFFFFu) - 0x00800000u) < 0x7E000000u) {
            float n0, n1;
            f2_unpack(f2_neg_rcp_rn_normal(f2_pack(x, -x), f2_pack(1.0f, 1.0f)), n0, n1);
            bad_x = bad_x || __float_as_uint(n0) != (__float_as_uint(b) ^ 0x80000000u) ||
                    __float_as_uint(n1) != __float_as_uint(b);
        }
        // the literal pair body's division for |x| in [2^-64, 2^64): two
        // quotients per x, one hard (next to a rounding midpoint) where x's
        // significand is odd (cr_divcheck.h)
        const uint32_t ef = ((uint32_t)i >> 23) & 0xFFu;
        if (ef >= 63u && ef <= 190u) {
            const float a0 = divcheck_numerator((uint32_t)i, true);
            const float a1 = divcheck_numerator((uint32_t)i, false);
            const uint64_t W = f2_pack(x, x);
            float nq0, nq1;
            f2_unpack(f2_neg_div_rn(f2_pack(a0, a1), W, f2_neg_rcp_rn_normal(W, f2_pack(1.0f, 1.0f))),
                      nq0, nq1);
            bad_x = bad_x || !divcheck_quotient_ok(__fdiv_rn(a0, x), nq0) ||
                    !divcheck_quotient_ok(__fdiv_rn(a1, x), nq1);
        }
        if (bad_x) {
            mine++;
            atomicMin(first, (uint32_t)i);
        }
    }
    if (mine) atomicAdd(bad, mine);
}

inline int blocks_for(int64_t n, int per) { return (int)((n + per - 1) / per); }

}  // namespace

int launch_file_records(const double view[16], const double proj[16], const double* box_min,
                        int32_t nfiles, FileRec* out, void* stream, int float_uniforms, int literal) {
    // the chunk travels by value in the kernel parameters: no staging buffer
    // whose lifetime would have to outlast the launch
    FileChunk c;
    c.float_uniforms = float_uniforms;
    c.literal = literal;
    for (int i = 0; i < 16; i++) {
        c.view[i] = view[i];
        c.proj[i] = proj[i];
    }
    for (int32_t first = 0; first < nfiles; first += kFilesPerLaunch) {
        c.first = first;
        c.count = std::min<int32_t>(kFilesPerLaunch, nfiles - first);
        for (int k = 0; k < 3 * c.count; k++) c.box_min[k] = box_min[3 * (int64_t)first + k];
        if (launch_k(k_file_records, blocks_for(c.count, 128), 128, (cudaStream_t)stream, c, out) != 0)
            return -1;
    }
    return 0;
}

int launch_cull(const ViewParams& vp, const cr_batch* batches, int64_t nb, int64_t capacity,
                int32_t quirks, uint32_t* scratch, void* stream, int64_t list_cap, int node_slices) {
    if (nb <= 0) return 0;
    return launch_k(k_cull, blocks_for(nb, 256), 256, (cudaStream_t)stream, vp, batches, nb,
                    capacity, quirks, scratch, list_cap < 0 ? nb : list_cap, (int32_t)node_slices);
}

template <int MODE, int PAYLOAD, int BLOCK, bool MANY, bool LIT>
static int occupancy_list1() {
    static const int n = [] {
        int k = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &k, k_batched<MODE, PAYLOAD, BLOCK, 1, MANY, LIT>, BLOCK, 0) == cudaSuccess && k > 0
                   ? k
                   : 1;
    }();
    return n;
}

// The (usually short) 20/30-bit list with a grid that is resident at once,
// then the 10-bit list as its programmatic dependent: it starts as soon as
// every list-1 CTA has started, on the SM room list 1 leaves.
template <int MODE, int PAYLOAD, int BLOCK, bool MANY, bool LIT = false>
static int launch_lists(const ViewParams& vp, const BatchedLaunch& bl, int grid, cudaStream_t s) {
    int device = 0, sms = 1;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return -1;
    const int grid1 = std::min(grid, sms * occupancy_list1<MODE, PAYLOAD, BLOCK, MANY, LIT>());
    PairParams pp;
    fill_pair_params(vp, &pp);
    if (launch_k(k_batched<MODE, PAYLOAD, BLOCK, 1, MANY, LIT>, grid1, BLOCK, s, vp, bl, pp) != 0) return -1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(BLOCK);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batched<MODE, PAYLOAD, BLOCK, 0, MANY, LIT>, vp, bl, pp) == cudaSuccess
               ? 0
               : -1;
}

template <int MODE, int PAYLOAD>
static int launch_batched_t(const ViewParams& vp, const BatchedLaunch& bl, int block, int grid,
                            cudaStream_t s) {
    // CR_QUIRK_LITERAL_ARITH, and clouds with more than kInlineFiles files:
    // 128-thread instances only
    if (bl.quirks & CR_QUIRK_LITERAL_ARITH) {
        if (vp.nfiles > kInlineFiles) return launch_lists<MODE, PAYLOAD, 128, true, true>(vp, bl, grid, s);
        return launch_lists<MODE, PAYLOAD, 128, false, true>(vp, bl, grid, s);
    }
    if (vp.nfiles > kInlineFiles) return launch_lists<MODE, PAYLOAD, 128, true>(vp, bl, grid, s);
    switch (block) {
        case 128: return launch_lists<MODE, PAYLOAD, 128, false>(vp, bl, grid, s);
        case 512: return launch_lists<MODE, PAYLOAD, 512, false>(vp, bl, grid, s);
        default: return launch_lists<MODE, PAYLOAD, 256, false>(vp, bl, grid, s);
    }
}

int launch_batched(const ViewParams& vp, const BatchedLaunch& bl, int block, int grid, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (bl.mode == kModeRaster) {
        if (bl.payload == CR_PAYLOAD_COLOR)
            return launch_batched_t<kModeRaster, CR_PAYLOAD_COLOR>(vp, bl, block, grid, s);
        return launch_batched_t<kModeRaster, CR_PAYLOAD_INDEX>(vp, bl, block, grid, s);
    }
    if (bl.mode == kModeHqsDepth) return launch_batched_t<kModeHqsDepth, CR_PAYLOAD_INDEX>(vp, bl, block, grid, s);
    return launch_batched_t<kModeHqsColor, CR_PAYLOAD_INDEX>(vp, bl, block, grid, s);
}

template <int MODE, int PAYLOAD>
static int occupancy_t(int block, bool many, bool literal) {
    int n = 0;
    cudaError_t e;
    if (literal) {
        e = many ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 128, 0, true, true>, 128, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 128, 0, false, true>, 128, 0);
        return e == cudaSuccess ? n : 1;
    }
    if (many) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 128, 0, true>, 128, 0);
        return e == cudaSuccess ? n : 1;
    }
    switch (block) {
        case 128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 128, 0, false>, 128, 0); break;
        case 512: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 512, 0, false>, 512, 0); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batched<MODE, PAYLOAD, 256, 0, false>, 256, 0); break;
    }
    return e == cudaSuccess ? n : 1;
}

int batched_blocks_per_sm(int mode, int payload, int block, bool many, bool literal) {
    if (mode == kModeRaster)
        return payload == CR_PAYLOAD_COLOR ? occupancy_t<kModeRaster, CR_PAYLOAD_COLOR>(block, many, literal)
                                           : occupancy_t<kModeRaster, CR_PAYLOAD_INDEX>(block, many, literal);
    if (mode == kModeHqsDepth) return occupancy_t<kModeHqsDepth, CR_PAYLOAD_INDEX>(block, many, literal);
    return occupancy_t<kModeHqsColor, CR_PAYLOAD_INDEX>(block, many, literal);
}

int launch_plain(const float T[16], int32_t W, int32_t H, const cr_vertex* v, int64_t n,
                 uint64_t* fb, int grid, int variant, void* stream, int literal) {
    if (n <= 0) return 0;
    PlainParams pp;
    for (int i = 0; i < 16; i++) pp.T[i] = T[i];
    pp.W = W;
    pp.H = H;
    int64_t need = (n + 255) / 256;
    if (need < grid) grid = (int)need;
    const uint4* v4 = reinterpret_cast<const uint4*>(v);
    cudaStream_t s = (cudaStream_t)stream;
    if (literal) {
        if (variant == 1) return launch_k(k_plain<256, 1, true>, grid, 256, s, pp, v4, n, fb);
        if (variant == 2) return launch_k(k_plain<256, 2, true>, grid, 256, s, pp, v4, n, fb);
        return launch_k(k_plain<256, 0, true>, grid, 256, s, pp, v4, n, fb);
    }
    if (variant == 1) return launch_k(k_plain<256, 1>, grid, 256, s, pp, v4, n, fb);
    if (variant == 2) return launch_k(k_plain<256, 2>, grid, 256, s, pp, v4, n, fb);
    return launch_k(k_plain<256, 0>, grid, 256, s, pp, v4, n, fb);
}

int launch_resolve_index(int32_t W, int32_t H, uint64_t* fb, const uint32_t* rgba,
                         int64_t rgba_words, uint32_t* image, int clear_after, uint64_t clear,
                         void* stream, int tiles) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = (P + 1) / 2 > tail ? (P + 1) / 2 : tail;
    return launch_k(k_resolve_index, blocks_for(threads, 256), 256, (cudaStream_t)stream, P, tail,
                    fb, rgba, rgba_words, image, clear_after, clear, W, H, tiles);
}

int launch_resolve_color(int32_t W, int32_t H, uint64_t* fb, uint32_t* image, int clear_after,
                         uint64_t clear, void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = (P + 1) / 2 > tail ? (P + 1) / 2 : tail;
    return launch_k(k_resolve_color, blocks_for(threads, 256), 256, (cudaStream_t)stream, P, tail,
                    fb, image, clear_after, clear);
}

int launch_resolve_plain(int32_t W, int32_t H, uint64_t* fb, uint32_t* image, int clear_after,
                         uint64_t clear, int tiles, int zero_rule, void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = P > tail ? P : tail;
    return launch_k(k_resolve_plain, blocks_for(threads, 256), 256, (cudaStream_t)stream, P, tail,
                    W, H, tiles, zero_rule, fb, image, clear_after, clear);
}

int launch_resolve_hqs(int32_t W, int32_t H, uint32_t* depth, uint64_t* accum, uint32_t* image,
                       int clear_after, void* stream) {
    int64_t P = (int64_t)W * H, tail = (int64_t)W + 1;
    int64_t threads = P > tail ? P : tail;
    return launch_k(k_resolve_hqs, blocks_for(threads, 256), 256, (cudaStream_t)stream, P, tail,
                    depth, accum, image, clear_after);
}

int launch_check_reciprocal(uint64_t* bad, uint32_t* first) {
    int device = 0, sms = 1;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return -1;
    if (launch_k(k_check_reciprocal, sms * 8, 256, (cudaStream_t)0,
                 reinterpret_cast<unsigned long long*>(bad), first) != 0)
        return -1;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

int launch_fill_u64(uint64_t* p, int64_t n, uint64_t v, void* stream) {
    if (n <= 0) return 0;
    int grid = blocks_for(n, 256);
    if (grid > 65535) grid = 65535;
    return launch_k(k_fill_u64, grid, 256, (cudaStream_t)stream, p, n, v);
}

int launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, void* stream) {
    if (n <= 0) return 0;
    int grid = blocks_for(n, 256);
    if (grid > 65535) grid = 65535;
    return launch_k(k_fill_u32, grid, 256, (cudaStream_t)stream, p, n, v);
}

}  // namespace cr
