// cr_multiview.cu -- many views of one cloud in one persistent launch
// (include/cr_raster.h, cr_mv_*), generalising the two-eye fetch of
// compute_loop_las_hqs_vr/depth.cs:374-412 to groups of up to 8 views.
//
//   k_mv_cull    one thread per (batch, view group): frustum test and
//                precision level per view; appends {batch, group, visible
//                mask, 3-bit level per view, w-safe bit per view at 24 + s}
//                to a work list.
//   k_mv_raster  persistent CTAs pull (batch, group) items, read the batch's
//                points once with 128-bit loads, decode them, and project and
//                splat every point into each visible view of the group at that
//                view's own level, through the per-CTA z-cache (tags are the
//                view's word offset plus the pixel id).
//   k_mv_resolve every view's pixels (grid y = view), fused re-clear.
// The arithmetic is the single-view kernels' (cr_device.cuh), so each view's
// framebuffer equals a cr_render of that view alone, bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cr_device.cuh"
#include "cr_filerec.h"
#include "cr_internal.h"

namespace cr {
namespace {

struct MVArgs {
    const MVView* views;
    const MVFile* files;
    int32_t nviews, nfiles, G;
    const cr_batch* batches;
    const uint32_t* lo;
    const uint32_t* md;
    const uint32_t* hi;
    const uint32_t* rgba;
    unsigned long long* fbs;
    uint32_t* scratch;
    int64_t list_cap;  // uint4 items in the list region: batches x groups
    int32_t quirks;
    const uint32_t* pairs;  // per group: bit s = views s, s + 1 share rows y and w (or NULL)
};

constexpr int kSlotWords = 16;  // per view slot in shared memory: T[12], Wf, Hf, W, fb_off

// The 12 transform entries of a view's T that the projection uses.
__host__ __device__ inline void mv_file_from_rec(const FileRec& r, MVFile* o) {
    const int pick[12] = {0, 1, 3, 4, 5, 7, 8, 9, 11, 12, 13, 15};
    for (int k = 0; k < 12; k++) o->T[k] = r.T[pick[k]];
    for (int k = 0; k < 24; k++) o->planes[k] = r.planes[k];
    for (int k = 0; k < 16; k++) o->VW[k] = r.VW[k];
}

// Per (view, file) records of a frame for clouds with more than kInlineFiles
// files (grid x: files, grid y strides over the views): the host's
// file_record on the device, bit for bit (cr_filerec.h).
__global__ void __launch_bounds__(128) k_mv_file_records(const double* __restrict__ mats,
                                                         const double* __restrict__ box,
                                                         int32_t nviews, int32_t nfiles,
                                                         MVFile* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfiles) return;
    double bmin[3];
    for (int k = 0; k < 3; k++) bmin[k] = box[3 * (int64_t)f + k];
    for (int v = blockIdx.y; v < nviews; v += gridDim.y) {
        double view[16], proj[16];
        for (int k = 0; k < 16; k++) {
            view[k] = mats[32 * (int64_t)v + k];
            proj[k] = mats[32 * (int64_t)v + 16 + k];
        }
        FileRec r;
        file_record(view, proj, bmin, &r);
        mv_file_from_rec(r, &out[(int64_t)v * nfiles + f]);
    }
}

__global__ void __launch_bounds__(256) k_mv_cull(const MVView* __restrict__ views,
                                                 const MVFile* __restrict__ files, int32_t nviews,
                                                 int32_t nfiles, int32_t G, int32_t ngroups,
                                                 const cr_batch* __restrict__ batches, int64_t nb,
                                                 int64_t capacity, int32_t quirks, int32_t culling,
                                                 int32_t lod_skip_level,
                                                 uint32_t* __restrict__ scratch) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    uint4 item = make_uint4(0, 0, 0, 0);
    if (idx < nb * ngroups) {
        const int64_t b = idx / ngroups;
        const int32_t g = (int32_t)(idx - b * ngroups);
        const int4* r4 = reinterpret_cast<const int4*>(batches + b);
        const int4 a = __ldg(r4), c = __ldg(r4 + 1), d = __ldg(r4 + 2);
        const float mnx = __int_as_float(a.y), mny = __int_as_float(a.z), mnz = __int_as_float(a.w);
        const float mxx = __int_as_float(c.x), mxy = __int_as_float(c.y), mxz = __int_as_float(c.z);
        const int32_t np = c.w, fp = d.x, fi = d.y;
        const int64_t count = points_in_batch(np, fp, quirks);
        const bool ok = np >= 0 && np <= kPointsPerBatch && fp >= 0 &&
                        (int64_t)fp + count + 4 <= capacity && fi >= 0 && fi < nfiles;
        if (!ok) {
            atomicOr(&scratch[kErrWord], kErrBadBatch);
        } else if (count > 0) {
            uint32_t vismask = 0, levels = 0;
            for (int s = 0; s < G; s++) {
                const int v = g * G + s;
                if (v >= nviews) break;
                const MVFile& f = files[(int64_t)v * nfiles + fi];
                const MVView& vw = views[v];
                if (culling && !intersects_frustum(f.planes, mnx, mny, mnz, mxx, mxy, mxz)) continue;
                const int level = precision_level(vw.P, f.VW, vw.W, vw.H, mnx, mny, mnz, mxx, mxy, mxz);
                if (lod_skip_level > 0 && level >= lod_skip_level) continue;  // nodes/render.cs:273
                vismask |= 1u << s;
                levels |= (uint32_t)level << (3 * s);
                // bit 24 + s: view s's clip w is proven to lie in [2^-120, 2^120]
                float tw[16];
                tw[3] = f.T[2];
                tw[7] = f.T[5];
                tw[11] = f.T[8];
                tw[15] = f.T[11];
                if (w_safe(tw, mnx, mny, mnz, mxx, mxy, mxz)) levels |= 1u << (24 + s);
            }
            keep = vismask != 0;
            item = make_uint4((uint32_t)b, (uint32_t)g, vismask, levels);
        }
    }
    // items whose visible views all decode at 10 bit to the front of the list
    // region, the others to the back (their kernel instance decodes 20/30 bit)
    bool all10 = true;
    for (int s = 0; s < G; s++)
        if (((item.z >> s) & 1u) && ((item.w >> (3 * s)) & 7u) < 2u) all10 = false;
    const bool front = keep && all10;
    const bool back = keep && !all10;
    uint4* list = reinterpret_cast<uint4*>(scratch + kScratchHead);
    const int64_t cap = nb * ngroups;
    const uint32_t lane = lane_id();
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t mf = __ballot_sync(kFull, front);
    if (mf) {
        const uint32_t leader = __ffs(mf) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&scratch[kItemCount], __popc(mf));
        base = __shfl_sync(kFull, base, leader);
        if (front) list[base + __popc(mf & below)] = item;
    }
    const uint32_t mb = __ballot_sync(kFull, back);
    if (mb) {
        const uint32_t leader = __ffs(mb) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&scratch[kItemCount2], __popc(mb));
        base = __shfl_sync(kFull, base, leader);
        if (back) list[cap - 1 - (int64_t)(base + __popc(mb & below))] = item;
    }
}

__device__ __forceinline__ void emit_mv(unsigned long long* fbs, unsigned long long* zc, bool ok,
                                        int32_t pix, uint32_t fb_off, uint32_t wbits,
                                        uint32_t payload) {
    const uint32_t tag = fb_off + (uint32_t)pix;
    const uint32_t slot = zslot(tag);
    const bool cand = ok && !zcache_rejects(zc, slot, tag, wbits);
    if (__any_sync(kFull, cand) && cand)
        submit_min<unsigned long long>(fbs + tag, zc, slot, tag,
                                       ((unsigned long long)wbits << 32) | payload, wbits);
}

struct Decoded {
    float x[4], y[4], z[4];
};

// Decodes the thread's 4 points at level class LC (2: 10 bit, 1: 20 bit, 0: 30 bit).
__device__ __forceinline__ void decode4(int LC, const uint4& w4, const uint4& w8, const uint4& w12,
                                        float mnx, float mny, float mnz, const float* s,
                                        bool l0_x12, Decoded& o) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint32_t a = u4get(w4, j);
        if (LC == 2) {
            o.x[j] = __fmaf_rn(small_u2f(a & 1023u), s[0], mnx);
            o.y[j] = __fmaf_rn(small_u2f((a >> 10) & 1023u), s[1], mny);
            o.z[j] = __fmaf_rn(small_u2f((a >> 20) & 1023u), s[2], mnz);
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
            o.x[j] = __fmaf_rn(__uint2float_rn(X), s[3], mnx);
            o.y[j] = __fmaf_rn(__uint2float_rn(Y), s[4], mny);
            o.z[j] = __fmaf_rn(__uint2float_rn(Z), s[5], mnz);
        }
    }
}

__device__ __forceinline__ int level_class(int level) { return level >= 2 ? 2 : level; }

// Projects the 4 decoded points into the view in shared-memory slot `sv` and
// splats them.  The slot holds T[12], then (Wf, Hf, W, fb_off), 16-byte aligned.
template <int PAYLOAD, bool SAFE>
__device__ __forceinline__ void splat_view(const MVArgs& a, unsigned long long* zc, const float* sv,
                                           const Decoded& d, uint32_t valid_mask, uint32_t idx0,
                                           const uint4& col) {
    const float4 t0 = reinterpret_cast<const float4*>(sv)[0];
    const float4 t1 = reinterpret_cast<const float4*>(sv)[1];
    const float4 t2 = reinterpret_cast<const float4*>(sv)[2];
    const float4 t3 = reinterpret_cast<const float4*>(sv)[3];
    BatchCtx c;
    c.T0 = t0.x; c.T1 = t0.y; c.T3 = t0.z; c.T4 = t0.w;
    c.T5 = t1.x; c.T7 = t1.y; c.T8 = t1.z; c.T9 = t1.w;
    c.T11 = t2.x; c.T12 = t2.y; c.T13 = t2.z; c.T15 = t2.w;
    c.Wf = t3.x;
    c.Hf = t3.y;
    c.W = __float_as_int(t3.z);
    const uint32_t fb_off = __float_as_uint(t3.w);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int32_t pix;
        uint32_t wbits;
        const bool ok = project<SAFE>(c, d.x[j], d.y[j], d.z[j], pix, wbits) && ((valid_mask >> j) & 1u);
        const uint32_t payload = (PAYLOAD == CR_PAYLOAD_COLOR) ? u4get(col, j) : idx0 + (uint32_t)j;
        emit_mv(a.fbs, zc, ok, pix, fb_off, wbits, payload);
    }
}

// Two views whose T rows y and w are bitwise equal (a stereo pair built as
// translate(-+ipd/2, 0, 0) * V_head, whose eyes differ in row x only) and whose
// slots hold the same Wf, Hf and W: y, w, 1/w, the inside test of y and the
// pixel row are computed once per point, x and the pixel column per view.
// Every value is the one splat_view computes (same operations, same operands),
// so both views' words are unchanged.
template <int PAYLOAD, bool SAFE>
__device__ __forceinline__ void splat_pair(const MVArgs& a, unsigned long long* zc, const float* sa,
                                           const float* sb, const Decoded& d, uint32_t valid_mask,
                                           uint32_t idx0, const uint4& col) {
    const float4 t0 = reinterpret_cast<const float4*>(sa)[0];
    const float4 t1 = reinterpret_cast<const float4*>(sa)[1];
    const float4 t2 = reinterpret_cast<const float4*>(sa)[2];
    const float4 t3 = reinterpret_cast<const float4*>(sa)[3];
    const float4 u0 = reinterpret_cast<const float4*>(sb)[0];
    const float4 u1 = reinterpret_cast<const float4*>(sb)[1];
    const float4 u2 = reinterpret_cast<const float4*>(sb)[2];
    const float4 u3 = reinterpret_cast<const float4*>(sb)[3];
    // slot layout T0 T1 T3 T4 | T5 T7 T8 T9 | T11 T12 T13 T15 | Wf Hf W fb_off
    const float aT0 = t0.x, aT1 = t0.y, aT3 = t0.z, aT4 = t0.w, aT5 = t1.x, aT7 = t1.y, aT8 = t1.z;
    const float aT9 = t1.w, aT11 = t2.x, aT12 = t2.y, aT13 = t2.z, aT15 = t2.w;
    const float bT0 = u0.x, bT4 = u0.w, bT8 = u1.z, bT12 = u2.y;
    const float Wf = t3.x, Hf = t3.y;
    const int32_t W = __float_as_int(t3.z);
    const uint32_t fa = __float_as_uint(t3.w), fb = __float_as_uint(u3.w);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float x = d.x[j], y = d.y[j], z = d.z[j];
        const float py = __fmaf_rn(aT9, z, __fmaf_rn(aT5, y, __fmaf_rn(aT1, x, aT13)));
        const float pw = __fmaf_rn(aT11, z, __fmaf_rn(aT7, y, __fmaf_rn(aT3, x, aT15)));
        const float rw = SAFE ? rcp_rn_normal(pw) : rcp_rn(pw);
        const float qy = fmul(py, rw);
        const bool yin = ((valid_mask >> j) & 1u) && (SAFE || pw > 0.0f) && qy >= -1.0f && qy <= 1.0f;
        const int32_t row = small_f2i(fmul(__fmaf_rn(qy, 0.5f, 0.5f), Hf)) * W;
        const uint32_t wbits = __float_as_uint(pw);
        const uint32_t payload = (PAYLOAD == CR_PAYLOAD_COLOR) ? u4get(col, j) : idx0 + (uint32_t)j;
        const float pxa = __fmaf_rn(aT8, z, __fmaf_rn(aT4, y, __fmaf_rn(aT0, x, aT12)));
        const float qxa = fmul(pxa, rw);
        const bool oka = yin && qxa >= -1.0f && qxa <= 1.0f;
        emit_mv(a.fbs, zc, oka, small_f2i(fmul(__fmaf_rn(qxa, 0.5f, 0.5f), Wf)) + row, fa, wbits, payload);
        const float pxb = __fmaf_rn(bT8, z, __fmaf_rn(bT4, y, __fmaf_rn(bT0, x, bT12)));
        const float qxb = fmul(pxb, rw);
        const bool okb = yin && qxb >= -1.0f && qxb <= 1.0f;
        emit_mv(a.fbs, zc, okb, small_f2i(fmul(__fmaf_rn(qxb, 0.5f, 0.5f), Wf)) + row, fb, wbits, payload);
    }
}

// LIST 0: items whose visible views all decode at 10 bit (only the low word
// stream is read); LIST 1: the others, each view decoded at its own level.
template <int PAYLOAD, int BLOCK, int LIST>
__device__ __forceinline__ void mv_raster_items(const MVArgs& a) {
    __shared__ uint32_t s_item[2];
    __shared__ __align__(16) float s_view[CR_MV_MAX_GROUP][kSlotWords];
    __shared__ unsigned long long s_zc[kZCacheSlots];
    uint32_t* cursor = a.scratch + (LIST == 0 ? kCursor0 : kCursor2);
    const uint32_t nitems =
        *reinterpret_cast<volatile uint32_t*>(a.scratch + (LIST == 0 ? kItemCount : kItemCount2));
    if (nitems == 0) return;
    const uint4* items = reinterpret_cast<const uint4*>(a.scratch + kScratchHead);
    for (int i = threadIdx.x; i < kZCacheSlots; i += BLOCK) s_zc[i] = 0xFFFFFFFFull;
    if (threadIdx.x == 0) s_item[0] = atomicAdd(cursor, 1u);
    __syncthreads();
    const bool l0_x12 = (a.quirks & CR_QUIRK_L0_X12) != 0;
    int buf = 0;
    while (true) {
        const uint32_t wi = s_item[buf];
        if (wi >= nitems) break;
        if (threadIdx.x == 0) s_item[buf ^ 1] = atomicAdd(cursor, 1u);
        const uint4 it = items[LIST == 0 ? (int64_t)wi : a.list_cap - 1 - (int64_t)wi];
        const uint32_t b = it.x, g = it.y, vismask = it.z, levels = it.w;
        const int4* r4 = reinterpret_cast<const int4*>(a.batches + b);
        const int4 ra = __ldg(r4), rc = __ldg(r4 + 1), rd = __ldg(r4 + 2);
        const float mnx = __int_as_float(ra.y), mny = __int_as_float(ra.z), mnz = __int_as_float(ra.w);
        const float mxx = __int_as_float(rc.x), mxy = __int_as_float(rc.y), mxz = __int_as_float(rc.z);
        const int64_t first = rd.x;
        const int32_t count = (int32_t)points_in_batch(rc.w, rd.x, a.quirks);
        const int fi = rd.y;
        // the group's visible views into shared memory
        for (int t = threadIdx.x; t < a.G * kSlotWords; t += BLOCK) {
            const int s = t / kSlotWords, k = t - s * kSlotWords;
            const int v = (int)g * a.G + s;
            if (((vismask >> s) & 1u) == 0u || v >= a.nviews) continue;
            float val;
            if (k < 12) val = a.files[(int64_t)v * a.nfiles + fi].T[k];
            else if (k == 12) val = (float)a.views[v].W;
            else if (k == 13) val = (float)a.views[v].H;
            else if (k == 14) val = __int_as_float(a.views[v].W);
            else val = __uint_as_float(a.views[v].fb_off);
            s_view[s][k] = val;
        }
        __syncthreads();
        uint32_t classes = 0;
        if (LIST == 1)
            for (int s = 0; s < a.G; s++)
                if ((vismask >> s) & 1u) classes |= 1u << level_class((levels >> (3 * s)) & 7u);
        const bool single = LIST == 0 || __popc(classes) == 1;
        const int only = LIST == 0 ? 2 : __ffs(classes) - 1;
        // shared pairs of this item: both views visible, at one level class,
        // with the same w-range proof
        uint32_t pairs = 0;
        if (a.pairs) {
            const uint32_t cand = a.pairs[g] & vismask & (vismask >> 1);
            for (int s = 0; s + 1 < a.G; s++) {
                if (((cand >> s) & 1u) == 0u) continue;
                const bool same_level =
                    LIST == 0 || level_class((levels >> (3 * s)) & 7u) == level_class((levels >> (3 * s + 3)) & 7u);
                const bool same_safe = (((levels >> (24 + s)) ^ (levels >> (25 + s))) & 1u) == 0u;
                if (same_level && same_safe) pairs |= 1u << s;
            }
        }
        const bool need8 = LIST == 1 && (classes & 3u) != 0;
        const bool need12 = LIST == 1 && (classes & 1u) != 0;
        float sc[6];
        const float sx = fsub(mxx, mnx), sy = fsub(mxy, mny), sz = fsub(mxz, mnz);
        // size / 1024 and size / 2^30 as products with the exact reciprocals
        // (the same real value, so the same rounding for every input)
        sc[0] = fmul(sx, 0x1p-10f); sc[1] = fmul(sy, 0x1p-10f); sc[2] = fmul(sz, 0x1p-10f);
        sc[3] = fmul(sx, 0x1p-30f); sc[4] = fmul(sy, 0x1p-30f); sc[5] = fmul(sz, 0x1p-30f);

        const int64_t v0 = first >> 2;
        const int32_t head = (int32_t)(first & 3);
        // CR_QUIRK_UVEC4_BASE (las2/render.cs:319-341), as in the single-view
        // raster: with firstPoint % 4 != 0 the vectors v % 128 == 0 (the
        // reference's thread 0) are skipped and none past 2559 is read
        const bool uvec4 = head != 0 && (a.quirks & CR_QUIRK_UVEC4_BASE) != 0;
        const int nv = uvec4 ? min((head + count + 3) >> 2, kPointsPerBatch / 4) : (head + count + 3) >> 2;
        const uint32_t index0 = (uint32_t)(first - head);
        const uint4* lo4 = reinterpret_cast<const uint4*>(a.lo) + v0;
        const uint4* md4 = reinterpret_cast<const uint4*>(a.md) + v0;
        const uint4* hi4 = reinterpret_cast<const uint4*>(a.hi) + v0;
        const uint4* co4 = reinterpret_cast<const uint4*>(a.rgba) + v0;
        const uint4 zero = make_uint4(0, 0, 0, 0);
        uint4 n4 = zero, n8 = zero, n12 = zero, ncol = zero;
        if ((int)threadIdx.x < nv) {
            n4 = ld_stream(lo4 + threadIdx.x);
            if (need8) n8 = ld_stream(md4 + threadIdx.x);
            if (need12) n12 = ld_stream(hi4 + threadIdx.x);
            if (PAYLOAD == CR_PAYLOAD_COLOR) ncol = ld_stream(co4 + threadIdx.x);
        }
        for (int base = 0; base < nv; base += BLOCK) {
            const int v = base + (int)threadIdx.x;
            const uint4 w4 = n4, w8 = n8, w12 = n12, col = ncol;
            const int vn = v + BLOCK;
            if (vn < nv) {
                n4 = ld_stream(lo4 + vn);
                if (need8) n8 = ld_stream(md4 + vn);
                if (need12) n12 = ld_stream(hi4 + vn);
                if (PAYLOAD == CR_PAYLOAD_COLOR) ncol = ld_stream(co4 + vn);
            }
            const int32_t rel0 = 4 * v - head;
            uint32_t valid_mask = 0;
#pragma unroll
            for (int j = 0; j < 4; j++)
                valid_mask |= ((uint32_t)(rel0 + j) < (uint32_t)count ? 1u : 0u) << j;
            if (uvec4 && (v & 127) == 0) valid_mask = 0;
            const uint32_t idx0 = index0 + 4u * (uint32_t)v;
            Decoded d;
            if (LIST == 0) decode4(2, w4, w8, w12, mnx, mny, mnz, sc, l0_x12, d);
            else if (single) decode4(only, w4, w8, w12, mnx, mny, mnz, sc, l0_x12, d);
            for (int s = 0; s < a.G; s++) {
                if (((vismask >> s) & 1u) == 0u) continue;
                if (LIST == 1 && !single)
                    decode4(level_class((levels >> (3 * s)) & 7u), w4, w8, w12, mnx, mny, mnz, sc,
                            l0_x12, d);
                // views whose w range is proven safe skip the reciprocal's range
                // test (measured 12 % faster on the 64-view frame)
                const bool safe = (levels >> (24 + s)) & 1u;
                if ((pairs >> s) & 1u) {
                    if (safe)
                        splat_pair<PAYLOAD, true>(a, s_zc, s_view[s], s_view[s + 1], d, valid_mask, idx0, col);
                    else
                        splat_pair<PAYLOAD, false>(a, s_zc, s_view[s], s_view[s + 1], d, valid_mask, idx0, col);
                    s++;
                } else if (safe) {
                    splat_view<PAYLOAD, true>(a, s_zc, s_view[s], d, valid_mask, idx0, col);
                } else {
                    splat_view<PAYLOAD, false>(a, s_zc, s_view[s], d, valid_mask, idx0, col);
                }
            }
        }
        __syncthreads();
        buf ^= 1;
    }
}

// List 1 is launched first and lets the list-0 grid start at once
// (programmatic dependent launch); every list-0 CTA waits for the list-1 grid
// before it exits, so the resolve that follows sees both lists' writes.
template <int PAYLOAD, int BLOCK, int LIST>
__global__ void __launch_bounds__(BLOCK) k_mv_raster(MVArgs a) {
    if (LIST == 1) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    mv_raster_items<PAYLOAD, BLOCK, LIST>(a);
    if (LIST == 0) asm volatile("griddepcontrol.wait;" ::: "memory");
}

__global__ void k_mv_resolve(const MVView* __restrict__ views, unsigned long long* fbs,
                             uint32_t* images, const uint32_t* __restrict__ rgba,
                             int64_t rgba_words, int32_t payload, int32_t clear_after,
                             unsigned long long clear) {
    const MVView vw = views[blockIdx.y];
    const int64_t P = (int64_t)vw.W * vw.H, tail = (int64_t)vw.W + 1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long* fb = fbs + vw.fb_off;
    if (t < P) {
        const unsigned long long w = fb[t];
        const float dpt = __uint_as_float((uint32_t)(w >> 32));
        const bool valid = dpt > 0.0f && dpt < 1000000.0f;  // resolve.cs:124
        uint32_t out;
        if (payload == CR_PAYLOAD_COLOR) {
            out = valid ? (uint32_t)w : kBackground;
        } else {
            const uint32_t id = valid ? (uint32_t)w : 0u;
            out = (id == 0u || id >= rgba_words) ? kBackground : __ldg(rgba + id);
        }
        images[vw.img_off + t] = out;
        if (clear_after) fb[t] = clear;
    }
    if (clear_after && t < tail) fb[P + t] = clear;
}

__global__ void k_mv_fill(unsigned long long* p, int64_t n, unsigned long long v) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// The clear of compute_loop_las.h:288-301 for every view of a frame (grid y =
// view): W*H+W+1 words each, the guard tail included.
__global__ void k_mv_fill_views(const MVView* __restrict__ views, unsigned long long* fbs,
                                unsigned long long v) {
    const MVView vw = views[blockIdx.y];
    const int64_t n = (int64_t)vw.W * vw.H + vw.W + 1;
    unsigned long long* fb = fbs + vw.fb_off;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        fb[i] = v;
}

// The 10-bit list, then the 20/30-bit list, on one stream.
template <int PAYLOAD, int BLOCK>
int mv_occupancy_list1() {
    static const int n = [] {
        int k = 0;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_mv_raster<PAYLOAD, BLOCK, 1>, BLOCK,
                                                             0) == cudaSuccess && k > 0
                   ? k
                   : 1;
    }();
    return n;
}

// The 20/30-bit list with a grid that is resident at once, then the 10-bit
// list as its programmatic dependent.
template <int PAYLOAD, int BLOCK>
cudaError_t launch_mv_lists(const MVArgs& a, int grid, cudaStream_t s) {
    int device = 0, sms = 1;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int grid1 = std::min(grid, sms * mv_occupancy_list1<PAYLOAD, BLOCK>());
    if (launch_k(k_mv_raster<PAYLOAD, BLOCK, 1>, grid1, BLOCK, s, a) != 0) return cudaErrorLaunchFailure;
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
    return cudaLaunchKernelEx(&cfg, k_mv_raster<PAYLOAD, BLOCK, 0>, a);
}

template <int PAYLOAD>
cudaError_t launch_mv_raster_t(const MVArgs& a, int block, int grid, cudaStream_t s) {
    switch (block) {
        case 64: return launch_mv_lists<PAYLOAD, 64>(a, grid, s);
        case 256: return launch_mv_lists<PAYLOAD, 256>(a, grid, s);
        default: return launch_mv_lists<PAYLOAD, 128>(a, grid, s);
    }
}

template <int PAYLOAD>
int mv_occupancy_t(int block) {
    int n = 0;
    cudaError_t e;
    switch (block) {
        case 64: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mv_raster<PAYLOAD, 64, 0>, 64, 0); break;
        case 256: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mv_raster<PAYLOAD, 256, 0>, 256, 0); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mv_raster<PAYLOAD, 128, 0>, 128, 0); break;
    }
    return e == cudaSuccess && n > 0 ? n : 1;
}

int64_t dispatched(const CloudInfo& ci, int quirks) {
    int64_t nb = ci.nb;
    if (quirks & CR_QUIRK_DISPATCH_BY_POINTS)
        nb = std::min<int64_t>(nb, (ci.n + kPointsPerBatch - 1) / kPointsPerBatch);
    return nb;
}

}  // namespace

int64_t mv_scratch_words(int64_t nb, int64_t nviews) { return kScratchHead + 4 * nb * nviews + 64; }

cr_status mv_fill_view(const cr_view* view, const CloudInfo& ci, MVView* out_view,
                       MVFile* out_files) {
    ViewParams vp;
    cr_status s = view_params_for(view, ci.box_min, ci.nfiles, 1, &vp);
    if (s != CR_OK) return s;
    std::memcpy(out_view->P, vp.P, sizeof(vp.P));
    out_view->W = view->width;
    out_view->H = view->height;
    if (ci.nfiles <= kInlineFiles)
        for (int f = 0; f < ci.nfiles; f++) mv_file_from_rec(vp.files[f], &out_files[f]);
    return CR_OK;
}

cr_status mv_enqueue(const MVFrame& f, void* stream, const char** what) {
    cudaStream_t st = (cudaStream_t)stream;
    auto fail = [&](const char* w) {
        if (what) *what = w;
        return CR_ERR_CUDA;
    };
    if (cudaMemsetAsync(f.scratch, 0, kCounterWords * 4, st) != cudaSuccess) return fail("counter reset");
    const int64_t words = std::max<int64_t>(f.max_words, 1);
    if (f.clear_before) {
        const unsigned gx = (unsigned)std::min<int64_t>((words + 255) / 256, 4096);
        if (launch_k(k_mv_fill_views, dim3(gx, (unsigned)f.nviews), 256, st, f.d_views,
                     reinterpret_cast<unsigned long long*>(f.fbs), f.clear_value) != 0)
            return fail("fill launch");
    }
    const int G = std::max(1, std::min(f.G, f.nviews));
    const int ngroups = (f.nviews + G - 1) / G;
    const int64_t nb = dispatched(f.ci, f.quirks);
    const int64_t threads = nb * ngroups;
    if (f.ci.nfiles > kInlineFiles) {
        if (!f.d_mats || !f.d_box) return fail("file records");
        const unsigned gy = (unsigned)std::min(f.nviews, 65535);
        if (launch_k(k_mv_file_records, dim3((unsigned)((f.ci.nfiles + 127) / 128), gy), 128, st,
                     f.d_mats, f.d_box, f.nviews, f.ci.nfiles, const_cast<MVFile*>(f.d_files)) != 0)
            return fail("file record launch");
    }
    if (threads > 0) {
        if (launch_k(k_mv_cull, (unsigned)((threads + 255) / 256), 256, st, f.d_views, f.d_files,
                     f.nviews, f.ci.nfiles, G, ngroups, f.ci.batches, nb, f.ci.capacity, f.quirks,
                     f.culling, f.lod_skip_level, f.scratch) != 0)
            return fail("cull launch");
        MVArgs a;
        a.views = f.d_views;
        a.files = f.d_files;
        a.nviews = f.nviews;
        a.nfiles = f.ci.nfiles;
        a.G = G;
        a.batches = f.ci.batches;
        a.lo = f.ci.lo;
        a.md = f.ci.md;
        a.hi = f.ci.hi;
        a.rgba = f.ci.rgba;
        a.fbs = reinterpret_cast<unsigned long long*>(f.fbs);
        a.scratch = f.scratch;
        a.list_cap = threads;  // k_mv_cull's list region: one item per (batch, group)
        a.quirks = f.quirks;
        a.pairs = f.d_pairs;
        const bool color = f.payload == CR_PAYLOAD_COLOR;
        const int per_sm = f.ctas_per_sm > 0 ? f.ctas_per_sm
                           : (color ? mv_occupancy_t<CR_PAYLOAD_COLOR>(f.block)
                                    : mv_occupancy_t<CR_PAYLOAD_INDEX>(f.block));
        const int grid = f.num_sms * per_sm;
        const cudaError_t e = color ? launch_mv_raster_t<CR_PAYLOAD_COLOR>(a, f.block, grid, st)
                                    : launch_mv_raster_t<CR_PAYLOAD_INDEX>(a, f.block, grid, st);
        if (e != cudaSuccess) return fail("raster launch");
    }
    if (f.resolve) {
        const unsigned gx = (unsigned)((words + 255) / 256);
        if (launch_k(k_mv_resolve, dim3(gx, (unsigned)f.nviews), 256, st, f.d_views,
                     reinterpret_cast<unsigned long long*>(f.fbs), f.images, f.ci.rgba, f.ci.capacity,
                     f.payload, f.clear_after, f.clear_value) != 0)
            return fail("resolve launch");
    }
    return CR_OK;
}

}  // namespace cr

using namespace cr;

struct cr_mv {
    cr_ctx* ctx = nullptr;
    const cr_cloud* cloud = nullptr;
    CloudInfo ci{};            // refreshed every frame (the loaded counts may grow)
    int64_t graph_n = -1, graph_nb = -1;  // loaded counts the captured graph dispatches
    int32_t nviews = 0;
    std::vector<int32_t> W, H;
    std::vector<int64_t> fb_off, img_off;
    int64_t total_words = 0, total_pixels = 0, max_words = 0;
    unsigned long long* fbs = nullptr;
    uint32_t* images = nullptr;
    MVView* d_views = nullptr;
    MVFile* d_files = nullptr;
    MVView* h_views = nullptr;  // pinned staging
    MVFile* h_files = nullptr;  // clouds of at most kInlineFiles files
    double* h_mats = nullptr;   // clouds with more files: view + proj per view,
    double* d_mats = nullptr;   // and every file's boxMin, from which each frame
    double* h_box = nullptr;    // computes d_files on the GPU
    double* d_box = nullptr;
    std::vector<uint8_t> eq_next;  // view v shares rows y and w with view v + 1
    uint32_t* h_pairs = nullptr;   // per group: bit s pairs views s, s + 1 (pinned)
    uint32_t* d_pairs = nullptr;
    int32_t shared_pairs = 0;
    uint32_t* scratch = nullptr;
    int num_sms = 0;
    cr_render_params params{};
    int G = 8, ngroups = 1, block = 128, quirks = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;
    bool pending = false;
    bool views_set = false;
    std::string err;
};

namespace {

cr_status mv_fail(cr_mv* mv, cr_status s, const std::string& msg) {
    if (mv) mv->err = msg;
    return s;
}

cr_status mv_cuda(cr_mv* mv, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return CR_OK;
    return mv_fail(mv, e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

void drop_graph(cr_mv* mv) {
    if (mv->exec) cudaGraphExecDestroy(mv->exec);
    if (mv->graph) cudaGraphDestroy(mv->graph);
    mv->exec = nullptr;
    mv->graph = nullptr;
}

// Greedy disjoint pairs (s, s + 1) inside each group of G views.
void update_pairs(cr_mv* mv) {
    if (!mv->h_pairs) return;
    mv->shared_pairs = 0;
    for (int g = 0; g < mv->ngroups; g++) {
        uint32_t mask = 0;
        for (int s = 0; s + 1 < mv->G; s++) {
            const int v = g * mv->G + s;
            if (v + 1 >= mv->nviews) break;
            if (mv->eq_next.size() > (size_t)v && mv->eq_next[v]) {
                mask |= 1u << s;
                ++mv->shared_pairs;
                ++s;
            }
        }
        mv->h_pairs[g] = mask;
    }
}

// Views v and v + 1 share their projected y, w: equal size and proj * view
// rows 1 and 3 bitwise equal.  Every file's transform row r is computed from
// row r of proj * view and the file's boxMin alone (file_record:
// (proj * view) * translate(boxMin)), so the float rows y and w of all the
// files' T then agree too.
bool shares_rows(const cr_view& a, const cr_view& b) {
    if (a.width != b.width || a.height != b.height) return false;
    double pa[16], pb[16];
    mat_mul(a.proj, a.view, pa);
    mat_mul(b.proj, b.view, pb);
    for (int c = 0; c < 4; c++)
        for (int row : {1, 3})
            if (std::memcmp(&pa[4 * c + row], &pb[4 * c + row], sizeof(double)) != 0) return false;
    return true;
}

cr_status apply_params(cr_mv* mv, const cr_render_params* p) {
    if (p->method != CR_METHOD_LOOP_LAS && p->method != CR_METHOD_LOOP_LAS_PREFETCH)
        return mv_fail(mv, CR_ERR_INVALID_ARG, "multi-view plans render loop_las / loop_las_prefetch");
    if (p->payload != CR_PAYLOAD_INDEX && p->payload != CR_PAYLOAD_COLOR)
        return mv_fail(mv, CR_ERR_INVALID_ARG, "unknown payload");
    if ((p->payload == CR_PAYLOAD_COLOR || p->resolve) && !mv->ci.rgba)
        return mv_fail(mv, CR_ERR_INVALID_ARG, "the color stream is required");
    int G = p->views_per_group > 0 ? p->views_per_group : CR_MV_MAX_GROUP;
    if (G > CR_MV_MAX_GROUP) return mv_fail(mv, CR_ERR_INVALID_ARG, "views_per_group must be <= 8");
    const int block = p->block_threads == 0 ? 128 : p->block_threads;
    if (block != 64 && block != 128 && block != 256)
        return mv_fail(mv, CR_ERR_INVALID_ARG, "block_threads must be 64, 128 or 256");
    const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? default_quirks_for(p->method) : p->quirks;
    if (quirks & CR_QUIRK_LITERAL_ARITH)
        return mv_fail(mv, CR_ERR_UNSUPPORTED, "multi-view plans follow the FMA contract (no CR_QUIRK_LITERAL_ARITH)");
    drop_graph(mv);
    mv->params = *p;
    mv->G = std::min(G, mv->nviews);
    mv->ngroups = (mv->nviews + mv->G - 1) / mv->G;
    mv->block = block;
    mv->quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? default_quirks_for(p->method) : p->quirks;
    update_pairs(mv);
    return CR_OK;
}

cr_status enqueue_frame(cr_mv* mv, cudaStream_t st) {
    const cr_render_params& p = mv->params;
    const bool many = mv->ci.nfiles > kInlineFiles;
    cudaError_t e = cudaMemcpyAsync(mv->d_views, mv->h_views, sizeof(MVView) * mv->nviews,
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !many)
        e = cudaMemcpyAsync(mv->d_files, mv->h_files,
                            sizeof(MVFile) * (size_t)mv->nviews * mv->ci.nfiles,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && many)
        e = cudaMemcpyAsync(mv->d_mats, mv->h_mats, sizeof(double) * 32 * (size_t)mv->nviews,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && many)
        e = cudaMemcpyAsync(mv->d_box, mv->h_box, sizeof(double) * 3 * (size_t)mv->ci.nfiles,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(mv->d_pairs, mv->h_pairs, sizeof(uint32_t) * (size_t)mv->ngroups,
                            cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return mv_cuda(mv, e, "frame setup");
    MVFrame f{};
    f.ci = mv->ci;
    f.d_views = mv->d_views;
    f.d_files = mv->d_files;
    f.nviews = mv->nviews;
    f.fbs = reinterpret_cast<uint64_t*>(mv->fbs);
    f.images = mv->images;
    f.scratch = mv->scratch;
    f.G = mv->G;
    f.block = mv->block;
    f.ctas_per_sm = p.ctas_per_sm;
    f.quirks = mv->quirks;
    f.payload = p.payload;
    f.culling = p.frustum_culling;
    f.lod_skip_level = p.lod_skip_level;
    f.num_sms = mv->num_sms;
    f.clear_before = 0;
    f.resolve = p.resolve;
    f.clear_after = p.clear_after;
    f.clear_value = p.clear_value;
    f.max_words = mv->max_words;
    f.d_mats = mv->d_mats;
    f.d_box = mv->d_box;
    f.d_pairs = mv->d_pairs;
    const char* what = "";
    const cr_status s = mv_enqueue(f, st, &what);
    if (s != CR_OK) return mv_fail(mv, s, std::string(what) + " failed");
    return CR_OK;
}

}  // namespace

extern "C" {

cr_status cr_mv_create(cr_ctx* ctx, const cr_cloud* cloud, int32_t nviews, const int32_t* widths,
                       const int32_t* heights, const cr_render_params* params, cr_mv** out) {
    if (!ctx || !cloud || !widths || !heights || !params || !out || nviews < 1 || nviews > 65536)
        return CR_ERR_INVALID_ARG;
    *out = nullptr;
    cr_mv* mv = new (std::nothrow) cr_mv();
    if (!mv) return CR_ERR_OUT_OF_MEMORY;
    mv->ctx = ctx;
    mv->cloud = cloud;
    if (!cloud_info(cloud, &mv->ci) || !mv->ci.md || !mv->ci.hi) {
        delete mv;
        return CR_ERR_INVALID_ARG;
    }
    mv->nviews = nviews;
    mv->num_sms = cr_ctx_num_sms(ctx);
    int64_t words = 0, pixels = 0;
    for (int v = 0; v < nviews; v++) {
        const int32_t w = widths[v], h = heights[v];
        if (w <= 0 || h <= 0 || w >= (1 << 22) || h >= (1 << 22) ||
            (int64_t)w * h + w + 1 >= ((int64_t)1 << 31)) {
            delete mv;
            return CR_ERR_INVALID_ARG;
        }
        mv->W.push_back(w);
        mv->H.push_back(h);
        mv->fb_off.push_back(words);
        mv->img_off.push_back(pixels);
        words += (int64_t)w * h + w + 1;
        pixels += (int64_t)w * h;
        mv->max_words = std::max<int64_t>(mv->max_words, (int64_t)w * h + w + 1);
    }
    if (words >= ((int64_t)1 << 32) - 1) {  // z-cache tags are 32-bit word offsets
        delete mv;
        return CR_ERR_INVALID_ARG;
    }
    mv->total_words = words;
    mv->total_pixels = pixels;
    mv->eq_next.assign(nviews, 0);
    cr_status s = apply_params(mv, params);
    if (s != CR_OK) {
        delete mv;
        return s;
    }
    cudaError_t e = cudaMalloc(&mv->fbs, words * 8);
    if (e == cudaSuccess) e = cudaMalloc(&mv->images, std::max<int64_t>(pixels, 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&mv->d_views, sizeof(MVView) * nviews);
    if (e == cudaSuccess) e = cudaMalloc(&mv->d_files, sizeof(MVFile) * (size_t)nviews * mv->ci.nfiles);
    if (e == cudaSuccess) e = cudaMalloc(&mv->scratch, mv_scratch_words(mv->ci.nb_total, nviews) * 4);
    if (e == cudaSuccess) e = cudaMemset(mv->scratch, 0, mv_scratch_words(mv->ci.nb_total, nviews) * 4);
    if (e == cudaSuccess) e = cudaHostAlloc(&mv->h_views, sizeof(MVView) * nviews, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc(&mv->d_pairs, sizeof(uint32_t) * nviews);
    if (e == cudaSuccess) e = cudaHostAlloc(&mv->h_pairs, sizeof(uint32_t) * nviews, cudaHostAllocDefault);
    if (e == cudaSuccess) {
        std::memset(mv->h_pairs, 0, sizeof(uint32_t) * nviews);
        update_pairs(mv);
    }
    if (mv->ci.nfiles <= kInlineFiles) {
        if (e == cudaSuccess)
            e = cudaHostAlloc(&mv->h_files, sizeof(MVFile) * (size_t)nviews * mv->ci.nfiles,
                              cudaHostAllocDefault);
    } else {
        if (e == cudaSuccess) e = cudaMalloc(&mv->d_mats, sizeof(double) * 32 * (size_t)nviews);
        if (e == cudaSuccess) e = cudaMalloc(&mv->d_box, sizeof(double) * 3 * (size_t)mv->ci.nfiles);
        if (e == cudaSuccess)
            e = cudaHostAlloc(&mv->h_mats, sizeof(double) * 32 * (size_t)nviews, cudaHostAllocDefault);
        if (e == cudaSuccess)
            e = cudaHostAlloc(&mv->h_box, sizeof(double) * 3 * (size_t)mv->ci.nfiles, cudaHostAllocDefault);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&mv->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cr_mv_destroy(mv);
        return e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA;
    }
    for (int v = 0; v < nviews; v++) {
        mv->h_views[v].W = mv->W[v];
        mv->h_views[v].H = mv->H[v];
        mv->h_views[v].fb_off = (uint32_t)mv->fb_off[v];
        mv->h_views[v].img_off = (uint32_t)mv->img_off[v];
    }
    *out = mv;
    return CR_OK;
}

cr_status cr_mv_destroy(cr_mv* mv) {
    if (!mv) return CR_ERR_INVALID_ARG;
    if (mv->pending) cudaEventSynchronize(mv->done);
    drop_graph(mv);
    void* dev[8] = {mv->fbs, mv->images, mv->d_views, mv->d_files, mv->scratch, mv->d_mats, mv->d_box,
                    mv->d_pairs};
    for (void* p : dev)
        if (p) cudaFree(p);
    void* host[5] = {mv->h_views, mv->h_files, mv->h_mats, mv->h_box, mv->h_pairs};
    for (void* p : host)
        if (p) cudaFreeHost(p);
    if (mv->done) cudaEventDestroy(mv->done);
    delete mv;
    return CR_OK;
}

const char* cr_mv_last_error(const cr_mv* mv) { return mv ? mv->err.c_str() : ""; }

cr_status cr_mv_set_params(cr_mv* mv, const cr_render_params* p) {
    if (!mv || !p) return CR_ERR_INVALID_ARG;
    if (mv->pending) cudaEventSynchronize(mv->done);
    return apply_params(mv, p);
}

cr_status cr_mv_get_params(const cr_mv* mv, cr_render_params* out) {
    if (!mv || !out) return CR_ERR_INVALID_ARG;
    *out = mv->params;
    out->views_per_group = mv->G;
    out->block_threads = mv->block;
    return CR_OK;
}

cr_status cr_mv_set_views(cr_mv* mv, const cr_view* views) {
    if (!mv || !views) return CR_ERR_INVALID_ARG;
    if (mv->pending) {
        cudaError_t e = cudaEventSynchronize(mv->done);
        if (e != cudaSuccess) return mv_cuda(mv, e, "waiting for the previous frame");
        mv->pending = false;
    }
    for (int v = 0; v < mv->nviews; v++) {
        if (views[v].width != mv->W[v] || views[v].height != mv->H[v])
            return mv_fail(mv, CR_ERR_INVALID_ARG, "view " + std::to_string(v) + " size differs from the plan");
        const bool many = mv->ci.nfiles > kInlineFiles;
        cr_status s = mv_fill_view(&views[v], mv->ci, &mv->h_views[v],
                                   many ? nullptr : &mv->h_files[(int64_t)v * mv->ci.nfiles]);
        if (s != CR_OK) return mv_fail(mv, s, "view " + std::to_string(v) + ": bad matrices");
        if (many) {
            std::memcpy(&mv->h_mats[32 * (int64_t)v], views[v].view, sizeof(double) * 16);
            std::memcpy(&mv->h_mats[32 * (int64_t)v + 16], views[v].proj, sizeof(double) * 16);
        }
    }
    // the files' boxMin as the frames of these views read them
    if (mv->h_box) std::memcpy(mv->h_box, mv->ci.box_min, sizeof(double) * 3 * (size_t)mv->ci.nfiles);
    for (int v = 0; v < mv->nviews; v++)
        mv->eq_next[v] = v + 1 < mv->nviews && shares_rows(views[v], views[v + 1]) ? 1 : 0;
    update_pairs(mv);
    mv->views_set = true;
    return CR_OK;
}

cr_status cr_mv_shared_pairs(const cr_mv* mv, int32_t* pairs) {
    if (!mv || !pairs) return CR_ERR_INVALID_ARG;
    *pairs = mv->shared_pairs;
    return CR_OK;
}

cr_status cr_mv_render(cr_mv* mv, int32_t use_graph, void* stream) {
    if (!mv) return CR_ERR_INVALID_ARG;
    const NvtxRange range("cr_mv_render");
    if (!mv->views_set) return mv_fail(mv, CR_ERR_INVALID_ARG, "cr_mv_set_views first");
    // the cloud's loaded counts may have grown since the last frame; a graph
    // captured for other counts is dropped and captured again
    if (!cloud_info(mv->cloud, &mv->ci)) return mv_fail(mv, CR_ERR_INVALID_ARG, "cloud");
    if (mv->exec && (mv->graph_n != mv->ci.n || mv->graph_nb != mv->ci.nb)) drop_graph(mv);
    cudaStream_t st = (cudaStream_t)stream;
    cr_status s = CR_OK;
    if (use_graph && st != nullptr) {
        if (!mv->exec) {
            cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return mv_cuda(mv, e, "begin capture");
            s = enqueue_frame(mv, st);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(st, &g);
            if (s != CR_OK) {
                if (g) cudaGraphDestroy(g);
                return s;
            }
            if (e != cudaSuccess) return mv_cuda(mv, e, "end capture");
            mv->graph = g;
            mv->graph_n = mv->ci.n;
            mv->graph_nb = mv->ci.nb;
            e = cudaGraphInstantiate(&mv->exec, g, 0);
            if (e != cudaSuccess) {
                drop_graph(mv);
                return mv_cuda(mv, e, "graph instantiate");
            }
        }
        cudaError_t e = cudaGraphLaunch(mv->exec, st);
        if (e != cudaSuccess) return mv_cuda(mv, e, "graph launch");
    } else {
        s = enqueue_frame(mv, st);
        if (s != CR_OK) return s;
    }
    cudaError_t e = cudaEventRecord(mv->done, st);
    if (e != cudaSuccess) return mv_cuda(mv, e, "event record");
    mv->pending = true;
    return CR_OK;
}

cr_status cr_mv_clear(cr_mv* mv, uint64_t value, void* stream) {
    if (!mv) return CR_ERR_INVALID_ARG;
    const int64_t n = mv->total_words;
    const int grid = (int)std::min<int64_t>((n + 255) / 256, 65535);
    if (launch_k(k_mv_fill, grid, 256, (cudaStream_t)stream, mv->fbs, n, value) != 0)
        return mv_fail(mv, CR_ERR_CUDA, "clear launch failed");
    return CR_OK;
}

cr_status cr_mv_read(cr_mv* mv, int32_t view, int32_t what, void* dst, int64_t bytes, void* stream) {
    if (!mv || !dst || view < 0 || view >= mv->nviews || bytes < 0) return CR_ERR_INVALID_ARG;
    const void* src;
    int64_t limit;
    if (what == CR_FB_WORDS) {
        src = mv->fbs + mv->fb_off[view];
        limit = ((int64_t)mv->W[view] * mv->H[view] + mv->W[view] + 1) * 8;
    } else if (what == CR_FB_IMAGE) {
        src = mv->images + mv->img_off[view];
        limit = (int64_t)mv->W[view] * mv->H[view] * 4;
    } else {
        return mv_fail(mv, CR_ERR_INVALID_ARG, "CR_FB_WORDS or CR_FB_IMAGE");
    }
    if (bytes > limit) return mv_fail(mv, CR_ERR_INVALID_ARG, "read past the view's buffer");
    return mv_cuda(mv, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost,
                                       (cudaStream_t)stream), "read");
}

cr_status cr_mv_autotune(cr_mv* mv, int32_t frames, void* stream, cr_render_params* best,
                         char* report, int32_t report_bytes) {
    if (!mv || frames < 1) return CR_ERR_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const cr_render_params base = mv->params;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return mv_fail(mv, CR_ERR_CUDA, "event create");
    std::string js = "{";
    float best_ms = 1e30f;
    cr_render_params best_p = base;
    const int blocks[3] = {64, 128, 256};
    const int groups[4] = {1, 2, 4, 8};
    cr_status s = CR_OK;
    for (int bi = 0; bi < 3 && s == CR_OK; bi++) {
        for (int gi = 0; gi < 4 && s == CR_OK; gi++) {
            if (groups[gi] > mv->nviews && groups[gi] > 1) continue;
            cr_render_params p = base;
            p.block_threads = blocks[bi];
            p.views_per_group = groups[gi];
            if ((s = cr_mv_set_params(mv, &p)) != CR_OK) break;
            for (int k = 0; k < 2 && s == CR_OK; k++) s = cr_mv_render(mv, 0, stream);
            cudaEventRecord(e0, st);
            for (int k = 0; k < frames && s == CR_OK; k++) s = cr_mv_render(mv, 0, stream);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) s = mv_fail(mv, CR_ERR_CUDA, "autotune sync");
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= frames;
            char buf[96];
            std::snprintf(buf, sizeof(buf), "%s\"block%d_group%d_ptsthread%d\": %.4f", js.size() > 1 ? ", " : "",
                          blocks[bi], groups[gi], kPointsPerBatch / blocks[bi], ms);
            js += buf;
            if (ms < best_ms) {
                best_ms = ms;
                best_p = p;
            }
        }
    }
    js += "}";
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != CR_OK) return s;
    s = cr_mv_set_params(mv, &best_p);
    if (best) *best = best_p;
    if (report && report_bytes > 0) {
        std::strncpy(report, js.c_str(), (size_t)report_bytes - 1);
        report[report_bytes - 1] = '\0';
    }
    return s;
}

}  // extern "C"
