// cr_synth.cu -- synthetic LAS clouds, Morton ordering and the GPU build of
// the LAS-derived batched layout (include/cr_synth.h).
//
// The generator is a pure function of (seed, point index) built from 64-bit
// integer hashing and IEEE double + - * / floor; the host and device paths
// share the __host__ __device__ code below and compile without contraction
// (-ffp-contract=off / -fmad=false), so they write identical records.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/cr_synth.h"
#include "cr_internal.h"
#include "cr_quant.h"

namespace {

constexpr int kRecBytes = CR_LAS_FORMAT2_BYTES;

// splitmix64 output function (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014).
__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xbf58476d1ce4e5b9ull;
    z ^= z >> 27;
    z *= 0x94d049bb133111ebull;
    z ^= z >> 31;
    return z;
}

__host__ __device__ inline uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
    return mix64(seed ^ mix64(a * 0x9E3779B97F4A7C15ull + b * 0xD6E8FEB86659FD93ull +
                              0x632BE59BD9B4E019ull));
}

__host__ __device__ inline double u53(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

// Value noise on the integer lattice with smoothstep interpolation.
__host__ __device__ inline double vnoise(double px, double py, uint64_t s) {
    const double fx = floor(px), fy = floor(py);
    const uint64_t ix = (uint64_t)(int64_t)fx, iy = (uint64_t)(int64_t)fy;
    const double tx = px - fx, ty = py - fy;
    const double v00 = u53(hash3(s, ix, iy)), v10 = u53(hash3(s, ix + 1, iy));
    const double v01 = u53(hash3(s, ix, iy + 1)), v11 = u53(hash3(s, ix + 1, iy + 1));
    const double sx = tx * tx * (3.0 - 2.0 * tx);
    const double sy = ty * ty * (3.0 - 2.0 * ty);
    const double a = v00 + sx * (v10 - v00);
    const double b = v01 + sx * (v11 - v01);
    return a + sy * (b - a);
}

// Fractional Brownian motion: octaves of halving amplitude, doubling frequency.
__host__ __device__ inline double fbm(double px, double py, uint64_t seed, int octaves) {
    double sum = 0.0, amp = 0.5, f = 1.0;
    for (int o = 0; o < octaves; o++) {
        sum = sum + amp * vnoise(px * f, py * f, seed + 0x1000ull * (uint64_t)(o + 1));
        amp = amp * 0.5;
        f = f * 2.0;
    }
    return sum;
}

// N(0, 1) by the Irwin-Hall sum of 12 uniforms.
__host__ __device__ inline double gauss(uint64_t seed, uint64_t i) {
    double s = 0.0;
    for (int k = 0; k < 3; k++) {
        const uint64_t h = hash3(seed, i, 10 + k);
        for (int j = 0; j < 4; j++)
            s = s + ((double)((h >> (16 * j)) & 0xFFFFu) * (1.0 / 65536.0) + (1.0 / 131072.0));
    }
    return s - 6.0;
}

__host__ __device__ inline int clamp255(int v) { return v < 0 ? 0 : (v > 255 ? 255 : v); }

struct GenPoint {
    double x, y, z;
    int r, g, b;
};

__host__ __device__ inline void terrain_color(const cr_synth_params& p, uint64_t i, double z, GenPoint& o) {
    double t = z / p.height;
    t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    const double c0[3] = {70.0, 110.0, 50.0}, c1[3] = {150.0, 120.0, 80.0}, c2[3] = {235.0, 235.0, 235.0};
    const uint64_t h = hash3(p.seed, i, 5);
    int c[3];
    for (int k = 0; k < 3; k++) {
        double v = t < 0.5 ? c0[k] + (c1[k] - c0[k]) * (2.0 * t) : c1[k] + (c2[k] - c1[k]) * (2.0 * t - 1.0);
        c[k] = clamp255((int)v + (int)((h >> (8 * k)) & 31u) - 16);
    }
    o.r = c[0];
    o.g = c[1];
    o.b = c[2];
}

__host__ __device__ inline void gen_point(const cr_synth_params& p, int64_t n, uint64_t i, GenPoint& o) {
    const int64_t box_total = (int64_t)p.num_boxes * p.points_per_box;
    const int64_t nbox_pts = p.kind == CR_SYNTH_TERRAIN_BOXES ? (box_total < n ? box_total : n) : 0;
    const int64_t nterrain = n - nbox_pts;
    const double inv_wl = 1.0 / p.wavelength;
    if ((int64_t)i < nterrain) {
        o.x = p.origin[0] + u53(hash3(p.seed, i, 0)) * p.extent;
        o.y = p.origin[1] + u53(hash3(p.seed, i, 1)) * p.extent;
        o.z = p.height * fbm(o.x * inv_wl, o.y * inv_wl, p.seed, p.octaves) + p.sigma * gauss(p.seed, i);
        terrain_color(p, i, o.z, o);
        return;
    }
    // points on the faces of axis-aligned boxes standing on the terrain
    const uint64_t k = i - (uint64_t)nterrain;
    const uint64_t bi = k / (uint64_t)p.points_per_box;
    const double cx = p.origin[0] + u53(hash3(p.seed ^ 0xB0C5ull, bi, 0)) * p.extent;
    const double cy = p.origin[1] + u53(hash3(p.seed ^ 0xB0C5ull, bi, 1)) * p.extent;
    const double wx = 10.0 + 30.0 * u53(hash3(p.seed ^ 0xB0C5ull, bi, 2));
    const double wy = 10.0 + 30.0 * u53(hash3(p.seed ^ 0xB0C5ull, bi, 3));
    const double h = p.box_min_height + (p.box_max_height - p.box_min_height) * u53(hash3(p.seed ^ 0xB0C5ull, bi, 4));
    const double z0 = p.height * fbm(cx * inv_wl, cy * inv_wl, p.seed, p.octaves);
    const double a_top = wx * wy, a_x = wy * h, a_y = wx * h;
    const double total = a_top + 2.0 * a_x + 2.0 * a_y;
    const double sel = u53(hash3(p.seed, i, 20)) * total;
    const double u = u53(hash3(p.seed, i, 21)), v = u53(hash3(p.seed, i, 22));
    const double x0 = cx - 0.5 * wx, y0 = cy - 0.5 * wy;
    if (sel < a_top) {
        o.x = x0 + u * wx; o.y = y0 + v * wy; o.z = z0 + h;
    } else if (sel < a_top + a_x) {
        o.x = x0; o.y = y0 + u * wy; o.z = z0 + v * h;
    } else if (sel < a_top + 2.0 * a_x) {
        o.x = x0 + wx; o.y = y0 + u * wy; o.z = z0 + v * h;
    } else if (sel < a_top + 2.0 * a_x + a_y) {
        o.x = x0 + u * wx; o.y = y0; o.z = z0 + v * h;
    } else {
        o.x = x0 + u * wx; o.y = y0 + wy; o.z = z0 + v * h;
    }
    const uint64_t hc = hash3(p.seed, i, 23);
    o.r = (int)(hc & 0xFFu);
    o.g = (int)((hc >> 8) & 0xFFu);
    o.b = (int)((hc >> 16) & 0xFFu);
}

__host__ __device__ inline void put_i32(uint8_t* d, int32_t v) {
    const uint32_t u = (uint32_t)v;
    for (int k = 0; k < 4; k++) d[k] = (uint8_t)(u >> (8 * k));
}
__host__ __device__ inline void put_u16(uint8_t* d, uint32_t v) {
    d[0] = (uint8_t)v;
    d[1] = (uint8_t)(v >> 8);
}
__host__ __device__ inline int32_t get_i32(const uint8_t* d) {
    return (int32_t)((uint32_t)d[0] | ((uint32_t)d[1] << 8) | ((uint32_t)d[2] << 16) | ((uint32_t)d[3] << 24));
}
__host__ __device__ inline uint32_t get_u16(const uint8_t* d) { return (uint32_t)d[0] | ((uint32_t)d[1] << 8); }

// floor(x / s + 0.5) (the LAS integer of a coordinate), bit for bit, with the
// division replaced by a multiplication with inv = RN(1/s) where that cannot
// change the result: x * inv lies within 3 ulps of RN(x / s) and
// r -> floor(RN(r + 0.5)) is monotone, so when both ends of a margin of 8
// ulps around the product give the same integer, so does RN(x / s).  Near a
// half-integer the division is done.  (Double division runs at a small
// fraction of the FP64 rate on this part.)
__host__ __device__ inline int32_t las_int(double x, double s, double inv) {
    const double r1 = x * inv;
    const double e = fabs(r1) * 0x1p-49;
    const double lo = floor((r1 - e) + 0.5), hi = floor((r1 + e) + 0.5);
    return (int32_t)(lo == hi ? lo : floor(x / s + 0.5));
}

// One LAS point-format-2 record (26 B).  Colors are stored as 16-bit values
// (c * 256) for 7 of 8 points and as plain 8-bit values for the rest, so both
// branches of the loader's `v < 256 ? v : v / 256` are exercised.
// inv_scale = 1 / p.las_scale.
__host__ __device__ inline void write_record(const cr_synth_params& p, double inv_scale, int64_t n,
                                             uint64_t i, uint8_t* d) {
    GenPoint g;
    gen_point(p, n, i, g);
    const int32_t X = las_int(g.x, p.las_scale, inv_scale);
    const int32_t Y = las_int(g.y, p.las_scale, inv_scale);
    const int32_t Z = las_int(g.z, p.las_scale, inv_scale);
    put_i32(d + 0, X);
    put_i32(d + 4, Y);
    put_i32(d + 8, Z);
    for (int k = 12; k < 20; k++) d[k] = 0;
    const bool wide = (hash3(p.seed, i, 6) & 7u) != 0u;
    const uint32_t m = wide ? 256u : 1u;
    put_u16(d + 20, (uint32_t)g.r * m);
    put_u16(d + 22, (uint32_t)g.g * m);
    put_u16(d + 24, (uint32_t)g.b * m);
}

// Sort_Frugal/src/main.cpp:58-77: 21 bits per axis, x at bit 0, y bit 1, z bit 2.
__host__ __device__ inline uint64_t spread3(uint32_t a) {
    uint64_t x = a & 0x1FFFFFu;
    x = (x | x << 32) & 0x1F00000000FFFFull;
    x = (x | x << 16) & 0x1F0000FF0000FFull;
    x = (x | x << 8) & 0x100F00F00F00F00Full;
    x = (x | x << 4) & 0x10C30C30C30C30C3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

struct MortonFrame {
    double min[3];
    double cube, inv;  // inv = RN(1 / cube)
    double scale[3];
    double offset[3];
    cr::QuantFx fx[3];  // the GPU keys' integer form of morton_axis (cr_quant.h)
};

// Sort_Frugal/src/main.cpp:82-105: normalise by the largest header extent.
// The tool passes 2^21 for a point on the cube's far face to a 21-bit mask,
// which wraps it to 0 and sorts it to the front; it is clamped to 2^21 - 1 here.
// uint32(((v - min) / cube) * 2^21) as one product with the reciprocal: d *
// inv lies within a few ulps of RN(d / cube), so when no integer lies within
// 16 ulps of t1 = d * inv * 2^21 both truncate to the same integer; otherwise
// (rarely) the division is done.  Same rule as the encoder's quantize30.
__host__ __device__ inline uint32_t morton_axis(const MortonFrame& f, int k, int32_t X) {
    const double v = (double)X * f.scale[k] + f.offset[k];
    const double d = v - f.min[k];
    const double t1 = (d * f.inv) * 2097152.0;
    const double e = t1 * 0x1p-49;
    double t = t1;
    if (!(floor(t1 - e) == floor(t1 + e))) t = (d / f.cube) * 2097152.0;
    const uint32_t u = (t >= 0.0) ? (t < 4294967295.0 ? (uint32_t)t : 0xFFFFFFFFu) : 0u;
    return u < 2097151u ? u : 2097151u;
}

__host__ __device__ inline uint64_t morton_of(const MortonFrame& f, const uint8_t* rec) {
    uint32_t q[3];
    for (int k = 0; k < 3; k++) q[k] = morton_axis(f, k, get_i32(rec + 4 * k));
    return spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
}

// The GPU keys: the cell in integer arithmetic where the error bound decides
// it (all but about one point in 10^5 per axis for LAS scales and extents),
// else the double chain.  The host sort keeps the chain, so every GPU/host
// comparison checks the integer form.
__device__ inline uint64_t morton_of_fast(const MortonFrame& f, const uint8_t* rec) {
    uint32_t q[3];
    for (int k = 0; k < 3; k++) {
        const int32_t X = get_i32(rec + 4 * k);
        if (!cr::quant_fast(f.fx[k], X, 2097151u, &q[k])) q[k] = morton_axis(f, k, X);
    }
    return spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
}

MortonFrame morton_frame(const cr_las_header* h) {
    MortonFrame f;
    double size[3];
    for (int k = 0; k < 3; k++) {
        f.min[k] = h->min[k];
        size[k] = h->max[k] - h->min[k];
        f.scale[k] = h->scale[k];
        f.offset[k] = h->offset[k];
    }
    f.cube = std::max(std::max(size[0], size[1]), size[2]);
    if (!(f.cube > 0.0)) f.cube = 1.0;
    f.inv = 1.0 / f.cube;
    for (int k = 0; k < 3; k++)
        f.fx[k] = cr::quant_setup(f.scale[k], f.offset[k], f.min[k], 0.0, false, f.cube, 21, INT32_MIN, INT32_MAX);
    return f;
}

void fill_header(const cr_synth_params* p, int64_t n, const int32_t mn[3], const int32_t mx[3],
                 cr_las_header* h) {
    h->num_points = n;
    h->point_format = 2;
    h->bytes_per_point = kRecBytes;
    for (int k = 0; k < 3; k++) {
        h->scale[k] = p->las_scale;
        h->offset[k] = 0.0;
        h->min[k] = (double)mn[k] * p->las_scale + 0.0;
        h->max[k] = (double)mx[k] * p->las_scale + 0.0;
    }
}

bool valid_params(const cr_synth_params* p) {
    return p && p->extent > 0.0 && p->height > 0.0 && p->wavelength > 0.0 && p->las_scale > 0.0 &&
           p->octaves >= 1 && p->octaves <= 16 &&
           (p->kind == CR_SYNTH_TERRAIN ||
            (p->kind == CR_SYNTH_TERRAIN_BOXES && p->num_boxes >= 0 && p->points_per_box > 0));
}

// ---- device kernels ------------------------------------------------------------

__global__ void k_gen(cr_synth_params p, double inv_scale, int64_t n, uint8_t* rec) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        write_record(p, inv_scale, n, (uint64_t)i, rec + i * kRecBytes);
}

__global__ void k_bounds(const uint8_t* rec, int64_t n, int32_t bpp, int32_t* mnmx) {
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; k++) {
            int32_t v = get_i32(rec + i * bpp + 4 * k);
            mn[k] = min(mn[k], v);
            mx[k] = max(mx[k], v);
        }
    }
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
            mx[k] = max(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; k++) {
            atomicMin(&mnmx[k], mn[k]);
            atomicMax(&mnmx[3 + k], mx[k]);
        }
}

__global__ void k_morton_keys(MortonFrame f, const uint8_t* rec, int64_t n, int32_t bpp,
                              unsigned long long* keys, uint32_t* idx) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = morton_of_fast(f, rec + i * bpp);
        idx[i] = (uint32_t)i;
    }
}

// dst[i] = src[perm[i]] for records of `bpp` bytes (even, <= kGatherMaxBpp).
// A warp gathers 32 records: each lane reads its source record as 16-bit
// words (records start on 2-byte boundaries), writes them into the warp's
// slice of shared memory at their destination offsets, and the warp stores the
// 32 * bpp contiguous destination bytes as 16-byte vectors (bpp is even, so
// 32 * bpp is a multiple of 16 and the warp's first byte is 16-byte aligned
// when dst is).  The tail warp (fewer than 32 records) stores 16-bit words.
constexpr int kGatherMaxBpp = 64;
constexpr int kGatherWarps = 8;
__global__ void __launch_bounds__(32 * kGatherWarps) k_gather(const uint8_t* __restrict__ src,
                                                              uint8_t* __restrict__ dst,
                                                              const uint32_t* __restrict__ perm,
                                                              int64_t n, int32_t bpp) {
    __shared__ __align__(16) uint16_t s_buf[kGatherWarps][32 * kGatherMaxBpp / 2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint16_t* buf = s_buf[warp];
    const int words = bpp >> 1;
    const int64_t nwarps = (int64_t)gridDim.x * kGatherWarps;
    for (int64_t w0 = ((int64_t)blockIdx.x * kGatherWarps + warp) * 32; w0 < n; w0 += nwarps * 32) {
        const int64_t i = w0 + lane;
        const int cnt = (int)min((int64_t)32, n - w0);
        if (lane < cnt) {
            const uint16_t* s = reinterpret_cast<const uint16_t*>(src + (int64_t)perm[i] * bpp);
            for (int k = 0; k < words; k++) buf[lane * words + k] = __ldg(s + k);
        }
        __syncwarp();
        uint8_t* d = dst + w0 * bpp;
        if (cnt == 32) {
            const int vecs = (32 * bpp) >> 4;
            for (int k = lane; k < vecs; k += 32)
                reinterpret_cast<uint4*>(d)[k] = reinterpret_cast<const uint4*>(buf)[k];
        } else {
            for (int k = lane; k < cnt * words; k += 32) reinterpret_cast<uint16_t*>(d)[k] = buf[k];
        }
        __syncwarp();
    }
}

struct EncodeArgs {
    double scale[3], offset[3], box_min[3];
    int64_t n, sparse_offset;
    int32_t bpp, rgb, file_index;
};

// LasLoaderSparse.cpp:146-148: min(uint32(((v - min) / size) * 2^30), 2^30 - 1)
// (NaN -> 0), bit for bit, with one multiplication by inv = RN(1/size) in
// place of the division where that cannot change the result: d * inv lies
// within 3 ulps of RN(d / size), so when no integer lies within 8 ulps of
// t1 = d * inv * 2^30 both truncate to the same integer.  Otherwise (a point
// on the box's far face, about one in 2^20 others, a zero or subnormal size)
// the division is done.
__device__ __forceinline__ uint32_t quantize30(double d, double size, double inv) {
    const double t1 = (d * inv) * 1073741824.0;
    const double e = t1 * 0x1p-49;
    double t = t1;
    if (!(floor(t1 - e) == floor(t1 + e))) t = (d / size) * 1073741824.0;
    const uint32_t u = (t != t) ? 0u : (uint32_t)t;
    return u < 1073741823u ? u : 1073741823u;
}

// LasLoaderSparse.cpp:84-199, one CTA per batch.
__global__ void __launch_bounds__(256) k_encode(EncodeArgs a, const uint8_t* __restrict__ rec,
                                                cr_batch* batches, uint32_t* lo, uint32_t* md,
                                                uint32_t* hi, uint32_t* rgba) {
    __shared__ int32_t s_red[6][8];
    __shared__ double s_box[9];
    __shared__ cr::QuantFx s_fx[3];
    const int64_t first = (int64_t)blockIdx.x * cr::kPointsPerBatch;
    const int64_t left = a.n - first;
    const int cnt = (int)(left < cr::kPointsPerBatch ? left : cr::kPointsPerBatch);
    // The batch AABB of v = double(X) * scale + offset - boxMin
    // (LasLoaderSparse.cpp:93-105): every step rounds monotonically, so v is
    // monotone in the integer X and the box is v at the integer extremes.
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const uint8_t* r = rec + (first + i) * a.bpp;
        for (int k = 0; k < 3; k++) {
            const int32_t X = get_i32(r + 4 * k);
            mn[k] = min(mn[k], X);
            mx[k] = max(mx[k], X);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; k++) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
            mx[k] = max(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
        }
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; k++) {
            s_red[k][warp] = mn[k];
            s_red[3 + k][warp] = mx[k];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        int32_t lo = s_red[k][0], hi = s_red[3 + k][0];
        for (int w = 1; w < nwarps; w++) {
            lo = min(lo, s_red[k][w]);
            hi = max(hi, s_red[3 + k][w]);
        }
        const double vlo = (double)lo * a.scale[k] + a.offset[k] - a.box_min[k];
        const double vhi = (double)hi * a.scale[k] + a.offset[k] - a.box_min[k];
        const double b0 = a.scale[k] < 0.0 ? vhi : vlo, b1 = a.scale[k] < 0.0 ? vlo : vhi;
        s_box[k] = b0;
        s_box[3 + k] = b1;
        s_box[6 + k] = 1.0 / (b1 - b0);
        s_fx[k] = cr::quant_setup(a.scale[k], a.offset[k], a.box_min[k], b0, true, b1 - b0, 30, lo, hi);
    }
    __syncthreads();
    const double bmin[3] = {s_box[0], s_box[1], s_box[2]};
    const double size[3] = {s_box[3] - s_box[0], s_box[4] - s_box[1], s_box[5] - s_box[2]};
    const double inv[3] = {s_box[6], s_box[7], s_box[8]};
    if (threadIdx.x == 0) {
        cr_batch b;
        memset(&b, 0, sizeof(b));
        b.min_x = (float)s_box[0]; b.min_y = (float)s_box[1]; b.min_z = (float)s_box[2];
        b.max_x = (float)s_box[3]; b.max_y = (float)s_box[4]; b.max_z = (float)s_box[5];
        b.num_points = cnt;
        b.first_point = (int32_t)(a.sparse_offset + first);
        b.file_index = a.file_index;
        batches[blockIdx.x] = b;
    }
    // Each coordinate's 30-bit cell in integer arithmetic where the error bound
    // decides it (cr_quant.h), else the double chain: the same integer either way.
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int64_t pi = first + i;
        const uint8_t* r = rec + pi * a.bpp;
        uint32_t q[3];
        for (int k = 0; k < 3; k++) {
            const int32_t X = get_i32(r + 4 * k);
            if (!cr::quant_fast(s_fx[k], X, 1073741823u, &q[k])) {
                const double v = (double)X * a.scale[k] + a.offset[k] - a.box_min[k];
                q[k] = quantize30(v - bmin[k], size[k], inv[k]);
            }
        }
        lo[pi] = ((q[0] >> 20) & 1023u) | (((q[1] >> 20) & 1023u) << 10) | (((q[2] >> 20) & 1023u) << 20);
        md[pi] = ((q[0] >> 10) & 1023u) | (((q[1] >> 10) & 1023u) << 10) | (((q[2] >> 10) & 1023u) << 20);
        hi[pi] = (q[0] & 1023u) | ((q[1] & 1023u) << 10) | ((q[2] & 1023u) << 20);
        if (a.rgb >= 0) {
            uint32_t R = get_u16(r + a.rgb), G = get_u16(r + a.rgb + 2), B = get_u16(r + a.rgb + 4);
            R = R < 256u ? R : R / 256u;
            G = G < 256u ? G : G / 256u;
            B = B < 256u ? B : B / 256u;
            rgba[pi] = R | (G << 8) | (B << 16);
        } else {
            rgba[pi] = 0u;
        }
    }
}

__host__ __device__ inline cr_vertex uniform_vertex(uint64_t seed, uint64_t i, float size) {
    const uint64_t h0 = hash3(seed, i, 0), h1 = hash3(seed, i, 1), h2 = hash3(seed, i, 2);
    const float k = 1.0f / 16777216.0f;
    cr_vertex v;
    v.x = ((float)(uint32_t)(h0 >> 40) * k) * size;
    v.y = ((float)(uint32_t)((h0 >> 16) & 0xFFFFFFu) * k) * size;
    v.z = ((float)(uint32_t)(h1 >> 40) * k) * size;
    v.color = (uint32_t)(h2 >> 32);
    return v;
}

__global__ void k_uniform(uint64_t seed, int64_t n, float size, cr_vertex* out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = uniform_vertex(seed, (uint64_t)i, size);
}

int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)std::min<int64_t>(std::max<int64_t>(g, 1), 65535);
}

template <typename F>
void parallel_for(int64_t n, F f) {
    unsigned t = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    if (n < 65536) t = 1;
    std::vector<std::thread> th;
    for (unsigned k = 0; k < t; k++)
        th.emplace_back([=] { f(n * k / t, n * (k + 1) / t); });
    for (auto& x : th) x.join();
}

cr_status cuda_status(cudaError_t e) {
    return e == cudaSuccess ? CR_OK : (e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA);
}

}  // namespace

cr_status cr::encode_records_device(const uint8_t* d_rec, int64_t n, int32_t bpp, int32_t rgb,
                                   const double scale[3], const double offset[3], const double box_min[3],
                                   int64_t sparse_offset, int32_t file_index, cr_batch* d_batches,
                                   uint32_t* d_lo, uint32_t* d_md, uint32_t* d_hi, uint32_t* d_rgba,
                                   void* stream) {
    if (n < 0 || (n > 0 && !d_rec) || bpp < 12 || !scale || !offset || !box_min || !d_batches || !d_lo ||
        !d_md || !d_hi || !d_rgba || sparse_offset < 0 || sparse_offset + n >= ((int64_t)1 << 31))
        return CR_ERR_INVALID_ARG;
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(scale[k]) || !std::isfinite(offset[k]) || !std::isfinite(box_min[k]))
            return CR_ERR_INVALID_ARG;
    if (rgb >= 0 && rgb + 6 > bpp) return CR_ERR_INVALID_ARG;
    const int64_t nb = cr_num_batches(n);
    if (nb == 0) return CR_OK;
    EncodeArgs a;
    for (int k = 0; k < 3; k++) {
        a.scale[k] = scale[k];
        a.offset[k] = offset[k];
        a.box_min[k] = box_min[k];
    }
    a.n = n;
    a.sparse_offset = sparse_offset;
    a.bpp = bpp;
    a.rgb = rgb < 0 ? -1 : rgb;
    a.file_index = file_index;
    k_encode<<<(unsigned)nb, 256, 0, (cudaStream_t)stream>>>(a, d_rec, d_batches, d_lo, d_md, d_hi, d_rgba);
    return cuda_status(cudaGetLastError());
}

extern "C" {

void cr_synth_params_default(int32_t kind, double extent, uint64_t seed, cr_synth_params* out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->kind = kind;
    out->octaves = 6;
    out->seed = seed;
    out->extent = extent;
    out->height = 20.0;
    out->sigma = 0.05;
    out->wavelength = extent / 4.0;
    out->las_scale = 0.001;
    out->num_boxes = 2000;
    out->points_per_box = 20000;
    out->box_min_height = 10.0;
    out->box_max_height = 60.0;
}

cr_status cr_synth_points_host(const cr_synth_params* p, int64_t n, uint8_t* rec, cr_las_header* hdr) {
    if (!valid_params(p) || n < 0 || (n > 0 && !rec) || !hdr) return CR_ERR_INVALID_ARG;
    const cr_synth_params pp = *p;
    const double inv = 1.0 / pp.las_scale;
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) write_record(pp, inv, n, (uint64_t)i, rec + i * kRecBytes);
    });
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            const int32_t v = get_i32(rec + i * kRecBytes + 4 * k);
            mn[k] = std::min(mn[k], v);
            mx[k] = std::max(mx[k], v);
        }
    if (n == 0)
        for (int k = 0; k < 3; k++) mn[k] = mx[k] = 0;
    fill_header(p, n, mn, mx, hdr);
    return CR_OK;
}

cr_status cr_morton_sort_host(uint8_t* rec, int64_t n, int32_t bpp, const cr_las_header* hdr) {
    if (n < 0 || (n > 0 && !rec) || bpp < 12 || !hdr || n >= ((int64_t)1 << 32)) return CR_ERR_INVALID_ARG;
    const MortonFrame f = morton_frame(hdr);
    std::vector<std::pair<uint64_t, uint32_t>> keys((size_t)n);
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) keys[i] = {morton_of(f, rec + i * bpp), (uint32_t)i};
    });
    std::sort(keys.begin(), keys.end());
    std::vector<uint8_t> tmp((size_t)n * bpp);
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++)
            std::memcpy(&tmp[(size_t)i * bpp], rec + (int64_t)keys[i].second * bpp, bpp);
    });
    std::memcpy(rec, tmp.data(), tmp.size());
    return CR_OK;
}

cr_status cr_synth_points_device(cr_ctx* ctx, const cr_synth_params* p, int64_t n, uint8_t* d_rec,
                                 cr_las_header* hdr, void* stream) {
    if (!ctx || !valid_params(p) || n < 0 || (n > 0 && !d_rec) || !hdr) return CR_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int32_t init[6] = {INT32_MAX, INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN, INT32_MIN};
    int32_t* d_mm = nullptr;
    cudaError_t e = cudaMalloc(&d_mm, sizeof(init));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_mm, init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n > 0) {
        k_gen<<<grid_for(n) * 4 > 65535 ? 65535 : grid_for(n) * 4, 256, 0, s>>>(*p, 1.0 / p->las_scale,
                                                                                 n, d_rec);
        k_bounds<<<grid_for(n) > 2048 ? 2048 : grid_for(n), 256, 0, s>>>(d_rec, n, kRecBytes, d_mm);
        e = cudaGetLastError();
    }
    int32_t mm[6];
    if (e == cudaSuccess) e = cudaMemcpyAsync(mm, d_mm, sizeof(mm), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (d_mm) cudaFree(d_mm);
    if (e != cudaSuccess) return cuda_status(e);
    if (n == 0)
        for (int k = 0; k < 6; k++) mm[k] = 0;
    fill_header(p, n, mm, mm + 3, hdr);
    return CR_OK;
}

cr_status cr_morton_sort_device(cr_ctx* ctx, uint8_t* d_rec, int64_t n, int32_t bpp,
                                const cr_las_header* hdr, void* stream) {
    if (!ctx || n < 0 || (n > 0 && !d_rec) || bpp < 12 || (bpp & 1) || bpp > kGatherMaxBpp || !hdr ||
        n >= ((int64_t)1 << 31))
        return CR_ERR_INVALID_ARG;
    if (n <= 1) return CR_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const MortonFrame f = morton_frame(hdr);
    unsigned long long *k0 = nullptr, *k1 = nullptr;
    uint32_t *v0 = nullptr, *v1 = nullptr;
    uint8_t* tmp = nullptr;
    void* cub_tmp = nullptr;
    size_t cub_bytes = 0;
    cudaError_t e = cudaMalloc(&k0, n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&k1, n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&v0, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&v1, n * 4);
    if (e == cudaSuccess) {
        k_morton_keys<<<grid_for(n), 256, 0, s>>>(f, d_rec, n, bpp, k0, v0);
        e = cudaGetLastError();
    }
    cub::DoubleBuffer<unsigned long long> keys(k0, k1);
    cub::DoubleBuffer<uint32_t> vals(v0, v1);
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, keys, vals, (int)n, 0, 63, s);
    if (e == cudaSuccess) e = cudaMalloc(&cub_tmp, cub_bytes);
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, keys, vals, (int)n, 0, 63, s);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, (size_t)n * bpp);
    if (e == cudaSuccess) {
        const int64_t warps = (n + 31) / 32;
        const int grid = (int)std::min<int64_t>((warps + kGatherWarps - 1) / kGatherWarps, 65535);
        k_gather<<<grid, 32 * kGatherWarps, 0, s>>>(d_rec, tmp, vals.Current(), n, bpp);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rec, tmp, (size_t)n * bpp, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    void* ptrs[6] = {k0, k1, v0, v1, tmp, cub_tmp};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    return cuda_status(e);
}

cr_status cr_encode_las_device(cr_ctx* ctx, const uint8_t* d_rec, int64_t n, int32_t bpp, int32_t fmt,
                               const double scale[3], const double offset[3], const double box_min[3],
                               int64_t sparse_offset, int32_t file_index, cr_batch* d_batches,
                               uint32_t* d_lo, uint32_t* d_md, uint32_t* d_hi, uint32_t* d_rgba,
                               void* stream) {
    if (!ctx) return CR_ERR_INVALID_ARG;
    // LasLoaderSparse.cpp:123-131: formats without RGB read their colour at byte 0
    const int rgb = fmt == 2 ? 20 : (fmt == 3 ? 28 : ((fmt == 7 || fmt == 8) ? 30 : 0));
    return cr::encode_records_device(d_rec, n, bpp, rgb, scale, offset, box_min, sparse_offset, file_index,
                                     d_batches, d_lo, d_md, d_hi, d_rgba, stream);
}

cr_status cr_synth_cloud_device(cr_ctx* ctx, const cr_synth_params* p, int64_t n, cr_cloud* cloud,
                                cr_las_header* hdr, void* stream) {
    if (!ctx || !valid_params(p) || !cloud || !hdr || n <= 0) return CR_ERR_INVALID_ARG;
    if (cr_cloud_num_points(cloud) != n || cr_cloud_num_batches(cloud) != cr_num_batches(n))
        return CR_ERR_INVALID_ARG;
    cr_batch* db;
    uint32_t *lo, *md, *hi, *rgba;
    cr_status st = cr_cloud_device(cloud, &db, &lo, &md, &hi, &rgba);
    if (st != CR_OK || !lo || !md || !hi || !rgba) return CR_ERR_INVALID_ARG;
    uint8_t* rec = nullptr;
    cudaError_t e = cudaMalloc(&rec, (size_t)n * kRecBytes);
    if (e != cudaSuccess) return cuda_status(e);
    st = cr_synth_points_device(ctx, p, n, rec, hdr, stream);
    if (st == CR_OK) st = cr_morton_sort_device(ctx, rec, n, kRecBytes, hdr, stream);
    if (st == CR_OK)
        st = cr_encode_las_device(ctx, rec, n, kRecBytes, 2, hdr->scale, hdr->offset, hdr->min, 0, 0, db,
                                  lo, md, hi, rgba, stream);
    if (st == CR_OK) st = cuda_status(cudaStreamSynchronize((cudaStream_t)stream));
    cudaFree(rec);
    if (st == CR_OK) st = cr_cloud_set_files(ctx, cloud, hdr->min);
    return st;
}

cr_status cr_synth_uniform_host(uint64_t seed, int64_t n, float size, cr_vertex* out) {
    if (n < 0 || (n > 0 && !out)) return CR_ERR_INVALID_ARG;
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; i++) out[i] = uniform_vertex(seed, (uint64_t)i, size);
    });
    return CR_OK;
}

cr_status cr_synth_uniform_device(cr_ctx* ctx, uint64_t seed, int64_t n, float size, cr_vertex* d_out,
                                  void* stream) {
    if (!ctx || n < 0 || (n > 0 && !d_out)) return CR_ERR_INVALID_ARG;
    if (n == 0) return CR_OK;
    k_uniform<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(seed, n, size, d_out);
    return cuda_status(cudaGetLastError());
}

}  // extern "C"
