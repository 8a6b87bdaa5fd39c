/*
 * oracle.h -- scalar CPU restatement of the point-rasterizer hot path of
 * m-schuetz/compute_rasterizer.  TEST INFRASTRUCTURE ONLY: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark load it as the
 * checker.  The product (compute_rasterizer_gb300) never links or calls it.
 *
 * Parity status: the reference's kernels are GLSL compute shaders, which need
 * an OpenGL context (none exists here), and its host loader needs
 * OpenGL/GLFW/ImGui headers.  What builds from its sources, by oracle/Makefile
 * into oracle/_ref: the vendored glm (the CPU tests pin this file's matrix
 * setup to it), Sort_Frugal's Morton code, the vendored LASzip, and the GLSL
 * shaders themselves, translated statement by statement to C++ against that
 * glm (glsl_cpp.py, glsl_prelude.hpp) and run on the CPU (shader_ref.cpp).
 * In its literal arithmetic mode (or_set_arith) this file equals those
 * shaders bit for bit (tests/test_cpu_shader_pin.py: loop_las, loop_las2,
 * HQS depth / color / resolve, the loop_las and early-z resolves, early-z,
 * the dedup and early-z & reduce warp variants, loop_nodes); the contract
 * mode below, which the kernels follow, differs from it only by the FMA and
 * reciprocal choices GLSL leaves to the driver.
 *
 * ARITHMETIC CONTRACT (GLSL leaves division, length() and contraction to the
 * driver; this contract fixes them, and the CUDA kernels follow it bit for bit):
 *   - IEEE binary32/binary64, round-to-nearest-even, no implicit contraction
 *     (compiled with -ffp-contract=off); every FMA below is written explicitly.
 *   - scalar x / y and sqrt: correctly rounded.  A vector divided by a scalar
 *     (v / s in GLSL) is v * RN(1/s): one correctly rounded reciprocal,
 *     multiplied into each component, which is how shader compilers emit it.
 *   - matrix * matrix (glm order): R[c][r] = ((A[0][r]*B[c][0] + A[1][r]*B[c][1])
 *     + A[2][r]*B[c][2]) + A[3][r]*B[c][3]; no FMA.  Matrices are column-major,
 *     element (c, r) stored at [c*4 + r].
 *   - per-batch math (frustum planes, cull, precision level): plain mul/add in
 *     the order GLSL writes them, dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z,
 *     length(v) = sqrt(dot(v, v)), mat4*vec4 = ((m0*v.x + m1*v.y) + m2*v.z) + m3*v.w.
 *   - per-point math (decode + project), explicit FMA:
 *       x  = fma(float(X), boxSize.x / STEPS, min.x)      (STEPS = 2^10 or 2^30)
 *       p.c = fma(T[2][c], z, fma(T[1][c], y, fma(T[0][c], x, T[3][c])))  c = x, y, w
 *       r  = 1 / p.w (correctly rounded);  q = p.x * r, p.y * r
 *       inside = w > 0 && -1 <= qx <= 1 && -1 <= qy <= 1   (NaN is outside)
 *       px = int(fma(qx, 0.5, 0.5) * float(W))  (truncation; same for y/H)
 *       pixel = px + py * W
 *     p.z is never used by the reference (only its division), so it is not formed.
 *   - framebuffers carry a guard tail of W + 1 entries past W*H: the reference
 *     writes pixel W*H + px when q == 1 exactly (render.cs:404-409) and relies
 *     on an over-allocated buffer (compute_loop_las.h:130-138).
 */
#ifndef CR_ORACLE_H
#define CR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 64 B batch record: render.cs:22-40, written by LasLoaderSparse.cpp:109-121. */
typedef struct or_batch {
    int32_t state;
    float min_x, min_y, min_z;
    float max_x, max_y, max_z;
    int32_t num_points;
    int32_t first_point;
    int32_t file_index;
    int32_t padding[6];
} or_batch;

/* Plain 16 B point: compute_2021_earlyz/render.cs:15-20. */
typedef struct or_vertex {
    float x, y, z;
    uint32_t color;
} or_vertex;

/* Per-file uniforms the shaders read (render.cs:44-49 File + UniformData). */
typedef struct or_file_frame {
    float transform[16];   /* mat4(proj * view * translate(boxMin)), double product then cast */
    float planes[6][4];    /* frustumPlanes(transformFrustum): normal.xyz, constant */
    float view_world[16];  /* uniforms.view * file.world, float product */
} or_file_frame;

/* Quirk switches (reference behaviours kept for drop-in parity). */
enum {
    OR_QUIRK_L0_X12 = 1,       /* H1: 30-bit decode uses X_12 for Y and Z (render.cs:352-353) */
    OR_QUIRK_INCLUSIVE_END = 2, /* H2: `localIndex > numPoints` bound (las2/render.cs:341, hqs/depth.cs:276) */
    OR_QUIRK_DISPATCH_BY_POINTS = 4, /* H3: dispatch ceil(numPoints/10240) batch records (compute_loop_las2.h:234) */
    OR_QUIRK_UVEC4_BASE = 8,  /* H6: las2's uvec4 addressing from firstPoint/4 (las2/render.cs:319-341) */
    OR_QUIRK_RESOLVE_TILES = 16, /* resolves cover floor(W/16) x floor(H/16) tiles (compute_2021_earlyz.h:161-163) */
    OR_QUIRK_NODE_LOOP = 32,     /* loop_nodes' per-node loop (compute_loop_nodes/render.cs:296-300) */
    OR_QUIRK_LEVEL4_80PX = 64,   /* level 4 below 80 px (compute_loop_nodes/render.cs:199) */
    OR_QUIRK_ONE_WORLD = 128     /* every batch uses file 0 (Potree batches hold the level there) */
};

enum { OR_PAYLOAD_INDEX = 0, OR_PAYLOAD_COLOR = 1 };

/* Arithmetic interpretation of the shader math (oracle.c, or_set_arith):
 * CONTRACT is the contract above (the kernels' arithmetic); LITERAL evaluates
 * the shader source operation by operation with glm's operators, as the
 * reference shaders compiled as C++ do (oracle/shader_ref.cpp), which pins
 * everything but the contract's FMA and reciprocal choices to the reference's
 * own source.  Returns the previous mode; process-wide, set it before
 * or_file_setup and the raster calls. */
enum { OR_ARITH_CONTRACT = 0, OR_ARITH_LITERAL = 1 };
int or_set_arith(int mode);

typedef struct or_frame {
    float proj[16];
    int32_t width, height;
    int32_t frustum_culling;
    int32_t quirks;
    int32_t payload;
    int32_t lod_skip_level; /* >0: skip batches at precision level >= this
                               (compute_loop_nodes/render.cs:273-276 uses 4) */
    int32_t num_files;
    const or_file_frame* files;
} or_frame;

/* ---- host matrix setup (A0) ---------------------------------------------- */
void or_mat4d_mul(const double* a, const double* b, double* out);
void or_mat4f_mul(const float* a, const float* b, float* out);
void or_perspective(double fovy_rad, double aspect, double znear, double zfar, double out[16]);
void or_look_at(const double eye[3], const double center[3], const double up[3], double out[16]);
void or_inverse(const double m[16], double out[16]);
void or_orbit_world(double yaw, double pitch, double radius, const double target[3], double out[16]);
void or_frustum_planes(const float m[16], float planes[6][4]);
void or_file_setup(const double view[16], const double proj[16], const double box_min[3],
                   or_file_frame* out);
/* compute_loop_nodes.h:128-139: the uniforms as float matrix products */
void or_file_setup_float(const double view[16], const double proj[16], const double box_min[3],
                         or_file_frame* out);
void or_proj_float(const double proj[16], float out[16]);

/* ---- per-batch culling and precision level (A4, A5) ----------------------- */
int or_intersects_frustum(const float planes[6][4], const float wmin[3], const float wmax[3]);
int or_precision_level(const or_frame* fr, const or_file_frame* file, const float wmin[3],
                       const float wmax[3]);

/* ---- batched atomicMin path: loop_las / loop_las_prefetch (A6-A9) --------- */
int64_t or_points_in_batch(const or_batch* b, int32_t quirks);
int64_t or_dispatch_batches(int64_t num_batch_records, int64_t num_points, int32_t quirks);
void or_raster_batched(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                       int64_t num_points, const uint32_t* xyz_low, const uint32_t* xyz_med,
                       const uint32_t* xyz_hig, const uint32_t* rgba, uint64_t* fb);
void or_raster_batched_mt(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                          int64_t num_points, const uint32_t* xyz_low, const uint32_t* xyz_med,
                          const uint32_t* xyz_hig, const uint32_t* rgba, uint64_t* fb,
                          int threads);
/* resolve.cs:100-193 (window 0): index payload -> ssRGBA gather, 0 -> background */
void or_resolve_index(int32_t width, int32_t height, const uint64_t* fb, const uint32_t* rgba,
                      uint32_t* out);
/* the same over the floor(W/16) x floor(H/16) tiles only (compute_loop_nodes.h:199-201):
 * other pixels of `out` keep their values */
void or_resolve_index_tiles(int32_t width, int32_t height, const uint64_t* fb,
                            const uint32_t* rgba, uint32_t* out);
/* color payload: the low word is already the color */
void or_resolve_color(int32_t width, int32_t height, const uint64_t* fb, uint32_t* out);
void or_fill_u64(uint64_t* buf, int64_t n, uint64_t value);

/* ---- HQS two-pass (A12-A15) ------------------------------------------------ */
void or_hqs_depth(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                  int64_t num_points, const uint32_t* xyz_low, const uint32_t* xyz_med,
                  const uint32_t* xyz_hig, uint32_t* depth);
void or_hqs_color(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                  int64_t num_points, const uint32_t* xyz_low, const uint32_t* xyz_med,
                  const uint32_t* xyz_hig, const uint32_t* rgba, const uint32_t* depth,
                  uint64_t* accum);
void or_hqs_resolve(int32_t width, int32_t height, const uint64_t* accum, uint32_t* out);

/* ---- plain 16 B path: compute_2021_earlyz (A16, A17) ---------------------- */
void or_plain_transform(const double view[16], const double proj[16], float out[16]);
void or_raster_plain(const float transform[16], int32_t width, int32_t height,
                     const or_vertex* v, int64_t n, uint64_t* fb);
/* compute_2021_dedup (variant 1) / compute_2021_earlyz_reduce (variant 2):
 * warp reductions over 32 consecutive points, key depth << 24 | color. */
void or_raster_plain_warp(const float T[16], int32_t W, int32_t H, const or_vertex* v, int64_t n,
                          uint64_t* fb, int32_t variant);
/* quirks: OR_QUIRK_RESOLVE_TILES; zero_rule: ucol == 0 resolves to (0,0,0,255)
 * (early-z and early-z & reduce; the dedup resolve has no such rule). */
void or_resolve_plain(int32_t width, int32_t height, uint64_t* fb, uint8_t* out_rgba8,
                      uint64_t reclear, int32_t quirks, int32_t zero_rule);

/* ---- LAS-derived layout builder: LasLoaderSparse.cpp:37-212 (A1, A2) ----- */
int64_t or_num_batches(int64_t n);
void or_encode_las(const uint8_t* records, int64_t n, int32_t bytes_per_point,
                   int32_t point_format, const double scale[3], const double offset[3],
                   const double box_min[3], int64_t sparse_offset, int32_t file_index,
                   or_batch* batches, uint32_t* xyz_low, uint32_t* xyz_med, uint32_t* xyz_hig,
                   uint32_t* rgba);
/* LasLoaderStandard.h:152-179: LAS -> 16 B float xyz + RGBA8 */
void or_encode_standard(const uint8_t* records, int64_t n, int32_t bytes_per_point,
                        int32_t point_format, const double scale[3], const double offset[3],
                        const double box_min[3], or_vertex* out);

/* ---- Morton order: tools/sort_points/Sort_Frugal/src/main.cpp:58-105 ------ */
uint64_t or_morton3(uint32_t x, uint32_t y, uint32_t z);

/* FNV-1a 64 over bytes: the golden-vector digest */
uint64_t or_fnv1a64(const void* data, int64_t bytes);

#ifdef __cplusplus
}
#endif
#endif
