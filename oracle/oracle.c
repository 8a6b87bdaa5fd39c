/*
 * oracle.c -- scalar C restatement of the compute_rasterizer hot path.
 * TEST INFRASTRUCTURE: loaded only by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker.  The arithmetic contract is
 * written in oracle.h.  Build: oracle/Makefile (gcc -O2 -ffp-contract=off).
 *
 * Every function names the reference file:line whose behaviour it restates
 * (paths relative to the m-schuetz/compute_rasterizer tree).
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#define STEPS_30BIT 1073741824.0
#define STEPS_10BIT 1024.0
#define MASK_10BIT 1023u
#define POINTS_PER_BATCH 10240 /* Resources.h:4-6: 80 points x 128 threads */

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* ------------------------------------------------------------------------- */
/* A0: host matrix setup                                                      */
/* ------------------------------------------------------------------------- */

/* glm mat4 * mat4 (type_mat4x4.inl operator*): column c of the result is
 * A[0]*B[c][0] + A[1]*B[c][1] + A[2]*B[c][2] + A[3]*B[c][3], summed left to right. */
void or_mat4d_mul(const double* a, const double* b, double* out) {
    double r[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            double s = a[0 * 4 + row] * b[c * 4 + 0];
            s = s + a[1 * 4 + row] * b[c * 4 + 1];
            s = s + a[2 * 4 + row] * b[c * 4 + 2];
            s = s + a[3 * 4 + row] * b[c * 4 + 3];
            r[c * 4 + row] = s;
        }
    memcpy(out, r, sizeof(r));
}

void or_mat4f_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            float s = a[0 * 4 + row] * b[c * 4 + 0];
            s = s + a[1 * 4 + row] * b[c * 4 + 1];
            s = s + a[2 * 4 + row] * b[c * 4 + 2];
            s = s + a[3 * 4 + row] * b[c * 4 + 3];
            r[c * 4 + row] = s;
        }
    memcpy(out, r, sizeof(r));
}

/* Camera.h:34-39 -> glm::perspective (right-handed, clip z in [-1, 1]). */
void or_perspective(double fovy, double aspect, double zn, double zf, double out[16]) {
    double t = tan(fovy / 2.0);
    memset(out, 0, 16 * sizeof(double));
    out[0] = 1.0 / (aspect * t);
    out[5] = 1.0 / t;
    out[10] = -(zf + zn) / (zf - zn);
    out[11] = -1.0;
    out[14] = -(2.0 * zf * zn) / (zf - zn);
}

static void vnorm3(const double v[3], double o[3]) {
    double d = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
    double inv = 1.0 / sqrt(d);
    o[0] = v[0] * inv; o[1] = v[1] * inv; o[2] = v[2] * inv;
}
static void vcross3(const double a[3], const double b[3], double o[3]) {
    double x = a[1] * b[2] - b[1] * a[2];
    double y = a[2] * b[0] - b[2] * a[0];
    double z = a[0] * b[1] - b[0] * a[1];
    o[0] = x; o[1] = y; o[2] = z;
}
static double vdot3(const double a[3], const double b[3]) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

/* Right-handed look-at view matrix (the config-1 camera). */
void or_look_at(const double eye[3], const double center[3], const double up[3], double out[16]) {
    double d[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    double f[3], s[3], u[3], t[3];
    vnorm3(d, f);
    vcross3(f, up, t);
    vnorm3(t, s);
    vcross3(s, f, u);
    memset(out, 0, 16 * sizeof(double));
    out[0] = s[0]; out[4] = s[1]; out[8] = s[2];
    out[1] = u[0]; out[5] = u[1]; out[9] = u[2];
    out[2] = -f[0]; out[6] = -f[1]; out[10] = -f[2];
    out[12] = -vdot3(s, eye);
    out[13] = -vdot3(u, eye);
    out[14] = vdot3(f, eye);
    out[15] = 1.0;
}

/* General 4x4 inverse by cofactors (2x2 minors of the lower and upper row
 * pairs), divided by the determinant.  Camera.h:35 `view = inverse(world)`. */
void or_inverse(const double m[16], double out[16]) {
#define M(c, r) m[(c) * 4 + (r)]
    /* 2x2 minors over rows (2,3) and rows (0,1), indexed by column pair */
    double s0 = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
    double s1 = M(0, 0) * M(2, 1) - M(2, 0) * M(0, 1);
    double s2 = M(0, 0) * M(3, 1) - M(3, 0) * M(0, 1);
    double s3 = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    double s4 = M(1, 0) * M(3, 1) - M(3, 0) * M(1, 1);
    double s5 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1);
    double c5 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    double c4 = M(1, 2) * M(3, 3) - M(3, 2) * M(1, 3);
    double c3 = M(1, 2) * M(2, 3) - M(2, 2) * M(1, 3);
    double c2 = M(0, 2) * M(3, 3) - M(3, 2) * M(0, 3);
    double c1 = M(0, 2) * M(2, 3) - M(2, 2) * M(0, 3);
    double c0 = M(0, 2) * M(1, 3) - M(1, 2) * M(0, 3);
    double det = (s0 * c5 - s1 * c4 + s2 * c3) + (s3 * c2 - s4 * c1 + s5 * c0);
    double id = 1.0 / det;
    double r[16];
#define R(c, rr) r[(c) * 4 + (rr)]
    R(0, 0) = (M(1, 1) * c5 - M(2, 1) * c4 + M(3, 1) * c3) * id;
    R(1, 0) = (-M(1, 0) * c5 + M(2, 0) * c4 - M(3, 0) * c3) * id;
    R(2, 0) = (M(1, 3) * s5 - M(2, 3) * s4 + M(3, 3) * s3) * id;
    R(3, 0) = (-M(1, 2) * s5 + M(2, 2) * s4 - M(3, 2) * s3) * id;
    R(0, 1) = (-M(0, 1) * c5 + M(2, 1) * c2 - M(3, 1) * c1) * id;
    R(1, 1) = (M(0, 0) * c5 - M(2, 0) * c2 + M(3, 0) * c1) * id;
    R(2, 1) = (-M(0, 3) * s5 + M(2, 3) * s2 - M(3, 3) * s1) * id;
    R(3, 1) = (M(0, 2) * s5 - M(2, 2) * s2 + M(3, 2) * s1) * id;
    R(0, 2) = (M(0, 1) * c4 - M(1, 1) * c2 + M(3, 1) * c0) * id;
    R(1, 2) = (-M(0, 0) * c4 + M(1, 0) * c2 - M(3, 0) * c0) * id;
    R(2, 2) = (M(0, 3) * s4 - M(1, 3) * s2 + M(3, 3) * s0) * id;
    R(3, 2) = (-M(0, 2) * s4 + M(1, 2) * s2 - M(3, 2) * s0) * id;
    R(0, 3) = (-M(0, 1) * c3 + M(1, 1) * c1 - M(2, 1) * c0) * id;
    R(1, 3) = (M(0, 0) * c3 - M(1, 0) * c1 + M(2, 0) * c0) * id;
    R(2, 3) = (-M(0, 3) * s3 + M(1, 3) * s1 - M(2, 3) * s0) * id;
    R(3, 3) = (M(0, 2) * s3 - M(1, 2) * s1 + M(2, 2) * s0) * id;
#undef R
#undef M
    memcpy(out, r, sizeof(r));
}

/* OrbitControls.h:116-135: world = translate(target) * rotZ(yaw) * rotX(pitch)
 * * flip * translate(0, 0, radius), with rotation entries as glm::rotate forms
 * them for the unit axes (diagonal term c + (1 - c) on the axis). */
void or_orbit_world(double yaw, double pitch, double radius, const double target[3], double out[16]) {
    double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, target[0], target[1], target[2], 1};
    double cy = cos(yaw), sy = sin(yaw), cp = cos(pitch), sp = sin(pitch);
    double Ry[16] = {cy, sy, 0, 0, -sy, cy, 0, 0, 0, 0, cy + (1.0 - cy), 0, 0, 0, 0, 1};
    double Rp[16] = {cp + (1.0 - cp), 0, 0, 0, 0, cp, sp, 0, 0, -sp, cp, 0, 0, 0, 0, 1};
    double F[16] = {1, 0, 0, 0, 0, 0, 1, 0, 0, -1, 0, 0, 0, 0, 0, 1};
    double Tr[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, radius, 1};
    double a[16], b[16], c[16], d[16];
    or_mat4d_mul(T, Ry, a);
    or_mat4d_mul(a, Rp, b);
    or_mat4d_mul(b, F, c);
    or_mat4d_mul(c, Tr, d);
    memcpy(out, d, sizeof(d));
}

/* Arithmetic interpretation (or_set_arith).  OR_ARITH_CONTRACT: the contract
 * in oracle.h, which the kernels follow.  OR_ARITH_LITERAL: the shader source
 * evaluated operation by operation in IEEE binary32 with glm's operators --
 * what the reference shaders compute when compiled as C++ against the
 * reference's glm (oracle/shader_ref.cpp): mul then add in the decode,
 * mat4 * vec4 = (m0 x + m1 y) + (m2 z + m3 w) (glm's type_mat4x4.inl), a vector
 * divided by a scalar divides each component.  Everything else is shared. */
static int g_arith = OR_ARITH_CONTRACT;
int or_set_arith(int mode) {
    const int old = g_arith;
    g_arith = mode;
    return old;
}

/* render.cs:134-143 createPlane + :145-174 frustumPlanes. */
static void create_plane(float x, float y, float z, float w, float out[4]) {
    float len = sqrtf((x * x + y * y) + z * z);
    if (g_arith == OR_ARITH_LITERAL) {
        out[0] = x / len;
        out[1] = y / len;
        out[2] = z / len;
    } else {
        float inv = 1.0f / len; /* vec3(x, y, z) / nLength: one reciprocal */
        out[0] = x * inv;
        out[1] = y * inv;
        out[2] = z * inv;
    }
    out[3] = w / len;
}

void or_frustum_planes(const float m[16], float planes[6][4]) {
    create_plane(m[3] - m[0], m[7] - m[4], m[11] - m[8], m[15] - m[12], planes[0]);
    create_plane(m[3] + m[0], m[7] + m[4], m[11] + m[8], m[15] + m[12], planes[1]);
    create_plane(m[3] + m[1], m[7] + m[5], m[11] + m[9], m[15] + m[13], planes[2]);
    create_plane(m[3] - m[1], m[7] - m[5], m[11] - m[9], m[15] - m[13], planes[3]);
    create_plane(m[3] - m[2], m[7] - m[6], m[11] - m[10], m[15] - m[14], planes[4]);
    create_plane(m[3] + m[2], m[7] + m[6], m[11] + m[10], m[15] + m[14], planes[5]);
}

/* compute_loop_las.h:141-200: per file, world = translate(boxMin) in double,
 * transform = mat4(proj * view * world), transformFrustum = transform,
 * fWorld = mat4(world); UBO view = mat4(view). */
void or_file_setup(const double view[16], const double proj[16], const double box_min[3],
                   or_file_frame* out) {
    double world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, box_min[0], box_min[1], box_min[2], 1};
    double pv[16], t[16];
    or_mat4d_mul(proj, view, pv);
    or_mat4d_mul(pv, world, t);
    float fview[16], fworld[16];
    for (int i = 0; i < 16; i++) {
        out->transform[i] = (float)t[i];
        fview[i] = (float)view[i];
        fworld[i] = (float)world[i];
    }
    or_frustum_planes(out->transform, out->planes);
    or_mat4f_mul(fview, fworld, out->view_world);
}

/* compute_loop_nodes.h:128-139: mat4 view, proj (float casts of the double
 * matrices), worldViewProj = proj * view * world in float. */
void or_file_setup_float(const double view[16], const double proj[16], const double box_min[3],
                         or_file_frame* out) {
    double world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, box_min[0], box_min[1], box_min[2], 1};
    float fv[16], fp[16], fw[16], pv[16];
    for (int i = 0; i < 16; i++) {
        fv[i] = (float)view[i];
        fp[i] = (float)proj[i];
        fw[i] = (float)world[i];
    }
    or_mat4f_mul(fp, fv, pv);
    or_mat4f_mul(pv, fw, out->transform);
    or_frustum_planes(out->transform, out->planes);
    or_mat4f_mul(fv, fw, out->view_world);
}

void or_proj_float(const double proj[16], float out[16]) {
    for (int i = 0; i < 16; i++) out[i] = (float)proj[i];
}

/* ------------------------------------------------------------------------- */
/* A4, A5: per-batch cull and precision level                                 */
/* ------------------------------------------------------------------------- */

/* render.cs:176-197 */
int or_intersects_frustum(const float planes[6][4], const float wmin[3], const float wmax[3]) {
    for (int i = 0; i < 6; i++) {
        const float* p = planes[i];
        float vx = p[0] > 0.0f ? wmax[0] : wmin[0];
        float vy = p[1] > 0.0f ? wmax[1] : wmin[1];
        float vz = p[2] > 0.0f ? wmax[2] : wmin[2];
        float d = ((p[0] * vx + p[1] * vy) + p[2] * vz) + p[3];
        if (d < 0.0f) return 0;
    }
    return 1;
}

static void mat4_vec4(const float m[16], const float v[4], float o[4]) {
    for (int r = 0; r < 4; r++) {
        if (g_arith == OR_ARITH_LITERAL) {
            o[r] = (m[0 * 4 + r] * v[0] + m[1 * 4 + r] * v[1]) + (m[2 * 4 + r] * v[2] + m[3 * 4 + r] * v[3]);
            continue;
        }
        float s = m[0 * 4 + r] * v[0];
        s = s + m[1 * 4 + r] * v[1];
        s = s + m[2 * 4 + r] * v[2];
        s = s + m[3 * 4 + r] * v[3];
        o[r] = s;
    }
}

/* render.cs:199-231 getPrecisionLevel */
int or_precision_level(const or_frame* fr, const or_file_frame* file, const float wmin[3],
                       const float wmax[3]) {
    float c[4] = {(wmin[0] + wmax[0]) / 2.0f, (wmin[1] + wmax[1]) / 2.0f,
                  (wmin[2] + wmax[2]) / 2.0f, 1.0f};
    float dx = wmin[0] - wmax[0], dy = wmin[1] - wmax[1], dz = wmin[2] - wmax[2];
    float radius = sqrtf((dx * dx + dy * dy) + dz * dz);
    float vc[4], ve[4], pc[4], pe[4];
    mat4_vec4(file->view_world, c, vc);
    ve[0] = vc[0] + radius; ve[1] = vc[1] + 0.0f; ve[2] = vc[2] + 0.0f; ve[3] = vc[3] + 0.0f;
    mat4_vec4(fr->proj, vc, pc);
    mat4_vec4(fr->proj, ve, pe);
    float pcx, pcy, pex, pey;
    if (g_arith == OR_ARITH_LITERAL) {
        pcx = pc[0] / pc[3]; pcy = pc[1] / pc[3];
        pex = pe[0] / pe[3]; pey = pe[1] / pe[3];
    } else {
        float rc = 1.0f / pc[3], re = 1.0f / pe[3]; /* xy / w: one reciprocal each */
        pcx = pc[0] * rc; pcy = pc[1] * rc;
        pex = pe[0] * re; pey = pe[1] * re;
    }
    float W = (float)fr->width, H = (float)fr->height;
    float scx = (W * (pcx + 1.0f)) / 2.0f, scy = (H * (pcy + 1.0f)) / 2.0f;
    float sex = (W * (pex + 1.0f)) / 2.0f, sey = (H * (pey + 1.0f)) / 2.0f;
    float ex = sex - scx, ey = sey - scy;
    float px = sqrtf(ex * ex + ey * ey);
    if (px < ((fr->quirks & OR_QUIRK_LEVEL4_80PX) ? 80.0f : 100.0f)) return 4;
    if (px < 200.0f) return 3;
    if (px < 500.0f) return 2;
    if (px < 10000.0f) return 1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* per-point decode + projection (A6, A7)                                     */
/* ------------------------------------------------------------------------- */

typedef struct {
    float minx, miny, minz;
    float sx, sy, sz; /* boxSize / STEPS for the batch's level */
    int level;
} batch_decode;

static void make_decode(const or_batch* b, int level, batch_decode* d) {
    float bx = b->max_x - b->min_x, by = b->max_y - b->min_y, bz = b->max_z - b->min_z;
    float steps = level >= 2 ? (float)STEPS_10BIT : (float)STEPS_30BIT;
    d->minx = b->min_x; d->miny = b->min_y; d->minz = b->min_z;
    d->sx = bx / steps; d->sy = by / steps; d->sz = bz / steps;
    d->level = level;
}

/* render.cs:333-397 (loop_las), compute_loop_las2/render.cs:319-469 */
static void decode_point(const batch_decode* d, int32_t quirks, int64_t idx, const uint32_t* lo,
                         const uint32_t* md, const uint32_t* hi, float p[3]) {
    uint32_t X, Y, Z;
    uint32_t b4 = lo[idx];
    if (d->level >= 2) {
        X = b4 & MASK_10BIT; Y = (b4 >> 10) & MASK_10BIT; Z = (b4 >> 20) & MASK_10BIT;
    } else {
        uint32_t b8 = md[idx];
        X = ((b4 & MASK_10BIT) << 20) | ((b8 & MASK_10BIT) << 10);
        Y = (((b4 >> 10) & MASK_10BIT) << 20) | (((b8 >> 10) & MASK_10BIT) << 10);
        Z = (((b4 >> 20) & MASK_10BIT) << 20) | (((b8 >> 20) & MASK_10BIT) << 10);
        if (d->level == 0) {
            uint32_t b12 = hi[idx];
            uint32_t x12 = b12 & MASK_10BIT;
            uint32_t y12 = (b12 >> 10) & MASK_10BIT;
            uint32_t z12 = (b12 >> 20) & MASK_10BIT;
            if (quirks & OR_QUIRK_L0_X12) { y12 = x12; z12 = x12; }
            X |= x12; Y |= y12; Z |= z12;
        }
    }
    if (g_arith == OR_ARITH_LITERAL) {
        p[0] = (float)X * d->sx + d->minx;
        p[1] = (float)Y * d->sy + d->miny;
        p[2] = (float)Z * d->sz + d->minz;
        return;
    }
    p[0] = fmaf((float)X, d->sx, d->minx);
    p[1] = fmaf((float)Y, d->sy, d->miny);
    p[2] = fmaf((float)Z, d->sz, d->minz);
}

/* render.cs:399-409: returns 1 and the pixel id if the point lands inside */
static int project(const float T[16], int32_t W, int32_t H, const float p[3], int32_t* pix,
                   float* w_out) {
    const int lit = g_arith == OR_ARITH_LITERAL;
    float x, y, w;
    if (lit) { /* file.transform * vec4(point, 1.0) in glm's association */
        x = (T[0] * p[0] + T[4] * p[1]) + (T[8] * p[2] + T[12] * 1.0f);
        y = (T[1] * p[0] + T[5] * p[1]) + (T[9] * p[2] + T[13] * 1.0f);
        w = (T[3] * p[0] + T[7] * p[1]) + (T[11] * p[2] + T[15] * 1.0f);
    } else {
        x = fmaf(T[8], p[2], fmaf(T[4], p[1], fmaf(T[0], p[0], T[12])));
        y = fmaf(T[9], p[2], fmaf(T[5], p[1], fmaf(T[1], p[0], T[13])));
        w = fmaf(T[11], p[2], fmaf(T[7], p[1], fmaf(T[3], p[0], T[15])));
    }
    /* render.cs:404 `!(w <= 0 || x < -1 || ...)`, written positively so that
     * a NaN position counts as outside */
    if (!(w > 0.0f)) return 0;
    float qx, qy;
    if (lit) {
        qx = x / w;
        qy = y / w;
    } else {
        float rw = 1.0f / w; /* pos.xyz / pos.w: one reciprocal of w */
        qx = x * rw;
        qy = y * rw;
    }
    if (!(qx >= -1.0f && qx <= 1.0f && qy >= -1.0f && qy <= 1.0f)) return 0;
    float fx = fmaf(qx, 0.5f, 0.5f) * (float)W;
    float fy = fmaf(qy, 0.5f, 0.5f) * (float)H;
    int32_t px = (int32_t)fx, py = (int32_t)fy;
    *pix = px + py * W;
    *w_out = w;
    return 1;
}

/* ------------------------------------------------------------------------- */
/* batched atomicMin path                                                     */
/* ------------------------------------------------------------------------- */

/* Points a batch's workgroup processes: render.cs:316 (`>=`, loop_las) or
 * las2/render.cs:341, hqs/depth.cs:276 (`>`, one past a partial batch), capped
 * by the 80 x 128 loop (Resources.h:4-6). */
int64_t or_points_in_batch(const or_batch* b, int32_t quirks) {
    int64_t n = b->num_points;
    if (quirks & OR_QUIRK_NODE_LOOP) {
        /* compute_loop_nodes/render.cs:296-300: loopSize = min(ceil(n / 128), 500)
         * + 4; i < loopSize / 4 iterations of one uvec4 per thread from
         * firstPoint / 4; `localIndex >= numPoints` skips (continue) */
        if (n < 0) return 0;
        int64_t loop = (n + 127) / 128;
        if (loop > 500) loop = 500;
        int64_t reach = 512 * ((loop + 4) / 4) - (b->first_point & 3);
        return n < reach ? n : reach;
    }
    if (quirks & OR_QUIRK_INCLUSIVE_END) n = n + 1;
    if (n > POINTS_PER_BATCH) n = POINTS_PER_BATCH;
    if (n < 0) n = 0;
    return n;
}

/* compute_loop_las.h:233 dispatches numBatchesLoaded workgroups;
 * compute_loop_las2.h:234 and compute_loop_las_hqs.h:238 ceil(numPoints/10240). */
int64_t or_dispatch_batches(int64_t num_records, int64_t num_points, int32_t quirks) {
    if (quirks & OR_QUIRK_DISPATCH_BY_POINTS) {
        int64_t n = (num_points + POINTS_PER_BATCH - 1) / POINTS_PER_BATCH;
        return n < num_records ? n : num_records;
    }
    return num_records;
}

typedef struct {
    const or_frame* fr;
    const or_batch* batches;
    int64_t b0, b1;
    const uint32_t *lo, *md, *hi, *rgba;
    uint64_t* fb;
    int atomic;
} raster_job;

static inline void min_u64(uint64_t* slot, uint64_t key, int atomic) {
    if (!atomic) {
        if (key < *slot) *slot = key;
        return;
    }
    _Atomic uint64_t* a = (_Atomic uint64_t*)slot;
    uint64_t cur = atomic_load_explicit(a, memory_order_relaxed);
    while (key < cur) {
        if (atomic_compare_exchange_weak_explicit(a, &cur, key, memory_order_relaxed,
                                                  memory_order_relaxed))
            break;
    }
}

/* render.cs:233-435 main(), one workgroup per batch record. */
static void raster_range(const raster_job* j) {
    const or_frame* fr = j->fr;
    for (int64_t bi = j->b0; bi < j->b1; bi++) {
        const or_batch* b = &j->batches[bi];
        const or_file_frame* file = &fr->files[(fr->quirks & OR_QUIRK_ONE_WORLD) ? 0 : b->file_index];
        float wmin[3] = {b->min_x, b->min_y, b->min_z};
        float wmax[3] = {b->max_x, b->max_y, b->max_z};
        if (fr->frustum_culling && !or_intersects_frustum(file->planes, wmin, wmax)) continue;
        int level = or_precision_level(fr, file, wmin, wmax);
        if (fr->lod_skip_level > 0 && level >= fr->lod_skip_level) continue;
        batch_decode d;
        make_decode(b, level, &d);
        int64_t count = or_points_in_batch(b, fr->quirks);
        /* H6, compute_loop_las2/render.cs:319-341: base = firstPoint / 4 + tid; thread
         * t's point (i, j) is index 4 * (base + 128 i) + j, i.e. batch point
         * l = 4 t + 512 i + j - r with r = firstPoint % 4.  Thread 0's first
         * localIndex (j - r) underflows the uint compare, so thread 0 returns at
         * once and every l with (l + r) % 512 < 4 is skipped; the threads reach
         * l = 10239 - r at most, so the last r points are never visited. */
        const int32_t r = (fr->quirks & OR_QUIRK_UVEC4_BASE) ? (b->first_point & 3) : 0;
        for (int64_t l = 0; l < count; l++) {
            if (r != 0 && (l >= POINTS_PER_BATCH - r || ((l + r) & 511) < 4)) continue;
            int64_t idx = (int64_t)b->first_point + l;
            float p[3], w;
            int32_t pix;
            decode_point(&d, fr->quirks, idx, j->lo, j->md, j->hi, p);
            if (!project(file->transform, fr->width, fr->height, p, &pix, &w)) continue;
            uint32_t payload = fr->payload == OR_PAYLOAD_COLOR ? j->rgba[idx] : (uint32_t)idx;
            uint64_t key = ((uint64_t)f2u(w) << 32) | payload;
            min_u64(&j->fb[pix], key, j->atomic);
        }
    }
}

void or_raster_batched(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                       int64_t num_points, const uint32_t* lo, const uint32_t* md,
                       const uint32_t* hi, const uint32_t* rgba, uint64_t* fb) {
    raster_job j = {fr, batches, 0, or_dispatch_batches(num_batches, num_points, fr->quirks),
                    lo, md, hi, rgba, fb, 0};
    raster_range(&j);
}

static void* raster_thread(void* arg) {
    raster_range((const raster_job*)arg);
    return NULL;
}

/* CPU baseline: the same loop over batch ranges on `threads` host threads with
 * a compare-and-swap min per pixel. */
void or_raster_batched_mt(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                          int64_t num_points, const uint32_t* lo, const uint32_t* md,
                          const uint32_t* hi, const uint32_t* rgba, uint64_t* fb, int threads) {
    int64_t nb = or_dispatch_batches(num_batches, num_points, fr->quirks);
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    raster_job jobs[256];
    for (int t = 0; t < threads; t++) {
        jobs[t] = (raster_job){fr, batches, nb * t / threads, nb * (t + 1) / threads,
                               lo, md, hi, rgba, fb, 1};
        pthread_create(&tid[t], NULL, raster_thread, &jobs[t]);
    }
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
}

/* resolve.cs:100-146, window = 0 */
void or_resolve_index(int32_t W, int32_t H, const uint64_t* fb, const uint32_t* rgba,
                      uint32_t* out) {
    int64_t P = (int64_t)W * H;
    for (int64_t p = 0; p < P; p++) {
        uint64_t v = fb[p];
        float depth = u2f((uint32_t)(v >> 32));
        uint32_t id = 0;
        if (depth > 0.0f && depth < 1000000.0f) id = (uint32_t)v;
        out[p] = id == 0 ? 0x00443322u : rgba[id];
    }
}

void or_resolve_index_tiles(int32_t W, int32_t H, const uint64_t* fb, const uint32_t* rgba,
                            uint32_t* out) {
    for (int32_t y = 0; y < H / 16 * 16; y++)
        for (int32_t x = 0; x < W / 16 * 16; x++) {
            const int64_t p = (int64_t)x + (int64_t)y * W;
            uint64_t v = fb[p];
            float depth = u2f((uint32_t)(v >> 32));
            uint32_t id = 0;
            if (depth > 0.0f && depth < 1000000.0f) id = (uint32_t)v;
            out[p] = id == 0 ? 0x00443322u : rgba[id];
        }
}

void or_resolve_color(int32_t W, int32_t H, const uint64_t* fb, uint32_t* out) {
    int64_t P = (int64_t)W * H;
    for (int64_t p = 0; p < P; p++) {
        uint64_t v = fb[p];
        float depth = u2f((uint32_t)(v >> 32));
        out[p] = (depth > 0.0f && depth < 1000000.0f) ? (uint32_t)v : 0x00443322u;
    }
}

void or_fill_u64(uint64_t* buf, int64_t n, uint64_t value) {
    for (int64_t i = 0; i < n; i++) buf[i] = value;
}

/* ------------------------------------------------------------------------- */
/* HQS                                                                        */
/* ------------------------------------------------------------------------- */

/* compute_loop_las_hqs/depth.cs:242-389 */
void or_hqs_depth(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                  int64_t num_points, const uint32_t* lo, const uint32_t* md, const uint32_t* hi,
                  uint32_t* depth) {
    int64_t nb = or_dispatch_batches(num_batches, num_points, fr->quirks);
    for (int64_t bi = 0; bi < nb; bi++) {
        const or_batch* b = &batches[bi];
        const or_file_frame* file = &fr->files[(fr->quirks & OR_QUIRK_ONE_WORLD) ? 0 : b->file_index];
        float wmin[3] = {b->min_x, b->min_y, b->min_z};
        float wmax[3] = {b->max_x, b->max_y, b->max_z};
        if (fr->frustum_culling && !or_intersects_frustum(file->planes, wmin, wmax)) continue;
        const int level = or_precision_level(fr, file, wmin, wmax);
        if (fr->lod_skip_level > 0 && level >= fr->lod_skip_level) continue;
        batch_decode d;
        make_decode(b, level, &d);
        int64_t count = or_points_in_batch(b, fr->quirks);
        for (int64_t l = 0; l < count; l++) {
            int64_t idx = (int64_t)b->first_point + l;
            float p[3], w;
            int32_t pix;
            decode_point(&d, fr->quirks, idx, lo, md, hi, p);
            if (!project(file->transform, fr->width, fr->height, p, &pix, &w)) continue;
            uint32_t dw = f2u(w);
            if (dw < depth[pix]) depth[pix] = dw;
        }
    }
}

/* compute_loop_las_hqs/color.cs:242-448: points within 1% of the pixel's min
 * depth add (R, G, B, 1); accumulators are two int64 per pixel holding
 * R | G << 32 and B | count << 32 (the resolve reads them as four uint32). */
void or_hqs_color(const or_frame* fr, const or_batch* batches, int64_t num_batches,
                  int64_t num_points, const uint32_t* lo, const uint32_t* md, const uint32_t* hi,
                  const uint32_t* rgba, const uint32_t* depth, uint64_t* accum) {
    int64_t nb = or_dispatch_batches(num_batches, num_points, fr->quirks);
    for (int64_t bi = 0; bi < nb; bi++) {
        const or_batch* b = &batches[bi];
        const or_file_frame* file = &fr->files[(fr->quirks & OR_QUIRK_ONE_WORLD) ? 0 : b->file_index];
        float wmin[3] = {b->min_x, b->min_y, b->min_z};
        float wmax[3] = {b->max_x, b->max_y, b->max_z};
        if (fr->frustum_culling && !or_intersects_frustum(file->planes, wmin, wmax)) continue;
        const int level = or_precision_level(fr, file, wmin, wmax);
        if (fr->lod_skip_level > 0 && level >= fr->lod_skip_level) continue;
        batch_decode d;
        make_decode(b, level, &d);
        int64_t count = or_points_in_batch(b, fr->quirks);
        for (int64_t l = 0; l < count; l++) {
            int64_t idx = (int64_t)b->first_point + l;
            float p[3], w;
            int32_t pix;
            decode_point(&d, fr->quirks, idx, lo, md, hi, p);
            if (!project(file->transform, fr->width, fr->height, p, &pix, &w)) continue;
            float bd = u2f(depth[pix]);
            if (!(w <= bd * 1.01f)) continue;
            uint32_t c = rgba[idx];
            uint64_t R = c & 0xFFu, G = (c >> 8) & 0xFFu, B = (c >> 16) & 0xFFu;
            accum[2 * (int64_t)pix + 0] += R | (G << 32);
            accum[2 * (int64_t)pix + 1] += B | ((uint64_t)1 << 32);
        }
    }
}

/* compute_loop_las_hqs/resolve.cs:62-130 */
void or_hqs_resolve(int32_t W, int32_t H, const uint64_t* accum, uint32_t* out) {
    int64_t P = (int64_t)W * H;
    for (int64_t p = 0; p < P; p++) {
        uint64_t a = accum[2 * p], b = accum[2 * p + 1];
        uint32_t R = (uint32_t)a, G = (uint32_t)(a >> 32);
        uint32_t B = (uint32_t)b, count = (uint32_t)(b >> 32);
        if (count == 0) {
            out[p] = 0x00443322u;
            continue;
        }
        uint32_t r = R / count, g = G / count, bb = B / count;
        out[p] = r | (g << 8) | (bb << 16);
    }
}

/* ------------------------------------------------------------------------- */
/* plain 16 B path: compute_2021_earlyz                                      */
/* ------------------------------------------------------------------------- */

/* compute_2021_earlyz.h:108-113: float mat4 product proj * view * world(identity) */
void or_plain_transform(const double view[16], const double proj[16], float out[16]) {
    float fv[16], fp[16], id[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}, pv[16];
    for (int i = 0; i < 16; i++) { fv[i] = (float)view[i]; fp[i] = (float)proj[i]; }
    or_mat4f_mul(fp, fv, pv);
    or_mat4f_mul(pv, id, out);
}

/* compute_2021_earlyz/render.cs:35-74.  The early-z filter there compares the
 * depth word only; equal-depth points that both pass it race into atomicMin,
 * so the full-key minimum is the reference's own outcome whenever the order is
 * not decisive.  This restatement keeps the per-pixel minimum key. */
void or_raster_plain(const float T[16], int32_t W, int32_t H, const or_vertex* v, int64_t n,
                     uint64_t* fb) {
    for (int64_t i = 0; i < n; i++) {
        float p[3] = {v[i].x, v[i].y, v[i].z}, w;
        int32_t pix;
        if (!project(T, W, H, p, &pix, &w)) continue;
        uint64_t key = ((uint64_t)f2u(w) << 32) | v[i].color;
        if (key < fb[pix]) fb[pix] = key;
    }
}

/* The two warp-reduction variants of the plain path, over subgroups of 32
 * consecutive points (gl_SubgroupSize on the reference's GPU; a subgroup op
 * sees only the invocations that did not return at the culling test).  Both
 * pack key = depth << 24 | color, the color's top byte overlapping the low
 * depth byte, so which points reach the atomic decides the result.
 *   variant 1: compute_2021_dedup/render.cs:33-69 -- partition by pixel id,
 *     lanes at their partition's minimum depth write.
 *   variant 2: compute_2021_earlyz_reduce/render.cs:44-82 -- if every active
 *     lane has the same pixel, only the subgroup's minimum depth writes;
 *     otherwise a lane writes unless its pair partner (lane ^ 1) is active, on
 *     the same pixel and strictly closer.
 * Points past n are not active (the reference reads past the bound range). */
void or_raster_plain_warp(const float T[16], int32_t W, int32_t H, const or_vertex* v, int64_t n,
                          uint64_t* fb, int32_t variant) {
    for (int64_t w0 = 0; w0 < n; w0 += 32) {
        int ok[32], write[32];
        int32_t pix[32];
        uint32_t depth[32];
        for (int l = 0; l < 32; l++) {
            const int64_t i = w0 + l;
            ok[l] = 0;
            write[l] = 0;
            pix[l] = 0;
            depth[l] = 0;
            if (i >= n) continue;
            float p[3] = {v[i].x, v[i].y, v[i].z}, w;
            ok[l] = project(T, W, H, p, &pix[l], &w);
            depth[l] = f2u(w);
        }
        if (variant == 1) {
            for (int l = 0; l < 32; l++) {
                if (!ok[l]) continue;
                uint32_t mind = depth[l];
                for (int m = 0; m < 32; m++)
                    if (ok[m] && pix[m] == pix[l] && depth[m] < mind) mind = depth[m];
                write[l] = depth[l] == mind;
            }
        } else {
            int first = -1, same = 1;
            uint32_t mind = 0xFFFFFFFFu;
            for (int l = 0; l < 32; l++) {
                if (!ok[l]) continue;
                if (first < 0) first = l;
                else if (pix[l] != pix[first]) same = 0;
                if (depth[l] < mind) mind = depth[l];
            }
            for (int l = 0; l < 32; l++) {
                if (!ok[l]) continue;
                const int q = l ^ 1;
                if (same) write[l] = depth[l] == mind;
                else write[l] = !ok[q] || pix[q] != pix[l] || depth[l] <= depth[q];
            }
        }
        for (int l = 0; l < 32; l++) {
            if (!write[l]) continue;
            const uint64_t key = ((uint64_t)depth[l] << 24) | v[w0 + l].color;
            if (key < fb[pix[l]]) fb[pix[l]] = key;
        }
    }
}

/* compute_2021_earlyz/resolve.cs:41-77: 24-bit color to RGBA8 through
 * unpackUnorm4x8 (c / 255) * 255, color 0 -> opaque black; then re-clear. */
/* compute_2021_earlyz/resolve.cs:41-77, compute_2021_dedup/resolve.cs:15-42,
 * compute_2021_earlyz_reduce/resolve.cs:41-77.  The reference dispatches
 * floor(W/16) x floor(H/16) groups of 16 x 16 threads (compute_2021_earlyz.h:
 * 161-163), so with OR_QUIRK_RESOLVE_TILES the pixels past the last full tile
 * keep their image and framebuffer words.  Without it every pixel is resolved
 * and the framebuffer's guard tail (W + 1 words past W*H) is re-cleared too. */
void or_resolve_plain(int32_t W, int32_t H, uint64_t* fb, uint8_t* out, uint64_t reclear,
                      int32_t quirks, int32_t zero_rule) {
    const int tiles = (quirks & OR_QUIRK_RESOLVE_TILES) != 0;
    const int32_t Wt = tiles ? W / 16 * 16 : W, Ht = tiles ? H / 16 * 16 : H;
    for (int32_t y = 0; y < Ht; y++) {
        for (int32_t x = 0; x < Wt; x++) {
            const int64_t p = (int64_t)x + (int64_t)y * W;
            uint32_t ucol = (uint32_t)(fb[p] & 0x00FFFFFFu);
            uint8_t* o = out + 4 * p;
            if (ucol == 0 && zero_rule) {
                o[0] = 0; o[1] = 0; o[2] = 0; o[3] = 255;
            } else {
                for (int k = 0; k < 4; k++) {
                    float c = (float)((ucol >> (8 * k)) & 0xFFu);
                    float f = 255.0f * (c / 255.0f);
                    o[k] = (uint8_t)(uint32_t)f;
                }
            }
            fb[p] = reclear;
        }
    }
    if (!tiles)
        for (int64_t t = 0; t <= W; t++) fb[(int64_t)W * H + t] = reclear;
}

/* ------------------------------------------------------------------------- */
/* LAS-derived layout builder                                                 */
/* ------------------------------------------------------------------------- */

int64_t or_num_batches(int64_t n) { return (n + POINTS_PER_BATCH - 1) / POINTS_PER_BATCH; }

static int32_t rd_i32(const uint8_t* p) { int32_t v; memcpy(&v, p, 4); return v; }
static uint16_t rd_u16(const uint8_t* p) { uint16_t v; memcpy(&v, p, 2); return v; }

static int rgb_offset_sparse(int fmt) {
    /* LasLoaderSparse.cpp:123-132 */
    if (fmt == 2) return 20;
    if (fmt == 3) return 28;
    if (fmt == 7) return 30;
    if (fmt == 8) return 30;
    return 0;
}

static uint32_t quantize30(double v, double lo, double size) {
    double t = ((v - lo) / size) * STEPS_30BIT;
    /* (x - min) / size is NaN for a zero-extent axis; the reference's
     * uint32_t(NaN) is undefined, defined here as 0. */
    uint32_t q = (t == t) ? (uint32_t)t : 0u;
    return q < (uint32_t)(STEPS_30BIT - 1) ? q : (uint32_t)(STEPS_30BIT - 1);
}

/* LasLoaderSparse.cpp:37-212 loadLas for one load task: batches of 10,240,
 * double AABB relative to boxMin, float AABB record, 30-bit quantisation split
 * into three 10-bit word streams, RGB16 -> RGB8. */
void or_encode_las(const uint8_t* rec, int64_t n, int32_t bpp, int32_t fmt, const double scale[3],
                   const double offset[3], const double box_min[3], int64_t sparse_offset,
                   int32_t file_index, or_batch* batches, uint32_t* lo, uint32_t* md, uint32_t* hi,
                   uint32_t* rgba) {
    int64_t nb = or_num_batches(n);
    int rgb = rgb_offset_sparse(fmt);
    for (int64_t bi = 0; bi < nb; bi++) {
        int64_t first = bi * POINTS_PER_BATCH;
        int64_t cnt = n - first < POINTS_PER_BATCH ? n - first : POINTS_PER_BATCH;
        double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t i = 0; i < cnt; i++) {
            const uint8_t* r = rec + (first + i) * bpp;
            for (int k = 0; k < 3; k++) {
                double v = (double)rd_i32(r + 4 * k) * scale[k] + offset[k] - box_min[k];
                mn[k] = v < mn[k] ? v : mn[k];
                mx[k] = mx[k] < v ? v : mx[k];
            }
        }
        double sz[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
        or_batch* b = &batches[bi];
        memset(b, 0, sizeof(*b));
        b->min_x = (float)mn[0]; b->min_y = (float)mn[1]; b->min_z = (float)mn[2];
        b->max_x = (float)mx[0]; b->max_y = (float)mx[1]; b->max_z = (float)mx[2];
        b->num_points = (int32_t)cnt;
        b->first_point = (int32_t)(sparse_offset + first);
        b->file_index = file_index;
        for (int64_t i = 0; i < cnt; i++) {
            int64_t pi = first + i;
            const uint8_t* r = rec + pi * bpp;
            uint32_t q[3];
            for (int k = 0; k < 3; k++) {
                double v = (double)rd_i32(r + 4 * k) * scale[k] + offset[k] - box_min[k];
                q[k] = quantize30(v, mn[k], sz[k]);
            }
            lo[pi] = ((q[0] >> 20) & MASK_10BIT) | (((q[1] >> 20) & MASK_10BIT) << 10) |
                     (((q[2] >> 20) & MASK_10BIT) << 20);
            md[pi] = ((q[0] >> 10) & MASK_10BIT) | (((q[1] >> 10) & MASK_10BIT) << 10) |
                     (((q[2] >> 10) & MASK_10BIT) << 20);
            hi[pi] = (q[0] & MASK_10BIT) | ((q[1] & MASK_10BIT) << 10) |
                     ((q[2] & MASK_10BIT) << 20);
            int R = rd_u16(r + rgb), G = rd_u16(r + rgb + 2), B = rd_u16(r + rgb + 4);
            R = R < 256 ? R : R / 256;
            G = G < 256 ? G : G / 256;
            B = B < 256 ? B : B / 256;
            rgba[pi] = (uint32_t)R | ((uint32_t)G << 8) | ((uint32_t)B << 16);
        }
    }
}

/* LasLoaderStandard.h:152-179 */
void or_encode_standard(const uint8_t* rec, int64_t n, int32_t bpp, int32_t fmt,
                        const double scale[3], const double offset[3], const double box_min[3],
                        or_vertex* out) {
    int rgb = fmt == 2 ? 20 : (fmt == 3 ? 28 : 0);
    for (int64_t i = 0; i < n; i++) {
        const uint8_t* r = rec + i * bpp;
        float xyz[3];
        for (int k = 0; k < 3; k++)
            xyz[k] = (float)((double)rd_i32(r + 4 * k) * scale[k] + offset[k] - box_min[k]);
        int R = rd_u16(r + rgb), G = rd_u16(r + rgb + 2), B = rd_u16(r + rgb + 4);
        uint32_t cr = (uint32_t)(R > 255 ? R / 256 : R) & 0xFFu;
        uint32_t cg = (uint32_t)(G > 255 ? G / 256 : G) & 0xFFu;
        uint32_t cb = (uint32_t)(B > 255 ? B / 256 : B) & 0xFFu;
        out[i].x = xyz[0]; out[i].y = xyz[1]; out[i].z = xyz[2];
        out[i].color = cr | (cg << 8) | (cb << 16) | (255u << 24);
    }
}

/* ------------------------------------------------------------------------- */

/* Sort_Frugal/src/main.cpp:58-77: 21 bits per axis, x in bit 0, y bit 1, z bit 2 */
static uint64_t spread3(uint32_t a) {
    uint64_t x = a & 0x1FFFFFu;
    uint64_t r = 0;
    for (int i = 0; i < 21; i++) r |= ((x >> i) & 1u) << (3 * i);
    return r;
}
uint64_t or_morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

uint64_t or_fnv1a64(const void* data, int64_t bytes) {
    const uint8_t* p = (const uint8_t*)data;
    uint64_t h = 0xcbf29ce484222325ull;
    for (int64_t i = 0; i < bytes; i++) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}
