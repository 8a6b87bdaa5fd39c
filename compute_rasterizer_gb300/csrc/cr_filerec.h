// cr_filerec.h -- the per-file uniforms of one view (compute_loop_las.h:166-200,
// render.cs:134-174), written once for host and device.  The host computes the
// records of the first kInlineFiles files into the kernel parameters; clouds
// with more files get every record computed on the GPU (k_file_records) into
// a device array the kernels index by `fileIndex`, as the reference's file
// SSBO is (render.cs:44-49, compute_loop_las.h:100,168-199).  Both sides
// compile with contraction off (-ffp-contract=off on the host, -fmad=false on
// the device) and IEEE division and square root, so the two agree bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "cr_internal.h"

namespace cr {

// glm operator*(mat4, mat4): column c = A[0]*B[c][0] + A[1]*B[c][1] + A[2]*B[c][2] + A[3]*B[c][3]
template <typename T>
__host__ __device__ inline void mat_mul(const T* a, const T* b, T* out) {
    T r[16];
    for (int c = 0; c < 4; c++) {
        for (int row = 0; row < 4; row++) {
            T s = a[row] * b[c * 4];
            s = s + a[4 + row] * b[c * 4 + 1];
            s = s + a[8 + row] * b[c * 4 + 2];
            s = s + a[12 + row] * b[c * 4 + 3];
            r[c * 4 + row] = s;
        }
    }
    for (int i = 0; i < 16; i++) out[i] = r[i];
}

// render.cs:134-174: planes from the rows of transformFrustum, normalised.
// literal (CR_QUIRK_LITERAL_ARITH): `vec3(x, y, z) / nLength` divides each
// component instead of multiplying by one reciprocal.
__host__ __device__ inline void frustum_planes(const float* m, float* planes, bool literal = false) {
    const float comb[6][4] = {
        {m[3] - m[0], m[7] - m[4], m[11] - m[8], m[15] - m[12]},
        {m[3] + m[0], m[7] + m[4], m[11] + m[8], m[15] + m[12]},
        {m[3] + m[1], m[7] + m[5], m[11] + m[9], m[15] + m[13]},
        {m[3] - m[1], m[7] - m[5], m[11] - m[9], m[15] - m[13]},
        {m[3] - m[2], m[7] - m[6], m[11] - m[10], m[15] - m[14]},
        {m[3] + m[2], m[7] + m[6], m[11] + m[10], m[15] + m[14]},
    };
    for (int i = 0; i < 6; i++) {
        const float* p = comb[i];
        const float len = sqrtf((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2]);
        // render.cs:139-140: vec3 / length is one reciprocal, w / length a division
        if (literal) {
            planes[4 * i + 0] = p[0] / len;
            planes[4 * i + 1] = p[1] / len;
            planes[4 * i + 2] = p[2] / len;
        } else {
            const float inv = 1.0f / len;
            planes[4 * i + 0] = p[0] * inv;
            planes[4 * i + 1] = p[1] * inv;
            planes[4 * i + 2] = p[2] * inv;
        }
        planes[4 * i + 3] = p[3] / len;
    }
}

// compute_loop_las.h:166-200 for one file: transform = mat4(proj * view *
// translate(boxMin)) in double, then the float planes and view * world.
__host__ __device__ inline void file_record(const double* view, const double* proj,
                                            const double* box_min, FileRec* out, bool literal = false) {
    const double world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0,
                              box_min[0], box_min[1], box_min[2], 1};
    double pv[16], t[16];
    mat_mul(proj, view, pv);
    mat_mul(pv, world, t);
    float fview[16], fworld[16];
    for (int i = 0; i < 16; i++) {
        out->T[i] = (float)t[i];
        fview[i] = (float)view[i];
        fworld[i] = (float)world[i];
    }
    frustum_planes(out->T, out->planes, literal);
    mat_mul(fview, fworld, out->VW);
}

// compute_loop_nodes.h:128-139: the same uniforms as float products,
// transform = (float(proj) * float(view)) * float(world), view * world in
// float (CR_QUIRK_FLOAT_UNIFORMS).
__host__ __device__ inline void file_record_float(const double* view, const double* proj,
                                                  const double* box_min, FileRec* out,
                                                  bool literal = false) {
    const double world[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0,
                              box_min[0], box_min[1], box_min[2], 1};
    float fv[16], fp[16], fw[16], pv[16];
    for (int i = 0; i < 16; i++) {
        fv[i] = (float)view[i];
        fp[i] = (float)proj[i];
        fw[i] = (float)world[i];
    }
    mat_mul(fp, fv, pv);
    mat_mul(pv, fw, out->T);
    frustum_planes(out->T, out->planes, literal);
    mat_mul(fv, fw, out->VW);
}

}  // namespace cr
