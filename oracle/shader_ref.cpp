// shader_ref.cpp -- runs the reference's own GLSL compute shaders on the CPU
// (TEST INFRASTRUCTURE: compiled by oracle/Makefile's `ref` target into
// oracle/_ref/libshaderref.so, loaded only by the CPU tests as the reference
// side of the oracle's parity pin; nothing in the product links it).
//
// Each shader is translated to C++ by oracle/glsl_cpp.py (written into
// oracle/_ref/, never committed) and included here under its own namespace.
// An entry point binds the shader's buffers and uniforms to caller arrays and
// runs its dispatch: every workgroup, and in it every invocation, one after
// another (the shaders use no barrier, shared memory or subgroup operation).
// The arithmetic is the shader's own, evaluated in IEEE binary32 without
// contraction, with glm's operators: the oracle's literal arithmetic mode.
#include <cstring>

#include "loop_las_render.cpp"
#include "loop_las2_render.cpp"
#include "hqs_depth.cpp"
#include "hqs_color.cpp"
#include "las_resolve.cpp"
#include "hqs_resolve.cpp"
#include "earlyz_render.cpp"
#include "earlyz_resolve.cpp"
#include "nodes_render.cpp"
#include "dedup_render.cpp"
#include "reduce_render.cpp"

namespace {

// A groups_x x groups_y dispatch of a 2-D workgroup shader.
template <class F>
void dispatch2d(uint groups_x, uint groups_y, uvec3 size, F&& shader_main) {
    for (uint gy = 0; gy < groups_y; gy++)
        for (uint gx = 0; gx < groups_x; gx++)
            for (uint ly = 0; ly < size.y; ly++)
                for (uint lx = 0; lx < size.x; lx++) {
                    gl_WorkGroupID = uvec3(gx, gy, 0u);
                    gl_LocalInvocationID = uvec3(lx, ly, 0u);
                    gl_GlobalInvocationID = uvec3(gx * size.x + lx, gy * size.y + ly, 0u);
                    shader_main();
                }
}

// A 1D dispatch of `groups` workgroups of 128 invocations in subgroups of 32
// run in lockstep (glsl_sg::run), the subgroup size of the reference's GPUs.
void dispatch_subgroups(int64_t groups, void (*shader_main)()) {
    static glsl_sg::Lockstep ls;
    uvec3 wg[32], local[32], global[32];
    for (int64_t b = 0; b < groups; b++)
        for (uint s = 0; s < 4; s++) {
            for (uint l = 0; l < 32; l++) {
                wg[l] = uvec3((uint)b, 0u, 0u);
                local[l] = uvec3(32u * s + l, 0u, 0u);
                global[l] = uvec3((uint)b * 128u + 32u * s + l, 0u, 0u);
            }
            glsl_sg::run(ls, shader_main, wg, local, global, &gl_WorkGroupID, &gl_LocalInvocationID,
                         &gl_GlobalInvocationID);
        }
}

}  // namespace

extern "C" {

// compute_loop_las/render.cs dispatched as compute_loop_las.h:233 does (one
// workgroup per batch record).  files: per file the shader's File record,
// mat4 transform, transformFrustum, world, padding (64 floats, column-major).
int ref_loop_las_render(const void* batches, int64_t num_batches, const uint32_t* lo,
                        const uint32_t* md, const uint32_t* hi, const void* files,
                        const float view[16], const float proj[16], int32_t width, int32_t height,
                        int32_t frustum_culling, int64_t num_points, uint64_t* fb) {
    using namespace loop_las;
    ssFramebuffer = fb;
    ssBatches = const_cast<Batch*>(static_cast<const Batch*>(batches));
    ssXyz_4b = const_cast<uint32_t*>(lo);
    ssXyz_8b = const_cast<uint32_t*>(md);
    ssXyz_12b = const_cast<uint32_t*>(hi);
    ssRGBA = nullptr;
    ssFiles = const_cast<File*>(static_cast<const File*>(files));
    std::memset(&debug, 0, sizeof(debug));
    std::memset(&boundingBoxes, 0, sizeof(boundingBoxes));
    std::memset(&uniforms, 0, sizeof(uniforms));
    std::memcpy(&uniforms.view[0][0], view, 16 * sizeof(float));
    std::memcpy(&uniforms.proj[0][0], proj, 16 * sizeof(float));
    uniforms.pointsPerThread = 80;  // compute_loop_las.h:155 (POINTS_PER_THREAD, Resources.h:4)
    uniforms.enableFrustumCulling = frustum_culling;
    uniforms.showBoundingBox = 0;
    uniforms.numPoints = (int)num_points;
    uniforms.imageSize = ivec2(width, height);
    uniforms.colorizeChunks = false;
    uniforms.colorizeOverdraw = false;
    for (int64_t b = 0; b < num_batches; b++)
        for (uint t = 0; t < gl_WorkGroupSize.x; t++) {
            gl_WorkGroupID = uvec3((uint)b, 0u, 0u);
            gl_LocalInvocationID = uvec3(t, 0u, 0u);
            gl_GlobalInvocationID = uvec3((uint)b * gl_WorkGroupSize.x + t, 0u, 0u);
            shader_main();
        }
    return 0;
}

// compute_loop_las2/render.cs dispatched as compute_loop_las2.h:234 does:
// ceil(numPointsLoaded / 10240) workgroups (-1 if that exceeds the records).
// The streams are read as uvec4 from firstPoint / 4 up to 10,240 words on, so
// each must hold the last record's firstPoint + 10,244 words.
int ref_loop_las2_render(const void* batches, int64_t num_batches, const uint32_t* lo,
                         const uint32_t* md, const uint32_t* hi, const void* files,
                         const float view[16], const float proj[16], int32_t width,
                         int32_t height, int32_t frustum_culling, int64_t num_points,
                         uint64_t* fb) {
    using namespace loop_las2;
    const int64_t dispatch = (num_points + 10239) / 10240;
    if (dispatch > num_batches) return -1;
    ssFramebuffer = fb;
    ssBatches = const_cast<Batch*>(static_cast<const Batch*>(batches));
    ssXyz_4b = reinterpret_cast<uvec4*>(const_cast<uint32_t*>(lo));
    ssXyz_8b = reinterpret_cast<uvec4*>(const_cast<uint32_t*>(md));
    ssXyz_12b = reinterpret_cast<uvec4*>(const_cast<uint32_t*>(hi));
    ssRGBA = nullptr;
    ssFiles = const_cast<File*>(static_cast<const File*>(files));
    std::memset(&debug, 0, sizeof(debug));
    std::memset(&boundingBoxes, 0, sizeof(boundingBoxes));
    std::memset(&uniforms, 0, sizeof(uniforms));
    std::memcpy(&uniforms.view[0][0], view, 16 * sizeof(float));
    std::memcpy(&uniforms.proj[0][0], proj, 16 * sizeof(float));
    uniforms.pointsPerThread = 80;  // compute_loop_las2.h:157
    uniforms.enableFrustumCulling = frustum_culling;
    uniforms.numPoints = (int)num_points;
    uniforms.imageSize = ivec2(width, height);
    for (int64_t b = 0; b < dispatch; b++)
        for (uint t = 0; t < gl_WorkGroupSize.x; t++) {
            gl_WorkGroupID = uvec3((uint)b, 0u, 0u);
            gl_LocalInvocationID = uvec3(t, 0u, 0u);
            gl_GlobalInvocationID = uvec3((uint)b * gl_WorkGroupSize.x + t, 0u, 0u);
            shader_main();
        }
    return 0;
}

// compute_loop_las_hqs: depth.cs then color.cs, each over ceil(numPoints /
// 10240) workgroups (compute_loop_las_hqs.h:238, :267; -1 if that exceeds the
// records).  depth: u32 per pixel; accum: two int64 per pixel (R | G << 32,
// B | count << 32), as the caller cleared them.
int ref_hqs_render(const void* batches, int64_t num_batches, const uint32_t* lo, const uint32_t* md,
                   const uint32_t* hi, const uint32_t* rgba, const void* files, const float view[16],
                   const float proj[16], int32_t width, int32_t height, int32_t frustum_culling,
                   int64_t num_points, uint32_t* depth, int64_t* accum) {
    const int64_t dispatch = (num_points + 10239) / 10240;
    if (dispatch > num_batches) return -1;
    {
        using namespace hqs_depth;
        ssFbo_depth = depth;
        ssFbo_rgba = accum;
        ssBatches = const_cast<Batch*>(static_cast<const Batch*>(batches));
        ssXyz_4b = const_cast<uint32_t*>(lo);
        ssXyz_8b = const_cast<uint32_t*>(md);
        ssXyz_12b = const_cast<uint32_t*>(hi);
        ssRGBA = const_cast<uint32_t*>(rgba);
        ssFiles = const_cast<File*>(static_cast<const File*>(files));
        std::memset(&debug, 0, sizeof(debug));
        std::memset(&boundingBoxes, 0, sizeof(boundingBoxes));
        std::memset(&uniforms, 0, sizeof(uniforms));
        std::memcpy(&uniforms.view[0][0], view, 16 * sizeof(float));
        std::memcpy(&uniforms.proj[0][0], proj, 16 * sizeof(float));
        uniforms.pointsPerThread = 80;  // compute_loop_las_hqs.h:162
        uniforms.enableFrustumCulling = frustum_culling;
        uniforms.numPoints = (int)num_points;
        uniforms.imageSize = ivec2(width, height);
        for (int64_t b = 0; b < dispatch; b++)
            for (uint t = 0; t < gl_WorkGroupSize.x; t++) {
                gl_WorkGroupID = uvec3((uint)b, 0u, 0u);
                gl_LocalInvocationID = uvec3(t, 0u, 0u);
                shader_main();
            }
    }
    {
        using namespace hqs_color;
        ssFbo_depth = depth;
        ssFbo_rgba = accum;
        ssBatches = const_cast<Batch*>(static_cast<const Batch*>(batches));
        ssXyz_4b = const_cast<uint32_t*>(lo);
        ssXyz_8b = const_cast<uint32_t*>(md);
        ssXyz_12b = const_cast<uint32_t*>(hi);
        ssRGBA = const_cast<uint32_t*>(rgba);
        ssFiles = const_cast<File*>(static_cast<const File*>(files));
        std::memset(&debug, 0, sizeof(debug));
        std::memset(&boundingBoxes, 0, sizeof(boundingBoxes));
        std::memset(&uniforms, 0, sizeof(uniforms));
        std::memcpy(&uniforms.view[0][0], view, 16 * sizeof(float));
        std::memcpy(&uniforms.proj[0][0], proj, 16 * sizeof(float));
        uniforms.pointsPerThread = 80;
        uniforms.enableFrustumCulling = frustum_culling;
        uniforms.numPoints = (int)num_points;
        uniforms.imageSize = ivec2(width, height);
        for (int64_t b = 0; b < dispatch; b++)
            for (uint t = 0; t < gl_WorkGroupSize.x; t++) {
                gl_WorkGroupID = uvec3((uint)b, 0u, 0u);
                gl_LocalInvocationID = uvec3(t, 0u, 0u);
                shader_main();
            }
    }
    return 0;
}

// compute_loop_las/resolve.cs over ceil(W/16) x ceil(H/16) groups
// (compute_loop_las.h:253-255).  Invocations past the image's right or bottom
// edge read framebuffer words beyond W*H (the caller pads fb) and store
// nothing.  image: W*H r32ui texels.
int ref_loop_las_resolve(uint64_t* fb, const uint32_t* rgba, int32_t width, int32_t height,
                         uint32_t* image) {
    using namespace las_resolve;
    ssFramebuffer = fb;
    ssRGBA = const_cast<uint32_t*>(rgba);
    std::memset(&debug, 0, sizeof(debug));
    std::memset(&uniforms, 0, sizeof(uniforms));
    uniforms.imageSize = ivec2(width, height);
    uOutput = uimage2D{image, width, height, 0};
    dispatch2d((uint)(width + 15) / 16, (uint)(height + 15) / 16, gl_WorkGroupSize, shader_main);
    return 0;
}

// compute_loop_las_hqs/resolve.cs over ceil(W/16) x ceil(H/16) groups
// (compute_loop_las_hqs.h:288-290); accum as 4 uint words per pixel (R, G, B,
// count: the two int64 accumulators), padded by the caller as fb above.
int ref_hqs_resolve(const uint32_t* accum, int32_t width, int32_t height, uint32_t* image) {
    using namespace hqs_resolve;
    ssRGBA = const_cast<uint32_t*>(accum);
    std::memset(&debug, 0, sizeof(debug));
    std::memset(&uniforms, 0, sizeof(uniforms));
    uniforms.imageSize = ivec2(width, height);
    uOutput = uimage2D{image, width, height, 0};
    dispatch2d((uint)(width + 15) / 16, (uint)(height + 15) / 16, gl_WorkGroupSize, shader_main);
    return 0;
}

// compute_2021_earlyz/render.cs: ceil(n / 128) groups over 16-byte points
// (compute_2021_earlyz.h:118-131; n below its 268M-point chunk).  transform:
// proj * view * world as the host computes it (compute_2021_earlyz.h:108-113).
// n must be a multiple of 128: the shader reads every invocation's point.
int ref_earlyz_render(const void* vertices_, int64_t n, const float transform[16], int32_t width,
                      int32_t height, uint64_t* fb) {
    using namespace earlyz_render;
    if (n % 128 != 0) return -1;
    vertices = const_cast<Vertex*>(static_cast<const Vertex*>(vertices_));
    ssFramebuffer = fb;
    std::memcpy(&uTransform[0][0], transform, 16 * sizeof(float));
    uImageSize = ivec2(width, height);
    for (int64_t b = 0; b < n / 128; b++)
        for (uint t = 0; t < gl_WorkGroupSize.x; t++) {
            gl_WorkGroupID = uvec3((uint)b, 0u, 0u);
            gl_LocalInvocationID = uvec3(t, 0u, 0u);
            shader_main();
        }
    return 0;
}

// compute_2021_earlyz/resolve.cs over floor(W/16) x floor(H/16) groups
// (compute_2021_earlyz.h:162-164): each resolved pixel's RGBA8 and the
// re-clear of its framebuffer word.  image: W*H rgba8ui texels.
int ref_earlyz_resolve(uint64_t* fb, int32_t width, int32_t height, uint8_t* image) {
    using namespace earlyz_resolve;
    ssFramebuffer = fb;
    vertices = nullptr;
    uOutput = uimage2D{image, width, height, 1};
    dispatch2d((uint)width / 16, (uint)height / 16, gl_WorkGroupSize, shader_main);
    return 0;
}

// compute_loop_nodes/render.cs (its PREFETCHED body) over one workgroup per
// node (compute_loop_nodes.h:180-181).  world is the identity and view, proj,
// transform = proj * view * world the float matrices compute_loop_nodes.h:
// 126-139 uploads; transformFrustum = transform.  The uvec4 reads run up to
// (min(ceil(n / 128), 500) + 4) / 4 vectors per invocation past a node's
// pointOffset / 4, so the caller pads the streams.
int ref_loop_nodes_render(const void* batches, int64_t num_batches, const uint32_t* lo,
                          const uint32_t* md, const uint32_t* hi, const float view[16],
                          const float proj[16], const float transform[16], int32_t width,
                          int32_t height, int32_t frustum_culling, int64_t num_points,
                          uint64_t* fb) {
    using namespace nodes_render;
    ssFramebuffer = fb;
    ssBatches = const_cast<Batch*>(static_cast<const Batch*>(batches));
    ssXyz_4b = reinterpret_cast<uvec4*>(const_cast<uint32_t*>(lo));
    ssXyz_8b = reinterpret_cast<uvec4*>(const_cast<uint32_t*>(md));
    ssXyz_12b = reinterpret_cast<uvec4*>(const_cast<uint32_t*>(hi));
    ssRGBA = nullptr;
    std::memset(&debug, 0, sizeof(debug));
    std::memset(&boundingBoxes, 0, sizeof(boundingBoxes));
    std::memset(&uniforms, 0, sizeof(uniforms));
    uniforms.world = mat4(1.0f);
    std::memcpy(&uniforms.view[0][0], view, 16 * sizeof(float));
    std::memcpy(&uniforms.proj[0][0], proj, 16 * sizeof(float));
    std::memcpy(&uniforms.transform[0][0], transform, 16 * sizeof(float));
    std::memcpy(&uniforms.transformFrustum[0][0], transform, 16 * sizeof(float));
    uniforms.pointsPerThread = 80;
    uniforms.enableFrustumCulling = frustum_culling;
    uniforms.numPoints = (int)num_points;
    uniforms.imageSize = ivec2(width, height);
    for (int64_t b = 0; b < num_batches; b++)
        for (uint t = 0; t < gl_WorkGroupSize.x; t++) {
            gl_WorkGroupID = uvec3((uint)b, 0u, 0u);
            gl_LocalInvocationID = uvec3(t, 0u, 0u);
            shader_main();
        }
    return 0;
}

// compute_2021_dedup/render.cs and compute_2021_earlyz_reduce/render.cs:
// ceil(n / 128) groups (compute_2021_dedup.h:129-131,
// compute_2021_earlyz_reduce.h:129-131), subgroups of 32 in lockstep; n a
// multiple of 128 as for ref_earlyz_render.
int ref_dedup_render(const void* vertices_, int64_t n, const float transform[16], int32_t width,
                     int32_t height, uint64_t* fb) {
    using namespace dedup_render;
    if (n % 128 != 0) return -1;
    vertices = const_cast<Vertex*>(static_cast<const Vertex*>(vertices_));
    ssFramebuffer = fb;
    std::memcpy(&uTransform[0][0], transform, 16 * sizeof(float));
    uImageSize = ivec2(width, height);
    dispatch_subgroups(n / 128, shader_main);
    return 0;
}
int ref_reduce_render(const void* vertices_, int64_t n, const float transform[16], int32_t width,
                      int32_t height, uint64_t* fb) {
    using namespace reduce_render;
    if (n % 128 != 0) return -1;
    vertices = const_cast<Vertex*>(static_cast<const Vertex*>(vertices_));
    ssFramebuffer = fb;
    std::memcpy(&uTransform[0][0], transform, 16 * sizeof(float));
    uImageSize = ivec2(width, height);
    dispatch_subgroups(n / 128, shader_main);
    return 0;
}

}  // extern "C"
