// glsl_prelude.hpp -- the GLSL compute-shader environment a reference shader
// needs to compile as C++ (TEST INFRASTRUCTURE: included only by the
// translations oracle/glsl_cpp.py writes into oracle/_ref/, which the CPU
// tests run as the reference side of a parity pin).
//
// Vector and matrix types, their operators and the built-in functions are the
// reference's vendored glm (GLSL semantics in C++, swizzles enabled).  A
// workgroup's invocations run one after another; the translated shaders use
// no barrier, shared memory or subgroup operation, so that order is one the
// GPU could have produced, and every atomic below is a plain read-modify-write.
// Floating point is IEEE binary32 without contraction (-ffp-contract=off):
// each GLSL operation rounds once, a vector divided by a scalar divides each
// component, and glm's matrix products keep glm's association.
#pragma once

#define GLM_FORCE_SWIZZLE
#include <array>
#include <cstdint>
#include <glm/glm.hpp>

// A swizzle combined with a scalar by + or / (`p.xy / p.w`, `p.xy + 1.0`; glm
// itself defines - and *): the swizzled vector's operator, element by
// element as GLSL defines it.
namespace glm {
namespace detail {
#define CR_GLSL_SWIZZLE_SCALAR_OP(OP)                                                            \
    template <int N, typename T, precision P, template <typename, precision> class V, int E0,   \
              int E1, int E2, int E3>                                                            \
    inline V<T, P> operator OP(_swizzle<N, T, P, V, E0, E1, E2, E3> const& a, T const& b) {     \
        return a() OP b;                                                                         \
    }                                                                                            \
    template <int N, typename T, precision P, template <typename, precision> class V, int E0,   \
              int E1, int E2, int E3>                                                            \
    inline V<T, P> operator OP(T const& a, _swizzle<N, T, P, V, E0, E1, E2, E3> const& b) {     \
        return a OP b();                                                                         \
    }
CR_GLSL_SWIZZLE_SCALAR_OP(+)
CR_GLSL_SWIZZLE_SCALAR_OP(/)
#undef CR_GLSL_SWIZZLE_SCALAR_OP
}  // namespace detail
}  // namespace glm

using namespace glm;
typedef unsigned int uint;

static uvec3 gl_WorkGroupID(0u), gl_LocalInvocationID(0u), gl_GlobalInvocationID(0u);

// barrier(): the invocations run one after another, so each has finished its
// previous loop steps when the next starts; the translated shaders share no
// memory through the barrier (hqs/depth.cs orders nothing with it).
inline void barrier() {}

// Subgroups of one invocation: a partition holds only the calling
// invocation, which leads it and owns its sums.  hqs/color.cs adds each
// partition's integer sums to the accumulators, so any grouping gives the
// same accumulators.
static const struct { uint x; } gl_SubgroupInvocationID = {0u};  // GLSL's scalar .x
template <class T>
inline uvec4 subgroupPartitionNV(T) {
    return uvec4(1u, 0u, 0u, 0u);
}
template <class T>
inline T subgroupPartitionedMinNV(T v, uvec4) {
    return v;
}
template <class T>
inline T subgroupPartitionedAddNV(T v, uvec4) {
    return v;
}

// A bound image: width x height texels, r32ui (one uint) or rgba8ui (four
// bytes).  GLSL drops stores outside the image.
struct uimage2D {
    void* data;
    int width, height;
    int rgba8;
};
typedef int sampler2D;  // bound but unread by the translated shaders
inline ivec2 imageSize(const uimage2D& im) { return ivec2(im.width, im.height); }
inline bool image_inside(const uimage2D& im, ivec2 p) {
    return p.x >= 0 && p.y >= 0 && p.x < im.width && p.y < im.height;
}
inline void imageStore(uimage2D& im, ivec2 p, uvec4 v) {
    if (!image_inside(im, p)) return;
    const size_t i = (size_t)p.y * (size_t)im.width + (size_t)p.x;
    if (im.rgba8) {
        uint8_t* t = static_cast<uint8_t*>(im.data) + 4 * i;
        const uint c[4] = {v.x, v.y, v.z, v.w};
        for (int k = 0; k < 4; k++) t[k] = (uint8_t)(c[k] < 255u ? c[k] : 255u);  // rgba8ui saturates
    } else {
        static_cast<uint*>(im.data)[i] = v.x;
    }
}
inline uint imageAtomicExchange(uimage2D& im, ivec2 p, uint v) {
    if (!image_inside(im, p) || im.rgba8) return 0u;
    uint* t = static_cast<uint*>(im.data) + (size_t)p.y * (size_t)im.width + (size_t)p.x;
    const uint old = *t;
    *t = v;
    return old;
}

// Unsigned division where GLSL leaves x / 0 undefined but does not trap
// (C++ would); the translated shaders overwrite such results.
inline uint glsl_udiv(uint a, uint b) { return b ? a / b : 0xFFFFFFFFu; }

template <class T, class U>
inline T atomicAdd(T& a, U v) {
    const T old = a;
    a = (T)(a + (T)v);
    return old;
}
template <class T, class U>
inline T atomicMin(T& a, U v) {
    const T old = a;
    if ((T)v < a) a = (T)v;
    return old;
}
template <class T, class U>
inline T atomicMax(T& a, U v) {
    const T old = a;
    if ((T)v > a) a = (T)v;
    return old;
}
