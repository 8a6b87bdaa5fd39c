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
#include <ucontext.h>

#include <algorithm>
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

// Subgroups.  Outside a lockstep run (below) a subgroup is the calling
// invocation alone: a partition holds only it, it leads it and owns its sums
// (hqs/color.cs adds each partition's integer sums to the accumulators, so any
// grouping gives the same accumulators).  Inside one, 32 invocations run as
// coroutines on this thread: an invocation reaching a subgroup operation
// yields, and once every invocation of the subgroup has yielded or finished
// the operation is evaluated over the invocations waiting at it -- the
// active invocations in GLSL's sense, invocations that returned or branched
// around it taking no part -- and they resume with its result.
static const struct { uint x; } gl_SubgroupInvocationID = {0u};  // GLSL's scalar .x

namespace glsl_sg {
enum Site { ALL_EQUAL, MIN, CLUSTERED_XOR, CLUSTERED_MIN, PARTITION, PARTITIONED_MIN };
enum State { READY, BLOCKED, DONE };
constexpr int kLanes = 32;
struct Lane {
    ucontext_t ctx;
    State state;
    Site site;
    int64_t a, b;
    int64_t result;
    uvec3 wg, local, global;
    char stack[1 << 16];
};
struct Lockstep {
    ucontext_t main;
    Lane lane[kLanes];
    int cur;
    void (*entry)();
};
static Lockstep* g_ls = nullptr;

// in an invocation: wait at the subgroup operation `site` with operands a, b
inline int64_t wait_op(Site site, int64_t a, int64_t b) {
    Lane& L = g_ls->lane[g_ls->cur];
    L.state = BLOCKED;
    L.site = site;
    L.a = a;
    L.b = b;
    swapcontext(&L.ctx, &g_ls->main);
    return L.result;
}
inline void trampoline() {
    g_ls->entry();
    g_ls->lane[g_ls->cur].state = DONE;  // uc_link resumes the scheduler
}
// Runs one subgroup: lanes 0..31 with their invocation ids.
inline void run(Lockstep& ls, void (*entry)(), const uvec3 wg[kLanes], const uvec3 local[kLanes],
                const uvec3 global[kLanes], uvec3* gl_wg, uvec3* gl_local, uvec3* gl_global) {
    g_ls = &ls;
    ls.entry = entry;
    for (int l = 0; l < kLanes; l++) {
        Lane& L = ls.lane[l];
        getcontext(&L.ctx);
        L.ctx.uc_stack.ss_sp = L.stack;
        L.ctx.uc_stack.ss_size = sizeof(L.stack);
        L.ctx.uc_link = &ls.main;
        makecontext(&L.ctx, trampoline, 0);
        L.state = READY;
        L.wg = wg[l];
        L.local = local[l];
        L.global = global[l];
    }
    while (true) {
        for (int l = 0; l < kLanes; l++) {
            if (ls.lane[l].state != READY) continue;
            ls.cur = l;
            *gl_wg = ls.lane[l].wg;
            *gl_local = ls.lane[l].local;
            *gl_global = ls.lane[l].global;
            swapcontext(&ls.main, &ls.lane[l].ctx);
        }
        int first = -1;
        for (int l = 0; l < kLanes && first < 0; l++)
            if (ls.lane[l].state == BLOCKED) first = l;
        if (first < 0) break;  // every lane done
        const Site site = ls.lane[first].site;
        uint32_t active = 0;
        for (int l = 0; l < kLanes; l++)
            if (ls.lane[l].state == BLOCKED && ls.lane[l].site == site) active |= 1u << l;
        for (int l = 0; l < kLanes; l++) {
            if (!((active >> l) & 1u)) continue;
            Lane& L = ls.lane[l];
            // the lanes the operation reads for this lane
            uint32_t from = active;
            if (site == CLUSTERED_XOR || site == CLUSTERED_MIN) from &= 3u << (l & ~1);  // clusters of 2
            if (site == PARTITIONED_MIN) from &= (uint32_t)L.b;
            int64_t r = site == ALL_EQUAL ? 1 : 0;
            bool any = false;
            for (int k = 0; k < kLanes; k++) {
                if (!((from >> k) & 1u)) continue;
                const int64_t v = ls.lane[k].a;
                switch (site) {
                    case ALL_EQUAL: r = r && v == L.a; break;
                    case MIN:
                    case CLUSTERED_MIN:
                    case PARTITIONED_MIN: r = any ? std::min(r, v) : v; break;
                    case CLUSTERED_XOR: r ^= v; break;
                    case PARTITION: r |= (int64_t)(v == L.a) << k; break;
                }
                any = true;
            }
            L.result = r;
        }
        for (int l = 0; l < kLanes; l++)
            if ((active >> l) & 1u) ls.lane[l].state = READY;
    }
    g_ls = nullptr;
}
}  // namespace glsl_sg

inline bool subgroupAllEqual(int v) {
    return glsl_sg::g_ls ? glsl_sg::wait_op(glsl_sg::ALL_EQUAL, v, 0) != 0 : true;
}
inline int subgroupMin(int v) {
    return glsl_sg::g_ls ? (int)glsl_sg::wait_op(glsl_sg::MIN, v, 0) : v;
}
inline int subgroupClusteredXor(int v, uint cluster_size) {
    return glsl_sg::g_ls && cluster_size == 2u ? (int)glsl_sg::wait_op(glsl_sg::CLUSTERED_XOR, v, 0) : v;
}
inline int subgroupClusteredMin(int v, uint cluster_size) {
    return glsl_sg::g_ls && cluster_size == 2u ? (int)glsl_sg::wait_op(glsl_sg::CLUSTERED_MIN, v, 0) : v;
}
template <class T>
inline uvec4 subgroupPartitionNV(T v) {
    if (!glsl_sg::g_ls) return uvec4(1u, 0u, 0u, 0u);
    return uvec4((uint)glsl_sg::wait_op(glsl_sg::PARTITION, (int64_t)v, 0), 0u, 0u, 0u);
}
template <class T>
inline T subgroupPartitionedMinNV(T v, uvec4 ballot) {
    if (!glsl_sg::g_ls) return v;
    return (T)glsl_sg::wait_op(glsl_sg::PARTITIONED_MIN, (int64_t)v, (int64_t)ballot.x);
}
template <class T>
inline T subgroupPartitionedAddNV(T v, uvec4) {
    return v;  // used outside lockstep runs only (hqs/color.cs)
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
