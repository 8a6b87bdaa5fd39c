// cr_noalloc.cu -- cr_render_batched_noalloc: the batched cull + raster on
// caller-owned device buffers, for callers that must not allocate device
// memory while rendering (an engine that owns the GPU memory budget, a plugin
// inside another application's frame loop, work recorded into a CUDA graph).
// The work list the cull kernel writes and the raster kernel reads lives in
// the fixed device array below instead of a cudaMalloc'd buffer.
#include <cuda_runtime.h>

#include <mutex>

#include "cr_internal.h"

namespace {

constexpr int64_t kNoallocWords = cr::kScratchHead + CR_NOALLOC_MAX_BATCHES;  // 512 KB
static_assert(kNoallocWords * 4 == 512 * 1024, "the no-alloc scratch is 512 KB");

// Counters (item count, work cursors) followed by the work list.  Every GPU
// that loads the library holds this array until the process exits, and every
// call shares it: calls that overlap on the GPU race.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoallocWords];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mutex;
uint32_t* g_addr[kMaxDevices] = {};

// In host code the array's name is only a stand-in; its device address is
// looked up once per device, with that device current.
cr_status scratch_address(int device, uint32_t** out) {
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CR_ERR_CUDA;
        g_addr[device] = static_cast<uint32_t*>(p);
    }
    *out = g_addr[device];
    return CR_OK;
}

}  // namespace

extern "C" cr_status cr_render_batched_noalloc(const cr_batch* d_batches, int64_t num_batches,
                                               int64_t num_points, const uint32_t* d_lo,
                                               const uint32_t* d_md, const uint32_t* d_hi,
                                               const uint32_t* d_rgba, int64_t stream_words,
                                               const double* box_min, int32_t num_files,
                                               const cr_view* view, const cr_render_params* p,
                                               uint64_t* d_fb, void* stream) {
    if (!d_batches || !d_lo || !d_md || !d_hi || !view || !p || !d_fb || !box_min)
        return CR_ERR_INVALID_ARG;
    if (num_batches < 0 || num_batches > CR_NOALLOC_MAX_BATCHES) return CR_ERR_INVALID_ARG;
    if (num_points < 0 || stream_words < num_points + cr::kStreamPad) return CR_ERR_INVALID_ARG;
    if (p->method != CR_METHOD_LOOP_LAS && p->method != CR_METHOD_LOOP_LAS_PREFETCH)
        return CR_ERR_INVALID_ARG;
    if (p->payload == CR_PAYLOAD_COLOR && !d_rgba) return CR_ERR_INVALID_ARG;
    const int32_t W = view->width, H = view->height;
    if (W <= 0 || H <= 0 || W >= (1 << 22) || H >= (1 << 22) ||
        (int64_t)W * H + W + 1 >= ((int64_t)1 << 31))
        return CR_ERR_INVALID_ARG;

    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
        return CR_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return CR_ERR_CUDA;
    uint32_t* scratch = nullptr;
    cr_status s = scratch_address(device, &scratch);
    if (s != CR_OK) return s;

    cr::ViewParams vp;
    s = cr::view_params_for(view, box_min, num_files, p->frustum_culling, &vp);
    if (s != CR_OK) return s;
    vp.lod_skip_level = p->lod_skip_level;
    const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT
                           ? (p->method == CR_METHOD_LOOP_LAS
                                  ? CR_QUIRK_L0_X12
                                  : CR_QUIRK_INCLUSIVE_END | CR_QUIRK_DISPATCH_BY_POINTS)
                           : p->quirks;
    int64_t nb = num_batches;
    if (quirks & CR_QUIRK_DISPATCH_BY_POINTS) {
        const int64_t by_points = (num_points + cr::kPointsPerBatch - 1) / cr::kPointsPerBatch;
        nb = by_points < nb ? by_points : nb;
    }

    // the counters start at zero on every call; the list needs no clearing
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(scratch, 0, cr::kCounterWords * 4, st) != cudaSuccess) return CR_ERR_CUDA;
    if (cr::launch_cull(vp, d_batches, nb, stream_words, quirks, scratch, stream) != 0)
        return CR_ERR_CUDA;
    cr::BatchedLaunch bl{};
    bl.batches = d_batches;
    bl.lo = d_lo;
    bl.md = d_md;
    bl.hi = d_hi;
    bl.rgba = d_rgba;
    bl.capacity = stream_words;
    bl.fb = d_fb;
    bl.scratch = scratch;
    bl.list_cap = nb;
    bl.quirks = quirks;
    bl.payload = p->payload;
    bl.mode = cr::kModeRaster;
    const int block = (p->block_threads == 256 || p->block_threads == 512) ? p->block_threads : 128;
    int per_sm = p->ctas_per_sm > 0 ? p->ctas_per_sm : cr::batched_blocks_per_sm(bl.mode, bl.payload, block);
    if (per_sm < 1) per_sm = 1;
    if (cr::launch_batched(vp, bl, block, sms * per_sm, stream) != 0) return CR_ERR_CUDA;
    return CR_OK;
}
