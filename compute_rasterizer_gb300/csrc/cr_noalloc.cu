// cr_noalloc.cu -- cr_render_batched_noalloc: the batched cull + raster on
// caller-owned device buffers, for callers that must not allocate device
// memory while rendering: an engine that owns the GPU memory budget and hands
// the renderer only the buffers it already placed, or a plugin running inside
// another application's frame loop, where a cudaMalloc or cudaFree would
// synchronise or disturb the host's device work.  The work list the cull
// kernel writes and the raster kernel reads, and the per-file records of
// clouds with more than 8 files, live in the fixed device array below instead
// of buffers this library would allocate.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "cr_internal.h"

namespace {

// [counters, error word, item list][file records], 16-byte aligned regions.
constexpr int64_t kListWords = cr::kScratchHead + CR_NOALLOC_MAX_BATCHES;
constexpr int64_t kFileWords = (int64_t)CR_NOALLOC_MAX_FILES * (sizeof(cr::FileRec) / 4);
constexpr int64_t kNoallocWords = kListWords + kFileWords;
static_assert(kListWords % 4 == 0 && sizeof(cr::FileRec) % 16 == 0, "regions stay 16-byte aligned");
static_assert(kNoallocWords * 4 == CR_NOALLOC_SCRATCH_BYTES, "the header states the array's size");

// Every GPU that loads the library holds this array until the process exits,
// and every call shares it: calls whose work overlaps on the GPU race.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoallocWords];

// In host code the array's name is only a host-side stand-in; its device
// address belongs to the CUDA context the module is loaded in.  The address
// is looked up once per context (the first call in that context, with the
// context current) and cached under the context's unique ID, which the driver
// never reuses within a process, so a destroyed and recreated context (or a
// second context on the same device, made with cuCtxCreate) gets its own
// lookup and never a stale address.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct AddrCache {
    std::mutex mu;
    bool resolved = false;
    CtxGetCurrentFn get_current = nullptr;
    CtxGetIdFn get_id = nullptr;
    std::vector<std::pair<unsigned long long, uint32_t*>> entries;
};
AddrCache g_cache;

bool resolve_driver_entry_points(AddrCache& c) {
    if (c.resolved) return c.get_current && c.get_id;
    c.resolved = true;
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) !=
            cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) !=
            cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess)
        return false;
    c.get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
    c.get_id = reinterpret_cast<CtxGetIdFn>(f1);
    return true;
}

// The array's device address in the calling thread's current context.
cr_status scratch_address(uint32_t** out) {
    std::lock_guard<std::mutex> lock(g_cache.mu);
    if (!resolve_driver_entry_points(g_cache)) return CR_ERR_CUDA;
    CUcontext cu = nullptr;
    if (g_cache.get_current(&cu) != CUDA_SUCCESS) return CR_ERR_CUDA;
    if (!cu) {
        // no context current yet: the runtime's lookup below makes the device's
        // primary context current, whose ID keys the entry
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CR_ERR_CUDA;
        if (g_cache.get_current(&cu) != CUDA_SUCCESS || !cu) return CR_ERR_CUDA;
    }
    unsigned long long id = 0;
    if (g_cache.get_id(cu, &id) != CUDA_SUCCESS) return CR_ERR_CUDA;
    for (const auto& e : g_cache.entries)
        if (e.first == id) {
            *out = e.second;
            return CR_OK;
        }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CR_ERR_CUDA;
    g_cache.entries.emplace_back(id, static_cast<uint32_t*>(p));
    *out = static_cast<uint32_t*>(p);
    return CR_OK;
}

}  // namespace

namespace cr {

// cr_ctx_check(NULL, stream): the array's sticky error word, read and cleared.
cr_status noalloc_check(void* stream) {
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return CR_ERR_CUDA;
    uint32_t* scratch = nullptr;
    const cr_status s = scratch_address(&scratch);
    if (s != CR_OK) return s;
    uint32_t flag = 0;
    if (cudaMemcpy(&flag, scratch + kErrWord, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return CR_ERR_CUDA;
    if (!flag) return CR_OK;
    const uint32_t zero = 0;
    if (cudaMemcpy(scratch + kErrWord, &zero, 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return CR_ERR_CUDA;
    return CR_ERR_DEVICE_FLAG;
}

}  // namespace cr

extern "C" cr_status cr_noalloc_scratch(void** device_address, int64_t* bytes) {
    if (!device_address || !bytes) return CR_ERR_INVALID_ARG;
    uint32_t* p = nullptr;
    const cr_status s = scratch_address(&p);
    if (s != CR_OK) return s;
    *device_address = p;
    *bytes = kNoallocWords * 4;
    return CR_OK;
}

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
    if (num_files < 1 || num_files > CR_NOALLOC_MAX_FILES) return CR_ERR_INVALID_ARG;
    if (num_points < 0 || stream_words < num_points + cr::kStreamPad) return CR_ERR_INVALID_ARG;
    if (p->method != CR_METHOD_LOOP_LAS && p->method != CR_METHOD_LOOP_LAS_PREFETCH)
        return CR_ERR_INVALID_ARG;
    // rasterizes only: a resolve or re-clear would need the image and color
    // buffers this call does not take
    if (p->resolve || p->clear_after) return CR_ERR_INVALID_ARG;
    if (p->payload == CR_PAYLOAD_COLOR && !d_rgba) return CR_ERR_INVALID_ARG;
    const int32_t W = view->width, H = view->height;
    if (W <= 0 || H <= 0 || W >= (1 << 22) || H >= (1 << 22) ||
        (int64_t)W * H + W + 1 >= ((int64_t)1 << 31))
        return CR_ERR_INVALID_ARG;

    const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? cr::default_quirks_for(p->method) : p->quirks;
    const int literal = (quirks & CR_QUIRK_LITERAL_ARITH) ? 1 : 0;
    cr::ViewParams vp;
    cr_status s = cr::view_params_for(view, box_min, num_files, p->frustum_culling, &vp, literal);
    if (s != CR_OK) return s;
    vp.lod_skip_level = p->lod_skip_level;

    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return CR_ERR_CUDA;
    uint32_t* scratch = nullptr;
    s = scratch_address(&scratch);
    if (s != CR_OK) return s;

    int64_t nb = num_batches;
    if (quirks & CR_QUIRK_DISPATCH_BY_POINTS) {
        const int64_t by_points = (num_points + cr::kPointsPerBatch - 1) / cr::kPointsPerBatch;
        nb = by_points < nb ? by_points : nb;
    }

    cudaStream_t st = (cudaStream_t)stream;
    const bool many = num_files > cr::kInlineFiles;
    if (many) {
        cr::FileRec* files = reinterpret_cast<cr::FileRec*>(scratch + kListWords);
        if (cr::launch_file_records(view->view, view->proj, box_min, num_files, files, stream, 0, literal) != 0)
            return CR_ERR_CUDA;
        vp.dfiles = files;
    }
    // the counters start at zero on every call; the list needs no clearing, and
    // the error word stays set until cr_ctx_check(NULL, stream) reads it
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
    int per_sm = p->ctas_per_sm > 0 ? p->ctas_per_sm
                                    : cr::batched_blocks_per_sm(bl.mode, bl.payload, block, many,
                                                                literal != 0);
    if (per_sm < 1) per_sm = 1;
    if (cr::launch_batched(vp, bl, block, sms * per_sm, stream) != 0) return CR_ERR_CUDA;
    return CR_OK;
}
