// cr_api.cpp -- host side of the C ABI (include/cr_raster.h): contexts,
// device-resident clouds and framebuffers, the per-frame uniform setup that
// compute_loop_las.h:117-304 does on the host, and the launch sequence
// cull -> raster -> resolve (-> clear) on the caller's stream.
//
// Host float math is compiled with -ffp-contract=off; matrix products follow
// glm's operand order so the float uniforms equal the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cr_filerec.h"
#include "cr_internal.h"

struct cr_frame_events {
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool ran[4] = {false, false, false, false};
};

struct cr_ctx {
    int device = 0;
    int num_sms = 0;
    uint32_t* scratch = nullptr;  // counters + work list
    int64_t scratch_words = 0;
    cr::FileRec* files = nullptr;  // per-file records of the frame's view (clouds > 8 files)
    int32_t files_cap = 0;
    int64_t last_dispatched = 0;  // batch records the last cull looked at
    int64_t last_list_cap = 0;    // words of its item-list region
    bool last_node_slices = false;
    std::vector<cr_frame_events> timing;  // GLTimerQueries-style event pairs
    int32_t timing_used = 0;
    std::string last_error;
};

struct cr_cloud {
    bool plain = false;
    int64_t n = 0;
    int64_t nb = 0;
    int32_t nfiles = 0;
    int32_t mask = 0;
    int64_t capacity = 0;  // words per stream incl. padding
    cr_batch* batches = nullptr;
    uint32_t* lo = nullptr;
    uint32_t* md = nullptr;
    uint32_t* hi = nullptr;
    uint32_t* rgba = nullptr;
    cr_vertex* verts = nullptr;
    std::vector<double> box_min;
    bool owned = true;  // false: arrays belong to the caller (cr_cloud_wrap)
    // points and batch records loaded so far (cr_cloud_set_loaded); -1 = all
    int64_t n_loaded = -1, nb_loaded = -1;
};

namespace {
int64_t loaded_points(const cr_cloud* c) { return c->n_loaded < 0 ? c->n : c->n_loaded; }
int64_t loaded_batches(const cr_cloud* c) { return c->nb_loaded < 0 ? c->nb : c->nb_loaded; }
}  // namespace

struct cr_fb {
    int32_t W = 0, H = 0, kind = 0;
    int64_t words = 0;  // W*H + W + 1
    uint64_t* fb = nullptr;
    uint32_t* depth = nullptr;
    uint64_t* accum = nullptr;
    uint32_t* image = nullptr;
};

namespace {

using namespace cr;

cr_status fail(cr_ctx* ctx, cr_status s, const char* fmt, const char* a = "", long long b = 0) {
    if (ctx) {
        char buf[512];
        std::snprintf(buf, sizeof(buf), fmt, a, b);
        ctx->last_error = buf;
    }
    return s;
}

cr_status cuda_fail(cr_ctx* ctx, cudaError_t e, const char* what) {
    if (ctx) ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA;
}

#define CR_CUDA(ctx, call, what)                         \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

// ---- host matrix setup ------------------------------------------------------

bool finite_all(const double* v, int n) {
    for (int i = 0; i < n; i++)
        if (!std::isfinite(v[i])) return false;
    return true;
}

cr_status build_view_params(cr_ctx* ctx, const cr_cloud* cloud, const cr_view* view, int culling,
                            int quirks, ViewParams* vp) {
    if (!finite_all(view->view, 16) || !finite_all(view->proj, 16))
        return fail(ctx, CR_ERR_INVALID_ARG, "view matrices must be finite%s", "");
    std::memset(vp, 0, sizeof(*vp));
    for (int i = 0; i < 16; i++) vp->P[i] = (float)view->proj[i];
    vp->W = view->width;
    vp->H = view->height;
    vp->nfiles = cloud->nfiles;
    vp->culling = culling ? 1 : 0;
    vp->level4_px = (quirks & CR_QUIRK_LEVEL4_80PX) ? 80.0f : 100.0f;
    vp->one_world = (quirks & CR_QUIRK_ONE_WORLD) ? 1 : 0;
    const bool literal = (quirks & CR_QUIRK_LITERAL_ARITH) != 0;
    vp->literal = literal ? 1 : 0;
    for (int f = 0; f < std::min(cloud->nfiles, kInlineFiles); f++) {
        if (quirks & CR_QUIRK_FLOAT_UNIFORMS)
            file_record_float(view->view, view->proj, &cloud->box_min[3 * f], &vp->files[f], literal);
        else
            file_record(view->view, view->proj, &cloud->box_min[3 * f], &vp->files[f], literal);
    }
    return CR_OK;
}

// Clouds with more than kInlineFiles files: every file's record of this view,
// computed on the GPU on `stream` into the context's record array.
cr_status enqueue_file_records(cr_ctx* ctx, const cr_cloud* cloud, const cr_view* view, int quirks,
                               ViewParams* vp, void* stream) {
    if (cloud->nfiles <= kInlineFiles) return CR_OK;
    if (ctx->files_cap < cloud->nfiles) {
        if (ctx->files) {
            // a frame still in flight may read the old array
            CR_CUDA(ctx, cudaDeviceSynchronize(), "synchronize");
            cudaFree(ctx->files);
            ctx->files = nullptr;
            ctx->files_cap = 0;
        }
        CR_CUDA(ctx, cudaMalloc(&ctx->files, sizeof(FileRec) * (size_t)cloud->nfiles), "file records");
        ctx->files_cap = cloud->nfiles;
    }
    if (launch_file_records(view->view, view->proj, cloud->box_min.data(), cloud->nfiles, ctx->files,
                            stream, (quirks & CR_QUIRK_FLOAT_UNIFORMS) ? 1 : 0,
                            (quirks & CR_QUIRK_LITERAL_ARITH) ? 1 : 0) != 0)
        return fail(ctx, CR_ERR_CUDA, "file record launch failed%s", "");
    vp->dfiles = ctx->files;
    return CR_OK;
}

cr_status check_size(cr_ctx* ctx, int32_t W, int32_t H) {
    // pixel ids stay below 2^31; W, H < 2^22 keeps (q * 0.5 + 0.5) * W below
    // 2^22, where a float still resolves fractions of a pixel
    if (W <= 0 || H <= 0 || W >= (1 << 22) || H >= (1 << 22) ||
        (int64_t)W * H + W + 1 >= ((int64_t)1 << 31))
        return fail(ctx, CR_ERR_INVALID_ARG, "bad framebuffer size %s%lld", "", (long long)W * H);
    return CR_OK;
}

cr_status ensure_scratch(cr_ctx* ctx, int64_t items) {
    int64_t need = kScratchHead + items + 64;
    if (need <= ctx->scratch_words) return CR_OK;
    if (ctx->scratch) {
        cudaDeviceSynchronize();
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_words = 0;
    }
    int64_t words = std::max<int64_t>(need, 1 << 16);
    CR_CUDA(ctx, cudaMalloc(&ctx->scratch, words * 4), "scratch allocation");
    CR_CUDA(ctx, cudaMemset(ctx->scratch, 0, words * 4), "scratch clear");
    ctx->scratch_words = words;
    return CR_OK;
}

constexpr int kNumMethods = 7;
const char* kNames[kNumMethods] = {"loop_las",       "loop_las_prefetch", "loop_las_hqs",
                                   "(2021) early-z", "(2021) dedup",      "(2021) early-z & reduce",
                                   "loop_nodes"};
const char* kGroups[kNumMethods] = {"10-10-10 bit encoded", "10-10-10 bit encoded", "10-10-10 bit encoded",
                                    "2021 method; standard 16 byte per point",
                                    "2021 method; standard 16 byte per point",
                                    "2021 method; standard 16 byte per point",
                                    "render Potree nodes"};
const char* kDescriptions[kNumMethods] = {
    "Batched atomicMin rasterizer over the 10-10-10 bit encoded layout; each batch picks 10, 20 "
    "or 30 bit coordinates from its projected size; point-index payload.",
    "Same algorithm reading four consecutive points per 128-bit load.",
    "High-quality shading: depth pass, then averaging of all points within 1% of the nearest "
    "depth.",
    "Plain 16 byte per point layout, one 64-bit atomicMin of depth|color per point.",
    "Plain 16 byte per point layout; the points of a warp are partitioned by pixel and only each "
    "partition's closest point is written (depth<<24|color).",
    "Plain 16 byte per point layout; a warp on one pixel writes only its closest point, otherwise "
    "pairs of lanes drop the farther of two points on one pixel (depth<<24|color).",
    "Potree octree nodes as batches of up to 64,512 points, 10/20/30 bit coordinates per node; "
    "nodes below 80 pixels (level 4) are skipped."};

bool plain_method(int32_t m) {
    return m == CR_METHOD_EARLYZ || m == CR_METHOD_DEDUP || m == CR_METHOD_EARLYZ_REDUCE;
}

int default_quirks(int32_t method) {
    switch (method) {
        case CR_METHOD_LOOP_LAS: return CR_QUIRK_L0_X12;
        case CR_METHOD_LOOP_LAS_PREFETCH:
            return CR_QUIRK_INCLUSIVE_END | CR_QUIRK_DISPATCH_BY_POINTS | CR_QUIRK_UVEC4_BASE;
        case CR_METHOD_LOOP_LAS_HQS:
            return CR_QUIRK_L0_X12 | CR_QUIRK_INCLUSIVE_END | CR_QUIRK_DISPATCH_BY_POINTS;
        case CR_METHOD_EARLYZ:
        case CR_METHOD_DEDUP:
        case CR_METHOD_EARLYZ_REDUCE: return CR_QUIRK_RESOLVE_TILES;
        case CR_METHOD_LOOP_NODES:
            return CR_QUIRK_NODE_LOOP | CR_QUIRK_LEVEL4_80PX | CR_QUIRK_ONE_WORLD |
                   CR_QUIRK_FLOAT_UNIFORMS | CR_QUIRK_RESOLVE_TILES;
        default: return 0;
    }
}

int read_i32(const uint8_t* p) { int32_t v; std::memcpy(&v, p, 4); return v; }
int read_u16(const uint8_t* p) { uint16_t v; std::memcpy(&v, p, 2); return v; }

}  // namespace

bool cr::cloud_info(const cr_cloud* c, CloudInfo* out) {
    if (!c || !out || c->plain) return false;
    out->batches = c->batches;
    out->lo = c->lo;
    out->md = c->md;
    out->hi = c->hi;
    out->rgba = c->rgba;
    out->n = loaded_points(c);
    out->nb = loaded_batches(c);
    out->n_total = c->n;
    out->nb_total = c->nb;
    out->capacity = c->capacity;
    out->nfiles = c->nfiles;
    out->box_min = c->box_min.data();
    return true;
}

int cr::default_quirks_for(int32_t method) { return default_quirks(method); }

int cr::ctx_device(const cr_ctx* ctx) { return ctx ? ctx->device : 0; }

cr_status cr::view_params_for(const cr_view* view, const double* box_min, int32_t num_files,
                              int32_t culling, ViewParams* vp, int literal) {
    if (!view || !box_min || !vp || num_files < 1 || num_files > kMaxFiles)
        return CR_ERR_INVALID_ARG;
    if (!finite_all(view->view, 16) || !finite_all(view->proj, 16) ||
        !finite_all(box_min, 3 * num_files))
        return CR_ERR_INVALID_ARG;
    std::memset(vp, 0, sizeof(*vp));
    for (int i = 0; i < 16; i++) vp->P[i] = (float)view->proj[i];
    vp->W = view->width;
    vp->H = view->height;
    vp->nfiles = num_files;
    vp->culling = culling ? 1 : 0;
    vp->level4_px = 100.0f;
    vp->literal = literal ? 1 : 0;
    for (int f = 0; f < std::min(num_files, kInlineFiles); f++)
        file_record(view->view, view->proj, &box_min[3 * f], &vp->files[f], literal != 0);
    return CR_OK;
}

// ============================================================================
extern "C" {

int32_t cr_abi_version(void) { return CR_ABI_VERSION; }

const char* cr_status_string(cr_status s) {
    switch (s) {
        case CR_OK: return "ok";
        case CR_ERR_INVALID_ARG: return "invalid argument";
        case CR_ERR_OUT_OF_MEMORY: return "out of device memory";
        case CR_ERR_ADMISSION_REJECTED: return "admission rejected";
        case CR_ERR_TIMEOUT: return "timeout";
        case CR_ERR_CUDA: return "CUDA error";
        case CR_ERR_DEVICE_FLAG: return "device error flag raised";
        case CR_ERR_UNSUPPORTED: return "unsupported";
        case CR_ERR_NOT_FOUND: return "not found";
        case CR_ERR_CORRUPT: return "corrupt data";
    }
    return "unknown status";
}

const char* cr_method_name(int32_t m) { return (m >= 0 && m < kNumMethods) ? kNames[m] : nullptr; }
const char* cr_method_group(int32_t m) { return (m >= 0 && m < kNumMethods) ? kGroups[m] : nullptr; }
const char* cr_method_description(int32_t m) {
    return (m >= 0 && m < kNumMethods) ? kDescriptions[m] : nullptr;
}

cr_status cr_method_find(const char* name, int32_t* method) {
    if (!name || !method) return CR_ERR_INVALID_ARG;
    for (int i = 0; i < kNumMethods; i++)
        if (std::strcmp(name, kNames[i]) == 0) {
            *method = i;
            return CR_OK;
        }
    return CR_ERR_NOT_FOUND;
}

void cr_render_params_default(int32_t method, cr_render_params* out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->method = method;
    out->payload = CR_PAYLOAD_INDEX;
    out->quirks = CR_QUIRKS_METHOD_DEFAULT;
    out->frustum_culling = 1;
    out->resolve = 1;
    out->clear_after = 1;
    out->clear_value = plain_method(method) ? kPlainReclear : kDefaultClear;
    if (method == CR_METHOD_LOOP_NODES) out->lod_skip_level = 4;  // compute_loop_nodes/render.cs:273
}

// ---- context ----------------------------------------------------------------

cr_status cr_ctx_create(int32_t device, cr_ctx** out) {
    if (!out) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return CR_ERR_CUDA;
    cr_ctx* ctx = new (std::nothrow) cr_ctx();
    if (!ctx) return CR_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        delete ctx;
        return CR_ERR_CUDA;
    }
    cr_status s = ensure_scratch(ctx, 1 << 16);
    if (s != CR_OK) {
        delete ctx;
        return s;
    }
    *out = ctx;
    return CR_OK;
}

static void destroy_timing(cr_ctx* ctx) {
    for (auto& f : ctx->timing)
        for (cudaEvent_t e : f.ev)
            if (e) cudaEventDestroy(e);
    ctx->timing.clear();
    ctx->timing_used = 0;
}

cr_status cr_timing_enable(cr_ctx* ctx, int32_t max_frames) {
    if (!ctx || max_frames < 0) return CR_ERR_INVALID_ARG;
    destroy_timing(ctx);
    ctx->timing.resize((size_t)max_frames);
    for (auto& f : ctx->timing)
        for (cudaEvent_t& e : f.ev) CR_CUDA(ctx, cudaEventCreate(&e), "event create");
    return CR_OK;
}

int32_t cr_timing_read(cr_ctx* ctx, int32_t stage, float* ms, int32_t max) {
    if (!ctx || stage < 0 || stage >= CR_NUM_STAGES || (max > 0 && !ms)) return -1;
    const int32_t n = std::min(ctx->timing_used, max);
    for (int32_t i = 0; i < n; i++) {
        const cr_frame_events& f = ctx->timing[i];
        ms[i] = 0.0f;
        if (!f.ran[stage]) continue;
        // the stage ends at the next boundary that was recorded after it
        int end = stage + 1;
        if (cudaEventSynchronize(f.ev[end]) != cudaSuccess) return -1;
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, f.ev[stage], f.ev[end]) != cudaSuccess) return -1;
        ms[i] = t;
    }
    return n;
}

cr_status cr_ctx_destroy(cr_ctx* ctx) {
    if (!ctx) return CR_ERR_INVALID_ARG;
    destroy_timing(ctx);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->files) cudaFree(ctx->files);
    delete ctx;
    return CR_OK;
}

const char* cr_last_error(const cr_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int32_t cr_ctx_num_sms(const cr_ctx* ctx) { return ctx ? ctx->num_sms : 0; }

cr_status cr_ctx_check(cr_ctx* ctx, void* stream) {
    if (!ctx) return noalloc_check(stream);
    CR_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream), "stream synchronize");
    uint32_t flag = 0;
    CR_CUDA(ctx, cudaMemcpy(&flag, ctx->scratch + kErrWord, 4, cudaMemcpyDeviceToHost), "flag read");
    if (flag) {
        uint32_t zero = 0;
        CR_CUDA(ctx, cudaMemcpy(ctx->scratch + kErrWord, &zero, 4, cudaMemcpyHostToDevice), "flag clear");
        return fail(ctx, CR_ERR_DEVICE_FLAG, "device error flag %s0x%llx", "", (long long)flag);
    }
    return CR_OK;
}

cr_status cr_check_reciprocal(cr_ctx* ctx, uint64_t* mismatches, uint32_t* first_mismatch) {
    if (!ctx || !mismatches || !first_mismatch) return CR_ERR_INVALID_ARG;
    uint64_t* d = nullptr;
    CR_CUDA(ctx, cudaMalloc(&d, 16), "check buffer");
    const uint64_t init[2] = {0ull, 0xFFFFFFFFull};
    cudaError_t e = cudaMemcpy(d, init, 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && launch_check_reciprocal(d, reinterpret_cast<uint32_t*>(d + 1)) != 0)
        e = cudaErrorLaunchFailure;
    uint64_t out[2] = {0ull, 0ull};
    if (e == cudaSuccess) e = cudaMemcpy(out, d, 16, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(ctx, CR_ERR_CUDA, "reciprocal check: %s", cudaGetErrorString(e));
    *mismatches = out[0];
    *first_mismatch = (uint32_t)out[1];
    return CR_OK;
}

// ---- clouds -------------------------------------------------------------------

cr_status cr_cloud_create(cr_ctx* ctx, int64_t n, int64_t nb, int32_t nfiles, int32_t mask,
                          cr_cloud** out) {
    if (!ctx || !out) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    if (n < 0 || nb < 0 || nb >= kMaxBatches || n >= ((int64_t)1 << 31) - kStreamPad ||
        nfiles < 1 || nfiles > kMaxFiles || (mask & CR_STREAM_LOW) == 0)
        return fail(ctx, CR_ERR_INVALID_ARG, "bad cloud shape %s(n=%lld)", "", (long long)n);
    cr_cloud* c = new (std::nothrow) cr_cloud();
    if (!c) return CR_ERR_OUT_OF_MEMORY;
    c->n = n;
    c->nb = nb;
    c->nfiles = nfiles;
    c->mask = mask;
    c->capacity = ((n + kStreamPad + 3) / 4) * 4;
    c->box_min.assign(3 * (size_t)nfiles, 0.0);
    const size_t bytes = (size_t)c->capacity * 4;
    cudaError_t e = cudaSuccess;
    uint32_t** streams[4] = {&c->lo, &c->md, &c->hi, &c->rgba};
    for (int i = 0; i < 4 && e == cudaSuccess; i++) {
        if (!(mask & (1 << i))) continue;
        e = cudaMalloc(streams[i], bytes);
        if (e == cudaSuccess) e = cudaMemset(*streams[i], 0, bytes);
    }
    if (e == cudaSuccess && nb > 0) {
        e = cudaMalloc(&c->batches, (size_t)nb * sizeof(cr_batch));
        if (e == cudaSuccess) e = cudaMemset(c->batches, 0, (size_t)nb * sizeof(cr_batch));
    }
    if (e != cudaSuccess) {
        cr_cloud_destroy(ctx, c);
        return cuda_fail(ctx, e, "cloud allocation");
    }
    *out = c;
    return CR_OK;
}

cr_status cr_cloud_upload(cr_ctx* ctx, cr_cloud* c, const cr_batch* batches, const uint32_t* lo,
                          const uint32_t* md, const uint32_t* hi, const uint32_t* rgba,
                          const double* box_min, void* stream) {
    if (!ctx || !c || c->plain) return CR_ERR_INVALID_ARG;
    if (!c->owned) return fail(ctx, CR_ERR_INVALID_ARG, "a wrapped cloud's arrays belong to the caller%s", "");
    cudaStream_t s = (cudaStream_t)stream;
    if (batches) {
        for (int64_t i = 0; i < c->nb; i++) {
            const cr_batch& b = batches[i];
            const float box[6] = {b.min_x, b.min_y, b.min_z, b.max_x, b.max_y, b.max_z};
            bool ok = b.num_points >= 0 && b.num_points <= kPointsPerBatch && b.first_point >= 0 &&
                      (int64_t)b.first_point + b.num_points <= c->n && b.file_index >= 0 &&
                      b.file_index < c->nfiles;
            for (int k = 0; k < 6 && ok; k++) ok = std::isfinite(box[k]);
            if (!ok) return fail(ctx, CR_ERR_INVALID_ARG, "invalid batch record %s%lld", "", (long long)i);
        }
        CR_CUDA(ctx, cudaMemcpyAsync(c->batches, batches, (size_t)c->nb * sizeof(cr_batch),
                                     cudaMemcpyHostToDevice, s), "batch upload");
    }
    const uint32_t* src[4] = {lo, md, hi, rgba};
    uint32_t* dst[4] = {c->lo, c->md, c->hi, c->rgba};
    for (int i = 0; i < 4; i++) {
        if (!src[i]) continue;
        if (!dst[i]) return fail(ctx, CR_ERR_INVALID_ARG, "stream %s%lld not allocated", "", (long long)i);
        CR_CUDA(ctx, cudaMemcpyAsync(dst[i], src[i], (size_t)c->n * 4, cudaMemcpyHostToDevice, s),
                "stream upload");
    }
    if (box_min) return cr_cloud_set_files(ctx, c, box_min);
    return CR_OK;
}

cr_status cr_cloud_set_files(cr_ctx* ctx, cr_cloud* c, const double* box_min) {
    if (!c || !box_min) return CR_ERR_INVALID_ARG;
    if (!finite_all(box_min, 3 * c->nfiles))
        return fail(ctx, CR_ERR_INVALID_ARG, "file boxMin must be finite%s", "");
    std::memcpy(c->box_min.data(), box_min, sizeof(double) * 3 * c->nfiles);
    return CR_OK;
}

cr_status cr_cloud_device(const cr_cloud* c, cr_batch** batches, uint32_t** lo, uint32_t** md,
                          uint32_t** hi, uint32_t** rgba) {
    if (!c || c->plain) return CR_ERR_INVALID_ARG;
    if (batches) *batches = c->batches;
    if (lo) *lo = c->lo;
    if (md) *md = c->md;
    if (hi) *hi = c->hi;
    if (rgba) *rgba = c->rgba;
    return CR_OK;
}

cr_status cr_cloud_read(cr_ctx* ctx, const cr_cloud* c, int32_t which, void* dst, int64_t bytes,
                        void* stream) {
    if (!ctx || !c || !dst || c->plain || bytes < 0) return CR_ERR_INVALID_ARG;
    const void* src = nullptr;
    int64_t limit = c->n * 4;
    switch (which) {
        case 0: src = c->batches; limit = c->nb * (int64_t)sizeof(cr_batch); break;
        case CR_STREAM_LOW: src = c->lo; break;
        case CR_STREAM_MED: src = c->md; break;
        case CR_STREAM_HIG: src = c->hi; break;
        case CR_STREAM_RGBA: src = c->rgba; break;
        default: return fail(ctx, CR_ERR_INVALID_ARG, "unknown cloud array %s%lld", "", (long long)which);
    }
    if (!src || bytes > limit) return fail(ctx, CR_ERR_INVALID_ARG, "bad cloud read %s%lld", "", (long long)bytes);
    // cudaMemcpyDefault: a wrapped cloud's arrays may be host memory
    CR_CUDA(ctx, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, (cudaStream_t)stream),
            "cloud read");
    return CR_OK;
}

int64_t cr_cloud_num_points(const cr_cloud* c) { return c ? c->n : -1; }

cr_status cr_cloud_set_loaded(cr_ctx* ctx, cr_cloud* c, int64_t points, int64_t batches) {
    if (!c) return CR_ERR_INVALID_ARG;
    if (points < 0 && batches < 0) {
        c->n_loaded = c->nb_loaded = -1;
        return CR_OK;
    }
    if (points < 0 || points > c->n || (!c->plain && (batches < 0 || batches > c->nb)))
        return fail(ctx, CR_ERR_INVALID_ARG, "loaded counts exceed the cloud%s", "");
    c->n_loaded = points;
    c->nb_loaded = c->plain ? -1 : batches;
    return CR_OK;
}
int64_t cr_cloud_num_batches(const cr_cloud* c) { return c ? c->nb : -1; }

cr_status cr_cloud_destroy(cr_ctx* ctx, cr_cloud* c) {
    if (!c) return CR_ERR_INVALID_ARG;
    if (c->owned) {
        void* ptrs[6] = {c->batches, c->lo, c->md, c->hi, c->rgba, c->verts};
        for (void* p : ptrs)
            if (p) cudaFree(p);
    }
    delete c;
    return CR_OK;
}

namespace {

// True when kernels on `device` may dereference p: device memory or pinned host
// memory mapped under unified addressing (the device pointer equals p), or any
// other host memory when the device reads pageable memory directly.
bool device_addressable(const void* p, int device) {
    cudaPointerAttributes a;
    std::memset(&a, 0, sizeof(a));
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
        return a.devicePointer == p && (a.type == cudaMemoryTypeManaged || a.device == device);
    if (a.type == cudaMemoryTypeHost) return a.devicePointer == p;
    int pageable = 0;
    return cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess &&
           pageable == 1;
}

}  // namespace

cr_status cr_cloud_wrap(cr_ctx* ctx, int64_t n, int64_t nb, int32_t nfiles, const cr_batch* batches,
                        const uint32_t* lo, const uint32_t* md, const uint32_t* hi,
                        const uint32_t* rgba, int64_t stream_words, cr_cloud** out) {
    if (!ctx || !out || !batches || !lo || n < 0 || nb < 0 || nb >= kMaxBatches ||
        n >= ((int64_t)1 << 31) ||
        nfiles < 1 || nfiles > kMaxFiles || stream_words < n + kStreamPad)
        return fail(ctx, CR_ERR_INVALID_ARG, "bad wrapped cloud arguments%s", "");
    *out = nullptr;
    const void* arrays[5] = {batches, lo, md, hi, rgba};
    const char* names[5] = {"batches", "xyz_low", "xyz_med", "xyz_hig", "rgba"};
    for (int i = 0; i < 5; i++)
        if (arrays[i] && !device_addressable(arrays[i], ctx->device))
            return fail(ctx, CR_ERR_INVALID_ARG, "%s is not memory the GPU can address", names[i]);
    cr_cloud* c = new (std::nothrow) cr_cloud();
    if (!c) return CR_ERR_OUT_OF_MEMORY;
    c->owned = false;
    c->n = n;
    c->nb = nb;
    c->nfiles = nfiles;
    c->capacity = stream_words;
    c->batches = const_cast<cr_batch*>(batches);
    c->lo = const_cast<uint32_t*>(lo);
    c->md = const_cast<uint32_t*>(md);
    c->hi = const_cast<uint32_t*>(hi);
    c->rgba = const_cast<uint32_t*>(rgba);
    c->mask = CR_STREAM_LOW | (md ? CR_STREAM_MED : 0) | (hi ? CR_STREAM_HIG : 0) | (rgba ? CR_STREAM_RGBA : 0);
    c->box_min.assign(3 * (size_t)nfiles, 0.0);
    *out = c;
    return CR_OK;
}

cr_status cr_cloud_create_plain(cr_ctx* ctx, int64_t n, cr_cloud** out) {
    if (!ctx || !out || n < 0 || n >= ((int64_t)1 << 33)) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    cr_cloud* c = new (std::nothrow) cr_cloud();
    if (!c) return CR_ERR_OUT_OF_MEMORY;
    c->plain = true;
    c->n = n;
    c->nfiles = 1;
    c->box_min.assign(3, 0.0);
    cudaError_t e = cudaMalloc(&c->verts, (size_t)std::max<int64_t>(n, 1) * sizeof(cr_vertex));
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(ctx, e, "plain cloud allocation");
    }
    *out = c;
    return CR_OK;
}

cr_status cr_cloud_upload_plain(cr_ctx* ctx, cr_cloud* c, const cr_vertex* v, void* stream) {
    if (!ctx || !c || !c->plain || !v) return CR_ERR_INVALID_ARG;
    CR_CUDA(ctx, cudaMemcpyAsync(c->verts, v, (size_t)c->n * sizeof(cr_vertex), cudaMemcpyHostToDevice,
                                 (cudaStream_t)stream), "vertex upload");
    return CR_OK;
}

cr_status cr_cloud_device_plain(const cr_cloud* c, cr_vertex** v) {
    if (!c || !c->plain || !v) return CR_ERR_INVALID_ARG;
    *v = c->verts;
    return CR_OK;
}

// ---- framebuffers -------------------------------------------------------------

cr_status cr_fb_create(cr_ctx* ctx, int32_t W, int32_t H, int32_t kind, cr_fb** out) {
    if (!ctx || !out || (kind != CR_FB_U64 && kind != CR_FB_HQS)) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    cr_status s = check_size(ctx, W, H);
    if (s != CR_OK) return s;
    cr_fb* f = new (std::nothrow) cr_fb();
    if (!f) return CR_ERR_OUT_OF_MEMORY;
    f->W = W;
    f->H = H;
    f->kind = kind;
    f->words = (int64_t)W * H + W + 1;
    cudaError_t e;
    if (kind == CR_FB_U64) {
        e = cudaMalloc(&f->fb, (size_t)f->words * 8);
    } else {
        e = cudaMalloc(&f->depth, (size_t)f->words * 4);
        if (e == cudaSuccess) e = cudaMalloc(&f->accum, (size_t)f->words * 16);
    }
    if (e == cudaSuccess) e = cudaMalloc(&f->image, (size_t)W * H * 4);
    // a new image starts at zero: pixels a resolve does not cover (the plain
    // methods' partial tiles) read back as 0, not as stale device memory
    if (e == cudaSuccess) e = cudaMemset(f->image, 0, (size_t)W * H * 4);
    if (e != cudaSuccess) {
        cr_fb_destroy(ctx, f);
        return cuda_fail(ctx, e, "framebuffer allocation");
    }
    *out = f;
    return CR_OK;
}

cr_status cr_fb_destroy(cr_ctx*, cr_fb* f) {
    if (!f) return CR_ERR_INVALID_ARG;
    void* ptrs[4] = {f->fb, f->depth, f->accum, f->image};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete f;
    return CR_OK;
}

cr_status cr_fb_clear(cr_ctx* ctx, cr_fb* f, uint64_t value, void* stream) {
    if (!ctx || !f) return CR_ERR_INVALID_ARG;
    int rc;
    if (f->kind == CR_FB_U64) {
        rc = launch_fill_u64(f->fb, f->words, value, stream);
    } else {
        rc = launch_fill_u32(f->depth, f->words, (uint32_t)value, stream);
        if (rc == 0) rc = launch_fill_u64(f->accum, 2 * f->words, 0ull, stream);
    }
    if (rc != 0) return fail(ctx, CR_ERR_CUDA, "clear launch failed%s", "");
    return CR_OK;
}

int64_t cr_fb_bytes(const cr_fb* f, int32_t what) {
    if (!f) return -1;
    switch (what) {
        case CR_FB_WORDS: return f->fb ? f->words * 8 : 0;
        case CR_FB_DEPTH: return f->depth ? f->words * 4 : 0;
        case CR_FB_ACCUM: return f->accum ? f->words * 16 : 0;
        case CR_FB_IMAGE: return (int64_t)f->W * f->H * 4;
    }
    return -1;
}

cr_status cr_fb_device(const cr_fb* f, int32_t what, void** p) {
    if (!f || !p) return CR_ERR_INVALID_ARG;
    switch (what) {
        case CR_FB_WORDS: *p = f->fb; break;
        case CR_FB_DEPTH: *p = f->depth; break;
        case CR_FB_ACCUM: *p = f->accum; break;
        case CR_FB_IMAGE: *p = f->image; break;
        default: return CR_ERR_INVALID_ARG;
    }
    return *p ? CR_OK : CR_ERR_INVALID_ARG;
}

cr_status cr_fb_read(cr_ctx* ctx, const cr_fb* f, int32_t what, void* dst, int64_t bytes, void* stream) {
    if (!ctx || !f || !dst) return CR_ERR_INVALID_ARG;
    void* src = nullptr;
    if (cr_fb_device(f, what, &src) != CR_OK || bytes < 0 || bytes > cr_fb_bytes(f, what))
        return fail(ctx, CR_ERR_INVALID_ARG, "bad fb read %s(%lld bytes)", "", (long long)bytes);
    CR_CUDA(ctx, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream),
            "fb read");
    return CR_OK;
}

// ---- rendering ------------------------------------------------------------------

cr_status cr_resolve(cr_ctx* ctx, const cr_cloud* cloud, const cr_render_params* p, cr_fb* fb,
                     void* stream) {
    if (!ctx || !p || !fb) return CR_ERR_INVALID_ARG;
    int rc;
    if (p->method == CR_METHOD_LOOP_LAS_HQS) {
        if (fb->kind != CR_FB_HQS) return fail(ctx, CR_ERR_INVALID_ARG, "HQS needs an HQS fb%s", "");
        rc = launch_resolve_hqs(fb->W, fb->H, fb->depth, fb->accum, fb->image, p->clear_after, stream);
    } else {
        if (fb->kind != CR_FB_U64) return fail(ctx, CR_ERR_INVALID_ARG, "method needs a u64 fb%s", "");
        if (plain_method(p->method)) {
            const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? default_quirks(p->method) : p->quirks;
            rc = launch_resolve_plain(fb->W, fb->H, fb->fb, fb->image, p->clear_after, p->clear_value,
                                      (quirks & CR_QUIRK_RESOLVE_TILES) != 0,
                                      p->method != CR_METHOD_DEDUP, stream);
        } else {
            const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? default_quirks(p->method) : p->quirks;
            const int tiles = (quirks & CR_QUIRK_RESOLVE_TILES) ? 1 : 0;
            if (p->payload == CR_PAYLOAD_COLOR && !tiles) {
                rc = launch_resolve_color(fb->W, fb->H, fb->fb, fb->image, p->clear_after, p->clear_value,
                                          stream);
            } else if (p->payload == CR_PAYLOAD_COLOR) {
                return fail(ctx, CR_ERR_UNSUPPORTED, "the tiled resolve reads the index payload%s", "");
            } else {
                if (!cloud || !cloud->rgba)
                    return fail(ctx, CR_ERR_INVALID_ARG, "index payload resolve needs the color stream%s", "");
                rc = launch_resolve_index(fb->W, fb->H, fb->fb, cloud->rgba, cloud->capacity, fb->image,
                                          p->clear_after, p->clear_value, stream, tiles);
            }
        }
    }
    if (rc != 0) return fail(ctx, CR_ERR_CUDA, "resolve launch failed%s", "");
    return CR_OK;
}

cr_status cr_render(cr_ctx* ctx, const cr_cloud* cloud, const cr_view* view,
                    const cr_render_params* p, cr_fb* fb, void* stream) {
    if (!ctx || !cloud || !view || !p || !fb) return CR_ERR_INVALID_ARG;
    const NvtxRange range("cr_render");
    if (p->method < 0 || p->method >= kNumMethods)
        return fail(ctx, CR_ERR_INVALID_ARG, "unknown method %s%lld", "", (long long)p->method);
    if (view->width != fb->W || view->height != fb->H)
        return fail(ctx, CR_ERR_INVALID_ARG, "view size differs from the framebuffer%s", "");
    cr_status s = check_size(ctx, view->width, view->height);
    if (s != CR_OK) return s;
    const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? default_quirks(p->method) : p->quirks;
    const bool plain = plain_method(p->method);
    const bool hqs = p->method == CR_METHOD_LOOP_LAS_HQS;

    // ---- validation before anything is enqueued
    if (plain) {
        if (!cloud->plain) return fail(ctx, CR_ERR_INVALID_ARG, "2021 methods need a plain cloud%s", "");
        if (fb->kind != CR_FB_U64) return fail(ctx, CR_ERR_INVALID_ARG, "2021 methods need a u64 fb%s", "");
        if (!finite_all(view->view, 16) || !finite_all(view->proj, 16))
            return fail(ctx, CR_ERR_INVALID_ARG, "view matrices must be finite%s", "");
    } else {
        if (cloud->plain) return fail(ctx, CR_ERR_INVALID_ARG, "method needs a LAS-derived cloud%s", "");
        if (!cloud->md || !cloud->hi)
            return fail(ctx, CR_ERR_INVALID_ARG, "batched methods need all three coordinate streams%s", "");
        if (hqs && fb->kind != CR_FB_HQS) return fail(ctx, CR_ERR_INVALID_ARG, "HQS needs an HQS fb%s", "");
        if (!hqs && fb->kind != CR_FB_U64) return fail(ctx, CR_ERR_INVALID_ARG, "method needs a u64 fb%s", "");
        if ((hqs || p->payload == CR_PAYLOAD_COLOR || p->resolve) && !cloud->rgba)
            return fail(ctx, CR_ERR_INVALID_ARG, "the color stream is required%s", "");
    }

    cudaStream_t st = (cudaStream_t)stream;
    cr_frame_events* fe = nullptr;
    if (ctx->timing_used < (int32_t)ctx->timing.size()) fe = &ctx->timing[ctx->timing_used++];
    auto mark = [&](int boundary, int stage_ran) {
        if (!fe) return;
        cudaEventRecord(fe->ev[boundary], st);
        if (stage_ran >= 0) fe->ran[stage_ran] = true;
    };
    mark(0, -1);

    if (plain) {
        // compute_2021_earlyz.h:108-113: float proj * view * identity
        float fv[16], fp[16], pv[16], T[16];
        const float id[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        for (int i = 0; i < 16; i++) {
            fv[i] = (float)view->view[i];
            fp[i] = (float)view->proj[i];
        }
        mat_mul(fp, fv, pv);
        mat_mul(pv, id, T);
        mark(1, -1);
        const int grid = ctx->num_sms * 8;
        const int variant = p->method == CR_METHOD_DEDUP ? 1 : (p->method == CR_METHOD_EARLYZ_REDUCE ? 2 : 0);
        if (launch_plain(T, fb->W, fb->H, cloud->verts, loaded_points(cloud), fb->fb, grid, variant,
                         stream, (quirks & CR_QUIRK_LITERAL_ARITH) ? 1 : 0) != 0)
            return fail(ctx, CR_ERR_CUDA, "plain raster launch failed%s", "");
        mark(2, CR_STAGE_RASTER);
        mark(3, -1);
        if (p->resolve) {
            s = cr_resolve(ctx, cloud, p, fb, stream);
            if (s != CR_OK) return s;
        }
        mark(4, p->resolve ? CR_STAGE_RESOLVE : -1);
        return CR_OK;
    }

    ViewParams vp;
    s = build_view_params(ctx, cloud, view, p->frustum_culling, quirks, &vp);
    if (s != CR_OK) return s;
    vp.lod_skip_level = p->lod_skip_level;
    s = enqueue_file_records(ctx, cloud, view, quirks, &vp, stream);
    if (s != CR_OK) return s;
    // the loader's numBatchesLoaded / numPointsLoaded (compute_loop_las.h:233,
    // compute_loop_las2.h:234)
    int64_t nb = loaded_batches(cloud);
    if (quirks & CR_QUIRK_DISPATCH_BY_POINTS)
        nb = std::min<int64_t>(nb, (loaded_points(cloud) + kPointsPerBatch - 1) / kPointsPerBatch);
    // loop_nodes: nodes of up to 64,512 points go out as kNodeSlice-point
    // slices, so a frame's few hundred nodes keep every SM busy.  (Slicing the
    // 10,240-point batches of small clouds too measured 3-9 % slower on the
    // 100M-point flight poses: the per-item cost outweighs the shorter tail.)
    const bool slices = (quirks & CR_QUIRK_NODE_LOOP) && nb <= (int64_t)kItemNodeMask + 1;
    const int64_t list_cap = slices ? nb * kMaxNodeSlices : nb;
    s = ensure_scratch(ctx, list_cap);
    if (s != CR_OK) return s;
    ctx->last_dispatched = nb;
    ctx->last_list_cap = list_cap;
    ctx->last_node_slices = slices;

    CR_CUDA(ctx, cudaMemsetAsync(ctx->scratch, 0, kCounterWords * 4, st), "counter reset");
    if (launch_cull(vp, cloud->batches, nb, cloud->capacity, quirks, ctx->scratch, stream, list_cap,
                    slices ? 1 : 0) != 0)
        return fail(ctx, CR_ERR_CUDA, "cull launch failed%s", "");
    mark(1, CR_STAGE_CULL);

    BatchedLaunch bl{};
    bl.batches = cloud->batches;
    bl.lo = cloud->lo;
    bl.md = cloud->md;
    bl.hi = cloud->hi;
    bl.rgba = cloud->rgba;
    bl.capacity = cloud->capacity;
    bl.fb = fb->fb;
    bl.depth = fb->depth;
    bl.accum = fb->accum;
    bl.scratch = ctx->scratch;
    bl.list_cap = list_cap;
    bl.node_slices = slices ? 1 : 0;
    bl.quirks = quirks;
    bl.payload = hqs ? CR_PAYLOAD_INDEX : p->payload;
    // 128 threads per CTA measured fastest for every payload at 1B points
    const int block = (p->block_threads == 256 || p->block_threads == 512) ? p->block_threads : 128;
    const int modes[2] = {hqs ? kModeHqsDepth : kModeRaster, kModeHqsColor};
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1 && !hqs) {
            mark(3, -1);
            break;
        }
        bl.mode = modes[pass];
        int per_sm = p->ctas_per_sm > 0 ? p->ctas_per_sm
                                         : batched_blocks_per_sm(bl.mode, bl.payload, block,
                                                                 cloud->nfiles > kInlineFiles,
                                                                 (quirks & CR_QUIRK_LITERAL_ARITH) != 0);
        if (per_sm < 1) per_sm = 1;
        const int grid = ctx->num_sms * per_sm;
        if (launch_batched(vp, bl, block, grid, stream) != 0)
            return fail(ctx, CR_ERR_CUDA, "batched raster launch failed%s", "");
        mark(2 + pass, pass == 0 ? CR_STAGE_RASTER : CR_STAGE_HQS_COLOR);
    }
    if (p->resolve) {
        s = cr_resolve(ctx, cloud, p, fb, stream);
        if (s != CR_OK) return s;
    }
    mark(4, p->resolve ? CR_STAGE_RESOLVE : -1);
    return CR_OK;
}

cr_status cr_last_frame_stats(cr_ctx* ctx, const cr_cloud* cloud, const cr_render_params* p,
                              cr_frame_stats* out) {
    if (!ctx || !cloud || !p || !out || cloud->plain) return CR_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    CR_CUDA(ctx, cudaDeviceSynchronize(), "synchronize");
    uint32_t counts[kCounterWords] = {};
    CR_CUDA(ctx, cudaMemcpy(counts, ctx->scratch, sizeof(counts), cudaMemcpyDeviceToHost), "count read");
    const uint32_t n_front = counts[kItemCount], n_back = counts[kItemCount2];
    const uint32_t count = n_front + n_back;
    std::vector<uint32_t> items(count);
    if (n_front)
        CR_CUDA(ctx, cudaMemcpy(items.data(), ctx->scratch + kScratchHead, (size_t)n_front * 4,
                                cudaMemcpyDeviceToHost), "item read");
    if (n_back)  // the 20/30-bit list fills the region from its end
        CR_CUDA(ctx, cudaMemcpy(items.data() + n_front,
                                ctx->scratch + kScratchHead + ctx->last_list_cap - n_back,
                                (size_t)n_back * 4, cudaMemcpyDeviceToHost), "item read");
    std::vector<cr_batch> recs((size_t)cloud->nb);
    if (cloud->nb)
        CR_CUDA(ctx, cudaMemcpy(recs.data(), cloud->batches, recs.size() * sizeof(cr_batch),
                                cudaMemcpyDeviceToHost), "batch read");
    const int quirks = p->quirks == CR_QUIRKS_METHOD_DEFAULT ? default_quirks(p->method) : p->quirks;
    const bool hqs = p->method == CR_METHOD_LOOP_LAS_HQS;
    const bool color = hqs || p->payload == CR_PAYLOAD_COLOR;
    out->batches_dispatched = ctx->last_dispatched;
    out->batches_visible = 0;
    for (uint32_t it : items) {
        const uint32_t b = it & (ctx->last_node_slices ? kItemNodeMask : kItemBatchMask);
        const int64_t slice = ctx->last_node_slices ? (int64_t)((it >> kItemSliceShift) & 31u) : 0;
        const int level = (int)(it >> 29);
        if (b >= recs.size() || level > 4) continue;
        int64_t n = recs[b].num_points;
        if (quirks & CR_QUIRK_NODE_LOOP) {  // compute_loop_nodes/render.cs:296-300
            const int64_t loop = std::min<int64_t>((n + 127) / 128, 500);
            n = std::min<int64_t>(n, 512 * ((loop + 4) / 4) - (recs[b].first_point & 3));
        } else {
            n = std::min<int64_t>(n + ((quirks & CR_QUIRK_INCLUSIVE_END) ? 1 : 0), kPointsPerBatch);
        }
        if (ctx->last_node_slices) {  // this item's slice of the node
            int64_t sf = 0;
            node_slice(recs[b].first_point, n, slice, &sf, &n);
        }
        const int words = level >= 2 ? 1 : (level == 1 ? 2 : 3);
        if (slice == 0) {
            out->batches_visible += 1;
            out->batches_per_level[level] += 1;
        }
        out->points_per_level[level] += n;
        // HQS reads the coordinates twice (depth and color pass) and colors once
        out->stream_bytes += (hqs ? 2 : 1) * (4 * words * n + (slice == 0 ? 64 : 0)) + (color ? 4 * n : 0);
    }
    return CR_OK;
}

// ---- host layout builders -----------------------------------------------------------

int64_t cr_num_batches(int64_t n) { return n <= 0 ? 0 : (n + kPointsPerBatch - 1) / kPointsPerBatch; }

// LasLoaderSparse.cpp:37-212 (loadLas) for one load task.
cr_status cr_encode_las(const uint8_t* rec, int64_t n, int32_t bpp, int32_t fmt, const double scale[3],
                        const double offset[3], const double box_min[3], int64_t sparse_offset,
                        int32_t file_index, cr_batch* batches, uint32_t* lo, uint32_t* md,
                        uint32_t* hi, uint32_t* rgba) {
    if ((n > 0 && !rec) || n < 0 || bpp < 12 || !scale || !offset || !box_min || !batches || !lo ||
        !md || !hi || !rgba || sparse_offset < 0 || sparse_offset + n >= ((int64_t)1 << 31) ||
        !finite_all(scale, 3) || !finite_all(offset, 3) || !finite_all(box_min, 3))
        return CR_ERR_INVALID_ARG;
    // LasLoaderSparse.cpp:123-132
    const int rgb = fmt == 2 ? 20 : (fmt == 3 ? 28 : ((fmt == 7 || fmt == 8) ? 30 : 0));
    if (rgb + 6 > bpp && rgb != 0) return CR_ERR_INVALID_ARG;
    const int64_t nb = cr_num_batches(n);
    const double steps = 1073741824.0;
    std::vector<double> xyz;
    for (int64_t bi = 0; bi < nb; bi++) {
        const int64_t first = bi * kPointsPerBatch;
        const int64_t cnt = std::min<int64_t>(kPointsPerBatch, n - first);
        xyz.resize((size_t)cnt * 3);
        double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t i = 0; i < cnt; i++) {
            const uint8_t* r = rec + (first + i) * bpp;
            for (int k = 0; k < 3; k++) {
                double v = (double)read_i32(r + 4 * k) * scale[k] + offset[k] - box_min[k];
                xyz[3 * i + k] = v;
                if (v < mn[k]) mn[k] = v;
                if (mx[k] < v) mx[k] = v;
            }
        }
        const double size[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
        cr_batch& b = batches[bi];
        std::memset(&b, 0, sizeof(b));
        b.min_x = (float)mn[0]; b.min_y = (float)mn[1]; b.min_z = (float)mn[2];
        b.max_x = (float)mx[0]; b.max_y = (float)mx[1]; b.max_z = (float)mx[2];
        b.num_points = (int32_t)cnt;
        b.first_point = (int32_t)(sparse_offset + first);
        b.file_index = file_index;
        for (int64_t i = 0; i < cnt; i++) {
            const int64_t pi = first + i;
            uint32_t q[3];
            for (int k = 0; k < 3; k++) {
                double t = ((xyz[3 * i + k] - mn[k]) / size[k]) * steps;
                uint32_t u = std::isnan(t) ? 0u : (uint32_t)t;  // zero-extent axis: 0/0
                q[k] = std::min<uint32_t>(u, 1073741823u);
            }
            lo[pi] = ((q[0] >> 20) & 1023u) | (((q[1] >> 20) & 1023u) << 10) | (((q[2] >> 20) & 1023u) << 20);
            md[pi] = ((q[0] >> 10) & 1023u) | (((q[1] >> 10) & 1023u) << 10) | (((q[2] >> 10) & 1023u) << 20);
            hi[pi] = (q[0] & 1023u) | ((q[1] & 1023u) << 10) | ((q[2] & 1023u) << 20);
            const uint8_t* r = rec + pi * bpp + rgb;
            int R = read_u16(r), G = read_u16(r + 2), B = read_u16(r + 4);
            R = R < 256 ? R : R / 256;
            G = G < 256 ? G : G / 256;
            B = B < 256 ? B : B / 256;
            rgba[pi] = (uint32_t)R | ((uint32_t)G << 8) | ((uint32_t)B << 16);
        }
    }
    return CR_OK;
}

// LasLoaderStandard.h:152-179
cr_status cr_encode_standard(const uint8_t* rec, int64_t n, int32_t bpp, int32_t fmt,
                             const double scale[3], const double offset[3], const double box_min[3],
                             cr_vertex* out) {
    if ((n > 0 && (!rec || !out)) || n < 0 || bpp < 12 || !scale || !offset || !box_min)
        return CR_ERR_INVALID_ARG;
    const int rgb = fmt == 2 ? 20 : (fmt == 3 ? 28 : 0);
    for (int64_t i = 0; i < n; i++) {
        const uint8_t* r = rec + i * bpp;
        float f[3];
        for (int k = 0; k < 3; k++)
            f[k] = (float)((double)read_i32(r + 4 * k) * scale[k] + offset[k] - box_min[k]);
        int R = read_u16(r + rgb), G = read_u16(r + rgb + 2), B = read_u16(r + rgb + 4);
        uint32_t cr_ = (uint32_t)(R > 255 ? R / 256 : R) & 0xFFu;
        uint32_t cg = (uint32_t)(G > 255 ? G / 256 : G) & 0xFFu;
        uint32_t cb = (uint32_t)(B > 255 ? B / 256 : B) & 0xFFu;
        out[i].x = f[0];
        out[i].y = f[1];
        out[i].z = f[2];
        out[i].color = cr_ | (cg << 8) | (cb << 16) | (255u << 24);
    }
    return CR_OK;
}

// ---- host matrices ---------------------------------------------------------------------

// glm::perspective, right-handed, clip z in [-1, 1] (Camera.h:38)
void cr_perspective(double fovy_deg, double aspect, double zn, double zf, double out[16]) {
    const double pi = 3.14159265358979323846264338327950288;
    const double fovy = pi * fovy_deg / 180.0;
    const double t = std::tan(fovy / 2.0);
    for (int i = 0; i < 16; i++) out[i] = 0.0;
    out[0] = 1.0 / (aspect * t);
    out[5] = 1.0 / t;
    out[10] = -(zf + zn) / (zf - zn);
    out[11] = -1.0;
    out[14] = -(2.0 * zf * zn) / (zf - zn);
}

static void normalize3(const double v[3], double o[3]) {
    const double inv = 1.0 / std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    o[0] = v[0] * inv;
    o[1] = v[1] * inv;
    o[2] = v[2] * inv;
}
static void cross3(const double a[3], const double b[3], double o[3]) {
    const double x = a[1] * b[2] - b[1] * a[2];
    const double y = a[2] * b[0] - b[2] * a[0];
    const double z = a[0] * b[1] - b[0] * a[1];
    o[0] = x;
    o[1] = y;
    o[2] = z;
}
static double dot3(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

void cr_look_at(const double eye[3], const double center[3], const double up[3], double out[16]) {
    const double d[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    double f[3], t[3], s[3], u[3];
    normalize3(d, f);
    cross3(f, up, t);
    normalize3(t, s);
    cross3(s, f, u);
    const double m[16] = {s[0], u[0], -f[0], 0, s[1], u[1], -f[1], 0, s[2], u[2], -f[2], 0,
                          -dot3(s, eye), -dot3(u, eye), dot3(f, eye), 1};
    std::memcpy(out, m, sizeof(m));
}

// Inverse by cofactors of 2x2 minors (row pairs 0-1 and 2-3), over the determinant.
static void inverse4(const double* m, double* out) {
    auto M = [&](int c, int r) { return m[c * 4 + r]; };
    const double s0 = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
    const double s1 = M(0, 0) * M(2, 1) - M(2, 0) * M(0, 1);
    const double s2 = M(0, 0) * M(3, 1) - M(3, 0) * M(0, 1);
    const double s3 = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    const double s4 = M(1, 0) * M(3, 1) - M(3, 0) * M(1, 1);
    const double s5 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1);
    const double c5 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    const double c4 = M(1, 2) * M(3, 3) - M(3, 2) * M(1, 3);
    const double c3 = M(1, 2) * M(2, 3) - M(2, 2) * M(1, 3);
    const double c2 = M(0, 2) * M(3, 3) - M(3, 2) * M(0, 3);
    const double c1 = M(0, 2) * M(2, 3) - M(2, 2) * M(0, 3);
    const double c0 = M(0, 2) * M(1, 3) - M(1, 2) * M(0, 3);
    const double det = (s0 * c5 - s1 * c4 + s2 * c3) + (s3 * c2 - s4 * c1 + s5 * c0);
    const double id = 1.0 / det;
    double r[16] = {
        (M(1, 1) * c5 - M(2, 1) * c4 + M(3, 1) * c3) * id,
        (-M(0, 1) * c5 + M(2, 1) * c2 - M(3, 1) * c1) * id,
        (M(0, 1) * c4 - M(1, 1) * c2 + M(3, 1) * c0) * id,
        (-M(0, 1) * c3 + M(1, 1) * c1 - M(2, 1) * c0) * id,
        (-M(1, 0) * c5 + M(2, 0) * c4 - M(3, 0) * c3) * id,
        (M(0, 0) * c5 - M(2, 0) * c2 + M(3, 0) * c1) * id,
        (-M(0, 0) * c4 + M(1, 0) * c2 - M(3, 0) * c0) * id,
        (M(0, 0) * c3 - M(1, 0) * c1 + M(2, 0) * c0) * id,
        (M(1, 3) * s5 - M(2, 3) * s4 + M(3, 3) * s3) * id,
        (-M(0, 3) * s5 + M(2, 3) * s2 - M(3, 3) * s1) * id,
        (M(0, 3) * s4 - M(1, 3) * s2 + M(3, 3) * s0) * id,
        (-M(0, 3) * s3 + M(1, 3) * s1 - M(2, 3) * s0) * id,
        (-M(1, 2) * s5 + M(2, 2) * s4 - M(3, 2) * s3) * id,
        (M(0, 2) * s5 - M(2, 2) * s2 + M(3, 2) * s1) * id,
        (-M(0, 2) * s4 + M(1, 2) * s2 - M(3, 2) * s0) * id,
        (M(0, 2) * s3 - M(1, 2) * s1 + M(2, 2) * s0) * id,
    };
    std::memcpy(out, r, sizeof(r));
}

// OrbitControls.h:116-135 world, inverted as Camera.h:35 does.
void cr_orbit_view(double yaw, double pitch, double radius, const double target[3], double out[16]) {
    const double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, target[0], target[1], target[2], 1};
    const double cy = std::cos(yaw), sy = std::sin(yaw), cp = std::cos(pitch), sp = std::sin(pitch);
    const double Ry[16] = {cy, sy, 0, 0, -sy, cy, 0, 0, 0, 0, cy + (1.0 - cy), 0, 0, 0, 0, 1};
    const double Rp[16] = {cp + (1.0 - cp), 0, 0, 0, 0, cp, sp, 0, 0, -sp, cp, 0, 0, 0, 0, 1};
    const double F[16] = {1, 0, 0, 0, 0, 0, 1, 0, 0, -1, 0, 0, 0, 0, 0, 1};
    const double Tr[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, radius, 1};
    double a[16], b[16], c[16], w[16];
    mat_mul(T, Ry, a);
    mat_mul(a, Rp, b);
    mat_mul(b, F, c);
    mat_mul(c, Tr, w);
    inverse4(w, out);
}

}  // extern "C"
