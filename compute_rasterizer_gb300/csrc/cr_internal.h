// cr_internal.h -- definitions shared by the host library (cr_api.cpp) and the
// CUDA kernels (cr_kernels.cu, cr_synth.cu).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include <nvtx3/nvToolsExt.h>

#include "../../include/cr_raster.h"

namespace cr {

// An NVTX range over a host call (the ranges profilers use to select a
// frame's launches; free unless a tool is attached).  The reference marks the
// same spans with GL timestamp queries (GLTimerQueries.cpp:6-22).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

constexpr int kPointsPerBatch = CR_POINTS_PER_BATCH;
constexpr int kInlineFiles = 8;       // per-file records passed in kernel parameters
constexpr int32_t kMaxFiles = CR_MAX_FILES;  // files per cloud (records in device memory past 8)
constexpr uint32_t kBackground = 0x00443322u;  // resolve.cs:141
constexpr uint64_t kDefaultClear = 0xFF800000FF800000ull;  // compute_loop_las.h:292-296
constexpr uint64_t kPlainReclear = 0xffffffffff3c321eull;  // compute_2021_earlyz/resolve.cs:77
constexpr uint32_t kHqsDepthClear = 0xFF800000u;           // compute_loop_las_hqs.h:336-340
// Zeroed words allocated past N in every stream: covers the 128-bit loads of
// a partial last batch and the one-past-the-end point of the inclusive bound.
constexpr int64_t kStreamPad = 64;

// Work items of the single-view lists (k_cull -> k_batched):
// batch index | kItemWSafe (the clip w of every point of the batch is proven
// to lie in [2^-120, 2^120]) | precision level << 29.
constexpr uint32_t kItemBatchMask = 0x0FFFFFFFu;
constexpr uint32_t kItemWSafe = 1u << 28;
constexpr int64_t kMaxBatches = (int64_t)1 << 28;
// With node slicing (loop_nodes, whose nodes hold up to 64,512 points), a
// node is handed out as items of kNodeSlice points: the slice in bits 23-27
// and the node's record index below.  Slices far smaller than a node spread
// the few hundred visible nodes of a typical octree frame over every SM.
// Slice boundaries sit at the node's first point rounded down to a 4-point
// vector plus multiples of kNodeSlice, so every slice but the first starts on
// a whole vector (node_slice()).
constexpr int kNodeSlice = 2560;
constexpr int kItemSliceShift = 23;
constexpr uint32_t kItemNodeMask = (1u << kItemSliceShift) - 1u;
constexpr int kMaxNodeSlices = 26;  // ceil((64,512 + 3) / kNodeSlice)

// Points [*first, *first + *count) of slice `slice` of a node of `count`
// points from `first` (host and device).
__host__ __device__ inline void node_slice(int64_t first, int64_t count, int64_t slice, int64_t* s_first,
                                          int64_t* s_count) {
    const int64_t base = (first & ~(int64_t)3) + slice * kNodeSlice;
    const int64_t lo = base > first ? base : first;
    const int64_t hi = base + kNodeSlice < first + count ? base + kNodeSlice : first + count;
    *s_first = lo;
    *s_count = hi > lo ? hi - lo : 0;
}
__host__ __device__ inline int64_t node_slices(int64_t first, int64_t count) {
    return count > 0 ? ((first & 3) + count + kNodeSlice - 1) / kNodeSlice : 0;
}

// Device error bits (ctx scratch word kErrWord).
enum : uint32_t {
    kErrBadBatch = 1u,   // record with num_points/first_point/file_index out of range
    kErrBadCount = 2u,   // work list overflow
};

// Per-(view, file) uniforms, computed on the host from double matrices
// (compute_loop_las.h:141-200 + render.cs:145-174): 56 floats.
struct FileRec {
    float T[16];       // transform = mat4(proj * view * translate(boxMin))
    float planes[24];  // frustumPlanes(transformFrustum): (nx, ny, nz, c) x 6
    float VW[16];      // uniforms.view * file.world (float product)
};

// Files [0, kInlineFiles) have their records in the kernel parameters; with
// more files, `dfiles` holds every file's record in device memory and files
// from kInlineFiles on are read from there (file_rec()).
struct ViewParams {
    float P[16];       // uniforms.proj
    int32_t W, H;
    int32_t nfiles;
    int32_t culling;
    int32_t lod_skip_level;  // >0: batches at level >= this are not rendered
    FileRec files[kInlineFiles];
    const FileRec* dfiles;   // nfiles records when nfiles > kInlineFiles, else null
    float level4_px;         // level 4 below this projected size (100; loop_nodes 80)
    int32_t one_world;       // every batch uses file 0's record (CR_QUIRK_ONE_WORLD)
    int32_t literal;         // CR_QUIRK_LITERAL_ARITH: the precision level as written
};

// Scratch words at the head of the ctx scratch buffer.  The cull kernel sorts
// visible batches into two lists sharing one region of `list_cap` words:
// 10-bit items grow from the front, 20/30-bit items from the back, so the
// common all-10-bit raster runs in a kernel instance without the wider decode.
enum : int {
    kItemCount = 0,   // items in the 10-bit list
    kCursor0 = 1,     // dynamic work cursor, 10-bit list, raster / HQS depth pass
    kCursor1 = 2,     // dynamic work cursor, 10-bit list, HQS color pass
    kItemCount2 = 3,  // items in the 20/30-bit list
    kCursor2 = 4,     // dynamic work cursor, 20/30-bit list, raster / HQS depth pass
    kCursor3 = 5,     // dynamic work cursor, 20/30-bit list, HQS color pass
    kCounterWords = 6,
    kErrWord = 7,     // sticky device error bits (cleared by cr_ctx_check)
    kScratchHead = 8  // item lists start here
};

enum Mode : int { kModeRaster = 0, kModeHqsDepth = 1, kModeHqsColor = 2 };

struct BatchedLaunch {
    const cr_batch* batches;
    const uint32_t* lo;
    const uint32_t* md;
    const uint32_t* hi;
    const uint32_t* rgba;
    int64_t capacity;      // allocated words per stream (N + padding)
    uint64_t* fb;          // u64 framebuffer (raster)
    uint32_t* depth;       // HQS depth
    uint64_t* accum;       // HQS accumulators
    uint32_t* scratch;     // counters + item lists
    int64_t list_cap;      // words of the item-list region
    int32_t quirks;
    int32_t payload;
    int32_t mode;
    int32_t node_slices;   // items are node slices (see kItemSliceShift)
};

// Host-callable launchers (cr_kernels.cu).
// Every file's record for one view, computed on the GPU from the double
// matrices and the files' boxMin (host array, passed to the kernels in their
// parameters, 1024 files per launch) into out[0, nfiles).
int launch_file_records(const double view[16], const double proj[16], const double* box_min,
                        int32_t nfiles, FileRec* out, void* stream, int float_uniforms = 0,
                        int literal = 0);
// list_cap: words of the item-list region (nb_dispatch, or nb_dispatch *
// kMaxNodeSlices with node_slices).
int launch_cull(const ViewParams& vp, const cr_batch* batches, int64_t nb_dispatch,
                int64_t capacity, int32_t quirks, uint32_t* scratch, void* stream,
                int64_t list_cap = -1, int node_slices = 0);
// bl.quirks & CR_QUIRK_LITERAL_ARITH selects the literal instances (128 threads)
int launch_batched(const ViewParams& vp, const BatchedLaunch& bl, int block, int grid,
                   void* stream);
// variant 0: early-z, 1: dedup, 2: early-z & reduce (the three plain methods);
// literal: CR_QUIRK_LITERAL_ARITH
int launch_plain(const float T[16], int32_t W, int32_t H, const cr_vertex* v, int64_t n,
                 uint64_t* fb, int grid, int variant, void* stream, int literal = 0);
// tiles: CR_QUIRK_RESOLVE_TILES (image words outside full 16x16 tiles kept)
int launch_resolve_index(int32_t W, int32_t H, uint64_t* fb, const uint32_t* rgba,
                         int64_t rgba_words, uint32_t* image, int clear_after, uint64_t clear,
                         void* stream, int tiles = 0);
int launch_resolve_color(int32_t W, int32_t H, uint64_t* fb, uint32_t* image, int clear_after,
                         uint64_t clear, void* stream);
// tiles: CR_QUIRK_RESOLVE_TILES; zero_rule: ucol == 0 resolves to opaque black
// (early-z, early-z & reduce; not dedup)
int launch_resolve_plain(int32_t W, int32_t H, uint64_t* fb, uint32_t* image, int clear_after,
                         uint64_t clear, int tiles, int zero_rule, void* stream);
int launch_resolve_hqs(int32_t W, int32_t H, uint32_t* depth, uint64_t* accum, uint32_t* image,
                       int clear_after, void* stream);
int launch_fill_u64(uint64_t* p, int64_t n, uint64_t v, void* stream);
int launch_fill_u32(uint32_t* p, int64_t n, uint32_t v, void* stream);
// rcp_rn against __frcp_rn over every float; counts into bad[0], the lowest
// mismatching bit pattern into *first (synchronous, default stream).
int launch_check_reciprocal(uint64_t* bad, uint32_t* first);
// many: the cloud has more than kInlineFiles files (its own kernel instances)
int batched_blocks_per_sm(int mode, int payload, int block, bool many = false, bool literal = false);

// Per-view uniforms from double matrices and per-file boxMin (cr_api.cpp):
// the records of the first min(num_files, kInlineFiles) files; dfiles is left
// null and must be set by the caller when num_files > kInlineFiles.
cr_status view_params_for(const cr_view* view, const double* box_min, int32_t num_files,
                          int32_t culling, ViewParams* out, int literal = 0);

// Read-only view of a LAS-derived cloud's device layout (cr_api.cpp).
struct CloudInfo {
    const cr_batch* batches;
    const uint32_t* lo;
    const uint32_t* md;
    const uint32_t* hi;
    const uint32_t* rgba;
    int64_t n, nb;              // points and batch records loaded (what frames dispatch)
    int64_t n_total, nb_total;  // allocated points and batch records
    int64_t capacity;
    int32_t nfiles;
    const double* box_min;  // 3 * nfiles
};
bool cloud_info(const cr_cloud* cloud, CloudInfo* out);
int default_quirks_for(int32_t method);
// cr_ctx_check(NULL, stream): the no-alloc array's error flag (cr_noalloc.cu)
cr_status noalloc_check(void* stream);

// k_encode over device records with the RGB triple at byte `rgb_offset` of a
// record, or colour 0 for rgb_offset < 0 (LAZ records without RGB, whose
// zeroed rgb loadLaz encodes); cr_encode_las_device derives the offset from
// the point format.
cr_status encode_records_device(const uint8_t* d_rec, int64_t n, int32_t bpp, int32_t rgb_offset,
                                const double scale[3], const double offset[3], const double box_min[3],
                                int64_t sparse_offset, int32_t file_index, cr_batch* d_batches,
                                uint32_t* d_lo, uint32_t* d_md, uint32_t* d_hi, uint32_t* d_rgba,
                                void* stream);
int ctx_device(const cr_ctx* ctx);

// ---- multi-view frames (cr_multiview.cu), shared by cr_mv plans and the server

// Per (view, file): the 12 transform entries the projection uses (T0, T1, T3,
// T4, T5, T7, T8, T9, T11, T12, T13, T15), the frustum planes, view * world.
struct MVFile {
    float T[12];
    float planes[24];
    float VW[16];
};

struct MVView {
    float P[16];
    int32_t W, H;
    uint32_t fb_off;   // u64 word offset of the view's framebuffer from MVFrame::fbs
    uint32_t img_off;  // u32 offset of the view's image from MVFrame::images
};

// Fills a view's P, W, H and, for clouds of at most kInlineFiles files, its
// per-file records from the double matrices (the single-view uniforms, so each
// view renders as cr_render would).  With more files the records are computed
// on the GPU each frame (MVFrame::d_mats, d_box) and out_files is not used.
cr_status mv_fill_view(const cr_view* view, const CloudInfo& ci, MVView* out_view,
                       MVFile* out_files);

// One multi-view frame over device-resident view records.
struct MVFrame {
    CloudInfo ci;
    const MVView* d_views;
    const MVFile* d_files;
    int32_t nviews;
    uint64_t* fbs;
    uint32_t* images;
    uint32_t* scratch;       // mv_scratch_words(ci.nb, nviews) words
    int32_t G, block, ctas_per_sm, quirks, payload, culling, num_sms;
    int32_t lod_skip_level;  // >0: a view skips batches at its level >= this
    int32_t clear_before;    // fill every view's W*H+W+1 words with clear_value first
    int32_t resolve, clear_after;
    uint64_t clear_value;
    int64_t max_words;       // max over the views of W*H+W+1
    // clouds with more than kInlineFiles files: per view the double view and
    // proj matrices (32 doubles), per file boxMin (3 doubles), both in device
    // memory; the frame computes d_files from them before the cull
    const double* d_mats;
    const double* d_box;
    // per view group, bit s: views s and s + 1 share their y / w rows (or NULL)
    const uint32_t* d_pairs;
};
int64_t mv_scratch_words(int64_t nb, int64_t nviews);
// Enqueues counter reset, [fill], cull, raster (both lists), [resolve] on stream.
cr_status mv_enqueue(const MVFrame& f, void* stream, const char** what);

}  // namespace cr
