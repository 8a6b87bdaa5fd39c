/*
 * cr_raster.h -- C ABI of the GB300 point-rasterizer hot path.
 *
 * This library replaces the render dispatches of the compute_rasterizer
 * `Method` plugins (include/Method.h:10-24) for the LAS-derived batched layout
 * ("loop_las", "loop_las_prefetch", "loop_las_hqs") and the plain 16-byte path
 * ("(2021) early-z").  Every entry point takes plain pointers and sizes, returns
 * a cr_status and never aborts; a failed call leaves a message that
 * cr_last_error() returns.  Device work is enqueued on the caller's CUDA stream
 * (`stream` arguments are cudaStream_t values passed as void*; NULL = legacy
 * default stream).
 *
 * Data layout (one GPU, device resident):
 *   batches   cr_batch[B]            64 B records, one per <= 10,240 points
 *   xyz_low   uint32[N]  10-bit x|y<<10|z<<20, bits 29..20 of the 30-bit coords
 *   xyz_med   uint32[N]  bits 19..10          (needed by levels 0-1)
 *   xyz_hig   uint32[N]  bits  9..0           (needed by level 0)
 *   rgba      uint32[N]  R | G<<8 | B<<16
 *   fb        uint64[W*H + W + 1]   depth-bits<<32 | payload, plus a guard tail
 * Streams are allocated with zeroed padding past N so that vector loads of a
 * partial last batch stay in bounds.
 */
#ifndef CR_RASTER_H
#define CR_RASTER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CR_ABI_VERSION 2
#define CR_POINTS_PER_BATCH 10240 /* Resources.h:4-6: POINTS_PER_THREAD 80 x WORKGROUP_SIZE 128 */
#define CR_MAX_POINTS_PER_LOAD 1024000 /* Resources.h:8 MAX_POINTS_PER_BATCH */
/* Files per cloud: each batch record names its file (`fileIndex`), whose
 * boxMin places it in the world (render.cs:44-49; the reference's file SSBO
 * holds 5,000 records, compute_loop_las.h:100).  The first 8 files' per-view
 * uniforms travel in kernel parameters; with more files every file's record
 * is computed on the GPU into device memory each frame. */
#define CR_MAX_FILES 65536

typedef enum cr_status {
    CR_OK = 0,
    CR_ERR_INVALID_ARG = 1,
    CR_ERR_OUT_OF_MEMORY = 2,
    CR_ERR_ADMISSION_REJECTED = 3,
    CR_ERR_TIMEOUT = 4,
    CR_ERR_CUDA = 5,
    CR_ERR_DEVICE_FLAG = 6, /* a kernel found an out-of-range record and skipped it */
    CR_ERR_UNSUPPORTED = 7,
    CR_ERR_NOT_FOUND = 8,
    CR_ERR_CORRUPT = 9 /* a compressed stream does not decode */
} cr_status;

/* Method ids; names as registered by the reference (compute_loop_las.h:82,
 * compute_loop_las2.h:82, compute_loop_las_hqs.h:88, compute_2021_earlyz.h:52,
 * compute_2021_dedup.h:52, compute_2021_earlyz_reduce.h:52,
 * compute_loop_nodes.h:76). */
typedef enum cr_method {
    CR_METHOD_LOOP_LAS = 0,          /* "loop_las" */
    CR_METHOD_LOOP_LAS_PREFETCH = 1, /* "loop_las_prefetch" */
    CR_METHOD_LOOP_LAS_HQS = 2,      /* "loop_las_hqs" */
    CR_METHOD_EARLYZ = 3,            /* "(2021) early-z" */
    CR_METHOD_DEDUP = 4,             /* "(2021) dedup" */
    CR_METHOD_EARLYZ_REDUCE = 5,     /* "(2021) early-z & reduce" */
    CR_METHOD_LOOP_NODES = 6         /* "loop_nodes": Potree octree nodes as batches (cr_potree.h) */
} cr_method;

typedef enum cr_payload {
    CR_PAYLOAD_INDEX = 0, /* low word = global point index; color gathered at resolve (render.cs:417) */
    CR_PAYLOAD_COLOR = 1  /* low word = the point's RGBA8 word */
} cr_payload;

/* Reference behaviours kept for drop-in parity (each method's default set is
 * what the reference does; pass 0 for the corrected behaviour). */
typedef enum cr_quirk {
    CR_QUIRK_L0_X12 = 1,             /* 30-bit decode takes Y, Z low bits from X (render.cs:352-353) */
    CR_QUIRK_INCLUSIVE_END = 2,      /* `localIndex > numPoints` (las2/render.cs:341, hqs/depth.cs:276) */
    CR_QUIRK_DISPATCH_BY_POINTS = 4, /* ceil(numPoints/10240) workgroups (compute_loop_las2.h:234) */
    /* loop_las_prefetch's uvec4 addressing from firstPoint/4 (las2/render.cs:319-341): when
     * firstPoint % 4 = r != 0, thread 0 underflows localIndex and returns, so the batch points
     * l with (l + r) % 512 < 4 are skipped, and the last r points (l >= 10240 - r) are never
     * visited.  Batched single-view, multi-view and server paths. */
    CR_QUIRK_UVEC4_BASE = 8,
    /* The resolve dispatches floor(W/16) x floor(H/16) groups of 16x16
     * (compute_2021_earlyz.h:161-163, compute_loop_nodes.h:199-201): pixels outside those
     * tiles keep their image words.  The 2021 methods re-clear in the resolve, so their
     * framebuffer words there keep their values too; loop_nodes clears its framebuffer
     * separately (compute_loop_nodes.h:239-251), every pixel. */
    CR_QUIRK_RESOLVE_TILES = 16,
    /* compute_loop_nodes/render.cs:296-300: a batch (an octree node) visits
     * min(numPoints, 512 * floor((min(ceil(numPoints / 128), 500) + 4) / 4) - firstPoint % 4)
     * points, so nodes hold up to 64,512 points, with no 10,240-point cap. */
    CR_QUIRK_NODE_LOOP = 32,
    /* compute_loop_nodes/render.cs:199: precision level 4 below 80 pixels (loop_las: 100). */
    CR_QUIRK_LEVEL4_80PX = 64,
    /* every batch rendered with file 0's world: Potree batches carry the node level in the
     * file_index slot (PotreeData.h:335-350), and loop_nodes has one world matrix. */
    CR_QUIRK_ONE_WORLD = 128,
    /* uniforms as float products: transform = float(proj) * float(view) * world
     * (compute_loop_nodes.h:128-139; loop_las forms them in double and casts). */
    CR_QUIRK_FLOAT_UNIFORMS = 256,
    /* The shader math evaluated as its GLSL source is written, each operation
     * rounded once: decode `float(X) * step + min` as a product then a sum,
     * `transform * vec4(p, 1)` as (m0 x + m1 y) + (m2 z + m3), `pos.xy / pos.w`
     * and `vec3 / length` as one division per component.  Off by default: the
     * kernels' own contract fuses the decode and projection into FMAs and
     * divides by one reciprocal (faster; GLSL leaves both choices to the
     * driver).  With it, frames equal the reference's shaders compiled as C++
     * against its glm, bit for bit.  Single-view methods only (cr_render and
     * the no-allocation entry); multi-view plans and the server refuse it. */
    CR_QUIRK_LITERAL_ARITH = 512
} cr_quirk;

#define CR_QUIRKS_METHOD_DEFAULT (-1)

/* 64-byte batch record: render.cs:22-40, LasLoaderSparse.cpp:109-121. */
typedef struct cr_batch {
    int32_t state;
    float min_x, min_y, min_z;
    float max_x, max_y, max_z;
    int32_t num_points;
    int32_t first_point; /* global index of the batch's first point */
    int32_t file_index;
    int32_t padding[6];
} cr_batch;

/* Plain 16-byte point: compute_2021_earlyz/render.cs:15-20. */
typedef struct cr_vertex {
    float x, y, z;
    uint32_t color;
} cr_vertex;

/* One view: Renderer.h:78-82 View{dmat4 view, proj} plus the framebuffer size.
 * Matrices are column-major doubles, like glm::dmat4. */
typedef struct cr_view {
    double view[16];
    double proj[16];
    int32_t width, height;
} cr_view;

typedef struct cr_render_params {
    int32_t method;          /* cr_method */
    int32_t payload;         /* cr_payload (batched methods) */
    int32_t quirks;          /* cr_quirk mask, or CR_QUIRKS_METHOD_DEFAULT */
    int32_t frustum_culling; /* Debug::frustumCullingEnabled (Debug.h:16-29), default 1 */
    int32_t resolve;         /* 1: resolve into the fb's RGBA8 image after rasterizing */
    int32_t clear_after;     /* 1: re-clear the fb after the resolve (compute_loop_las.h:288-301) */
    uint64_t clear_value;    /* fb clear word; default 0xFF800000FF800000 (-inf bits x2) */
    int32_t block_threads;   /* threads per CTA for the batched kernels; 0 = tuned default */
    int32_t ctas_per_sm;     /* persistent CTAs per SM; 0 = tuned default */
    int32_t views_per_group; /* multi-view: views sharing one point fetch; 0 = tuned default */
    int32_t lod_skip_level;  /* >0: skip batches whose precision level is >= this, the level-of-
                                detail cut of compute_loop_nodes/render.cs:273-276 (loop_nodes'
                                default: 4); 0 = render every visible batch, as the loop_las
                                methods do */
    int32_t reserved[4];
} cr_render_params;

typedef struct cr_ctx cr_ctx;
typedef struct cr_cloud cr_cloud;
typedef struct cr_fb cr_fb;

/* ---- library ------------------------------------------------------------- */
int32_t cr_abi_version(void);
const char* cr_status_string(cr_status s);
const char* cr_method_name(int32_t method);                 /* Method::name */
const char* cr_method_group(int32_t method);                /* Method::group */
const char* cr_method_description(int32_t method);          /* Method::description */
cr_status cr_method_find(const char* name, int32_t* method); /* Runtime.h:43-49 by name */
void cr_render_params_default(int32_t method, cr_render_params* out);

/* ---- context (one per device; not thread-safe per handle) ---------------- */
cr_status cr_ctx_create(int32_t device, cr_ctx** out);
cr_status cr_ctx_destroy(cr_ctx* ctx);
const char* cr_last_error(const cr_ctx* ctx);
/* Waits for `stream`, then reports a device-side error flag raised since the
 * last check (CR_ERR_DEVICE_FLAG) and clears it.  ctx = NULL checks the flag
 * of cr_render_batched_noalloc's fixed array in the current CUDA context. */
cr_status cr_ctx_check(cr_ctx* ctx, void* stream);
/* Self-check of the kernels' reciprocal (the correctly rounded 1/w that every
 * `xy / w` uses, render.cs:402): runs it against CUDA's __frcp_rn over all 2^32
 * float bit patterns on the context's device, the paired form of the 10-bit
 * raster over every float with |w| in [2^-126, 2^126), and the paired division
 * of CR_QUIRK_LITERAL_ARITH against __fdiv_rn on two quotients per float with
 * |w| in [2^-64, 2^64) (one of them next to a rounding midpoint where w's
 * significand is odd), and reports the mismatching patterns (NaN matches NaN)
 * and the lowest one (0xFFFFFFFF if none). */
cr_status cr_check_reciprocal(cr_ctx* ctx, uint64_t* mismatches, uint32_t* first_mismatch);
int32_t cr_ctx_num_sms(const cr_ctx* ctx);

/* ---- clouds: the LAS-derived layout (LasLoaderSparse.h:86-91) ------------ */
enum { CR_STREAM_LOW = 1, CR_STREAM_MED = 2, CR_STREAM_HIG = 4, CR_STREAM_RGBA = 8, CR_STREAM_ALL = 15 };

/* Allocates device storage for `num_points` points in `num_batches` records
 * across `num_files` files (per-file boxMin feeds the world matrix).
 * num_points < 2^31 - 64, num_batches < 2^28 and 1 <= num_files <=
 * CR_MAX_FILES (cr_cloud_wrap alike). */
cr_status cr_cloud_create(cr_ctx* ctx, int64_t num_points, int64_t num_batches, int32_t num_files,
                          int32_t stream_mask, cr_cloud** out);
/* Host -> device copies (pinned or pageable).  Any stream pointer may be NULL
 * to leave that stream untouched.  Records are validated on the host:
 * 0 <= num_points <= 10240, first_point + num_points <= N, file_index < files,
 * finite AABB. */
cr_status cr_cloud_upload(cr_ctx* ctx, cr_cloud* cloud, const cr_batch* batches,
                          const uint32_t* xyz_low, const uint32_t* xyz_med,
                          const uint32_t* xyz_hig, const uint32_t* rgba,
                          const double* file_box_min /* [3 * num_files] */, void* stream);
/* Device pointers of a cloud, for GPU-side writers (the GPU encoder). */
cr_status cr_cloud_device(const cr_cloud* cloud, cr_batch** batches, uint32_t** xyz_low,
                          uint32_t** xyz_med, uint32_t** xyz_hig, uint32_t** rgba);
cr_status cr_cloud_set_files(cr_ctx* ctx, cr_cloud* cloud, const double* file_box_min);
/* Device -> host copy of one array of the layout (CR_STREAM_LOW/MED/HIG/RGBA,
 * or 0 for the batch records), enqueued on `stream` (caller syncs). */
cr_status cr_cloud_read(cr_ctx* ctx, const cr_cloud* cloud, int32_t which, void* host_dst,
                        int64_t bytes, void* stream);
int64_t cr_cloud_num_points(const cr_cloud* cloud);
/* The loader's numPointsLoaded / numBatchesLoaded (LasLoaderSparse.h:77-91):
 * frames dispatch only the first `batches` records (or, for the methods that
 * dispatch by points, ceil(points / 10240) of them: compute_loop_las2.h:234),
 * so a cloud can be drawn while its load tasks are still arriving.  Records
 * past `batches` are not read.  points <= the cloud's points, batches <= its
 * records (a plain cloud ignores batches); both negative: everything, the
 * default. */
cr_status cr_cloud_set_loaded(cr_ctx* ctx, cr_cloud* cloud, int64_t points, int64_t batches);
int64_t cr_cloud_num_batches(const cr_cloud* cloud);
cr_status cr_cloud_destroy(cr_ctx* ctx, cr_cloud* cloud);

/* A cloud over caller-owned arrays of the layout above, for clouds kept in
 * host memory.  The reference's loader uploads every stream of every file into
 * GPU buffers (LasLoaderSparse.cpp:653-713); here, where kernels can read host
 * memory (pinned memory under unified addressing, or any memory where the
 * device reports pageable-memory access, as over NVLink-C2C on Grace), a
 * frame reads only the words its visible batches need across the link, and a
 * cloud is no longer bounded by device memory.  Each array may be device
 * memory or such host memory: the library checks that the GPU can address
 * every one (CR_ERR_INVALID_ARG if not) and never copies, writes or frees
 * them; the caller keeps them alive and unchanged while frames read them.
 * Streams hold stream_words >= num_points + 64 words, the words past
 * num_points zero.  xyz_med, xyz_hig and rgba may be NULL where no method
 * needs them.  cr_cloud_upload is refused for such a cloud; set each file's
 * boxMin with cr_cloud_set_files; cr_cloud_destroy releases only the handle. */
cr_status cr_cloud_wrap(cr_ctx* ctx, int64_t num_points, int64_t num_batches, int32_t num_files,
                        const cr_batch* batches, const uint32_t* xyz_low, const uint32_t* xyz_med,
                        const uint32_t* xyz_hig, const uint32_t* rgba, int64_t stream_words,
                        cr_cloud** out);

/* Plain 16 B/point clouds (LasLoaderStandard.h). */
cr_status cr_cloud_create_plain(cr_ctx* ctx, int64_t num_points, cr_cloud** out);
cr_status cr_cloud_upload_plain(cr_ctx* ctx, cr_cloud* cloud, const cr_vertex* vertices,
                                void* stream);
cr_status cr_cloud_device_plain(const cr_cloud* cloud, cr_vertex** vertices);

/* ---- framebuffers --------------------------------------------------------- */
enum { CR_FB_U64 = 0, CR_FB_HQS = 1 };
enum { CR_FB_WORDS = 0, CR_FB_DEPTH = 1, CR_FB_ACCUM = 2, CR_FB_IMAGE = 3 };

/* u64: W*H + W + 1 words + RGBA8 image (u32 per pixel).
 * HQS: u32 depth [W*H + W + 1], u64 accumulators [2 * (W*H + W + 1)], image. */
cr_status cr_fb_create(cr_ctx* ctx, int32_t width, int32_t height, int32_t kind, cr_fb** out);
cr_status cr_fb_destroy(cr_ctx* ctx, cr_fb* fb);
/* u64 kind: every word = value.  HQS: depth = low 32 bits of value, accum = 0. */
cr_status cr_fb_clear(cr_ctx* ctx, cr_fb* fb, uint64_t value, void* stream);
/* Size in bytes of one of the fb's buffers (CR_FB_WORDS/DEPTH/ACCUM/IMAGE). */
int64_t cr_fb_bytes(const cr_fb* fb, int32_t what);
/* Device -> host copy of one buffer, enqueued on `stream` (caller syncs). */
cr_status cr_fb_read(cr_ctx* ctx, const cr_fb* fb, int32_t what, void* host_dst, int64_t bytes,
                     void* stream);
cr_status cr_fb_device(const cr_fb* fb, int32_t what, void** device_ptr);

/* ---- rendering: Method::render (compute_loop_las.h:117-304 and siblings) --
 * Rasterizes `cloud` for `view` into `fb`; with params->resolve, resolves the
 * image; with params->clear_after, re-clears the fb for the next frame.  A new
 * fb must be cleared once with cr_fb_clear before its first frame. */
cr_status cr_render(cr_ctx* ctx, const cr_cloud* cloud, const cr_view* view,
                    const cr_render_params* params, cr_fb* fb, void* stream);

/* Resolve only (resolve.cs); `cloud` supplies the color stream for the index
 * payload and may be NULL otherwise. */
cr_status cr_resolve(cr_ctx* ctx, const cr_cloud* cloud, const cr_render_params* params,
                     cr_fb* fb, void* stream);

/* ---- many views of one cloud in one persistent launch ------------------------
 * The reference renders two eyes from one fetch of each point
 * (compute_loop_las_hqs_vr/depth.cs:374-412).  A multi-view plan generalises
 * that to any number of views of uneven size, in groups of up to
 * CR_MV_MAX_GROUP views: each work item is (batch, view group); a CTA fetches
 * the batch's points once and splats them into every view of the group whose
 * frustum the batch AABB intersects, each view at its own precision level, so
 * every view's framebuffer is bit-identical to a cr_render of that view alone.
 * The plan owns one framebuffer (u64 words + RGBA8 image) per view.  Its
 * frame (uniform upload, counter reset, cull, raster, resolve + re-clear) can
 * be captured once into a CUDA graph and replayed. */
#define CR_MV_MAX_GROUP 8
typedef struct cr_mv cr_mv;
/* params: method loop_las or loop_las_prefetch; payload, quirks, culling,
 * resolve, clear_after, clear_value as for cr_render; views_per_group 1..8
 * (0 = 8); block_threads 64/128/256 (0 = 128); ctas_per_sm (0 = occupancy). */
cr_status cr_mv_create(cr_ctx* ctx, const cr_cloud* cloud, int32_t num_views,
                       const int32_t* widths, const int32_t* heights,
                       const cr_render_params* params, cr_mv** out);
cr_status cr_mv_destroy(cr_mv* mv);
const char* cr_mv_last_error(const cr_mv* mv);
/* Replaces the launch parameters (drops a captured graph). */
cr_status cr_mv_set_params(cr_mv* mv, const cr_render_params* params);
cr_status cr_mv_get_params(const cr_mv* mv, cr_render_params* out);
/* Sets all num_views cameras (sizes must match the plan).  Waits for the
 * previous frame's uniform upload before overwriting the staging copy.
 * Adjacent views of a group whose proj * view rows y and w are bitwise equal
 * (the eyes of a stereo pair built as translate(-+ipd/2, 0, 0) * V_head, of
 * equal size) become a shared pair: each point's y, w, 1/w and pixel row are
 * computed once for both, x and the pixel column per eye -- the same
 * operations on the same operands, so the words do not change. */
cr_status cr_mv_set_views(cr_mv* mv, const cr_view* views);
/* Number of view pairs the current views and views_per_group share. */
cr_status cr_mv_shared_pairs(const cr_mv* mv, int32_t* pairs);
/* Enqueues one frame on `stream`.  use_graph = 1 captures the frame into a
 * CUDA graph on the first call and replays it afterwards (needs a stream
 * other than the legacy default stream). */
cr_status cr_mv_render(cr_mv* mv, int32_t use_graph, void* stream);
/* Every view's words = value (the start state of the first frame). */
cr_status cr_mv_clear(cr_mv* mv, uint64_t value, void* stream);
/* Device -> host copy of one view's CR_FB_WORDS or CR_FB_IMAGE (caller syncs). */
cr_status cr_mv_read(cr_mv* mv, int32_t view, int32_t what, void* host_dst, int64_t bytes,
                     void* stream);
/* Autotuner: times `frames` frames of every block size {64, 128, 256} x views
 * per group {1, 2, 4, 8} (points per thread 160, 80, 40) for the current
 * views, keeps the fastest in the plan, returns it in *best and a JSON report
 * of every configuration's milliseconds in `report` (may be NULL). */
cr_status cr_mv_autotune(cr_mv* mv, int32_t frames, void* stream, cr_render_params* best,
                         char* report, int32_t report_bytes);

/* ---- rasterizing without allocating ------------------------------------------
 * No counterpart in the reference (its Methods own GL buffers created at
 * start-up).  For callers that must not allocate device memory while they
 * render: a host engine that owns the GPU memory budget and hands the renderer
 * only buffers it already placed, or a plugin running inside someone else's
 * frame loop, where a cudaMalloc or cudaFree would synchronise the device or
 * disturb the host application's own work.  Same cull + raster as cr_render
 * for the batched methods (loop_las, loop_las_prefetch; no resolve, no HQS)
 * on caller-owned device buffers.  Its work list and, for clouds with more
 * than 8 files, the per-file records live in one fixed device array inside
 * the library (CR_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the
 * library until the process exits), sized for at most CR_NOALLOC_MAX_BATCHES
 * batch records and CR_NOALLOC_MAX_FILES files.  It allocates nothing: no
 * cudaMalloc, cudaFree or allocating library call.
 *   - `fb` holds width*height + width + 1 words, already cleared by the caller.
 *   - streams hold `stream_words` words each, with at least 64 zeroed words
 *     past the last point (the padding cr_cloud_create adds).
 *   - `file_box_min` is a host array of 3 * num_files doubles.
 *   - params->resolve and params->clear_after must be 0.
 *   - The first call in each CUDA context (the device's primary context, or
 *     one the caller made with cuCtxCreate and made current) looks up the
 *     array's device address in that context; make that first call before any
 *     stream capture.
 *   - Every call shares the one array, which keeps the previous call's
 *     contents (each call resets what must start at zero), so calls whose work
 *     overlaps on the GPU (other streams, other threads) race; serialise them
 *     on one stream.
 *   - A batch record out of range (num_points, first_point + num_points past
 *     stream_words, file_index >= num_files) is skipped without a fault and
 *     sets the array's error flag, which cr_ctx_check(NULL, stream) reports
 *     (CR_ERR_DEVICE_FLAG) and clears.
 * Returns CR_ERR_INVALID_ARG past the size limits or for bad arguments. */
#define CR_NOALLOC_MAX_BATCHES 131064
#define CR_NOALLOC_MAX_FILES 1024
#define CR_NOALLOC_SCRATCH_BYTES 753664 /* (8 + 131064) * 4 + 1024 * 224 */
cr_status cr_render_batched_noalloc(const cr_batch* d_batches, int64_t num_batches,
                                    int64_t num_points, const uint32_t* d_xyz_low,
                                    const uint32_t* d_xyz_med, const uint32_t* d_xyz_hig,
                                    const uint32_t* d_rgba, int64_t stream_words,
                                    const double* file_box_min, int32_t num_files,
                                    const cr_view* view, const cr_render_params* params,
                                    uint64_t* d_fb, void* stream);
/* The fixed array's device address in the calling thread's current CUDA
 * context (looked up there on first use, as by the render call) and its size
 * in bytes, for callers that account for device memory. */
cr_status cr_noalloc_scratch(void** device_address, int64_t* bytes);

/* ---- timer queries and frame counters --------------------------------------
 * GLTimerQueries::timestamp pairs (src/GLTimerQueries.cpp:6-22) around the
 * dispatches become CUDA events: while timing is on, every cr_render records
 * an event at each stage boundary.  Stages: 0 cull, 1 raster (HQS: depth),
 * 2 HQS color, 3 resolve. */
enum { CR_STAGE_CULL = 0, CR_STAGE_RASTER = 1, CR_STAGE_HQS_COLOR = 2, CR_STAGE_RESOLVE = 3,
       CR_NUM_STAGES = 4 };
cr_status cr_timing_enable(cr_ctx* ctx, int32_t max_frames); /* 0 disables; resets */
/* Synchronizes, then writes up to `max` per-frame milliseconds of `stage`
 * (frames that did not run the stage report 0) and returns the frame count. */
int32_t cr_timing_read(cr_ctx* ctx, int32_t stage, float* ms, int32_t max);

/* Debug counters of the last cull (compute_loop_las.h:54-62 DebugData):
 * visible batches and points per precision level and the bytes the raster
 * reads for them.  Synchronizes. */
typedef struct cr_frame_stats {
    int64_t batches_dispatched;
    int64_t batches_visible;
    int64_t batches_per_level[5];
    int64_t points_per_level[5];
    int64_t stream_bytes;      /* coordinate words + color words (if read) + 64 B records */
} cr_frame_stats;
cr_status cr_last_frame_stats(cr_ctx* ctx, const cr_cloud* cloud, const cr_render_params* params,
                              cr_frame_stats* out);

/* ---- host-side layout builders (LasLoaderSparse.cpp:37-212) --------------- */
int64_t cr_num_batches(int64_t num_points);
/* Encodes `n` LAS point records (raw bytes, `bytes_per_point` stride) of one
 * load task into batch records and the four streams.  `sparse_offset` is the
 * global index of the first record (LasFile::sparse_point_offset + firstPoint). */
cr_status cr_encode_las(const uint8_t* records, int64_t n, int32_t bytes_per_point,
                        int32_t point_format, const double scale[3], const double offset[3],
                        const double box_min[3], int64_t sparse_offset, int32_t file_index,
                        cr_batch* batches, uint32_t* xyz_low, uint32_t* xyz_med,
                        uint32_t* xyz_hig, uint32_t* rgba);
/* LasLoaderStandard.h:152-179: LAS records -> 16 B vertices. */
cr_status cr_encode_standard(const uint8_t* records, int64_t n, int32_t bytes_per_point,
                             int32_t point_format, const double scale[3], const double offset[3],
                             const double box_min[3], cr_vertex* out);

/* ---- host matrix setup (Camera.h:34-39, OrbitControls.h:116-135) ----------- */
void cr_perspective(double fovy_deg, double aspect, double znear, double zfar, double out[16]);
void cr_look_at(const double eye[3], const double center[3], const double up[3], double out[16]);
void cr_orbit_view(double yaw, double pitch, double radius, const double target[3],
                   double out_view[16]);

#ifdef __cplusplus
}
#endif
#endif
