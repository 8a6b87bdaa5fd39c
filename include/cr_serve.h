/*
 * cr_serve.h -- C ABI of the frame server: many clients' views of resident
 * clouds rendered by one GPU.
 *
 * The reference renders one camera per frame from its main loop: every frame
 * it calls the selected Method's update() and render() (main.cpp:342, :455)
 * for Renderer::views[0] (Renderer.h:78-82), over the clouds the loader keeps
 * on the GPU (LasLoaderSparse.h:23-44).  The server keeps that per-view
 * arithmetic -- each served image equals cr_render + cr_resolve of the same
 * view alone, bit for bit -- and schedules many requests at once:
 *
 *   resident clouds   cr_cloud handles registered once (cr_server_add_cloud)
 *   admission         every request needs (W*H+W+1)*8 B of framebuffer plus
 *                     W*H*4 B of image from one device pool (default 8 GiB);
 *                     cr_server_submit refuses a request that can never fit or
 *                     that finds the queue full (CR_ERR_ADMISSION_REJECTED);
 *                     queued requests wait for pool memory in arrival order
 *   continuous        a dispatcher thread launches whatever is queued for the
 *   batching          oldest request's cloud, up to max_batch_views views, as
 *                     one multi-view frame (one cull, one persistent raster,
 *                     one resolve) as soon as one of max_inflight launch slots
 *                     (each its own CUDA stream) is free; requests that arrive
 *                     during a launch join the next one
 *   plain arm         plain_launches = 1 renders every request by itself with
 *                     the single-view kernels (one cr_render per request), the
 *                     baseline the batched arm is measured against
 *
 * Threads: submit, poll, replay and stats may be called from any thread;
 * destroy must not race with them.  Times are microseconds on the server's
 * steady clock (cr_server_now_us).
 */
#ifndef CR_SERVE_H
#define CR_SERVE_H

#include "cr_raster.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CR_SERVE_MAX_POOL_BYTES (16LL << 30) /* u32 image offsets into the pool */
#define CR_SERVE_MAX_BATCH_VIEWS 256

typedef struct cr_server cr_server;

typedef struct cr_server_config {
    int64_t pool_bytes;       /* framebuffer + image pool; 0 = 8 GiB; <= CR_SERVE_MAX_POOL_BYTES */
    int32_t max_batch_views;  /* views per multi-view launch; 0 = 16 */
    int32_t max_inflight;     /* launch slots (streams) in flight; 0 = 4 */
    int32_t max_queued;       /* queued requests before submit refuses; 0 = 65536 */
    int32_t plain_launches;   /* 1: one single-view render per request */
    int32_t method;           /* CR_METHOD_LOOP_LAS or CR_METHOD_LOOP_LAS_PREFETCH */
    int32_t payload;          /* cr_payload */
    int32_t quirks;           /* cr_quirk mask, or CR_QUIRKS_METHOD_DEFAULT */
    int32_t frustum_culling;  /* 1 = on */
    int32_t views_per_group;  /* multi-view group size; 0 = 8 */
    int32_t block_threads;    /* 0 = tuned default */
    int32_t reserved[6];
} cr_server_config;

typedef struct cr_request {
    int32_t cloud;            /* id from cr_server_add_cloud */
    int32_t reserved0;
    cr_view view;
    uint32_t* host_image;     /* W*H RGBA8 words written before completion, or NULL */
    uint64_t user_tag;        /* returned in the completion */
} cr_request;

typedef struct cr_completion {
    uint64_t ticket;
    uint64_t user_tag;
    int32_t status;           /* CR_OK, CR_ERR_ADMISSION_REJECTED, CR_ERR_CUDA, ... */
    int32_t batch_views;      /* views that shared the request's launch */
    double t_arrival_us;      /* when the request arrived (submit, or its replay time) */
    double t_launch_us;       /* when its launch was enqueued */
    double t_done_us;         /* when the server saw the launch (and copy) finish */
} cr_completion;

typedef struct cr_server_stats {
    int64_t submitted, rejected, completed, failed;
    int64_t launches, views_launched;
    int64_t pool_bytes, pool_used_bytes, pool_peak_bytes;
    int32_t max_views_in_launch, queued;
    double gpu_ms;            /* summed CUDA-event time of all launches (overlap counted twice) */
} cr_server_stats;

/* Starts the dispatcher thread on ctx's device. */
cr_status cr_server_create(cr_ctx* ctx, const cr_server_config* cfg, cr_server** out);
/* Finishes every accepted request, stops the thread, frees the pool. */
cr_status cr_server_destroy(cr_server* s);
const char* cr_server_last_error(const cr_server* s);
double cr_server_now_us(const cr_server* s);

/* Registers a LAS-derived cloud (it must outlive the server). */
cr_status cr_server_add_cloud(cr_server* s, const cr_cloud* cloud, int32_t* id);

/* Queues one request.  CR_ERR_ADMISSION_REJECTED: its buffers exceed the pool
 * or the queue is full; CR_ERR_INVALID_ARG: bad cloud id or view. */
cr_status cr_server_submit(cr_server* s, const cr_request* r, uint64_t* ticket);

/* Pops up to `max` completions, waiting up to wait_ms for the first one. */
cr_status cr_server_poll(cr_server* s, cr_completion* out, int32_t max, int32_t* n,
                         int32_t wait_ms);

/* Waits until every accepted request has completed (CR_ERR_TIMEOUT after
 * timeout_ms; <0 = no limit).  Completions stay queued for cr_server_poll. */
cr_status cr_server_drain(cr_server* s, int32_t timeout_ms);

/* Open-loop replay: submits reqs[i] at arrival_us[i] after the call starts,
 * from the calling thread, then waits for all of them.  out[i] receives
 * request i's completion (status CR_ERR_ADMISSION_REJECTED if refused).  The
 * server must have no other requests outstanding. */
cr_status cr_server_replay(cr_server* s, const cr_request* reqs, const double* arrival_us,
                           int64_t n, cr_completion* out);

cr_status cr_server_stats_get(const cr_server* s, cr_server_stats* out);

/* Host-side fault injection for tests: the next `count` launches fail as if
 * their device allocation had failed (CR_INJECT_LAUNCH_ALLOC), before any
 * device work; their requests complete with CR_ERR_OUT_OF_MEMORY and the loop
 * carries on with the next launch.  Nothing faults on the device. */
enum { CR_INJECT_NONE = 0, CR_INJECT_LAUNCH_ALLOC = 1 };
cr_status cr_server_inject(cr_server* s, int32_t what, int32_t count);

#ifdef __cplusplus
}
#endif

#endif /* CR_SERVE_H */
