// cr_serve.cpp -- the frame server of include/cr_serve.h.
//
// One dispatcher thread per server owns the GPU side: it moves submitted
// requests into its queue, reaps finished launch slots (cudaEventQuery on the
// slot's last event), and starts new launches while a slot is free.  A launch
// takes the oldest queued request's cloud and every queued request for that
// cloud, in arrival order, up to max_batch_views, as long as each one's
// framebuffer + image chunk fits in the pool; the first that does not fit
// ends the batch (arrival order is kept, so a large request is not starved).
// The chunks return to the pool when the launch's event completes.
//
// Per request the device work is the reference frame (compute_loop_las.h:
// 288-301 clear, render.cs cull + raster, resolve.cs), so every image equals
// cr_render + cr_resolve of the same view alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/cr_serve.h"
#include "cr_internal.h"

namespace {

using cr::CloudInfo;
using cr::MVFile;
using cr::MVView;

constexpr int64_t kGranule = 256;

int64_t round_up(int64_t n) { return (n + kGranule - 1) / kGranule * kGranule; }

// First-fit allocator over [0, size) with coalescing on release.
class PoolAlloc {
  public:
    void init(int64_t size) {
        free_.clear();
        free_[0] = size;
        size_ = size;
        used_ = peak_ = 0;
    }
    bool alloc(int64_t n, int64_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const int64_t o = it->first, rest = it->second - n;
            free_.erase(it);
            if (rest > 0) free_[o + n] = rest;
            *off = o;
            used_ += n;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(int64_t off, int64_t n) {
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    int64_t size() const { return size_; }
    int64_t used() const { return used_; }
    int64_t peak() const { return peak_; }

  private:
    std::map<int64_t, int64_t> free_;
    int64_t size_ = 0, used_ = 0, peak_ = 0;
};

struct Pending {
    uint64_t ticket = 0;
    cr_request r{};
    int64_t fb_bytes = 0, bytes = 0;  // chunk: [fb words, rounded][image]
    double t_arrival = 0.0;
    MVView view{};
    MVFile files[cr::kInlineFiles];  // clouds of at most kInlineFiles files; with
                                     // more, the GPU computes them from r.view
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t* scratch = nullptr;
    int64_t scratch_words = 0;
    MVView* d_views = nullptr;
    MVFile* d_files = nullptr;
    MVView* h_views = nullptr;  // pinned
    MVFile* h_files = nullptr;  // pinned
    uint32_t* h_err = nullptr;  // pinned copy of the device error word
    // clouds with more than kInlineFiles files: view + proj per request
    // (pinned and device), every file's boxMin (pinned and device), the
    // multi-view records (d_files, files_cap per view) and the single-view
    // records (d_frec), grown to the largest file count launched
    double* h_mats = nullptr;
    double* d_mats = nullptr;
    double* h_box = nullptr;
    double* d_box = nullptr;
    cr::FileRec* d_frec = nullptr;
    int32_t files_cap = cr::kInlineFiles;  // files per view d_files / h_files hold
    int32_t many_cap = 0;                  // files h_box, d_box and d_frec hold
    bool busy = false;
    std::vector<Pending> reqs;
    std::vector<int64_t> offs;
    double t_launch = 0.0;
};

}  // namespace

struct cr_server {
    cr_ctx* ctx = nullptr;
    int device = 0, num_sms = 0;
    cr_server_config cfg{};
    int quirks = 0;
    std::chrono::steady_clock::time_point t0;

    std::mutex cloud_mu;
    std::vector<CloudInfo> clouds;        // as registered (layout, files)
    std::vector<const cr_cloud*> handles;  // re-read per launch: loaded counts may grow

    uint64_t* pool = nullptr;
    PoolAlloc alloc;  // dispatcher thread only
    std::vector<Slot> slots;

    std::mutex in_mu;
    std::condition_variable in_cv;
    std::deque<Pending> incoming;
    bool stop = false;  // under in_mu

    std::mutex done_mu;
    std::condition_variable done_cv;
    std::deque<cr_completion> done;
    int64_t outstanding = 0;  // accepted, not yet completed (under done_mu)

    std::atomic<int32_t> queued{0};
    std::atomic<uint64_t> next_ticket{1};
    std::atomic<int32_t> inject_alloc_failures{0};  // cr_server_inject

    mutable std::mutex stats_mu;
    cr_server_stats stats{};

    mutable std::mutex err_mu;
    mutable std::string err;

    std::thread th;
};

namespace {

double now_us(const cr_server* s) {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - s->t0).count();
}

cr_status set_err(const cr_server* s, cr_status st, const std::string& msg) {
    std::lock_guard<std::mutex> lk(s->err_mu);
    s->err = msg;
    return st;
}

int64_t dispatched_batches(const CloudInfo& ci, int quirks) {
    int64_t nb = ci.nb;
    if (quirks & CR_QUIRK_DISPATCH_BY_POINTS)
        nb = std::min<int64_t>(nb, (ci.n + cr::kPointsPerBatch - 1) / cr::kPointsPerBatch);
    return nb;
}

void complete(cr_server* s, const std::vector<Pending>& reqs, int32_t status, int32_t views,
              double t_launch, double t_done) {
    std::lock_guard<std::mutex> lk(s->done_mu);
    for (const Pending& p : reqs) {
        cr_completion c{};
        c.ticket = p.ticket;
        c.user_tag = p.r.user_tag;
        c.status = status;
        c.batch_views = views;
        c.t_arrival_us = p.t_arrival;
        c.t_launch_us = t_launch;
        c.t_done_us = t_done;
        s->done.push_back(c);
        s->outstanding--;
    }
    s->done_cv.notify_all();
}

// Reaps a slot whose last event completed (or failed).
void finish(cr_server* s, Slot& sl, cudaError_t e) {
    const double t = now_us(s);
    float ms = 0.0f;
    int32_t status = CR_OK;
    if (e != cudaSuccess) {
        status = CR_ERR_CUDA;
        set_err(s, CR_ERR_CUDA, std::string("launch failed: ") + cudaGetErrorString(e));
    } else {
        cudaEventElapsedTime(&ms, sl.ev0, sl.ev1);
        if (*sl.h_err != 0) status = CR_ERR_DEVICE_FLAG;
    }
    for (size_t i = 0; i < sl.reqs.size(); i++) s->alloc.release(sl.offs[i], sl.reqs[i].bytes);
    {
        std::lock_guard<std::mutex> lk(s->stats_mu);
        s->stats.completed += status == CR_OK ? (int64_t)sl.reqs.size() : 0;
        s->stats.failed += status == CR_OK ? 0 : (int64_t)sl.reqs.size();
        s->stats.gpu_ms += ms;
        s->stats.pool_used_bytes = s->alloc.used();
    }
    complete(s, sl.reqs, status, (int32_t)sl.reqs.size(), sl.t_launch, t);
    sl.reqs.clear();
    sl.offs.clear();
    sl.busy = false;
}

cudaError_t ensure_slot_scratch(Slot& sl, int64_t words) {
    if (sl.scratch_words >= words) return cudaSuccess;
    if (sl.scratch) cudaFree(sl.scratch);
    sl.scratch = nullptr;
    sl.scratch_words = 0;
    // no clearing: each launch zeroes the counters on the slot's stream, and
    // the cull writes every list item before the raster reads it
    const cudaError_t e = cudaMalloc(&sl.scratch, words * 4);
    if (e == cudaSuccess) sl.scratch_words = words;
    return e;
}

// Grows a free slot's per-file buffers to `nfiles` files (its stream is idle).
cudaError_t ensure_slot_files(Slot& sl, int32_t nfiles, int maxv) {
    cudaError_t e = cudaSuccess;
    if (nfiles > sl.files_cap) {
        if (sl.d_files) cudaFree(sl.d_files);
        sl.d_files = nullptr;
        e = cudaMalloc(&sl.d_files, sizeof(MVFile) * (size_t)maxv * nfiles);
        if (e != cudaSuccess) return e;
        sl.files_cap = nfiles;
    }
    if (nfiles > cr::kInlineFiles && nfiles > sl.many_cap) {
        if (sl.h_box) cudaFreeHost(sl.h_box);
        if (sl.d_box) cudaFree(sl.d_box);
        if (sl.d_frec) cudaFree(sl.d_frec);
        sl.h_box = nullptr;
        sl.d_box = nullptr;
        sl.d_frec = nullptr;
        sl.many_cap = 0;
        e = cudaHostAlloc(&sl.h_box, sizeof(double) * 3 * (size_t)nfiles, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_box, sizeof(double) * 3 * (size_t)nfiles);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_frec, sizeof(cr::FileRec) * (size_t)nfiles);
        if (e != cudaSuccess) return e;
        sl.many_cap = nfiles;
    }
    return cudaSuccess;
}

// Enqueues the frame of the requests in sl.reqs (chunks at sl.offs).
cr_status enqueue(cr_server* s, Slot& sl, const CloudInfo& ci, const char** what) {
    const cr_server_config& c = s->cfg;
    const int n = (int)sl.reqs.size();
    uint32_t* images = reinterpret_cast<uint32_t*>(s->pool);
    const int64_t nb = dispatched_batches(ci, s->quirks);
    // a launch of one request uses the single-view kernels: same image, and
    // faster than the multi-view raster at one view per group
    const bool single = c.plain_launches || n == 1;
    int32_t injected = s->inject_alloc_failures.load();
    while (injected > 0 && !s->inject_alloc_failures.compare_exchange_weak(injected, injected - 1)) {
    }
    cudaError_t e = injected > 0 ? cudaErrorMemoryAllocation
                                 : ensure_slot_scratch(sl, cr::mv_scratch_words(nb, single ? 1 : n));
    if (e == cudaSuccess)
        e = ensure_slot_files(sl, ci.nfiles, c.plain_launches ? 1 : c.max_batch_views);
    if (e != cudaSuccess) {
        *what = "scratch allocation";
        return CR_ERR_OUT_OF_MEMORY;
    }
    cudaEventRecord(sl.ev0, sl.st);
    // sticky error word and counters start at zero for this launch
    if (cudaMemsetAsync(sl.scratch, 0, cr::kScratchHead * 4, sl.st) != cudaSuccess) {
        *what = "scratch reset";
        return CR_ERR_CUDA;
    }
    if (single) {
        // one reference frame per request: clear, cull, raster, resolve
        for (int i = 0; i < n; i++) {
            const Pending& p = sl.reqs[i];
            const int32_t W = p.r.view.width, H = p.r.view.height;
            uint64_t* fb = s->pool + sl.offs[i] / 8;
            uint32_t* img = images + (sl.offs[i] + p.fb_bytes) / 4;
            cr::ViewParams vp;
            if (cr::view_params_for(&p.r.view, ci.box_min, ci.nfiles, c.frustum_culling, &vp) != CR_OK) {
                *what = "view matrices";
                return CR_ERR_INVALID_ARG;
            }
            if (ci.nfiles > cr::kInlineFiles) {
                if (cr::launch_file_records(p.r.view.view, p.r.view.proj, ci.box_min, ci.nfiles,
                                            sl.d_frec, sl.st) != 0) {
                    *what = "file record launch";
                    return CR_ERR_CUDA;
                }
                vp.dfiles = sl.d_frec;
            }
            if (cr::launch_fill_u64(fb, (int64_t)W * H + W + 1, cr::kDefaultClear, sl.st) != 0 ||
                cudaMemsetAsync(sl.scratch, 0, cr::kCounterWords * 4, sl.st) != cudaSuccess ||
                cr::launch_cull(vp, ci.batches, nb, ci.capacity, s->quirks, sl.scratch, sl.st) != 0) {
                *what = "plain frame setup";
                return CR_ERR_CUDA;
            }
            cr::BatchedLaunch bl{};
            bl.batches = ci.batches;
            bl.lo = ci.lo;
            bl.md = ci.md;
            bl.hi = ci.hi;
            bl.rgba = ci.rgba;
            bl.capacity = ci.capacity;
            bl.fb = fb;
            bl.scratch = sl.scratch;
            bl.list_cap = nb;
            bl.quirks = s->quirks;
            bl.payload = c.payload;
            bl.mode = cr::kModeRaster;
            const int block = c.plain_launches && c.block_threads > 0 ? c.block_threads : 128;
            const int per_sm = std::max(
                1, cr::batched_blocks_per_sm(bl.mode, bl.payload, block, ci.nfiles > cr::kInlineFiles));
            if (cr::launch_batched(vp, bl, block, s->num_sms * per_sm, sl.st) != 0) {
                *what = "plain raster launch";
                return CR_ERR_CUDA;
            }
            const int r = c.payload == CR_PAYLOAD_COLOR
                              ? cr::launch_resolve_color(W, H, fb, img, 0, cr::kDefaultClear, sl.st)
                              : cr::launch_resolve_index(W, H, fb, ci.rgba, ci.capacity, img, 0,
                                                         cr::kDefaultClear, sl.st);
            if (r != 0) {
                *what = "plain resolve launch";
                return CR_ERR_CUDA;
            }
        }
    } else {
        const bool many = ci.nfiles > cr::kInlineFiles;
        int64_t max_words = 1;
        for (int i = 0; i < n; i++) {
            const Pending& p = sl.reqs[i];
            sl.h_views[i] = p.view;
            sl.h_views[i].fb_off = (uint32_t)(sl.offs[i] / 8);
            sl.h_views[i].img_off = (uint32_t)((sl.offs[i] + p.fb_bytes) / 4);
            if (many) {
                std::memcpy(&sl.h_mats[32 * (int64_t)i], p.r.view.view, sizeof(double) * 16);
                std::memcpy(&sl.h_mats[32 * (int64_t)i + 16], p.r.view.proj, sizeof(double) * 16);
            } else {
                std::memcpy(&sl.h_files[(int64_t)i * ci.nfiles], p.files, sizeof(MVFile) * ci.nfiles);
            }
            const int64_t W = p.r.view.width, H = p.r.view.height;
            max_words = std::max(max_words, W * H + W + 1);
        }
        e = cudaMemcpyAsync(sl.d_views, sl.h_views, sizeof(MVView) * n, cudaMemcpyHostToDevice, sl.st);
        if (e == cudaSuccess && !many)
            e = cudaMemcpyAsync(sl.d_files, sl.h_files, sizeof(MVFile) * (size_t)n * ci.nfiles,
                                cudaMemcpyHostToDevice, sl.st);
        if (e == cudaSuccess && many) {
            std::memcpy(sl.h_box, ci.box_min, sizeof(double) * 3 * (size_t)ci.nfiles);
            e = cudaMemcpyAsync(sl.d_mats, sl.h_mats, sizeof(double) * 32 * (size_t)n,
                                cudaMemcpyHostToDevice, sl.st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(sl.d_box, sl.h_box, sizeof(double) * 3 * (size_t)ci.nfiles,
                                    cudaMemcpyHostToDevice, sl.st);
        }
        if (e != cudaSuccess) {
            *what = "view upload";
            return CR_ERR_CUDA;
        }
        cr::MVFrame f{};
        f.ci = ci;
        f.d_views = sl.d_views;
        f.d_files = sl.d_files;
        f.nviews = n;
        f.fbs = s->pool;
        f.images = images;
        f.scratch = sl.scratch;
        f.G = c.views_per_group;
        f.block = c.block_threads > 0 ? c.block_threads : 128;
        f.ctas_per_sm = 0;
        f.quirks = s->quirks;
        f.payload = c.payload;
        f.culling = c.frustum_culling;
        f.num_sms = s->num_sms;
        f.clear_before = 1;
        f.clear_value = cr::kDefaultClear;
        f.resolve = 1;
        f.clear_after = 0;
        f.max_words = max_words;
        f.d_mats = sl.d_mats;
        f.d_box = sl.d_box;
        const cr_status st = cr::mv_enqueue(f, sl.st, what);
        if (st != CR_OK) return st;
    }
    for (int i = 0; i < n; i++) {
        const Pending& p = sl.reqs[i];
        if (!p.r.host_image) continue;
        const size_t bytes = (size_t)p.r.view.width * p.r.view.height * 4;
        if (cudaMemcpyAsync(p.r.host_image, images + (sl.offs[i] + p.fb_bytes) / 4, bytes,
                            cudaMemcpyDeviceToHost, sl.st) != cudaSuccess) {
            *what = "image readback";
            return CR_ERR_CUDA;
        }
    }
    if (cudaMemcpyAsync(sl.h_err, sl.scratch + cr::kErrWord, 4, cudaMemcpyDeviceToHost, sl.st) !=
            cudaSuccess ||
        cudaEventRecord(sl.ev1, sl.st) != cudaSuccess) {
        *what = "completion record";
        return CR_ERR_CUDA;
    }
    return CR_OK;
}

// Starts one launch from the queue on a free slot; false if nothing could start.
bool launch(cr_server* s, Slot& sl, std::deque<Pending>& queue) {
    const int cloud = queue.front().r.cloud;
    const int maxv = s->cfg.plain_launches ? 1 : s->cfg.max_batch_views;
    std::deque<Pending> rest;
    while (!queue.empty()) {
        Pending p = std::move(queue.front());
        queue.pop_front();
        int64_t off = 0;
        if ((int)sl.reqs.size() < maxv && p.r.cloud == cloud && s->alloc.alloc(p.bytes, &off)) {
            sl.reqs.push_back(std::move(p));
            sl.offs.push_back(off);
            continue;
        }
        const bool blocked = p.r.cloud == cloud && (int)sl.reqs.size() < maxv;
        rest.push_back(std::move(p));
        if (blocked) break;  // keeps arrival order for this cloud: the rest waits
    }
    while (!queue.empty()) {
        rest.push_back(std::move(queue.front()));
        queue.pop_front();
    }
    queue.swap(rest);
    if (sl.reqs.empty()) return false;
    s->queued -= (int32_t)sl.reqs.size();

    CloudInfo ci;
    {
        std::lock_guard<std::mutex> lk(s->cloud_mu);
        ci = s->clouds[cloud];
        cr::cloud_info(s->handles[cloud], &ci);
    }
    const char* what = "";
    sl.t_launch = now_us(s);
    const cr_status st = [&] {
        const cr::NvtxRange range("cr_server launch");
        return enqueue(s, sl, ci, &what);
    }();
    if (st != CR_OK) {
        // nothing of this batch is waited for: drain the stream, fail its requests
        set_err(s, st, std::string("launch: ") + what);
        cudaStreamSynchronize(sl.st);
        for (size_t i = 0; i < sl.reqs.size(); i++) s->alloc.release(sl.offs[i], sl.reqs[i].bytes);
        {
            std::lock_guard<std::mutex> lk(s->stats_mu);
            s->stats.failed += (int64_t)sl.reqs.size();
        }
        complete(s, sl.reqs, st, (int32_t)sl.reqs.size(), sl.t_launch, now_us(s));
        sl.reqs.clear();
        sl.offs.clear();
        return true;
    }
    sl.busy = true;
    std::lock_guard<std::mutex> lk(s->stats_mu);
    s->stats.launches++;
    s->stats.views_launched += (int64_t)sl.reqs.size();
    s->stats.max_views_in_launch = std::max<int32_t>(s->stats.max_views_in_launch, (int32_t)sl.reqs.size());
    s->stats.pool_used_bytes = s->alloc.used();
    s->stats.pool_peak_bytes = s->alloc.peak();
    return true;
}

void dispatcher(cr_server* s) {
    cudaSetDevice(s->device);
    std::deque<Pending> queue;
    while (true) {
        bool stop = false, progressed = false;
        {
            std::lock_guard<std::mutex> lk(s->in_mu);
            while (!s->incoming.empty()) {
                queue.push_back(std::move(s->incoming.front()));
                s->incoming.pop_front();
            }
            stop = s->stop;
        }
        bool busy = false;
        for (Slot& sl : s->slots) {
            if (!sl.busy) continue;
            const cudaError_t e = cudaEventQuery(sl.ev1);
            if (e == cudaErrorNotReady) {
                busy = true;
                continue;
            }
            if (e != cudaSuccess) cudaGetLastError();
            finish(s, sl, e);
            progressed = true;
        }
        for (Slot& sl : s->slots) {
            if (queue.empty()) break;
            if (sl.busy) continue;
            if (!launch(s, sl, queue)) break;
            progressed = true;
            busy = busy || sl.busy;
        }
        if (stop && queue.empty() && !busy) {
            std::lock_guard<std::mutex> lk(s->in_mu);
            if (s->incoming.empty()) break;
            continue;
        }
        if (progressed) continue;
        if (busy) {
            std::this_thread::yield();  // a launch is in flight: poll its event
        } else {
            std::unique_lock<std::mutex> lk(s->in_mu);
            s->in_cv.wait_for(lk, std::chrono::milliseconds(5),
                              [&] { return !s->incoming.empty() || s->stop; });
        }
    }
}

void free_server(cr_server* s) {
    for (Slot& sl : s->slots) {
        if (sl.st) cudaStreamSynchronize(sl.st);
        if (sl.scratch) cudaFree(sl.scratch);
        if (sl.d_views) cudaFree(sl.d_views);
        if (sl.d_files) cudaFree(sl.d_files);
        if (sl.h_views) cudaFreeHost(sl.h_views);
        if (sl.h_files) cudaFreeHost(sl.h_files);
        if (sl.h_err) cudaFreeHost(sl.h_err);
        if (sl.h_mats) cudaFreeHost(sl.h_mats);
        if (sl.d_mats) cudaFree(sl.d_mats);
        if (sl.h_box) cudaFreeHost(sl.h_box);
        if (sl.d_box) cudaFree(sl.d_box);
        if (sl.d_frec) cudaFree(sl.d_frec);
        if (sl.ev0) cudaEventDestroy(sl.ev0);
        if (sl.ev1) cudaEventDestroy(sl.ev1);
        if (sl.st) cudaStreamDestroy(sl.st);
    }
    if (s->pool) cudaFree(s->pool);
    delete s;
}

}  // namespace

extern "C" {

cr_status cr_server_create(cr_ctx* ctx, const cr_server_config* cfg, cr_server** out) {
    if (!ctx || !cfg || !out) return CR_ERR_INVALID_ARG;
    *out = nullptr;
    cr_server_config c = *cfg;
    if (c.pool_bytes == 0) c.pool_bytes = 8LL << 30;
    // measured on the serving workload: 16-view launches, 4 in flight
    if (c.max_batch_views == 0) c.max_batch_views = 16;
    if (c.max_inflight == 0) c.max_inflight = 4;
    if (c.max_queued == 0) c.max_queued = 65536;
    if (c.views_per_group == 0) c.views_per_group = CR_MV_MAX_GROUP;
    if (c.pool_bytes < kGranule || c.pool_bytes > CR_SERVE_MAX_POOL_BYTES) return CR_ERR_INVALID_ARG;
    if (c.max_batch_views < 1 || c.max_batch_views > CR_SERVE_MAX_BATCH_VIEWS) return CR_ERR_INVALID_ARG;
    if (c.max_inflight < 1 || c.max_inflight > 16 || c.max_queued < 1) return CR_ERR_INVALID_ARG;
    if (c.views_per_group < 1 || c.views_per_group > CR_MV_MAX_GROUP) return CR_ERR_INVALID_ARG;
    if (c.block_threads != 0 && c.block_threads != 64 && c.block_threads != 128 &&
        c.block_threads != 256)
        return CR_ERR_INVALID_ARG;
    if (c.plain_launches && c.block_threads == 64) return CR_ERR_INVALID_ARG;
    if (c.method != CR_METHOD_LOOP_LAS && c.method != CR_METHOD_LOOP_LAS_PREFETCH)
        return CR_ERR_INVALID_ARG;
    if (c.payload != CR_PAYLOAD_COLOR && c.payload != CR_PAYLOAD_INDEX) return CR_ERR_INVALID_ARG;
    c.pool_bytes = c.pool_bytes / kGranule * kGranule;

    const int quirks = c.quirks == CR_QUIRKS_METHOD_DEFAULT ? cr::default_quirks_for(c.method) : c.quirks;
    if (quirks & CR_QUIRK_LITERAL_ARITH) return CR_ERR_UNSUPPORTED;  // the server renders by the FMA contract
    cr_server* s = new (std::nothrow) cr_server();
    if (!s) return CR_ERR_OUT_OF_MEMORY;
    s->ctx = ctx;
    s->cfg = c;
    s->device = cr::ctx_device(ctx);
    s->num_sms = cr_ctx_num_sms(ctx);
    s->quirks = c.quirks == CR_QUIRKS_METHOD_DEFAULT ? cr::default_quirks_for(c.method) : c.quirks;
    s->t0 = std::chrono::steady_clock::now();
    s->stats.pool_bytes = c.pool_bytes;
    if (cudaSetDevice(s->device) != cudaSuccess) {
        delete s;
        return CR_ERR_CUDA;
    }
    cudaError_t e = cudaMalloc(&s->pool, c.pool_bytes);
    s->alloc.init(c.pool_bytes);
    s->slots.resize(c.max_inflight);
    const int maxv = c.plain_launches ? 1 : c.max_batch_views;
    for (Slot& sl : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&sl.ev1);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_views, sizeof(MVView) * maxv);
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_files, sizeof(MVFile) * maxv * cr::kInlineFiles);
        if (e == cudaSuccess) e = cudaHostAlloc(&sl.h_views, sizeof(MVView) * maxv, cudaHostAllocDefault);
        if (e == cudaSuccess)
            e = cudaHostAlloc(&sl.h_files, sizeof(MVFile) * maxv * cr::kInlineFiles, cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaHostAlloc(&sl.h_err, 4, cudaHostAllocDefault);
        if (e == cudaSuccess) *sl.h_err = 0;
        if (e == cudaSuccess) e = cudaMalloc(&sl.d_mats, sizeof(double) * 32 * maxv);
        if (e == cudaSuccess) e = cudaHostAlloc(&sl.h_mats, sizeof(double) * 32 * maxv, cudaHostAllocDefault);
    }
    if (e != cudaSuccess) {
        const cr_status st = e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA;
        cudaGetLastError();
        free_server(s);
        return st;
    }
    s->th = std::thread(dispatcher, s);
    *out = s;
    return CR_OK;
}

cr_status cr_server_destroy(cr_server* s) {
    if (!s) return CR_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->in_mu);
        s->stop = true;
    }
    s->in_cv.notify_all();
    if (s->th.joinable()) s->th.join();
    free_server(s);
    return CR_OK;
}

const char* cr_server_last_error(const cr_server* s) {
    if (!s) return "";
    std::lock_guard<std::mutex> lk(s->err_mu);
    return s->err.c_str();
}

double cr_server_now_us(const cr_server* s) { return s ? now_us(s) : 0.0; }

cr_status cr_server_add_cloud(cr_server* s, const cr_cloud* cloud, int32_t* id) {
    if (!s || !cloud || !id) return CR_ERR_INVALID_ARG;
    CloudInfo ci;
    if (!cr::cloud_info(cloud, &ci) || !ci.md || !ci.hi || !ci.rgba)
        return set_err(s, CR_ERR_INVALID_ARG, "the server renders LAS-derived clouds with all four streams");
    std::lock_guard<std::mutex> lk(s->cloud_mu);
    *id = (int32_t)s->clouds.size();
    s->clouds.push_back(ci);
    s->handles.push_back(cloud);
    return CR_OK;
}

}  // extern "C"

namespace {

cr_status submit_at(cr_server* s, const cr_request* r, double t_arrival, uint64_t* ticket) {
    if (!s || !r) return CR_ERR_INVALID_ARG;
    Pending p;
    p.r = *r;
    CloudInfo ci;
    {
        std::lock_guard<std::mutex> lk(s->cloud_mu);
        if (r->cloud < 0 || r->cloud >= (int32_t)s->clouds.size())
            return set_err(s, CR_ERR_INVALID_ARG, "unknown cloud id");
        ci = s->clouds[r->cloud];
    }
    const int64_t W = r->view.width, H = r->view.height;
    if (W <= 0 || H <= 0 || W >= (1 << 22) || H >= (1 << 22) || W * H + W + 1 >= ((int64_t)1 << 31))
        return set_err(s, CR_ERR_INVALID_ARG, "view size out of range");
    if (cr::mv_fill_view(&r->view, ci, &p.view, p.files) != CR_OK)
        return set_err(s, CR_ERR_INVALID_ARG, "view matrices must be finite");
    p.fb_bytes = round_up((W * H + W + 1) * 8);
    p.bytes = p.fb_bytes + round_up(W * H * 4);
    p.t_arrival = t_arrival;
    if (p.bytes > s->cfg.pool_bytes || s->queued.load() >= s->cfg.max_queued) {
        std::lock_guard<std::mutex> lk(s->stats_mu);
        s->stats.rejected++;
        return set_err(s, CR_ERR_ADMISSION_REJECTED,
                       p.bytes > s->cfg.pool_bytes ? "request exceeds the framebuffer pool"
                                                   : "queue full");
    }
    p.ticket = s->next_ticket++;
    if (ticket) *ticket = p.ticket;
    {
        std::lock_guard<std::mutex> lk(s->done_mu);
        s->outstanding++;
    }
    {
        std::lock_guard<std::mutex> lk(s->stats_mu);
        s->stats.submitted++;
    }
    s->queued++;
    {
        std::lock_guard<std::mutex> lk(s->in_mu);
        s->incoming.push_back(std::move(p));
    }
    s->in_cv.notify_one();
    return CR_OK;
}

}  // namespace

extern "C" {

cr_status cr_server_submit(cr_server* s, const cr_request* r, uint64_t* ticket) {
    return submit_at(s, r, s ? now_us(s) : 0.0, ticket);
}

cr_status cr_server_poll(cr_server* s, cr_completion* out, int32_t max, int32_t* n, int32_t wait_ms) {
    if (!s || !out || !n || max < 1) return CR_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->done_mu);
    if (s->done.empty() && wait_ms > 0)
        s->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
    int32_t k = 0;
    while (k < max && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *n = k;
    return CR_OK;
}

cr_status cr_server_drain(cr_server* s, int32_t timeout_ms) {
    if (!s) return CR_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->done_mu);
    auto pred = [&] { return s->outstanding == 0; };
    if (timeout_ms < 0) {
        s->done_cv.wait(lk, pred);
        return CR_OK;
    }
    return s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred) ? CR_OK : CR_ERR_TIMEOUT;
}

cr_status cr_server_replay(cr_server* s, const cr_request* reqs, const double* arrival_us,
                           int64_t n, cr_completion* out) {
    if (!s || n < 0 || (n > 0 && (!reqs || !arrival_us || !out))) return CR_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->done_mu);
        if (s->outstanding != 0 || !s->done.empty())
            return set_err(s, CR_ERR_INVALID_ARG, "replay needs an idle server with no completions queued");
    }
    std::unordered_map<uint64_t, int64_t> index;
    index.reserve((size_t)n * 2);
    const double t0 = now_us(s);
    int64_t accepted = 0;
    for (int64_t i = 0; i < n; i++) {
        const double target = t0 + arrival_us[i];
        double t = now_us(s);
        if (target - t > 300.0)
            std::this_thread::sleep_for(std::chrono::duration<double, std::micro>(target - t - 200.0));
        while (now_us(s) < target) {
        }
        uint64_t ticket = 0;
        const cr_status st = submit_at(s, &reqs[i], target, &ticket);
        if (st == CR_OK) {
            index[ticket] = i;
            accepted++;
        } else {
            out[i] = cr_completion{};
            out[i].user_tag = reqs[i].user_tag;
            out[i].status = st;
            out[i].t_arrival_us = target;
        }
    }
    int64_t got = 0;
    std::unique_lock<std::mutex> lk(s->done_mu);
    while (got < accepted) {
        s->done_cv.wait(lk, [&] { return !s->done.empty(); });
        while (!s->done.empty()) {
            const cr_completion c = s->done.front();
            s->done.pop_front();
            auto it = index.find(c.ticket);
            if (it == index.end()) continue;
            out[it->second] = c;
            got++;
        }
    }
    return CR_OK;
}

cr_status cr_server_inject(cr_server* s, int32_t what, int32_t count) {
    if (!s || count < 0 || (what != CR_INJECT_NONE && what != CR_INJECT_LAUNCH_ALLOC))
        return CR_ERR_INVALID_ARG;
    s->inject_alloc_failures.store(what == CR_INJECT_LAUNCH_ALLOC ? count : 0);
    return CR_OK;
}

cr_status cr_server_stats_get(const cr_server* s, cr_server_stats* out) {
    if (!s || !out) return CR_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->stats_mu);
    *out = s->stats;
    out->queued = s->queued.load();
    return CR_OK;
}

}  // extern "C"
