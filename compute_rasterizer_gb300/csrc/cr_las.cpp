// cr_las.cpp -- LAS header parsing and file ingest (include/cr_las.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "../../include/cr_las.h"
#include "../../include/cr_synth.h"
#include "cr_internal.h"

namespace {

template <typename T>
T get(const uint8_t* p, int64_t off) {
    T v;
    std::memcpy(&v, p + off, sizeof(T));  // LAS is little-endian, as both hosts are
    return v;
}

}  // namespace

extern "C" {

// LasLoaderSparse.cpp:493-526
cr_status cr_las_parse_header(const void* header, int64_t size, cr_las_info* out) {
    if (!header || !out || size < CR_LAS_MIN_HEADER) return CR_ERR_INVALID_ARG;
    const uint8_t* h = static_cast<const uint8_t*>(header);
    if (std::memcmp(h, "LASF", 4) != 0) return CR_ERR_INVALID_ARG;
    cr_las_info info;
    std::memset(&info, 0, sizeof(info));
    info.version_major = get<uint8_t>(h, 24);
    info.version_minor = get<uint8_t>(h, 25);
    if (info.version_major == 1 && info.version_minor < 4) {
        info.num_points = get<uint32_t>(h, 107);
    } else {
        if (size < CR_LAS_14_HEADER) return CR_ERR_INVALID_ARG;
        const uint64_t n = get<uint64_t>(h, 247);
        info.num_points = n > 1000000000ull ? 1000000000ll : (int64_t)n;
    }
    info.num_points = std::min<int64_t>(info.num_points, 1000000000ll);
    info.offset_to_points = get<uint32_t>(h, 96);
    info.point_format = get<uint8_t>(h, 104) % 128;
    info.bytes_per_point = get<uint16_t>(h, 105);
    for (int k = 0; k < 3; k++) {
        info.scale[k] = get<double>(h, 131 + 8 * k);
        info.offset[k] = get<double>(h, 155 + 8 * k);
        info.max[k] = get<double>(h, 179 + 16 * k);
        info.min[k] = get<double>(h, 187 + 16 * k);
    }
    if (info.bytes_per_point < 12) return CR_ERR_INVALID_ARG;
    *out = info;
    return CR_OK;
}

int64_t cr_las_num_batches(int64_t n) {
    if (n <= 0) return 0;
    const int64_t task = CR_MAX_POINTS_PER_LOAD;
    const int64_t full = n / task, rest = n - full * task;
    return full * cr_num_batches(task) + cr_num_batches(rest);
}

// LasLoaderSparse.cpp:556-575 (load tasks), :37-212 (loadLas), :653-713 (upload)
cr_status cr_cloud_load_las(cr_ctx* ctx, cr_cloud* cloud, const void* records, int64_t n,
                            const cr_las_info* info, int64_t point_offset, int64_t batch_offset,
                            int32_t file_index, void* stream) {
    if (!ctx || !cloud || !info || n < 0 || (n > 0 && !records) || point_offset < 0 ||
        batch_offset < 0 || file_index < 0 || info->bytes_per_point < 12)
        return CR_ERR_INVALID_ARG;
    if (point_offset + n > cr_cloud_num_points(cloud) ||
        batch_offset + cr_las_num_batches(n) > cr_cloud_num_batches(cloud))
        return CR_ERR_INVALID_ARG;
    if (n == 0) return CR_OK;
    cr_batch* batches = nullptr;
    uint32_t *lo = nullptr, *md = nullptr, *hi = nullptr, *rgba = nullptr;
    cr_status s = cr_cloud_device(cloud, &batches, &lo, &md, &hi, &rgba);
    if (s != CR_OK || !lo || !md || !hi || !rgba) return CR_ERR_INVALID_ARG;

    const int64_t bpp = info->bytes_per_point;
    const int64_t task = CR_MAX_POINTS_PER_LOAD;
    uint8_t* staging = nullptr;
    if (cudaMalloc(&staging, (size_t)(std::min(n, task) * bpp)) != cudaSuccess) {
        cudaGetLastError();
        return CR_ERR_OUT_OF_MEMORY;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const uint8_t* src = static_cast<const uint8_t*>(records);
    int64_t b = batch_offset;
    for (int64_t first = 0; first < n && s == CR_OK; first += task) {
        const int64_t cnt = std::min(task, n - first);
        if (cudaMemcpyAsync(staging, src + first * bpp, (size_t)(cnt * bpp), cudaMemcpyHostToDevice, st) !=
            cudaSuccess) {
            s = CR_ERR_CUDA;
            break;
        }
        const int64_t p = point_offset + first;
        s = cr_encode_las_device(ctx, staging, cnt, (int32_t)bpp, info->point_format, info->scale,
                                 info->offset, info->min, p, file_index, batches + b, lo + p, md + p,
                                 hi + p, rgba + p, stream);
        b += cr_num_batches(cnt);
        // the staging buffer is reused by the next task
        if (s == CR_OK && cudaStreamSynchronize(st) != cudaSuccess) s = CR_ERR_CUDA;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess && s == CR_OK) s = CR_ERR_CUDA;
    cudaFree(staging);
    cudaGetLastError();
    return s;
}

}  // extern "C"
