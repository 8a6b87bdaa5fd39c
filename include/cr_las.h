/*
 * cr_las.h -- LAS file ingest into the batched layout (C ABI).
 *
 * The reference's loader reads each dropped file's header
 * (LasLoaderSparse.cpp:477-526), splits its points into load tasks of at most
 * MAX_POINTS_PER_BATCH = 1,024,000 points (:556-575, Resources.h:8), encodes
 * each task with loadLas (:37-212) and uploads the task's batch records and
 * word streams at the file's sparse point offset (:653-713); files are
 * numbered in drop order and their points laid out back to back.  Here the
 * caller reads the file bytes (any I/O it likes) and the library parses the
 * header and encodes every load task on the GPU into a cr_cloud.
 */
#ifndef CR_LAS_H
#define CR_LAS_H

#include "cr_raster.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CR_LAS_MIN_HEADER 227 /* LAS 1.0-1.3 public header block */
#define CR_LAS_14_HEADER 375  /* LAS 1.4 public header block */

typedef struct cr_las_info {
    int64_t num_points;       /* header count (u32 @107, or u64 @247 for 1.4), at most 1e9 */
    int64_t offset_to_points; /* u32 @96 */
    int32_t version_major;    /* u8 @24 */
    int32_t version_minor;    /* u8 @25 */
    int32_t point_format;     /* u8 @104, modulo 128 (the compression bit of LAZ) */
    int32_t bytes_per_point;  /* u16 @105 */
    double scale[3];          /* @131, 139, 147 */
    double offset[3];         /* @155, 163, 171 */
    double min[3];            /* @187, 203, 219 */
    double max[3];            /* @179, 195, 211 */
} cr_las_info;

/* Parses the public header block.  CR_ERR_INVALID_ARG if the bytes do not
 * start with "LASF", are shorter than the version's header, or describe
 * records shorter than 12 bytes. */
cr_status cr_las_parse_header(const void* header, int64_t size, cr_las_info* out);

/* Encodes `n` point records of one file (host memory, `bytes_per_point` each,
 * the file's point data from offset_to_points on) into `cloud` on the GPU:
 * points go to [point_offset, point_offset + n), batch records to
 * [batch_offset, batch_offset + cr_las_num_batches(n)), with file index
 * `file_index`.  Load tasks of CR_MAX_POINTS_PER_LOAD points are staged
 * through device memory; the call synchronizes `stream` before returning.
 * Set the file's boxMin with cr_cloud_set_files (info->min). */
cr_status cr_cloud_load_las(cr_ctx* ctx, cr_cloud* cloud, const void* records, int64_t n,
                            const cr_las_info* info, int64_t point_offset, int64_t batch_offset,
                            int32_t file_index, void* stream);

/* Batch records the load tasks of an n-point file produce: ceil per task of
 * CR_MAX_POINTS_PER_LOAD points (that size is a multiple of 10,240, so only
 * the file's last batch is partial). */
int64_t cr_las_num_batches(int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* CR_LAS_H */
