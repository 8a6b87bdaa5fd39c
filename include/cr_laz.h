/*
 * cr_laz.h -- LAZ (LASzip-compressed LAS) ingest into the batched layout, and
 * a LAZ writer (C ABI).
 *
 * Replaces loadLaz (LasLoaderSparse.cpp:214-429), which opens each load task's
 * file through the vendored LASzip (laszip_open_reader, laszip_seek_point),
 * reads the task's points one by one (laszip_read_point,
 * laszip_get_coordinates, the point's rgb) and encodes them like loadLas:
 * double coordinates X * scale + offset - boxMin, per-batch AABB, 30-bit
 * quantisation, 10-bit word split, colours v < 256 ? v : v / 256 without an
 * alpha byte.  A LAZ file's header is read like a LAS file's
 * (LasLoaderSparse.cpp:493-526; the point format modulo 128 clears the
 * compression bit); its points are split into the same load tasks.
 *
 * Here the chunks of the LAZ stream decode in parallel on host threads (every
 * chunk restarts the entropy coder) and each load task is encoded on the GPU
 * exactly as cr_cloud_load_las encodes the same records, except that point
 * formats without RGB get colour 0, as LASzip's zeroed rgb gives loadLaz.
 *
 * Supported streams (decoding): the LASzip point-wise coders, chunked
 * (compressor 2, the default for point formats 0-5, fixed or variable chunk
 * sizes) or not (compressor 1), with version-2 items POINT10, GPSTIME11,
 * RGB12 and BYTE (LAS point formats 0-3 plus extra bytes); and the layered
 * coder of LAS 1.4 (compressor 3) with version-3 items POINT14, RGB14,
 * RGBNIR14 and BYTE14 (point formats 6, 7 and 8 plus extra bytes), as
 * LASzip 3.4 writes them, and their version-4 revision.  Version-1 items and
 * wave packets (formats 4, 5, 9, 10) return CR_ERR_UNSUPPORTED.  The writer
 * produces point formats 0-3.
 */
#ifndef CR_LAZ_H
#define CR_LAZ_H

#include "cr_las.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CR_LAZ_MAX_ITEMS 8
/* LASzip item types (laszip.hpp LASitem::Type) */
enum {
    CR_LAZ_ITEM_BYTE = 0, CR_LAZ_ITEM_POINT10 = 6, CR_LAZ_ITEM_GPSTIME11 = 7, CR_LAZ_ITEM_RGB12 = 8,
    CR_LAZ_ITEM_POINT14 = 10, CR_LAZ_ITEM_RGB14 = 11, CR_LAZ_ITEM_RGBNIR14 = 12, CR_LAZ_ITEM_BYTE14 = 14
};
/* LASzip compressors */
enum { CR_LAZ_POINTWISE = 1, CR_LAZ_POINTWISE_CHUNKED = 2, CR_LAZ_LAYERED_CHUNKED = 3 };
#define CR_LAZ_DEFAULT_CHUNK 50000 /* LASzip's default chunk size */
#define CR_LAZ_VARIABLE_CHUNKS (-1)

typedef struct cr_laz_info {
    cr_las_info las;           /* the public header block, as cr_las_parse_header */
    int32_t compressor;        /* CR_LAZ_POINTWISE, _POINTWISE_CHUNKED or _LAYERED_CHUNKED */
    int32_t num_items;
    int32_t item_type[CR_LAZ_MAX_ITEMS];
    int32_t item_size[CR_LAZ_MAX_ITEMS];
    int32_t item_version[CR_LAZ_MAX_ITEMS];
    int32_t version_major, version_minor; /* of the LASzip that wrote the file */
    int64_t chunk_size;        /* points per chunk, CR_LAZ_VARIABLE_CHUNKS, or num_points unchunked */
    int64_t num_chunks;        /* chunks located; 0 when the file has no chunk table */
    int64_t points_at;         /* offset to point data */
} cr_laz_info;

typedef struct cr_laz cr_laz;

/* Parses the header, the LASzip VLR (user "laszip encoder", record 22204) and
 * the chunk table of a LAZ file held in memory.  `file` must stay valid and
 * unchanged until cr_laz_close.  CR_ERR_INVALID_ARG if the bytes are not a
 * LAS file with a LASzip VLR, CR_ERR_UNSUPPORTED for the coders above,
 * CR_ERR_CORRUPT if the chunk table does not decode. */
cr_status cr_laz_open(const void* file, int64_t size, cr_laz** out, cr_laz_info* info);
cr_status cr_laz_close(cr_laz* laz);

/* Decompresses points [first, first + n) into LAS records (bytes_per_point
 * each, the file's record layout) on up to `threads` host threads (<= 0: all
 * cores).  CR_ERR_CORRUPT if a chunk does not decode to its table extent. */
cr_status cr_laz_decode(const cr_laz* laz, int64_t first, int64_t n, void* records, int32_t threads);

/* Decodes the whole file and encodes it into `cloud` on the GPU: points to
 * [point_offset, point_offset + num_points), cr_las_num_batches(num_points)
 * batch records from batch_offset, file index `file_index`.  Decoding of the
 * next window of chunks overlaps the upload and encoding of the last one;
 * synchronizes `stream` before returning.  Set the file's boxMin with
 * cr_cloud_set_files (info.las.min). */
cr_status cr_cloud_load_laz(cr_ctx* ctx, cr_cloud* cloud, const cr_laz* laz, int64_t point_offset,
                            int64_t batch_offset, int32_t file_index, int32_t threads, void* stream);

/* Writer.  The LASzip VLR payload for LAS point format 0-3 records of
 * bytes_per_point bytes (extra bytes become a BYTE item) with the given chunk
 * size (or CR_LAZ_VARIABLE_CHUNKS); *len receives its size (34 + 6 per item). */
cr_status cr_laz_vlr(int32_t point_format, int32_t bytes_per_point, int64_t chunk_size, uint8_t* out,
                     int64_t cap, int64_t* len);
/* Compresses n records into the point data area of a LAZ file that starts at
 * file offset `points_at` (the chunk table pointer is absolute): the 8-byte
 * pointer, the chunks, the chunk table.  Chunks are compressed in parallel on
 * up to `threads` host threads; the bytes equal those LASzip writes for the
 * same records and chunking.  With CR_LAZ_VARIABLE_CHUNKS a chunk is closed
 * after every `var_chunk` points.  *len receives the size; CR_ERR_INVALID_ARG
 * if it exceeds cap (bound: cr_laz_compress_bound). */
cr_status cr_laz_compress(const void* records, int64_t n, int32_t point_format, int32_t bytes_per_point,
                          int64_t chunk_size, int64_t var_chunk, int64_t points_at, uint8_t* out,
                          int64_t cap, int64_t* len, int32_t threads);
int64_t cr_laz_compress_bound(int64_t n, int32_t bytes_per_point, int64_t chunk_size);

#ifdef __cplusplus
}
#endif

#endif /* CR_LAZ_H */
