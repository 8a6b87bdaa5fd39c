/*
 * cr_synth.h -- seeded synthetic point clouds in the LAS record format, the
 * Morton ordering the reference's offline sorter applies, and the GPU build of
 * the LAS-derived batched layout.
 *
 * The reference loads real LAS files: LasLoaderSparse::add parses the header
 * (LasLoaderSparse.cpp:477-595), loadLas encodes (:37-212), and the offline
 * tool tools/sort_points/Sort_Frugal orders points by a 3 x 21-bit Morton code
 * (main.cpp:58-141).  The generators here produce LAS point-format-2 records
 * (26 bytes: int32 X, Y, Z, ..., uint16 R, G, B at byte 20) from a
 * counter-based hash of (seed, point index), so the host and device versions
 * produce identical bytes for any thread count.
 */
#ifndef CR_SYNTH_H
#define CR_SYNTH_H

#include "cr_raster.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CR_LAS_FORMAT2_BYTES 26

/* The fields of a LAS public header block the loader reads (:497-526). */
typedef struct cr_las_header {
    int64_t num_points;
    int32_t point_format;
    int32_t bytes_per_point;
    double scale[3];
    double offset[3];
    double min[3];
    double max[3];
} cr_las_header;

enum { CR_SYNTH_TERRAIN = 0, CR_SYNTH_TERRAIN_BOXES = 1 };

typedef struct cr_synth_params {
    int32_t kind;           /* CR_SYNTH_TERRAIN / CR_SYNTH_TERRAIN_BOXES */
    int32_t octaves;        /* fbm octaves (6) */
    uint64_t seed;
    double extent;          /* terrain side in metres (1000, 10000) */
    double height;          /* z = height * fbm(x, y) + N(0, sigma) (20) */
    double sigma;           /* 0.05 */
    double wavelength;      /* wavelength of the first octave, metres */
    double las_scale;       /* LAS coordinate scale (0.001 = mm) */
    int32_t num_boxes;      /* boxes kind: 2000 */
    int32_t points_per_box; /* boxes kind: 20000 */
    double box_min_height;  /* 10 */
    double box_max_height;  /* 60 */
    double origin[2];       /* x, y of the square's corner (0, 0); the height field is absolute */
} cr_synth_params;

void cr_synth_params_default(int32_t kind, double extent, uint64_t seed, cr_synth_params* out);

/* Host generator: points [0, n) as format-2 records, in generation order;
 * fills the header (bounds from the quantised coordinates). */
cr_status cr_synth_points_host(const cr_synth_params* p, int64_t n, uint8_t* records,
                               cr_las_header* hdr);
/* Host Morton sort of records in place: key over the header's bounding cube
 * (Sort_Frugal/src/main.cpp:79-105), ties in original order. */
cr_status cr_morton_sort_host(uint8_t* records, int64_t n, int32_t bytes_per_point,
                              const cr_las_header* hdr);

/* Device generator into caller-allocated device records; computes the header
 * bounds on the device and synchronizes `stream` to return them. */
cr_status cr_synth_points_device(cr_ctx* ctx, const cr_synth_params* p, int64_t n,
                                 uint8_t* d_records, cr_las_header* hdr, void* stream);
/* Device Morton sort (stable radix sort of (code, index), then a gather);
 * records of an even bytes_per_point in [12, 64], as LAS point formats are. */
cr_status cr_morton_sort_device(cr_ctx* ctx, uint8_t* d_records, int64_t n,
                                int32_t bytes_per_point, const cr_las_header* hdr, void* stream);
/* GPU encoder: loadLas (LasLoaderSparse.cpp:37-212) over device records, one
 * CTA per 10,240-point batch; bit-identical to cr_encode_las. */
cr_status cr_encode_las_device(cr_ctx* ctx, const uint8_t* d_records, int64_t n,
                               int32_t bytes_per_point, int32_t point_format,
                               const double scale[3], const double offset[3],
                               const double box_min[3], int64_t sparse_offset,
                               int32_t file_index, cr_batch* d_batches, uint32_t* d_xyz_low,
                               uint32_t* d_xyz_med, uint32_t* d_xyz_hig, uint32_t* d_rgba,
                               void* stream);
/* Whole pipeline on the GPU: generate, sort, encode into `cloud` (file 0; the
 * cloud must hold n points and cr_num_batches(n) records). */
cr_status cr_synth_cloud_device(cr_ctx* ctx, const cr_synth_params* p, int64_t n, cr_cloud* cloud,
                                cr_las_header* hdr, void* stream);

/* Plain 16 B points: xyz ~ U[0, size)^3 (float), 32 random color bits. */
cr_status cr_synth_uniform_host(uint64_t seed, int64_t n, float size, cr_vertex* out);
cr_status cr_synth_uniform_device(cr_ctx* ctx, uint64_t seed, int64_t n, float size,
                                  cr_vertex* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
