/*
 * cr_potree.h -- Potree 2.0 octrees into the batched layout, for the
 * "loop_nodes" method ("render Potree nodes").
 *
 * Replaces PotreeData (modules/compute/PotreeData.h): loadMetadata (:143-184)
 * reads metadata.json, loadHierarchy (:186-315) walks hierarchy.bin (22-byte
 * node entries in chunks, proxy nodes pointing at further chunks), and the
 * loader thread (:317-474) reads octree.bin and encodes every node as one
 * batch record over the word streams.  A node's record is its octree box
 * (relative to the dataset's boxMin, children halved in float as
 * createChildAABB does, :112-140), its point count, its first point
 * (byteOffset / bytesPerPoint) and, in the file_index slot, its level
 * (:335-350); nodes are ordered by byteOffset.  Points are quantised to 30
 * bits against their node's box in double.
 *
 * The ordinary batched methods need nodes of at most 10,240 points; render
 * these clouds with CR_METHOD_LOOP_NODES, whose defaults reproduce
 * compute_loop_nodes (cr_raster.h).
 */
#ifndef CR_POTREE_H
#define CR_POTREE_H

#include "cr_raster.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Loader behaviours of PotreeData.h, on by default (quirks = -1): */
enum {
    /* the 12b stream receives bits 19..10, like the 8b one (PotreeData.h:441-449) */
    CR_POTREE_QUIRK_12B_FROM_8B = 1,
    /* uint32(t) & MASK_30BIT instead of a clamp: a point on a node's far face
     * wraps to 0 (PotreeData.h:420-422); without it the value is clamped to
     * 2^30 - 1 as loadLas does */
    CR_POTREE_QUIRK_WRAP30 = 2
};
#define CR_POTREE_QUIRKS_DEFAULT (-1)

typedef struct cr_potree_info {
    int64_t num_points;      /* metadata "points" */
    int64_t num_nodes;       /* nodes of the hierarchy = batch records */
    int64_t octree_bytes;    /* bytes of octree.bin the nodes cover */
    int32_t bytes_per_point; /* sum of the attribute sizes */
    int32_t rgb_offset;      /* byte offset of "rgb" in a point record; -1 without one */
    int32_t max_level;
    int32_t reserved;
    int64_t max_node_points;
    double scale[3], offset[3];
    double box_min[3], box_max[3]; /* metadata boundingBox */
    double spacing;
} cr_potree_info;

typedef struct cr_potree_node {
    int32_t level;
    int32_t type;            /* 0 inner, 1 leaf (2, proxy, is resolved while loading) */
    int32_t child_mask;
    int32_t reserved;
    int64_t num_points;
    int64_t byte_offset;     /* into octree.bin */
    int64_t byte_size;
    double min[3], max[3];   /* the node's box relative to boxMin */
} cr_potree_node;

typedef struct cr_potree cr_potree;

/* Reads <dir>/metadata.json and <dir>/hierarchy.bin. */
cr_status cr_potree_open(const char* dir, cr_potree** out, cr_potree_info* info);
cr_status cr_potree_close(cr_potree* p);
/* The nodes in batch order (sorted by byte_offset); returns CR_ERR_INVALID_ARG
 * if `max` is below the node count. */
cr_status cr_potree_nodes(const cr_potree* p, cr_potree_node* out, int64_t max);
/* Host encoder: octree.bin bytes [0, bytes) -> num_nodes batch records and
 * num_points words per stream (PotreeData.h:361-452).  quirks: cr_potree
 * quirk mask or CR_POTREE_QUIRKS_DEFAULT. */
cr_status cr_potree_encode(const cr_potree* p, const uint8_t* octree, int64_t bytes, int32_t quirks,
                           cr_batch* batches, uint32_t* xyz_low, uint32_t* xyz_med,
                           uint32_t* xyz_hig, uint32_t* rgba);
/* Reads <dir>/octree.bin, encodes it and uploads a cloud of num_points points
 * and num_nodes records with one file at boxMin (0, 0, 0): the nodes' boxes
 * are already relative to the dataset's boxMin, and compute_loop_nodes
 * renders with an identity world matrix. */
cr_status cr_potree_load(cr_ctx* ctx, const cr_potree* p, int32_t quirks, cr_cloud** out,
                         void* stream);

#ifdef __cplusplus
}
#endif
#endif
