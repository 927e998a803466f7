/* lpm_octree.h -- the Morton octree of pbosler/lpmKokkos built on the GPU.
 *
 * Replaces Lpm::Octree::Tree(const ko::View<Real*[3]>& p, const Int& md) (src/LpmOctree.hpp:22-87,
 * src/LpmOctree.cpp:21-117): leaves at max_depth holding every point (NodeArrayD,
 * src/LpmNodeArrayD.cpp:14-117), complete sibling sets at every level, internal levels and the
 * root (NodeArrayInternal, src/LpmNodeArrayInternal.cpp:13-186), all levels concatenated at
 * base_address[l], and the 27-neighbour lists of each node (NeighborhoodFunctor,
 * src/LpmOctreeKernels.hpp:371-400).  Node keys are the reference's shuffled x-y-z keys at
 * max_depth resolution; node_pt_inds, node_parents, node_kids and node_neighbors hold the same
 * values as the reference's views (-1 = NULL_IND; parents, kids and neighbours are level-local
 * indices), with two corrections: neighbours at levels >= 2 read the parent level at its base
 * address (the reference reads level-local indices as global rows), and ChildLUT row 0,
 * columns 18-20 and 24-26 carry the +x bit the reference's table omits.
 *
 * All returned arrays are DEVICE memory owned by the tree (valid until lpm_octree_destroy).
 */
#ifndef LPM_OCTREE_H
#define LPM_OCTREE_H

#include <stdint.h>

#include "lpm_bve.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lpm_octree lpm_octree;

/* Build the tree of n DEVICE points (point i, component c at x[i*x_si + c*x_sc]; 1 <= n < 2^31)
 * with leaves at max_depth (1..10, MAX_OCTREE_DEPTH).  `neighbors` is a bit set:
 *   LPM_OCTREE_NEIGHBORS    also fill the neighbour lists;
 *   LPM_OCTREE_FIXED_LEVELS the sync-free build the tree code uses: nothing is read back and the
 *                           stream is not synchronised; level l sits at a fixed base with room for
 *                           min(8^l, 8 n) nodes (base_address and nnodes_total from
 *                           lpm_octree_info describe that layout), its first nnodes_per_level[l]
 *                           nodes hold the same values as the concatenated build's level l, and
 *                           the rest have an empty point range (count 0).  No neighbour lists;
 *                           n < 2^28.  lpm_octree_info then synchronises the device to read the
 *                           level counts and the box.
 * Without LPM_OCTREE_FIXED_LEVELS the build synchronises `stream` (the level sizes are read back). */
#define LPM_OCTREE_NEIGHBORS    1
#define LPM_OCTREE_FIXED_LEVELS 2
int lpm_octree_build(const double* x, int64_t x_si, int64_t x_sc, int64_t n, int max_depth, int neighbors,
                     lpm_octree** out, lpm_stream_t stream);

/* Sizes: nnodes_per_level and base_address have max_depth + 1 entries; box = the points'
 * bounding box (xmin, xmax, ymin, ymax, zmin, zmax) before box2cube.  Any pointer may be NULL. */
int lpm_octree_info(const lpm_octree* t, int* max_depth, int64_t* nnodes_total, int64_t* npoints,
                    int32_t* nnodes_per_level, int32_t* base_address, double* box);

/* Device arrays, concatenated over levels 0..max_depth:
 *   keys (nnodes), pt_inds (nnodes x 2: first sorted point or -1, count), parents (nnodes),
 *   kids (nnodes x 8), neighbors (nnodes x 27; NULL unless built with neighbours);
 * per point: sorted_pts (n x 3, row-major), orig_ids (sorted -> input index),
 *   pt_in_leaf (level-local leaf of each sorted point).  Any pointer may be NULL. */
int lpm_octree_arrays(const lpm_octree* t, const uint32_t** keys, const int32_t** pt_inds, const int32_t** parents,
                      const int32_t** kids, const int32_t** neighbors, const double** sorted_pts,
                      const int32_t** orig_ids, const int32_t** pt_in_leaf);

int lpm_octree_destroy(lpm_octree* t);

#ifdef __cplusplus
}
#endif

#endif /* LPM_OCTREE_H */
