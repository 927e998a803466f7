// tree.hpp -- tree-code evaluation of the BVE direct sums (LPM_BVE_TREECODE, FP32C).
//
// The far field of well-separated source clusters is replaced by a barycentric Lagrange
// interpolant in a gnomonic chart of each cluster: the cluster's sources y_j (weights w_j) act
// on a target x through sum_j w_j F(x, y_j), F = y / (1 - x.y + eps^2) (and log(...) for psi).
// With (xi, eta) the gnomonic coordinates of y about the cluster's centre direction,
// F(x, y(xi, eta)) is smooth on the cluster's chart rectangle when x is far, so
//   sum_j w_j F(x, y_j) ~ sum_ab Q_ab F(x, y_ab),   Q_ab = sum_j w_j L_a(xi_j) L_b(eta_j),
// with y_ab the chart's (n+1) x (n+1) Chebyshev points mapped back to the unit sphere.  The
// proxies y_ab are ordinary sources of the pair kernel (same FP32C records), so one kernel
// evaluates near sources and far proxies alike.  Interpolating in the chart instead of in the
// octree cube matters: off the sphere 1/(1 - x.y) is singular on the tangent plane at x, which
// passes R^2/2 above a cluster at chord distance R, while in the chart the singularity stays
// ~R away (the usual tree-code regime).
//
// Clusters are the nodes of the reference's Morton octree (octree.hpp) over the stage positions
// of the sources; target batches ("tiles") are runs of at most 256 target slots of the plan's
// Morton order that stay inside one level-3 Morton cell.  A tile takes a cluster
// as far field when (r_tile + r_node) < theta |c_tile - c_node| and the node has more than
// (n+1)^2 sources and a valid chart; otherwise it recurses into the kids, or takes the node's
// sources directly at a leaf or when the node is accepted but too small to approximate.
//
// Per evaluation: source positions -> octree -> sources gathered into key order -> upward pass
// (centres, radii, charts, proxies) -> tile geometry -> traversal (counts, offsets, index lists)
// -> gathered pair kernel -> the usual epilogue.
#pragma once

#include <cstdint>

#include "engine.hpp"
#include "octree.hpp"

namespace lpm {

struct TreeParams {
  int degree = 8;          // interpolation degree n per chart axis: (n+1)^2 proxies per cluster
  double theta = 0.6;      // opening parameter of the acceptance test
  int leafPoints = 512;    // target mean sources per octree leaf (sets the octree depth)
  double minPairs = 1e9;   // solves with fewer target x source pairs use the direct sum
};

// Device description of one tree evaluation for the gathered pair kernel.
struct TreeDev {
  const double* tx;        // [3][nslots] target stage positions (SoA)
  const float4* sp0;       // [ns + nprox] sorted sources, then proxies: (x_hi, y_hi, z_hi, w)
  const float4* sp1;       // (x_lo, y_lo, z_lo, D)
  const int* self;         // [nslots] sorted index of the same particle, -1 if none
  const int* srcSlot;      // [ns] slot of the same particle as sorted source k, -1 if none
  const int2* tiles;       // [ntiles] {first slot, count} (runs inside one level-3 Morton cell)
  const int* tileCentre;   // [ntiles] centre slot of the tile (as in the direct kernel)
  const int64_t* listOff;  // [ntiles] offset of each tile's list in `list`
  const int64_t* listLen;  // [ntiles] its length
  const int* list;         // flattened per-tile source indices into sp0/sp1
  const int* order;        // [ntiles * nchunks] work items (tile * nchunks + part), longest first
  double* partial;         // [nchunks][ncomp][nslots]: part c of every tile's list sums into chunk c
  int nslots, ntiles, nchunks, ns;
  double eps2;
};

struct TreeStats {
  int depth = 0;
  int64_t nodes = 0, farClusters = 0;
  double pairs = 0, directPairs = 0, farPairs = 0;  // target x source(or proxy) pairs, last evaluation
  // CUDA-event times of the last timed evaluation (ms): octree build, upward pass, tile geometry
  // and interaction lists (both traversals); the pair kernel is in the context's pair timer.
  double buildMs = 0, upwardMs = 0, listMs = 0;
};

cudaError_t launchTreePair(const PairShape& shape, bool psi, bool precise, bool rcpApprox, const TreeDev* dev,
                           int nitems, int* counter, int grid, cudaStream_t s);
// The tree kernel's launch shape: 32 threads x 4 targets (128-target tiles), 128-record source
// blocks, 12 CTAs per SM (160-168 registers, 10.8 KB of shared memory).  Smaller tiles take fewer
// pairs (a tile's near field shrinks with its radius): 16.5 % fewer than 256-target tiles at
// icosahedral level 8, 13.5 % at level 7.
inline constexpr PairShape kTreeShape{32, 4, 128, 12};
bool treePairShapeSupported(const PairShape& shape);

}  // namespace lpm
