// octree.hpp -- the Morton octree of pbosler/lpmKokkos (src/LpmOctree.cpp:21-117,
// src/LpmNodeArrayD.cpp, src/LpmNodeArrayInternal.cpp, src/LpmOctreeKernels.hpp:27-400) built on
// the device, and its use as the source hierarchy of the tree-code evaluation.
//
// Layout (device, levels 0..depth concatenated at base[l], as Tree::initNodes stores them):
//   keys    uint32 per node      Morton key at max-depth resolution (x y z bits per level)
//   ptInds  int2 per node        {first sorted point or -1, point count}
//   parents int per node         level-local index of the parent, -1 for the root
//   kids    8 int per node       level-local indices of the children, -1 for leaves / empty nodes
//   nbrs    27 int per node      level-local neighbour indices (optional), -1 where none
//   sorted  3 double per point   points in key order (row-major)
//   origIds int per point        sorted -> input index
//   ptInLeaf int per point       sorted point -> level-local leaf index
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace lpm {

constexpr int kOctreeMaxDepth = 10;  // MAX_OCTREE_DEPTH, src/LpmOctreeUtil.hpp:24-28

class Octree {
 public:
  Octree() = default;
  ~Octree();
  Octree(const Octree&) = delete;
  Octree& operator=(const Octree&) = delete;

  // Builds the tree of n points x[i*si + c*sc] (device) with leaves at `depth`.  Reads the level
  // sizes back (synchronises `s`); buffers are reused by later builds when large enough.
  // hostBox = false leaves `box` stale and returns with the last copies still queued on `s`
  // (for a caller that reads only device arrays and synchronises later).
  void build(const double* x, int64_t si, int64_t sc, int64_t n, int depth, bool neighbors, cudaStream_t s,
             bool hostBox = true);

  // Sync-free build for the tree code: the same tree, its levels stored at fixed capacities --
  // level l at gbase[l] (= base[l]) with room for min(8^l, 8 n) nodes, nnodes = the total
  // capacity -- and the node counts kept on the device (dcount[0..depth]); nodes past a level's
  // count have an empty point range (ptInds.y = 0) and are never reached from the root.  Nothing
  // is read back, and a rebuild with the same n and depth allocates nothing, so after a first
  // build the call can be captured in a CUDA graph.  No neighbour lists.
  void buildOnDevice(const double* x, int64_t si, int64_t sc, int64_t n, int depth, cudaStream_t s);
  // Frees every buffer in stream order on `s` (after the work queued there); the object can be
  // built again or destroyed without a device synchronisation.
  void release(cudaStream_t s);
  int gbase[kOctreeMaxDepth + 2] = {};
  int* dcount = nullptr;              // device [depth + 2]: node counts per level, then the unique leaf keys

  int depth = 0;
  int64_t n = 0, nnodes = 0;
  int base[kOctreeMaxDepth + 1] = {};
  int npl[kOctreeMaxDepth + 1] = {};
  double box[6] = {};                 // reduced bounding box (host copy)

  uint32_t* keys = nullptr;
  int2* ptInds = nullptr;
  int* parents = nullptr;
  int* kids = nullptr;
  int* nbrs = nullptr;                // null unless built with neighbours
  double* sorted = nullptr;
  int* origIds = nullptr;
  int* ptInLeaf = nullptr;
  const double* dbox = nullptr;       // device copy of the box

 private:
  struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
  };
  template <typename T>
  T* grow(Buf& b, size_t count, cudaStream_t s);
  void releaseAll();

  Buf bKeys, bPt, bPar, bKids, bNbrs, bSorted, bOrig, bLeaf, bBox;
  Buf bCodes, bCodes2, bFlag, bScan, bUKeys, bUStart, bUCount, bNodeOf, bSib, bTemp, bPart, bCount;
  Buf bLevKeys[kOctreeMaxDepth + 1], bLevPt[kOctreeMaxDepth + 1], bLevPar[kOctreeMaxDepth + 1],
      bLevKids[kOctreeMaxDepth + 1], bLevNbrs[kOctreeMaxDepth + 1];
  std::vector<Buf*> all_;
  bool registered_ = false;
};

}  // namespace lpm
