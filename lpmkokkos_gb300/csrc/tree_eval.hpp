// tree_eval.hpp -- host side of the tree-code evaluation (tree.hpp describes the method).
#pragma once

#include "engine_core.hpp"
#include "octree.hpp"
#include "tree.hpp"

namespace lpm {

class TreeEval {
 public:
  // One evaluation for the solve P: builds the source octree over the stage positions the prep
  // kernel wrote, the proxies and the per-tile index lists, and runs the gathered pair kernel
  // into this object's partial buffer ([nchunks()][ncomp][slot]), which the epilogue then sums.
  // Synchronises `s` (octree level sizes, list lengths).
  void evaluate(SolvePlan& P, const TreeParams& tp, const PairShape& shape, bool psi, bool precise, bool rcpApprox,
                int slots, PairTimer* timer, cudaStream_t s);
  // Records that this solve's evaluation used the direct sum (smaller than TreeParams::minPairs).
  void markDirect(const SolvePlan& P) {
    stats_ = TreeStats{};
    stats_.pairs = stats_.directPairs = (double)P.nslots * P.ns;
  }
  double* partial() const { return partial_; }
  int nchunks() const { return nchunks_; }
  const TreeStats& stats() const { return stats_; }

 private:
  struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
  };
  template <typename T>
  T* grow(Buf& b, size_t count, cudaStream_t s);

 public:
  TreeEval() = default;
  ~TreeEval();
  TreeEval(const TreeEval&) = delete;
  TreeEval& operator=(const TreeEval&) = delete;

 private:
  Octree tree_;
  TreeStats stats_;
  Buf bPos, bSp0, bSp1, bInv, bSelf, bGeom, bApprox, bTileGeom, bLen, bFar, bOff, bOrder, bList, bPartial,
      bDev, bCounter, bErr, bSlot;
  std::vector<Buf*> all_{&bPos, &bSp0, &bSp1, &bInv, &bSelf, &bGeom, &bApprox, &bTileGeom, &bLen,
                         &bFar, &bOff, &bOrder, &bList, &bPartial, &bDev, &bCounter, &bErr, &bSlot};
  double* partial_ = nullptr;
  int nchunks_ = 1;
  // host source of the last upload (an evaluation synchronises before it rewrites it)
  TreeDev hDev_{};
  std::vector<int64_t> hLen_, hFar_, hOff_;
  std::vector<int2> hTiles_;
  std::vector<int> hOrder_;
  std::vector<uint64_t> hKey_;  // tiles by descending list length (then tile index), for the order
};

// Octree depth whose leaves hold about `leafPoints` of n points on the sphere: the nonempty
// cells of level d number ~4.7 * 4^d (a sphere of radius 1 in a cube of side 2).
int treeDepthFor(int64_t n, int leafPoints);

}  // namespace lpm
