// tree_eval.hpp -- host side of the tree-code evaluation (tree.hpp describes the method).
#pragma once

#include "engine_core.hpp"
#include "octree.hpp"
#include "tree.hpp"

namespace lpm {

class TreeEval {
 public:
  // One evaluation for the single solve P: builds the source octree over the stage positions
  // the prep kernel wrote, the proxies and the per-tile index lists, and runs the gathered pair
  // kernel into this object's one-chunk partial buffer.  The epilogue then reads stageDev().
  // Synchronises `s` (octree level sizes, list lengths).
  void evaluate(SolvePlan& P, const TreeParams& tp, const PairShape& shape, bool psi, bool precise, bool rcpApprox,
                int slots, PairTimer* timer, cudaStream_t s);
  const SolveStage* stageDev() const { return stageDev_; }
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
  Buf bPos, bSp0, bSp1, bInv, bSelf, bGeom, bApprox, bTileGeom, bTileSelf, bLen, bFar, bOff, bOrder, bList, bPartial,
      bDev, bStage, bCounter, bErr;
  std::vector<Buf*> all_{&bPos, &bSp0, &bSp1, &bInv, &bSelf, &bGeom, &bApprox, &bTileGeom, &bTileSelf, &bLen,
                         &bFar, &bOff, &bOrder, &bList, &bPartial, &bDev, &bStage, &bCounter, &bErr};
  SolveStage* stageDev_ = nullptr;
  // host sources of the last uploads (an evaluation synchronises before it rewrites them)
  TreeDev hDev_{};
  SolveStage hStage_{};
  std::vector<int64_t> hLen_, hFar_, hOff_;
  std::vector<int2> hTiles_;
  const int2* tilesOf_ = nullptr;  // plan whose tile sizes hTiles_ holds
  std::vector<int> hOrder_;
};

// Octree depth whose leaves hold about `leafPoints` of n points on the sphere: the nonempty
// cells of level d number ~4.7 * 4^d (a sphere of radius 1 in a cube of side 2).
int treeDepthFor(int64_t n, int leafPoints);

}  // namespace lpm
