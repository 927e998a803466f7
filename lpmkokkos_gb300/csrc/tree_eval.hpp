// tree_eval.hpp -- host side of the tree-code evaluation (tree.hpp describes the method).
#pragma once

#include "engine_core.hpp"
#include "octree.hpp"
#include "tree.hpp"

namespace lpm {

// What an evaluation reports back to the host without a synchronisation: device writes into
// mapped host memory, read before a later evaluation or a graph replay.
struct TreeWatch {
  int overflow;        // a list total exceeded the buffer (that evaluation summed every source)
  int stackErr;        // a traversal stack overflowed (cannot happen for depth <= 10)
  long long maxTotal;  // largest list total seen
};

class TreeEval {
 public:
  // One evaluation for the solve P: builds the source octree over the stage positions the prep
  // kernel wrote, the proxies and the per-tile index lists, and runs the gathered pair kernel
  // into this object's partial buffer ([nchunks()][ncomp][slot]), which the epilogue then sums.
  // Nothing is read back except on the first evaluation (the list total that sizes the list
  // buffer): sizes and counts stay on the device, the lists go to a buffer of fixed capacity,
  // and an evaluation whose lists do not fit sums every source directly (exact) and reports the
  // overflow, so the buffer grows before the next one.  After the first evaluation, and while
  // generation() stays the same, a call queues the same launches with the same arguments: the
  // calls can be captured in a CUDA graph and replayed.  `slots` (resident CTAs of the whole
  // GPU) sets how each tile's list is cut into work items, and so the summation order; `grid`
  // caps the pair kernel's persistent grid (0: slots), which changes no result.
  void evaluate(SolvePlan& P, const TreeParams& tp, const PairShape& shape, bool psi, bool precise, bool rcpApprox,
                int slots, int grid, PairTimer* timer, cudaStream_t s);
  // Applies the reports of evaluations since the last call (no synchronisation): grows the list
  // buffer after an overflow; true if that changed the launch arguments (a captured graph of
  // the evaluation must then be rebuilt).  Throws on a traversal stack overflow.
  bool poll();
  // Ready to be captured: sized by a first evaluation, no overflow reported since the last poll,
  // and the list buffer already grown to the capacity a poll set (an evaluation grows it).
  bool ready() const {
    return direct_ || (listCap_ > 0 && bList.bytes >= sizeof(int) * (size_t)listCap_ && !(watch_ && watch_->overflow));
  }
  // Changes whenever buffers or launch arguments change (graphs capture them).
  int generation() const { return generation_; }
  // Records that this solve's evaluation used the direct sum (smaller than TreeParams::minPairs).
  void markDirect(const SolvePlan& P) {
    direct_ = true;
    statsOnDevice_ = false;
    stats_ = TreeStats{};
    stats_.pairs = stats_.directPairs = (double)P.nslots * P.ns;
  }
  double* partial() const { return partial_; }
  int nchunks() const { return nchunks_; }
  // Statistics of the last evaluation (reads the device: synchronises).
  const TreeStats& stats();
  // Frees every device buffer in stream order on `s` and hands the report slot back to its pool
  // from a host function queued there, so that neither this call nor the destructor waits for
  // the device.  A later evaluation starts over (sizing pass included).
  void release(cudaStream_t s);

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
  void ensureWatch();
  Buf bPos, bSp0, bSp1, bInv, bSelf, bGeom, bApprox, bTileGeom, bLen, bFar, bOff, bOrder, bList, bPartial,
      bDev, bCounter, bErr, bSlot, bKey, bKey2, bTemp, bStats;
  std::vector<Buf*> all_{&bPos, &bSp0, &bSp1, &bInv, &bSelf, &bGeom, &bApprox, &bTileGeom, &bLen, &bFar, &bOff,
                         &bOrder, &bList, &bPartial, &bDev, &bCounter, &bErr, &bSlot, &bKey, &bKey2, &bTemp, &bStats};
  double* partial_ = nullptr;
  int nchunks_ = 1;
  int64_t listCap_ = 0;          // entries of the list buffer (0: not sized yet)
  bool direct_ = false;          // the solve is below the size threshold (direct sum)
  int generation_ = 0;
  bool statsOnDevice_ = false;
  TreeWatch* watch_ = nullptr;   // mapped host memory
  TreeWatch* dWatch_ = nullptr;  // its device address
  // the uploaded kernel description (re-uploaded only when it changes)
  TreeDev hDev_{};
  TreeDev* devAt_ = nullptr;
};

// Octree depth whose leaves hold about `leafPoints` of n points on the sphere: the nonempty
// cells of level d number ~4.7 * 4^d (a sphere of radius 1 in a cube of side 2).
int treeDepthFor(int64_t n, int leafPoints);

}  // namespace lpm
