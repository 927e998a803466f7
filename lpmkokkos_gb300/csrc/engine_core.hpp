// engine_core.hpp -- internals of the host engine shared by engine.cpp and server.cpp:
// error handling, device arenas, per-solve plans and batches, and the functions that build
// plans and queue one evaluation or one RK4 step of a batch.
#pragma once

#include "lpm_bve.h"
#include "engine.hpp"
#include "tree.hpp"

#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <exception>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace lpm {

// ---------------------------------------------------------------------------------------
// small utilities
// ---------------------------------------------------------------------------------------
struct Error {
  int code;
  std::string msg;
};

#define LPM_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw Error{LPM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)};            \
  } while (0)

[[noreturn]] inline void fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw Error{code, buf};
}

// Owns a set of device buffers.  By default they come from cudaMalloc/cudaFree; after
// streamOrdered(a, f, pool) they come from `pool` in stream order on `a` and are freed in
// stream order on `f` (the stream of their last use), so neither call waits for work in flight.
// A standard-library exception as a status of the C ABI: no exception may cross extern "C".
inline Error fromStd(const std::exception& e) {
  if (dynamic_cast<const std::bad_alloc*>(&e)) return Error{LPM_ERR_OUT_OF_MEMORY, "host memory exhausted"};
  return Error{LPM_ERR_INTERNAL, e.what()};
}

class DeviceArena {
 public:
  ~DeviceArena() { release(); }
  void streamOrdered(cudaStream_t allocStream, cudaStream_t freeStream, cudaMemPool_t pool) {
    async_ = true;
    allocS_ = allocStream;
    freeS_ = freeStream;
    pool_ = pool;
  }
  template <typename T>
  T* alloc(size_t count) {
    if (count == 0) count = 1;
    void* p = nullptr;
    const cudaError_t e =
        async_ ? cudaMallocFromPoolAsync(&p, count * sizeof(T), pool_, allocS_) : cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      fail(e == cudaErrorMemoryAllocation ? LPM_ERR_OUT_OF_MEMORY : LPM_ERR_CUDA, "device allocation (%zu bytes): %s",
           count * sizeof(T), cudaGetErrorString(e));
    }
    ptrs_.push_back(p);
    bytes_ += count * sizeof(T);
    return static_cast<T*>(p);
  }
  void release() {
    for (void* p : ptrs_) {
      if (async_) cudaFreeAsync(p, freeS_);
      else cudaFree(p);
    }
    ptrs_.clear();
    bytes_ = 0;
  }
  size_t bytes() const { return bytes_; }

 private:
  std::vector<void*> ptrs_;
  size_t bytes_ = 0;
  bool async_ = false;
  cudaStream_t allocS_ = nullptr, freeS_ = nullptr;
  cudaMemPool_t pool_ = nullptr;
};

template <typename T>
inline void upload(T* dst, const std::vector<T>& src, cudaStream_t s) {
  if (!src.empty()) LPM_CUDA(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

// Copy n strided 3-vectors from the device to a host row-major array (synchronises s).
std::vector<double> fetchPoints(const double* p, int64_t n, int64_t si, int64_t sc, cudaStream_t s);

inline uint32_t spread3(uint32_t x) {  // 10-bit value -> every third bit
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
inline uint32_t mortonKey(const double* x) {
  uint32_t q[3];
  for (int c = 0; c < 3; ++c) {
    double t = (x[c] + 1.05) * (1024.0 / 2.1);
    if (!(t >= 0.0)) t = 0.0;  // also catches NaN
    if (t > 1023.0) t = 1023.0;
    q[c] = (uint32_t)t;
  }
  return spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
}

void checkVec(const char* name, const void* p, int64_t n, int64_t si, int64_t sc);

// ---------------------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------------------
enum class Mode { Distinct = 0, Collocated = 1, RK4 = 2 };

// Launch shape used when the autotuner is off: 128 threads x 8 targets (four target pairs per
// thread), 256-source tiles, 2 resident CTAs per SM -- the fastest instantiated shape on GB300
// at icosahedral levels 6 and 7 (RK4 pair launches: 76.7 ms at level 7 against 77.1-80.8 ms for
// the others).  The autotuner may choose another one per problem size.
inline constexpr PairShape kDefaultFP32C{128, 8, 256, 1};
inline constexpr PairShape kFP64Shape{128, 1, 128, 1};

struct SolvePlan {
  Mode mode = Mode::Distinct;
  Precision prec = Precision::FP64;
  ParticleIO io;
  const uint8_t* mask = nullptr;
  bool skipMasked = false, sorted = true;
  int nslots = 0, ns = 0, ntiles = 0, nchunks = 1, tileSize = 1, chunkLen = 0;
  double eps2 = 0.0;
  std::vector<int2> tileSelfHost;
  std::vector<int> tileStart;  // [ntiles + 1] first slot of each target tile (tiles never straddle leaf0)
  int leaf0 = -1;  // symmetric layout: slots [leaf0, nslots) are the sources in source order
  bool symWanted = false;      // the plan was built asking for the symmetric layout ...
  int64_t symMin = 0;          // ... for solves of at least this many leaf sources
  // tree-code target tiles: runs of <= tileSize slots inside one level-3 Morton cell
  int nTreeTiles = 0;
  int2* treeTiles = nullptr;    // [nTreeTiles] {first slot, count}
  int* treeCentres = nullptr;   // [nTreeTiles] centre slot
  DeviceArena mem;
  bool partialReady = false;  // partial-sum buffer allocated (once per plan)
  SolveStage stage{};
  SolveDev dev{};
};

// CUDA-event timing of the pair-kernel launches (enabled by lpm_bve_ctx_set_timing).
struct PairTimer {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
  std::vector<cudaEvent_t> pool;
  double totalMs = 0.0;
  int64_t launches = 0;
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    LPM_CUDA(cudaEventCreate(&e));
    return e;
  }
  void collect() {
    for (auto& pr : pending) {
      LPM_CUDA(cudaEventSynchronize(pr.second));
      float ms = 0.f;
      LPM_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
      totalMs += ms;
      launches += 1;
      pool.push_back(pr.first);
      pool.push_back(pr.second);
    }
    pending.clear();
  }
  ~PairTimer() {
    for (auto& pr : pending) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

class TreeEval;

struct Batch {
  PairTimer* timer = nullptr;  // non-null: bracket each pair launch with events (direct launches only)
  std::vector<std::unique_ptr<SolvePlan>> owned;  // plans owned by this batch (single solves, ensembles)
  std::vector<SolvePlan*> solves;                 // the batch's solves in solve-index order (not owned)
  Precision prec = Precision::FP64;
  PairShape shape = kFP64Shape;
  bool rk4 = false;
  bool precise = false;    // FP32C hi/lo differences (arbitrary distinct targets)
  bool rcpApprox = false;  // FP32C without the Newton step (LPM_BVE_RCP_APPROX)
  int nitems = 0, grid = 0, nPrepBlocks = 0, nSlotBlocks = 0;
  // symmetric leaf x leaf evaluation (single FP32C solves with the symmetric layout): the direct
  // kernel's items over the non-leaf slots and the symmetric kernel's items, each run with its
  // own persistent grid and work counter (counter[0], counter[1])
  bool sym = false;
  WorkItem* symDirectItems = nullptr;
  WorkItem* symItems = nullptr;
  int nSymDirectItems = 0, nSymItems = 0, symDirectGrid = 0, symGrid = 0, symGridPsi = 0;
  std::vector<double> itemPairs;  // target-source pairs of each work item (host, launch order)
  DeviceArena mem;
  WorkItem* items = nullptr;
  SolveDev* solveDev = nullptr;
  SolveStage* stageDev = nullptr;
  int4* prepMap = nullptr;
  int4* slotMap = nullptr;
  int* counter = nullptr;
  // tree code (LPM_BVE_TREECODE): one evaluation state per solve, created on first use, and the
  // epilogue's stage table pointing at their partial sums
  std::vector<std::shared_ptr<TreeEval>> trees;
  SolveStage* treeStageDev = nullptr;
  std::vector<SolveStage> treeStageHost;
  std::vector<char> treeDirect;        // per solve: below TreeParams::minPairs, direct sum
  double treeDirectFor = -1.0;         // minPairs the subset below was built for
  WorkItem* directItems = nullptr;     // pair-kernel items of the direct solves
  int nDirectItems = 0;
  DeviceArena directMem;
  bool treeMode = false;
  TreeParams treeParams;
  int treeGrid = 0;  // cap of the tree pair kernel's persistent grid (0: slots)
  // several tree-code solves: their evaluations run on up to kTreeLanes side streams forked from
  // the batch's stream after the prep kernel and joined before the epilogue (in a captured step,
  // parallel branches), so that one solve's small octree and list kernels overlap another's
  std::vector<cudaStream_t> treeLanes;
  cudaEvent_t treeFork = nullptr;
  std::vector<cudaEvent_t> treeJoin;
  int slots = 0;  // resident CTA slots of the pair kernels (SMs x CTAs per SM)
  // captured RK4 step
  cudaGraphExec_t graph = nullptr;
  bool graphQuirk = false, graphRenorm = false, graphRcp = false, graphTree = false;
  int graphTreeGen = 0;  // the tree evaluations' generation the graph was captured with
  ~Batch() {
    if (graph) cudaGraphExecDestroy(graph);
    for (cudaEvent_t e : treeJoin) cudaEventDestroy(e);
    if (treeFork) cudaEventDestroy(treeFork);
    for (cudaStream_t l : treeLanes) cudaStreamDestroy(l);  // released once their work completes
  }
};

struct DeviceInfo {
  int device = 0, sms = 0;
};


// Shape-independent part of a plan, computed on the host: target slot order, compacted
// source list, and the maps between them.
struct HostPlan {
  int64_t na = 0, nb = 0;
  std::vector<uint8_t> hmask;
  std::vector<int> ids, srcFace, self, srcSlot;
  std::vector<uint32_t> slotKeys;  // Morton key of each slot (sorted plans only)
  int leaf0 = -1;                  // symmetric layout: first leaf slot (-1: plain layout)
  bool symWanted = false;
  int64_t symMin = 0;
};

// symLayout (collocated / RK4 plans, sorted): the non-leaf target slots (vertices, masked faces)
// first in Morton order, then every leaf in source order, so that leaf slot leaf0 + k is source
// k -- the layout of the symmetric leaf x leaf kernel.
// The layout is taken only by solves with at least symMinLeaves leaf sources (below that the
// second launch per evaluation costs more than the halved leaf pairs save).
HostPlan prepareHost(Mode mode, const ParticleIO& io, const uint8_t* mask, bool skipMasked, bool sort,
                     cudaStream_t s, bool symLayout = false, int64_t symMinLeaves = 0);
// Same from host arrays: ha (na x 3) and hb (nb x 3) row-major positions, hmask (nb bytes).
HostPlan prepareHostFromHost(Mode mode, int64_t na, int64_t nb, const double* ha, const double* hb,
                             const uint8_t* hmask, bool skipMasked, bool sort, bool symLayout = false,
                             int64_t symMinLeaves = 0);
// Default symMinLeaves: 64 leaf tiles (icosahedral level 6, cubed sphere level 7 and up).
constexpr int64_t kSymMinLeaves = 65536;
void buildSolve(SolvePlan& P, Mode mode, Precision prec, const ParticleIO& io, const uint8_t* mask, bool skipMasked,
                bool sort, double eps, int tileSize, const HostPlan& H, cudaStream_t s);
int chunkLength(int ns, int srcTile);
// Allocates a plan's partial buffer on first use; builds items, block maps and device tables.
void finalizeBatch(Batch& B, const DeviceInfo& dev, cudaStream_t s);
void refreshTables(Batch& B, cudaStream_t s);
struct EvalNames;
// names: profiler range names of the evaluation's launches (nullptr: no ranges)
void enqueueEval(Batch& B, int prepStage, int stageOut, bool psi, bool velocity, cudaStream_t s,
                 const EvalNames* names = nullptr);
void enqueueStep(Batch& B, bool quirk, bool renorm, cudaStream_t s);
// Uploads a tree-code batch's epilogue stage table when it changed.
void treeStageTable(Batch& B, cudaStream_t s);
// Puts a finalized batch in tree-code mode with evaluators the caller keeps (one per solve, in
// solve order): buffers, list capacity and octree carry over from batch to batch.  Every solve
// takes the tree code.  `s` is the stream the batch will run on (its side streams, created here
// so that a first step can be captured, take its priority).
void attachTrees(Batch& B, const std::vector<std::shared_ptr<TreeEval>>& trees, const TreeParams& tp,
                 cudaStream_t s);

// Snapshot file of a state held in host row-major arrays (snapshot.cpp).
void writeSnapshotHost(const char* path, int seed, int level, int vpf, int64_t nv, int64_t nf, double t, double dt,
                       double omega, const double* vx, const double* vzeta, const double* vvel, const double* fx,
                       const double* fzeta, const double* fvel, const double* farea, const uint8_t* fmask);

}  // namespace lpm
