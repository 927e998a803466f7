// server.cpp -- continuous-batching BVE solve server (include/lpm_bve_server.h).
//
// Two host threads share one GPU:
//   prep       admits queued requests first-come first-served while their estimated device
//              footprint fits the HBM budget, then builds the mesh (cached per seed/level/
//              flags together with its target/source plan) and the pinned host buffer of the
//              initial state (initial vorticity on the host only with the host_ic option).
//   gpu        owns every device object.  It uploads the requests that became ready (upload
//              stream, stream-ordered allocation from a private pool), evaluates their initial
//              vorticity and velocity, and advances every running solve.  Running solves are
//              grouped in size classes (log4 of pairs per evaluation); a class is one batch
//              whose RK4 step is one CUDA graph of 13 launches, each of the four evaluations one
//              pair-kernel launch over all the class's solves, run on the class's lane -- a
//              compute stream whose priority falls with the cost.  Classes advance at their own
//              pace, so a small request does not wait for the steps of a large one.  A class's
//              batch (work items, tables, graph) is rebuilt only when its membership changes.
//              A solve that has taken its steps is copied back into its pinned buffer and its
//              device memory is freed in stream order; the thread sleeps until a host function
//              queued behind a burst of steps, or a new request, wakes it.
// A host function queued on a request's lane behind its copy-back marks it done, returns its
// budget reservation and wakes waiters and the admission loop.
// With LPM_BVE_TREECODE two more threads, tree, take the requests of at least 1e9 pairs per
// evaluation from the gpu thread, upload them and compute their initial velocity with the tree
// code on their own streams -- the first evaluation of a solve sizes its interaction lists, the
// tree code's one read-back -- and hand them back.  The gpu thread then steps them in size
// classes of their own (tree classes: batches in tree-code mode whose steps are captured graphs,
// like the direct classes').  A solve's tree evaluator (octree, lists, buffers) stays with the
// request across batch rebuilds and is freed in stream order when it finishes.  A list that
// outgrows its buffer is summed directly for that evaluation (exact) and flagged; the class then
// runs one step uncaptured, which grows the buffer, and captures its step again.
// A solve's result is bit-identical alone or in any mix: its plan, work items, chunking and
// summation order depend on nothing but its own mesh and the launch shape, fixed per server.

#include "lpm_bve_server.h"
#include "engine_core.hpp"
#include "tree_eval.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <tuple>

struct lpm_bve_server;

namespace lpm {
namespace server {

using Clock = std::chrono::steady_clock;

// One mesh on the host with its RK4 plan (slot order, compacted sources), shared by every
// request on the same (seed, level, skip-masked) key.
struct MeshHost {
  int64_t nv = 0, nf = 0, nl = 0;
  std::vector<double> vx, fx, farea;
  std::vector<uint8_t> fmask;
  HostPlan plan;
};

// Per-request state layout, identical on the host (pinned) and on the device: doubles
// [vx 3nv | vvel 3nv | vzeta nv | fx 3nf | fvel 3nf | fzeta nf | farea nf], then nf mask bytes.
// Vectors are row-major (stride 3, 1), the LayoutRight views of the reference.
struct Layout {
  size_t vx, vvel, vzeta, fx, fvel, fzeta, farea, ndoubles, maskByte, bytes;
  Layout(int64_t nv, int64_t nf) {
    vx = 0;
    vvel = 3 * (size_t)nv;
    vzeta = 6 * (size_t)nv;
    fx = 7 * (size_t)nv;
    fvel = fx + 3 * (size_t)nf;
    fzeta = fvel + 3 * (size_t)nf;
    farea = fzeta + (size_t)nf;
    ndoubles = farea + (size_t)nf;
    maskByte = ndoubles * sizeof(double);
    bytes = (maskByte + (size_t)nf + 255) / 256 * 256;
  }
};

// Page-locked host memory for request states.  cudaHostAlloc is an implicit synchronisation
// point (work issued after it does not overlap work issued before it) and cudaFreeHost waits
// for the device, so requests never call either: they take blocks of slabs that are allocated
// only when the pool must grow (at least kSlabBytes at a time) and kept until the server is
// destroyed.  First fit over an address-ordered free list, neighbours coalesced on free.
class PinnedPool {
 public:
  static constexpr size_t kSlabBytes = size_t(256) << 20;
  static constexpr size_t kAlign = 256;
  ~PinnedPool() {
    for (auto& sl : slabs_) cudaFreeHost(sl.first);
  }
  char* alloc(size_t bytes) {
    bytes = (bytes + kAlign - 1) / kAlign * kAlign;
    std::lock_guard<std::mutex> lk(mu_);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        char* p = it->first;
        const size_t rest = it->second - bytes;
        free_.erase(it);
        if (rest) free_[p + bytes] = rest;
        used_[p] = bytes;
        return p;
      }
    }
    const size_t slab = std::max(kSlabBytes, bytes);
    void* q = nullptr;
    const cudaError_t e = cudaHostAlloc(&q, slab, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      fail(LPM_ERR_OUT_OF_MEMORY, "pinned host memory (%zu bytes): %s", slab, cudaGetErrorString(e));
    }
    char* p = static_cast<char*>(q);
    slabs_.emplace_back(p, slab);
    if (slab > bytes) free_[p + bytes] = slab - bytes;
    used_[p] = bytes;
    return p;
  }
  void release(char* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    auto u = used_.find(p);
    if (u == used_.end()) return;
    size_t len = u->second;
    used_.erase(u);
    auto next = free_.lower_bound(p);
    if (next != free_.end() && p + len == next->first && sameSlab(p, next->first)) {
      len += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == p && sameSlab(prev->first, p)) {
        prev->second += len;
        return;
      }
    }
    free_[p] = len;
  }

 private:
  bool sameSlab(const char* a, const char* b) const {
    for (const auto& sl : slabs_) {
      const bool ina = a >= sl.first && a < sl.first + sl.second, inb = b >= sl.first && b < sl.first + sl.second;
      if (ina || inb) return ina && inb;
    }
    return false;
  }
  std::mutex mu_;
  std::vector<std::pair<char*, size_t>> slabs_;
  std::map<char*, size_t> free_, used_;
};

struct Req {
  int64_t id = 0;
  lpm_bve_request r{};
  int state = LPM_REQ_QUEUED;
  std::string err;
  Clock::time_point tSubmit, tStart, tDone;
  size_t est = 0;
  int64_t nv = 0, nf = 0, nl = 0;
  std::shared_ptr<const MeshHost> mesh;  // held from preparation until the upload
  char* host = nullptr;                  // pinned state buffer (Layout)
  std::vector<double> gc, ga;            // Gaussian-vortex centres (ng x 3) and amplitudes
  // owned by the gpu thread while running
  int cls = 0;                     // size class: log4 of pairs per evaluation
  cudaStream_t lane = nullptr;     // compute stream of its size class
  std::unique_ptr<SolvePlan> plan;
  std::shared_ptr<TreeEval> tree;  // tree-code requests: the solve's evaluator, kept across batches
  DeviceArena mem;
  char* dev = nullptr;
  int stepsDone = 0;
  double pairsPerEval = 0.0;
  lpm_bve_server* owner = nullptr;  // for the host function that marks the request done
};

}  // namespace server
}  // namespace lpm

using namespace lpm;
using namespace lpm::server;

struct lpm_bve_server {
  DeviceInfo dev;
  unsigned flags = 0;
  Precision prec = Precision::FP32C;
  PairShape shape = kDefaultFP32C;
  double eps = 0.0;
  bool skip = false, quirk = true, renorm = false, rcp = false, hostIc = false;
  size_t budget = 0;
  int maxActive = 0;
  cudaStream_t up = nullptr, cap = nullptr;
  std::map<int, cudaStream_t> lanes;  // compute stream per size class (gpu thread creates them)
  int prioLeast = 0, prioGreatest = 0;  // stream priority range of the device
  int slots = 1;                         // resident CTAs of the pair kernel on the whole GPU
  cudaMemPool_t pool = nullptr;
  std::unique_ptr<PinnedPool> pinned = std::make_unique<PinnedPool>();
  // wake-ups of the gpu thread: new requests, finished bursts (host callbacks), stop
  std::mutex wmu;
  std::condition_variable cvWork;
  uint64_t wakeups = 0;

  std::mutex mu;
  std::condition_variable cvPrep, cvDone;
  bool stop = false;
  std::string fatal;  // non-empty once a CUDA error made the server unusable
  std::string err;    // last error of an API call
  int64_t nextId = 1;
  std::map<int64_t, std::unique_ptr<Req>> reqs;
  std::deque<Req*> queued, prepared;
  std::set<Req*> finishing;  // last step and copy-back queued, not yet complete
  size_t reserved = 0;
  int inflight = 0;  // admitted and not finished
  lpm_bve_server_counters st{};
  std::vector<double> latencies;
  std::map<std::tuple<int, int, int>, std::shared_ptr<const MeshHost>> meshes;  // prep thread only
  std::deque<std::tuple<int, int, int>> meshOrder;
  // tree code (LPM_BVE_TREECODE): requests of at least treeMinPairs pairs per evaluation go to a
  // tree thread for their setup and initial velocity, then back to the gpu thread (treeReady)
  bool tree = false;
  double treeMinPairs = 1e9;
  TreeParams treeParams;       // degree 8, theta 0.6, 512 sources per leaf
  int treeSlots = 1;           // resident CTAs of the tree pair kernel on the whole GPU
  std::deque<Req*> treeQueue;  // under mu
  std::deque<Req*> treeReady;  // under mu
  std::condition_variable cvTree;
  std::thread prepT, gpuT;
  std::vector<std::thread> treeT;
};

namespace lpm {
namespace server {
namespace {

double seconds(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

constexpr size_t kMeshCache = 16;

// Device bytes of one request: state, plan (targets, sources, RK4 increments, partial sums)
// and its share of the batch tables; 5 % + 1 MiB for pool granularity.
size_t estimateBytes(Precision prec, const PairShape& shape, bool skip, int64_t nv, int64_t nf, int64_t nl) {
  const Layout L(nv, nf);
  const size_t nslots = (size_t)nv + (size_t)(skip ? nl : nf), ns = (size_t)nl;
  const size_t ts = (size_t)shape.tileSize(), ntiles = (nslots + ts - 1) / ts;
  const int chunk = chunkLength((int)ns, shape.srcTile);
  const size_t nchunks = ns > 0 ? (ns + chunk - 1) / chunk : 1;
  const size_t ncomp = (size_t)pairNumComponents(prec, true);
  size_t plan = 8 * nslots + 12 * ntiles + 8 * ns + 24 * nslots + (prec == Precision::FP32C ? 64 + 28 : 32) * ns +
                4 * 32 * nslots + 8 * nchunks * ncomp * nslots;
  const size_t bs = (size_t)stageBlockSize();
  size_t tables = 2 * (ntiles * nchunks * sizeof(WorkItem) + (2 * nslots / bs + ns / bs + 4) * sizeof(int4) +
                       sizeof(SolveDev) + sizeof(SolveStage));
  const size_t raw = L.bytes + plan + tables;
  return raw + raw / 20 + (1u << 20);
}

// Empty when the request is well formed, else the reason.
std::string validate(const lpm_bve_request& q) {
  if ((q.seed != LPM_SEED_ICOS_TRI && q.seed != LPM_SEED_CUBED) || q.level < 0 || q.level > 10)
    return "seed must be LPM_SEED_ICOS_TRI/CUBED and level 0..10";
  if (q.nsteps < 0 || !std::isfinite(q.dt) || !std::isfinite(q.omega)) return "nsteps must be >= 0 and dt, omega finite";
  if (q.n_gaussians < 0 || q.n_gaussians > LPM_IC_MAX_GAUSSIANS || (q.n_gaussians > 0 && !(q.gauss_width > 0.0)))
    return "0..LPM_IC_MAX_GAUSSIANS Gaussians with a positive width";
  return std::string();
}

int setErr(lpm_bve_server* S, int code, const std::string& msg) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->err = msg;
  return code;
}

// Marks a request failed and returns its reservation (caller holds the lock).
void failLocked(lpm_bve_server* S, Req* r, const std::string& msg) {
  if (r->state == LPM_REQ_DONE || r->state == LPM_REQ_FAILED || r->state == LPM_REQ_CANCELLED) return;
  const bool admitted = r->state != LPM_REQ_QUEUED;
  r->state = LPM_REQ_FAILED;
  r->err = msg;
  r->tDone = Clock::now();
  if (admitted) {
    S->reserved -= r->est;
    S->inflight -= 1;
  }
  S->st.failed += 1;
  S->cvDone.notify_all();
  S->cvPrep.notify_all();
}

// Requests this large take the tree code (LPM_BVE_TREECODE servers).
bool treeSized(const lpm_bve_server* S, int64_t nv, int64_t nf, int64_t nl) {
  return S->tree && (double)(nv + (S->skip ? nl : nf)) * (double)nl >= S->treeMinPairs;
}

std::shared_ptr<const MeshHost> meshFor(lpm_bve_server* S, int seed, int level) {
  const auto key = std::make_tuple(seed, level, S->skip ? 1 : 0);
  auto it = S->meshes.find(key);
  if (it != S->meshes.end()) return it->second;
  auto M = std::make_shared<MeshHost>();
  if (lpm_mesh_counts(seed, level, &M->nv, &M->nf, &M->nl) != LPM_OK)
    fail(LPM_ERR_INVALID_ARGUMENT, "mesh seed %d level %d", seed, level);
  M->vx.resize(3 * (size_t)M->nv);
  M->fx.resize(3 * (size_t)M->nf);
  M->farea.resize((size_t)M->nf);
  M->fmask.resize((size_t)M->nf);
  if (lpm_mesh_build(seed, level, M->vx.data(), M->fx.data(), M->farea.data(), M->fmask.data()) != LPM_OK)
    fail(LPM_ERR_INVALID_ARGUMENT, "mesh seed %d level %d", seed, level);
  // FP32C solves take the symmetric layout (leaf x leaf pairs once) unless the server was created
  // with LPM_BVE_NO_SYMMETRIC or the tree code takes the solve (its tiles follow the Morton order)
  const bool sym = S->prec == Precision::FP32C && !(S->flags & LPM_BVE_NO_SYMMETRIC) &&
                   !treeSized(S, M->nv, M->nf, M->nl);
  M->plan = prepareHostFromHost(Mode::RK4, M->nv, M->nf, M->vx.data(), M->fx.data(), M->fmask.data(), S->skip, true,
                                sym, kSymMinLeaves);
  S->meshes[key] = M;
  S->meshOrder.push_back(key);
  if (S->meshOrder.size() > kMeshCache) {
    S->meshes.erase(S->meshOrder.front());
    S->meshOrder.pop_front();
  }
  return M;
}

// Host side of a request: mesh, pinned buffer, Gaussian-vortex parameters, and -- with the
// host_ic option -- the initial vorticity (RH54 + seeded Gaussian vortices, as
// BVESphere::init_vorticity evaluates an initial condition at vertices and faces); otherwise
// the GPU evaluates it after the upload.  Velocity starts at zero and is computed on the GPU
// before the first step.
void prepare(lpm_bve_server* S, Req* r) {
  r->mesh = meshFor(S, r->r.seed, r->r.level);
  const MeshHost& M = *r->mesh;
  const Layout L(M.nv, M.nf);
  r->host = S->pinned->alloc(L.bytes);
  double* d = reinterpret_cast<double*>(r->host);
  std::memcpy(d + L.vx, M.vx.data(), sizeof(double) * M.vx.size());
  std::memcpy(d + L.fx, M.fx.data(), sizeof(double) * M.fx.size());
  std::memcpy(d + L.farea, M.farea.data(), sizeof(double) * M.farea.size());
  std::memcpy(r->host + L.maskByte, M.fmask.data(), M.fmask.size());
  std::fill(d + L.vvel, d + L.vvel + 3 * M.nv, 0.0);
  std::fill(d + L.fvel, d + L.fvel + 3 * M.nf, 0.0);
  const int ng = r->r.n_gaussians;
  r->gc.assign(3 * (size_t)ng, 0.0);
  r->ga.assign((size_t)ng, 0.0);
  if (ng > 0) lpm_ic_gaussian_params(r->r.ic_seed, ng, -2.0, 2.0, r->gc.data(), r->ga.data());
  if (S->hostIc) {
    lpm_ic_rh54(d + L.vx, M.nv, d + L.vzeta);
    lpm_ic_rh54(d + L.fx, M.nf, d + L.fzeta);
    if (ng > 0) {
      lpm_ic_gaussians_add(d + L.vx, M.nv, r->gc.data(), r->ga.data(), ng, r->r.gauss_width, d + L.vzeta);
      lpm_ic_gaussians_add(d + L.fx, M.nf, r->gc.data(), r->ga.data(), ng, r->r.gauss_width, d + L.fzeta);
    }
  } else {
    std::fill(d + L.vzeta, d + L.vzeta + M.nv, 0.0);
    std::fill(d + L.fzeta, d + L.fzeta + M.nf, 0.0);
  }
}

// Wakes the gpu thread (new work, a finished burst, stop).  Also the host function queued
// behind each burst: it takes only wmu, which no thread holds across a CUDA call.
void wakeGpu(lpm_bve_server* S) {
  {
    std::lock_guard<std::mutex> lk(S->wmu);
    S->wakeups += 1;
  }
  S->cvWork.notify_one();
}
void CUDART_CB burstDone(void* p) { wakeGpu(static_cast<lpm_bve_server*>(p)); }

void prepLoop(lpm_bve_server* S) {
  cudaSetDevice(S->dev.device);
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cvPrep.wait(lk, [&] {
        if (S->stop) return true;
        if (S->queued.empty() || !S->fatal.empty()) return false;
        const Req* h = S->queued.front();
        return S->reserved + h->est <= S->budget && (S->maxActive <= 0 || S->inflight < S->maxActive);
      });
      if (S->stop) return;
      r = S->queued.front();
      S->queued.pop_front();
      r->state = LPM_REQ_PREPARING;
      S->reserved += r->est;
      S->inflight += 1;
    }
    try {
      prepare(S, r);
      {
        std::lock_guard<std::mutex> lk(S->mu);
        if (!S->fatal.empty()) {
          r->mesh.reset();
          failLocked(S, r, "server stopped after a device error: " + S->fatal);
          continue;
        }
        S->prepared.push_back(r);
      }
      wakeGpu(S);
    } catch (const Error& e) {
      std::lock_guard<std::mutex> lk(S->mu);
      r->mesh.reset();
      failLocked(S, r, e.msg);
    } catch (const std::exception& e) {
      std::lock_guard<std::mutex> lk(S->mu);
      r->mesh.reset();
      failLocked(S, r, "preparing the request: " + fromStd(e).msg);
    }
  }
}

int costClass(double pairsPerEval) {
  int c = 0;
  while (pairsPerEval >= 4.0 && c < 40) {
    pairsPerEval /= 4.0;
    ++c;
  }
  return c;
}

// Compute stream of a size class, created on first use: one stream per class, so classes of
// equal priority still run side by side; two classes (a factor 16 in pairs, one mesh level)
// per priority level, the cheapest (up to icosahedral level 4) on the highest priority.
cudaStream_t laneOf(lpm_bve_server* S, int cls) {
  auto it = S->lanes.find(cls);
  if (it != S->lanes.end()) return it->second;
  const int levels = S->prioLeast - S->prioGreatest + 1;
  const int i = std::max(0, std::min(levels - 1, (cls - 11) / 2));
  cudaStream_t l = nullptr;
  LPM_CUDA(cudaStreamCreateWithPriority(&l, cudaStreamNonBlocking, S->prioGreatest + i));
  S->lanes[cls] = l;
  return l;
}

// Uploads a prepared request and builds its plan on stream `s` (stream-ordered allocation, freed
// in order on `freeS`), with target tiles of `tileSize` slots.
void uploadAndPlan(lpm_bve_server* S, Req* r, cudaStream_t s, cudaStream_t freeS, int tileSize) {
  const MeshHost& M = *r->mesh;
  r->nv = M.nv;
  r->nf = M.nf;
  const Layout L(M.nv, M.nf);
  r->mem.streamOrdered(s, freeS, S->pool);
  r->dev = r->mem.alloc<char>(L.bytes);
  LPM_CUDA(cudaMemcpyAsync(r->dev, r->host, L.maskByte + (size_t)M.nf, cudaMemcpyHostToDevice, s));
  double* d = reinterpret_cast<double*>(r->dev);
  if (!S->hostIc) {
    const int ng = r->r.n_gaussians;
    for (const auto& part : {std::make_pair(L.vx, L.vzeta), std::make_pair(L.fx, L.fzeta)}) {
      const int64_t n = part.first == L.vx ? M.nv : M.nf;
      const int rc = lpm_ic_rh54_gaussians_device(d + part.first, n, 3, 1, r->gc.data(), r->ga.data(), ng,
                                                  r->r.gauss_width, d + part.second, (lpm_stream_t)s);
      if (rc != LPM_OK) fail(rc, "initial vorticity on the device: %s", cudaGetErrorString(cudaGetLastError()));
    }
  }
  ParticleIO io;
  io.na = M.nv;
  io.nb = M.nf;
  io.ax = DVec{d + L.vx, 3, 1};
  io.au = DVec{d + L.vvel, 3, 1};
  io.azeta = d + L.vzeta;
  io.bx = DVec{d + L.fx, 3, 1};
  io.bu = DVec{d + L.fvel, 3, 1};
  io.bzeta = d + L.fzeta;
  io.barea = d + L.farea;
  const uint8_t* mask = reinterpret_cast<const uint8_t*>(r->dev + L.maskByte);
  r->plan.reset(new SolvePlan());
  r->plan->mem.streamOrdered(s, freeS, S->pool);
  buildSolve(*r->plan, Mode::RK4, S->prec, io, mask, S->skip, true, S->eps, tileSize, M.plan, s);
  r->plan->stage.dt = r->r.dt;
  r->plan->stage.omega = r->r.omega;
  r->pairsPerEval = (double)r->plan->nslots * r->plan->ns;
}

// A direct-sum request: its size class and lane, then the upload (upload stream, freed in order
// on the lane).
void setupSolve(lpm_bve_server* S, Req* r) {
  const MeshHost& M = *r->mesh;
  r->cls = costClass((double)(M.nv + (S->skip ? M.nl : M.nf)) * (double)M.nl);
  r->lane = laneOf(S, r->cls);
  uploadAndPlan(S, r, S->up, r->lane, S->shape.tileSize());
}

// A batch over solves of one lane, built on stream `s`.  Its pair grid is set by shareSlots before
// its step is captured (initial-velocity batches keep the persistent grid finalizeBatch chose).
// Tree-code requests (each with its evaluator) make a tree-code batch.
std::unique_ptr<Batch> makeBatch(lpm_bve_server* S, const std::vector<Req*>& rs, cudaStream_t lane,
                                 cudaStream_t s) {
  const bool tree = rs.front()->tree != nullptr;
  auto B = std::make_unique<Batch>();
  B->prec = S->prec;
  B->shape = tree ? kTreeShape : S->shape;
  B->rk4 = true;
  B->rcpApprox = S->rcp;
  B->mem.streamOrdered(s, lane, S->pool);
  for (Req* r : rs) B->solves.push_back(r->plan.get());
  B->sym = false;  // solves below the layout's size threshold keep the plain kernel in the same batch
  if (!tree)
    for (const SolvePlan* p : B->solves) B->sym = B->sym || (p->leaf0 >= 0 && p->ns > 0);
  finalizeBatch(*B, S->dev, s);
  if (tree) {
    std::vector<std::shared_ptr<TreeEval>> trees;
    for (Req* r : rs) trees.push_back(r->tree);
    attachTrees(*B, trees, S->treeParams, lane);
    bool sized = true;
    for (Req* r : rs) sized = sized && r->tree->ready();
    if (sized) treeStageTable(*B, s);  // else the first (uncaptured) evaluation uploads it
  }
  return B;
}

// Resident tree pair-kernel CTAs that take the place of `slots` CTAs of the direct kernel.
int treeGridFor(const lpm_bve_server* S, int slots) {
  return std::max(1, (int)((int64_t)slots * S->treeSlots / std::max(1, S->slots)));
}

// Captures one RK4 step of B and installs it in `exec`: updated in place when exec exists (the
// update affects only later launches, so launches in flight keep their parameters), instantiated
// otherwise.  Membership changes then never instantiate or destroy an executable graph.
void installStep(lpm_bve_server* S, Batch& B, cudaGraphExec_t& exec) {
  cudaGraph_t g = nullptr;
  LPM_CUDA(cudaStreamBeginCapture(S->cap, cudaStreamCaptureModeThreadLocal));
  try {
    enqueueStep(B, S->quirk, S->renorm, S->cap);
  } catch (...) {
    cudaStreamEndCapture(S->cap, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  LPM_CUDA(cudaStreamEndCapture(S->cap, &g));
  cudaError_t ie = cudaSuccess;
  if (exec) {
    cudaGraphExecUpdateResultInfo info{};
    if (cudaGraphExecUpdate(exec, g, &info) != cudaSuccess) {  // topology changed: rebuild
      (void)cudaGetLastError();
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
  }
  if (!exec) ie = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  LPM_CUDA(ie);
}

// Host function queued on a request's lane behind its copy-back: the request is done.  It runs
// on a CUDA thread and takes only S->mu, which no thread holds across a CUDA call.
void CUDART_CB requestDone(void* p) {
  Req* r = static_cast<Req*>(p);
  lpm_bve_server* S = r->owner;
  std::lock_guard<std::mutex> lk(S->mu);
  S->finishing.erase(r);
  if (r->state != LPM_REQ_RUNNING) return;  // failed meanwhile by a device error
  r->state = LPM_REQ_DONE;
  r->tDone = Clock::now();
  S->reserved -= r->est;
  S->inflight -= 1;
  S->st.completed += 1;
  S->latencies.push_back(seconds(r->tSubmit, r->tDone));
  S->cvDone.notify_all();
  S->cvPrep.notify_all();
}

// Queues the copy of a finished solve's state into its pinned buffer, frees its device memory
// in stream order, and queues requestDone behind both on the request's lane.
void finish(lpm_bve_server* S, Req* r) {
  const Layout L(r->nv, r->nf);
  LPM_CUDA(cudaMemcpyAsync(r->host, r->dev, L.ndoubles * sizeof(double), cudaMemcpyDeviceToHost, r->lane));
  if (r->tree) {  // the tree evaluator's buffers, in stream order (a batch may still hold it)
    r->tree->release(r->lane);
    r->tree.reset();
  }
  r->plan.reset();
  r->mem.release();
  r->dev = nullptr;
  r->owner = S;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->finishing.insert(r);
  }
  LPM_CUDA(cudaLaunchHostFunc(r->lane, requestDone, r));
}

// Size classes and lanes.  Solves are grouped by cost (log4 of target-source pairs per
// evaluation); a class is one batch whose RK4 step is one captured graph, launched on the
// class's own stream (lane).  Every class advances at its own pace: up to kMaxInflight bursts
// in flight, a burst being as many steps as take about kBurstMs (measured per class, moving
// average), capped by the fewest steps any of its solves has left.
//
// The classes share the GPU in space, not in time: each class's pair kernel is persistent
// with a grid from shareSlots, which splits the resident CTA slots water-filling by demand
// (classes with few work items get what they need, the rest is split evenly).  Measured on
// GB300, stream priorities do not let a later kernel overtake the pending CTAs of a running
// grid: a level-7 step beside non-persistent level-8 kernels took as long as a level-8 step.
// With disjoint slot shares every class's kernels are resident at once, and a class's
// prep / epilogue kernels run in the slots its own pair kernel frees; a small reserve of
// slots stays out of every share for newcomers.  A host function queued
// behind each burst wakes this thread when it completes.
constexpr int kMaxInflight = 2;
constexpr int kTreeClass = 64;    // tree classes: kTreeClass + log4 of the direct-sum pairs
constexpr int kReserveFrac = 38;  // 1/38 of the slots: 8 of the 304 of the default shape
constexpr double kLongStepMs = 50.0;
constexpr double kBurstMs = 10.0;
constexpr int kMaxStepsPerBurst = 256;

struct Burst {
  cudaEvent_t e0, e1;
  int steps;
};

struct SizeClass {
  std::vector<Req*> solves;
  std::unique_ptr<Batch> batch;
  cudaStream_t lane = nullptr;
  bool changed = false;
  bool tree = false;   // a tree class (tree-code batch)
  bool stale = false;  // tree class: the captured step predates the batch or its grid
  int treeGen = -1;    // tree class: the evaluators' generations the step was captured with
  double msPerStep = -1.0;  // moving average of measured step time (-1: not measured yet)
  double pairsPerStep = 0.0;
  std::deque<Burst> inflight;
};

// Step time of a class before it has been measured: 4 evaluations at a nominal pair rate plus
// the 13 launches of a graph-replayed step.
double modelMs(const lpm_bve_server* S, double pairsPerStep) {
  const double rate = S->prec == Precision::FP32C ? 2.2e12 : 1.2e10;
  return pairsPerStep / rate * 1e3 + 0.06;
}

// Pair-kernel grid of every class with a batch: water-filling of the resident CTA slots by
// demand (work items), cheapest demand first.
std::map<int, int> shareSlots(const std::map<int, SizeClass>& classes, int slots) {
  std::vector<std::pair<int, int>> demand;  // (work items, class)
  for (const auto& kv : classes)
    if (kv.second.batch) demand.emplace_back(std::max(1, kv.second.batch->nitems), kv.first);
  std::sort(demand.begin(), demand.end());
  std::map<int, int> grid;
  int remaining = slots;
  for (size_t i = 0; i < demand.size(); ++i) {
    const int share = std::max(1, remaining / (int)(demand.size() - i));
    const int g = std::min(demand[i].first, share);
    grid[demand[i].second] = g;
    remaining = std::max(0, remaining - g);
  }
  return grid;
}

// The tree thread: uploads a tree-code request and builds its plan on this thread's stream,
// computes the initial velocity with a one-solve tree-code batch -- the solve's first evaluation,
// which sizes its interaction lists (one read-back of this stream) -- and hands the request to
// the gpu thread, whose tree classes step it.  Its result depends on nothing but the request.
void treeSetup(lpm_bve_server* S, cudaStream_t ts, Req* r) {
  {
    std::lock_guard<std::mutex> lk(S->mu);
    r->state = LPM_REQ_RUNNING;
    r->tStart = Clock::now();
  }
  uploadAndPlan(S, r, ts, ts, kTreeShape.tileSize());
  r->tree = std::make_shared<TreeEval>();
  {
    std::unique_ptr<Batch> B = makeBatch(S, {r}, ts, ts);
    enqueueEval(*B, 0, 0, false, true, ts);
  }
  LPM_CUDA(cudaStreamSynchronize(ts));
  std::lock_guard<std::mutex> lk(S->mu);
  S->st.tree_equiv_pairs += r->pairsPerEval;
  if (S->stop) {  // the gpu thread has gone: nobody steps it
    r->tree->release(ts);
    r->tree.reset();
    r->plan.reset();
    r->mem.release();
    failLocked(S, r, "server destroyed before the request ran");
    return;
  }
  S->treeReady.push_back(r);
}

void treeLoop(lpm_bve_server* S) {
  cudaSetDevice(S->dev.device);
  cudaStream_t ts = nullptr;
  std::string setupErr;
  if (cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking) != cudaSuccess) setupErr = "tree thread: no stream";
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cvTree.wait(lk, [&] { return S->stop || !S->treeQueue.empty(); });
      if (S->stop) {
        for (Req* q : S->treeQueue) failLocked(S, q, "server destroyed before the request ran");
        S->treeQueue.clear();
        break;
      }
      r = S->treeQueue.front();
      S->treeQueue.pop_front();
    }
    std::string err;
    try {
      if (!setupErr.empty()) fail(LPM_ERR_INTERNAL, "%s", setupErr.c_str());
      treeSetup(S, ts, r);
    } catch (const Error& e) {
      err = e.msg;
    } catch (const std::exception& e) {
      err = fromStd(e).msg;
    }
    r->mesh.reset();
    if (!err.empty()) {
      if (ts) cudaStreamSynchronize(ts);
      r->tree.reset();
      r->plan.reset();
      r->mem.release();
      std::lock_guard<std::mutex> lk(S->mu);
      failLocked(S, r, "tree code: " + err);
    }
    wakeGpu(S);
  }
  if (ts) {
    cudaStreamSynchronize(ts);
    cudaStreamDestroy(ts);
  }
}

void gpuLoop(lpm_bve_server* S) {
  cudaSetDevice(S->dev.device);
  std::map<int, SizeClass> classes;  // key: size class
  std::map<int, cudaGraphExec_t> execs;  // captured step per size class, kept while the server lives
  int nActive = 0;
  cudaEvent_t upEv = nullptr;
  std::vector<cudaEvent_t> evPool;
  uint64_t seenWakeups = 0;
  Clock::time_point tick = Clock::now();
  auto getEvent = [&]() {
    if (!evPool.empty()) {
      cudaEvent_t e = evPool.back();
      evPool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    LPM_CUDA(cudaEventCreate(&e));
    return e;
  };
  auto allActive = [&]() {
    std::vector<Req*> v;
    for (auto& kv : classes) v.insert(v.end(), kv.second.solves.begin(), kv.second.solves.end());
    return v;
  };
  std::string fatal;
  try {
    LPM_CUDA(cudaEventCreateWithFlags(&upEv, cudaEventDisableTiming));
    for (;;) {
      std::vector<Req*> joiners, treeJoin;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) break;
        joiners.assign(S->prepared.begin(), S->prepared.end());
        S->prepared.clear();
        treeJoin.assign(S->treeReady.begin(), S->treeReady.end());
        S->treeReady.clear();
        const Clock::time_point now = Clock::now();
        if (nActive > 0) S->st.busy_s += seconds(tick, now);
        tick = now;
      }
      // 1. upload the newcomers (a failure that leaves the context usable fails the request only)
      std::vector<Req*> ok;
      auto failJoiner = [&](Req* r, const std::string& msg) {
        cudaStreamSynchronize(S->up);  // copies into the request's memory may be queued
        r->plan.reset();
        r->mem.release();
        std::lock_guard<std::mutex> lk(S->mu);
        failLocked(S, r, msg);
      };
      for (Req* r : joiners) {
        if (treeSized(S, r->mesh->nv, r->mesh->nf, r->mesh->nl)) {
          std::lock_guard<std::mutex> lk(S->mu);  // large enough for the tree code: a tree thread
          S->treeQueue.push_back(r);
          S->cvTree.notify_one();
          continue;
        }
        try {
          setupSolve(S, r);
          ok.push_back(r);
        } catch (const Error& e) {
          if (e.code == LPM_ERR_CUDA) throw;
          failJoiner(r, e.msg);
        } catch (const std::exception& e) {
          failJoiner(r, fromStd(e).msg);
        }
        r->mesh.reset();
      }
      std::map<int, std::vector<Req*>> byClass;
      for (Req* r : ok) byClass[r->cls].push_back(r);
      std::vector<std::pair<cudaStream_t, std::unique_ptr<Batch>>> inits;  // initial velocity per class
      std::vector<Req*> noSteps;
      // tree-code requests arrive set up, with their initial velocity: straight into a tree class
      for (Req* r : treeJoin) {
        r->cls = kTreeClass + costClass(r->pairsPerEval);
        r->lane = laneOf(S, r->cls);
        r->mem.streamOrdered(S->up, r->lane, S->pool);  // freed in order on the lane from now on
        r->plan->mem.streamOrdered(S->up, r->lane, S->pool);
        if (r->r.nsteps > 0) {
          SizeClass& C = classes[r->cls];
          C.lane = r->lane;
          C.tree = true;
          C.solves.push_back(r);
          C.changed = true;
          ++nActive;
        } else {
          noSteps.push_back(r);
        }
      }
      for (auto& kv : byClass) {
        const cudaStream_t lane = kv.second.front()->lane;
        inits.emplace_back(lane, makeBatch(S, kv.second, lane, S->up));
        for (Req* r : kv.second) {
          if (r->r.nsteps > 0) {
            SizeClass& C = classes[kv.first];
            C.lane = lane;
            C.solves.push_back(r);
            C.changed = true;
            ++nActive;
          } else {
            noSteps.push_back(r);
          }
        }
      }
      // 2. rebuild the batches of classes whose membership changed
      std::vector<cudaStream_t> waiting;
      for (auto it = classes.begin(); it != classes.end();) {
        SizeClass& C = it->second;
        if (C.changed) {
          C.batch.reset();  // an in-flight graph is freed when it completes; tables in stream order
          C.pairsPerStep = 0.0;
          for (Req* r : C.solves) C.pairsPerStep += 4.0 * r->pairsPerEval;
          if (!C.solves.empty()) {
            C.batch = makeBatch(S, C.solves, C.lane, S->up);
            C.batch->grid = 0;  // installed below with its share of the slots
            C.stale = true;
            waiting.push_back(C.lane);
          }
          C.changed = false;
        }
        if (C.solves.empty() && C.inflight.empty()) {
          it = classes.erase(it);
        } else {
          ++it;
        }
      }
      // the SM slots of the pair kernels, shared among the classes with a batch; kReserveFrac of
      // them stay free so that a class that arrives while a long step is in flight (launched
      // with the old shares) finds resident room at once
      const int reserve = std::max(1, S->slots / kReserveFrac);
      for (const auto& kg : shareSlots(classes, std::max(1, S->slots - reserve))) {
        SizeClass& C = classes[kg.first];
        if (C.batch->grid != kg.second) {
          C.batch->grid = kg.second;
          // the symmetric evaluation's two launches run one after the other on the class's lane,
          // each within the same share
          C.batch->symDirectGrid = std::min(C.batch->nSymDirectItems, kg.second);
          C.batch->symGrid = std::min(C.batch->nSymItems, kg.second);
          C.batch->symGridPsi = std::min(C.batch->nSymItems, kg.second);
          C.batch->treeGrid = treeGridFor(S, kg.second);
          if (C.tree)
            C.stale = true;  // captured before its next burst, once every list is sized
          else
            installStep(S, *C.batch, execs[kg.first]);
        }
      }
      for (auto& in : inits) waiting.push_back(in.first);
      if (!waiting.empty()) {
        LPM_CUDA(cudaEventRecord(upEv, S->up));
        std::sort(waiting.begin(), waiting.end());
        waiting.erase(std::unique(waiting.begin(), waiting.end()), waiting.end());
        for (cudaStream_t l : waiting) LPM_CUDA(cudaStreamWaitEvent(l, upEv, 0));
      }
      for (auto& in : inits) {
        enqueueEval(*in.second, 0, 0, false, true, in.first);
        in.second.reset();
      }
      if (!ok.empty() || !treeJoin.empty()) {
        std::lock_guard<std::mutex> lk(S->mu);
        const Clock::time_point now = Clock::now();
        for (Req* r : ok) {
          r->state = LPM_REQ_RUNNING;
          r->tStart = now;
          S->st.pairs += r->pairsPerEval;
        }
        S->st.max_running_seen = std::max<int>(S->st.max_running_seen, nActive);
      }
      for (Req* r : noSteps) finish(S, r);
      // 3. fold in the bursts that have completed
      for (auto& kv : classes) {
        SizeClass& C = kv.second;
        while (!C.inflight.empty()) {
          const cudaError_t q = cudaEventQuery(C.inflight.front().e1);
          if (q == cudaErrorNotReady) break;
          LPM_CUDA(q);
          const Burst b = C.inflight.front();
          C.inflight.pop_front();
          float ms = 0.f;
          LPM_CUDA(cudaEventElapsedTime(&ms, b.e0, b.e1));
          const double per = ms / b.steps;
          C.msPerStep = C.msPerStep > 0 ? 0.5 * (C.msPerStep + per) : per;
          evPool.push_back(b.e0);
          evPool.push_back(b.e1);
        }
      }
      // 4. launch bursts on every lane that has room
      bool launched = false;
      double pairs = 0.0, treePairs = 0.0;
      int64_t solveSteps = 0, classSteps = 0;
      for (auto& kv : classes) {
        SizeClass& C = kv.second;
        for (;;) {
          if (!C.batch || C.solves.empty()) break;
          const double est = C.msPerStep > 0 ? C.msPerStep : modelMs(S, C.pairsPerStep);
          // a class with long steps keeps one in flight, so a new slot share applies sooner
          const int maxInflight = est >= kLongStepMs ? 1 : kMaxInflight;
          if ((int)C.inflight.size() >= maxInflight) break;
          int left = INT_MAX;
          for (Req* r : C.solves) left = std::min(left, r->r.nsteps - r->stepsDone);
          // a tree class whose lists outgrew their buffers since the last burst runs one step
          // uncaptured (its evaluations grow them); otherwise its step is captured again when
          // the batch, its grid or an evaluator's buffers changed
          bool uncaptured = false;
          if (C.tree) {
            bool ready = true;
            int gen = 0;
            for (Req* r : C.solves) {
              r->tree->poll();
              ready = ready && r->tree->ready();
              gen += r->tree->generation();
            }
            if (!ready) {
              uncaptured = true;
            } else if (C.stale || gen != C.treeGen || !execs[kv.first]) {
              treeStageTable(*C.batch, C.lane);
              installStep(S, *C.batch, execs[kv.first]);
              C.stale = false;
              C.treeGen = gen;
            }
          }
          const int k = uncaptured ? 1 : std::max(1, std::min({(int)(kBurstMs / est), left, kMaxStepsPerBurst}));
          Burst b{getEvent(), getEvent(), k};
          LPM_CUDA(cudaEventRecord(b.e0, C.lane));
          if (uncaptured) {
            enqueueStep(*C.batch, S->quirk, S->renorm, C.lane);
          } else {
            const cudaGraphExec_t exec = execs[kv.first];
            for (int j = 0; j < k; ++j) LPM_CUDA(cudaGraphLaunch(exec, C.lane));
          }
          LPM_CUDA(cudaEventRecord(b.e1, C.lane));
          LPM_CUDA(cudaLaunchHostFunc(C.lane, burstDone, S));
          C.inflight.push_back(b);
          launched = true;
          classSteps += k;
          std::vector<Req*> still;
          for (Req* r : C.solves) {
            r->stepsDone += k;
            (C.tree ? treePairs : pairs) += 4.0 * k * r->pairsPerEval;  // tree: direct-sum equivalent
            solveSteps += k;
            if (r->stepsDone >= r->r.nsteps) {
              finish(S, r);
              C.changed = true;
              --nActive;
            } else {
              still.push_back(r);
            }
          }
          C.solves.swap(still);
          if (C.changed) {
            C.batch.reset();
            break;  // rebuilt before its next burst
          }
        }
      }
      if (launched) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->st.steps_run += classSteps;
        S->st.solve_steps += solveSteps;
        S->st.pairs += pairs;
        S->st.tree_equiv_pairs += treePairs;
      }
      bool rebuild = false;
      for (auto& kv : classes) rebuild |= kv.second.changed;
      if (launched || rebuild || !ok.empty() || !treeJoin.empty()) continue;
      // 5. nothing to launch: sleep until a burst completes or work arrives (bounded wait)
      {
        std::unique_lock<std::mutex> lk(S->wmu);
        S->cvWork.wait_for(lk, std::chrono::milliseconds(nActive > 0 ? 50 : 500),
                           [&] { return S->wakeups != seenWakeups; });
        seenWakeups = S->wakeups;
      }
      for (auto& ln : S->lanes) {  // a device error stops the host functions: find it here
        const cudaError_t q = cudaStreamQuery(ln.second);
        if (q != cudaErrorNotReady) LPM_CUDA(q);
      }
    }
  } catch (const Error& e) {
    fatal = e.msg;
  } catch (const std::exception& e) {
    fatal = fromStd(e).msg;
  }
  if (!fatal.empty()) {  // every request not yet done fails; submit refuses new ones
    std::lock_guard<std::mutex> lk(S->mu);
    S->fatal = fatal;
    for (Req* r : allActive()) failLocked(S, r, "server stopped: " + fatal);
    for (Req* r : S->prepared) failLocked(S, r, "server stopped: " + fatal);
    for (Req* r : S->queued) failLocked(S, r, "server stopped: " + fatal);
    for (Req* r : S->finishing) failLocked(S, r, "server stopped: " + fatal);
    S->prepared.clear();
    S->queued.clear();
    S->finishing.clear();
    S->cvDone.notify_all();
  }
  std::vector<Req*> active = allActive();
  {
    std::lock_guard<std::mutex> lk(S->mu);  // set up by a tree thread, not yet in a class
    active.insert(active.end(), S->treeReady.begin(), S->treeReady.end());
    S->treeReady.clear();
  }
  for (auto& kv : classes) kv.second.batch.reset();
  for (auto& ln : S->lanes) cudaStreamSynchronize(ln.second);
  cudaStreamSynchronize(S->up);
  for (Req* r : active) {  // abandoned at shutdown
    r->tree.reset();
    r->plan.reset();
    r->mem.release();
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (Req* r : active) failLocked(S, r, "server destroyed while the request was running");
  }
  for (auto& kv : classes)
    for (auto& b : kv.second.inflight) {
      cudaEventDestroy(b.e0);
      cudaEventDestroy(b.e1);
    }
  for (cudaEvent_t e : evPool) cudaEventDestroy(e);
  for (auto& kv : execs)
    if (kv.second) cudaGraphExecDestroy(kv.second);
  if (upEv) cudaEventDestroy(upEv);
}

Req* findLocked(lpm_bve_server* S, int64_t id) {
  auto it = S->reqs.find(id);
  return it == S->reqs.end() ? nullptr : it->second.get();
}

}  // namespace
}  // namespace server
}  // namespace lpm

extern "C" {

int lpm_bve_server_create(const lpm_bve_server_opts* opts, lpm_bve_server** out) {
  if (!out) return LPM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::unique_ptr<lpm_bve_server> S;
  auto undo = [&](const Error& e) {
    std::fprintf(stderr, "lpm_bve_server_create: %s\n", e.msg.c_str());
    if (S && S->pool) cudaMemPoolDestroy(S->pool);
    if (S)
      for (cudaStream_t s : {S->up, S->cap})
        if (s) cudaStreamDestroy(s);
    return e.code;
  };
  try {
    S = std::make_unique<lpm_bve_server>();
    int dev = opts ? opts->device : -1;
    if (dev < 0) LPM_CUDA(cudaGetDevice(&dev));
    LPM_CUDA(cudaSetDevice(dev));
    S->dev.device = dev;
    LPM_CUDA(cudaDeviceGetAttribute(&S->dev.sms, cudaDevAttrMultiProcessorCount, dev));
    int major = 0, minor = 0;
    LPM_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    LPM_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3)
      fail(LPM_ERR_NOT_SUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a (GB300) only", dev, major,
           minor);
    const unsigned flags = opts ? opts->flags : LPM_BVE_FP32C;
    const double eps = opts ? opts->eps : 0.0;
    if (!(eps >= 0.0) || !std::isfinite(eps)) fail(LPM_ERR_INVALID_ARGUMENT, "server: eps must be finite and >= 0");
    if ((flags & LPM_BVE_TREECODE) && !(flags & LPM_BVE_FP32C))
      fail(LPM_ERR_NOT_SUPPORTED, "server: the tree code needs LPM_BVE_FP32C");
    S->tree = flags & LPM_BVE_TREECODE;
    S->flags = flags;
    S->prec = (flags & LPM_BVE_FP32C) ? Precision::FP32C : Precision::FP64;
    S->shape = S->prec == Precision::FP32C ? kDefaultFP32C : kFP64Shape;
    S->eps = eps;
    S->skip = flags & LPM_BVE_SKIP_MASKED_TARGETS;
    S->quirk = !(flags & LPM_BVE_RK4_FIX_QUIRK);
    S->renorm = flags & LPM_BVE_RENORM;
    S->rcp = flags & LPM_BVE_RCP_APPROX;
    S->hostIc = opts && opts->host_ic;
    S->maxActive = opts ? opts->max_active : 0;
    size_t freeB = 0, totalB = 0;
    LPM_CUDA(cudaMemGetInfo(&freeB, &totalB));
    S->budget = (opts && opts->hbm_budget_bytes) ? opts->hbm_budget_bytes : freeB / 10 * 8;
    S->st.budget_bytes = S->budget;
    int leastP = 0, greatestP = 0;
    LPM_CUDA(cudaDeviceGetStreamPriorityRange(&leastP, &greatestP));
    // uploads, initial-vorticity kernels and plan tables: small and waited for by the gpu
    // thread, so they take the highest priority (else they queue behind a large class's CTAs)
    LPM_CUDA(cudaStreamCreateWithPriority(&S->up, cudaStreamNonBlocking, greatestP));
    S->prioLeast = leastP;
    S->prioGreatest = greatestP;
    S->slots = std::max(1, pairBlocksPerSM(S->prec, S->shape, false) * S->dev.sms);
    S->treeParams.minPairs = 0.0;  // the server routes by treeMinPairs; a tree class takes the tree code
    S->treeSlots = kTreeShape.minBlocks * S->dev.sms;
    LPM_CUDA(cudaStreamCreateWithFlags(&S->cap, cudaStreamNonBlocking));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    LPM_CUDA(cudaMemPoolCreate(&S->pool, &props));
    uint64_t keep = UINT64_MAX;  // keep freed blocks for the next requests
    LPM_CUDA(cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  } catch (const Error& e) {
    return undo(e);
  } catch (const std::exception& e) {
    return undo(fromStd(e));
  }
  lpm_bve_server* raw = S.release();
  try {
    raw->prepT = std::thread(prepLoop, raw);
    raw->gpuT = std::thread(gpuLoop, raw);
    // two tree threads: a large request's setup need not wait for another's (each thread has
    // its own stream)
    if (raw->tree)
      for (int k = 0; k < 2; ++k) raw->treeT.emplace_back(treeLoop, raw);
  } catch (const std::exception& e) {  // no thread: stop and join the one that started
    std::fprintf(stderr, "lpm_bve_server_create: %s\n", e.what());
    lpm_bve_server_destroy(raw);
    return LPM_ERR_INTERNAL;
  }
  *out = raw;
  return LPM_OK;
}

int lpm_bve_server_submit(lpm_bve_server* S, const lpm_bve_request* req, int64_t* id) {
  if (!S || !req) return LPM_ERR_INVALID_ARGUMENT;
  const lpm_bve_request& q = *req;
  const std::string bad = validate(q);
  if (!bad.empty()) return setErr(S, LPM_ERR_INVALID_ARGUMENT, "submit: " + bad);
  int64_t nv = 0, nf = 0, nl = 0;
  lpm_mesh_counts(q.seed, q.level, &nv, &nf, &nl);
  try {
    auto r = std::make_unique<Req>();
    r->r = q;
    r->nv = nv;
    r->nf = nf;
    r->nl = nl;
    r->est = estimateBytes(S->prec, S->shape, S->skip, nv, nf, nl);
    r->tSubmit = Clock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->fatal.empty()) {
      S->err = "server stopped after a device error: " + S->fatal;
      return LPM_ERR_CUDA;
    }
    if (r->est > S->budget) {
      char buf[192];
      std::snprintf(buf, sizeof(buf), "submit: request needs about %zu bytes, the HBM budget is %zu", r->est,
                    S->budget);
      S->err = buf;
      return LPM_ERR_ADMISSION;
    }
    Req* raw = r.get();
    raw->id = S->nextId;
    S->reqs.emplace(raw->id, std::move(r));  // a throw here changes nothing
    try {
      S->queued.push_back(raw);
    } catch (...) {
      S->reqs.erase(raw->id);
      throw;
    }
    S->nextId += 1;
    if (id) *id = raw->id;
    S->st.submitted += 1;
    S->cvPrep.notify_one();
    return LPM_OK;
  } catch (const std::exception& e) {
    const Error x = fromStd(e);
    return setErr(S, x.code, "submit: " + x.msg);
  }
}

int lpm_bve_server_estimate(const lpm_bve_server_opts* opts, const lpm_bve_request* req, size_t* bytes) {
  if (!req || !bytes) return LPM_ERR_INVALID_ARGUMENT;
  if (!validate(*req).empty()) return LPM_ERR_INVALID_ARGUMENT;
  const unsigned flags = opts ? opts->flags : LPM_BVE_FP32C;
  const Precision prec = (flags & LPM_BVE_FP32C) ? Precision::FP32C : Precision::FP64;
  int64_t nv = 0, nf = 0, nl = 0;
  lpm_mesh_counts(req->seed, req->level, &nv, &nf, &nl);
  *bytes = estimateBytes(prec, prec == Precision::FP32C ? kDefaultFP32C : kFP64Shape,
                         flags & LPM_BVE_SKIP_MASKED_TARGETS, nv, nf, nl);
  return LPM_OK;
}

int lpm_bve_server_wait(lpm_bve_server* S, int64_t id, double timeout_s) {
  if (!S) return LPM_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(S->mu);
  Req* r = findLocked(S, id);
  if (!r) {
    S->err = "wait: unknown request id";
    return LPM_ERR_STATE;
  }
  auto finished = [&] { return r->state == LPM_REQ_DONE || r->state == LPM_REQ_FAILED || r->state == LPM_REQ_CANCELLED; };
  if (timeout_s < 0) {
    S->cvDone.wait(lk, finished);
  } else if (!S->cvDone.wait_for(lk, std::chrono::duration<double>(timeout_s), finished)) {
    return LPM_ERR_TIMEOUT;
  }
  if (r->state != LPM_REQ_DONE) {
    S->err = r->state == LPM_REQ_CANCELLED ? "request was cancelled" : "request failed: " + r->err;
    return LPM_ERR_STATE;
  }
  return LPM_OK;
}

int lpm_bve_server_status(lpm_bve_server* S, int64_t id, int* state) {
  if (!S || !state) return LPM_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->mu);
  Req* r = findLocked(S, id);
  if (!r) return LPM_ERR_STATE;
  *state = r->state;
  return LPM_OK;
}

int lpm_bve_server_cancel(lpm_bve_server* S, int64_t id) {
  if (!S) return LPM_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->mu);
  Req* r = findLocked(S, id);
  if (!r || r->state != LPM_REQ_QUEUED) {
    S->err = "cancel: only a request still waiting for admission can be cancelled";
    return LPM_ERR_STATE;
  }
  S->queued.erase(std::find(S->queued.begin(), S->queued.end(), r));
  r->state = LPM_REQ_CANCELLED;
  r->tDone = Clock::now();
  S->st.cancelled += 1;
  S->cvDone.notify_all();
  S->cvPrep.notify_all();
  return LPM_OK;
}

int lpm_bve_server_result(lpm_bve_server* S, int64_t id, int64_t* nverts, int64_t* nfaces, double* vx, double* vzeta,
                          double* vvel, double* fx, double* fzeta, double* fvel) {
  if (!S) return LPM_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->mu);
  Req* r = findLocked(S, id);
  if (!r) {
    S->err = "result: unknown request id";
    return LPM_ERR_STATE;
  }
  if (nverts) *nverts = r->nv;
  if (nfaces) *nfaces = r->nf;
  if (!vx && !vzeta && !vvel && !fx && !fzeta && !fvel) return LPM_OK;
  if (r->state != LPM_REQ_DONE || !r->host) {
    S->err = "result: request has not finished (or was released)";
    return LPM_ERR_STATE;
  }
  const Layout L(r->nv, r->nf);
  const double* d = reinterpret_cast<const double*>(r->host);
  auto put = [](double* dst, const double* src, size_t n) {
    if (dst) std::memcpy(dst, src, n * sizeof(double));
  };
  put(vx, d + L.vx, 3 * (size_t)r->nv);
  put(vvel, d + L.vvel, 3 * (size_t)r->nv);
  put(vzeta, d + L.vzeta, (size_t)r->nv);
  put(fx, d + L.fx, 3 * (size_t)r->nf);
  put(fvel, d + L.fvel, 3 * (size_t)r->nf);
  put(fzeta, d + L.fzeta, (size_t)r->nf);
  return LPM_OK;
}

int lpm_bve_server_snapshot(lpm_bve_server* S, int64_t id, const char* path) {
  if (!S || !path) return LPM_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->mu);
  Req* r = findLocked(S, id);
  if (!r || r->state != LPM_REQ_DONE || !r->host) {
    S->err = "snapshot: request has not finished (or was released)";
    return LPM_ERR_STATE;
  }
  try {
    const Layout L(r->nv, r->nf);
    const double* d = reinterpret_cast<const double*>(r->host);
    int vpf = 0;
    lpm_mesh_face_verts(r->r.seed, r->r.level, nullptr, &vpf);
    writeSnapshotHost(path, r->r.seed, r->r.level, vpf, r->nv, r->nf, r->r.nsteps * r->r.dt, r->r.dt, r->r.omega,
                      d + L.vx, d + L.vzeta, d + L.vvel, d + L.fx, d + L.fzeta, d + L.fvel, d + L.farea,
                      reinterpret_cast<const uint8_t*>(r->host + L.maskByte));
  } catch (const Error& e) {
    S->err = e.msg;
    return e.code;
  } catch (const std::exception& e) {
    const Error x = fromStd(e);
    S->err = x.msg;
    return x.code;
  }
  return LPM_OK;
}

int lpm_bve_server_release(lpm_bve_server* S, int64_t id) {
  if (!S) return LPM_ERR_INVALID_ARGUMENT;
  std::unique_ptr<Req> r;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return LPM_ERR_STATE;
    const int st = it->second->state;
    if (st != LPM_REQ_DONE && st != LPM_REQ_FAILED && st != LPM_REQ_CANCELLED) {
      S->err = "release: request has not finished";
      return LPM_ERR_STATE;
    }
    r = std::move(it->second);
    S->reqs.erase(it);
  }
  S->pinned->release(r->host);
  return LPM_OK;
}

int lpm_bve_server_timing(lpm_bve_server* S, int64_t id, double* total_s, double* wait_s, double* run_s) {
  if (!S) return LPM_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->mu);
  Req* r = findLocked(S, id);
  if (!r || r->state != LPM_REQ_DONE) return LPM_ERR_STATE;
  if (total_s) *total_s = seconds(r->tSubmit, r->tDone);
  if (wait_s) *wait_s = seconds(r->tSubmit, r->tStart);
  if (run_s) *run_s = seconds(r->tStart, r->tDone);
  return LPM_OK;
}

int lpm_bve_server_latency(lpm_bve_server* S, const double* q, int nq, double* out) {
  if (!S || (nq > 0 && (!q || !out))) return LPM_ERR_INVALID_ARGUMENT;
  std::vector<double> v;
  try {
    std::lock_guard<std::mutex> lk(S->mu);
    v = S->latencies;
  } catch (const std::exception& e) {
    const Error x = fromStd(e);
    return setErr(S, x.code, "latency: " + x.msg);
  }
  if (v.empty()) return LPM_ERR_STATE;
  std::sort(v.begin(), v.end());
  for (int i = 0; i < nq; ++i) {  // nearest-rank quantile
    if (!(q[i] >= 0.0 && q[i] <= 1.0)) return LPM_ERR_INVALID_ARGUMENT;
    const size_t k = (size_t)std::ceil(q[i] * (double)v.size());
    out[i] = v[k == 0 ? 0 : k - 1];
  }
  return LPM_OK;
}

int lpm_bve_server_stats(lpm_bve_server* S, lpm_bve_server_counters* out) {
  if (!S || !out) return LPM_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  out->queued = (int64_t)S->queued.size();
  int64_t running = 0;
  for (auto& kv : S->reqs) running += kv.second->state == LPM_REQ_RUNNING;
  out->running = running;
  out->reserved_bytes = S->reserved;
  out->budget_bytes = S->budget;
  return LPM_OK;
}

const char* lpm_bve_server_last_error(lpm_bve_server* S) { return S ? S->err.c_str() : "null server"; }

int lpm_bve_server_destroy(lpm_bve_server* S) {
  if (!S) return LPM_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cvPrep.notify_all();
  S->cvTree.notify_all();
  wakeGpu(S);
  if (S->prepT.joinable()) S->prepT.join();
  if (S->gpuT.joinable()) S->gpuT.join();
  for (auto& t : S->treeT)
    if (t.joinable()) t.join();
  cudaSetDevice(S->dev.device);
  for (auto& ln : S->lanes) cudaStreamSynchronize(ln.second);
  cudaStreamSynchronize(S->up);
  for (auto& kv : S->reqs) {
    kv.second->tree.reset();
    kv.second->plan.reset();
    kv.second->mem.release();
  }
  for (auto& ln : S->lanes) cudaStreamSynchronize(ln.second);
  S->reqs.clear();
  S->pinned.reset();
  cudaMemPoolDestroy(S->pool);
  cudaStreamDestroy(S->up);
  for (auto& ln : S->lanes) cudaStreamDestroy(ln.second);
  cudaStreamDestroy(S->cap);
  delete S;
  return LPM_OK;
}

}  // extern "C"
