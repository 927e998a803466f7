// engine.cpp -- host engine of the BVE path: contexts, plans, RK4 driver, CUDA graphs,
// and the C ABI of include/lpm_bve.h.
//
// A plan fixes everything about a problem that does not change from step to step: the
// spatially sorted target slots, the compacted (unmasked) source list, the per-tile
// self-exclusion ranges and the work items of the pair kernel.  Building it copies the
// positions and the mask to the host once; later calls with the same geometry only queue
// kernels.  One RK4 step is 13 launches (prep, pair, epilogue per evaluation plus the
// combine); it is captured once into a CUDA graph and replayed.

#include "lpm_bve.h"
#include "lpm_bve_ensemble.h"
#include "engine.hpp"
#include "engine_core.hpp"
#include "tree_eval.hpp"
#include "nvtx.hpp"

#include <algorithm>
#include <array>
#include <map>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace lpm {

// Copy n strided 3-vectors from the device to a host row-major array (synchronises s).
std::vector<double> fetchPoints(const double* p, int64_t n, int64_t si, int64_t sc, cudaStream_t s) {
  std::vector<double> out(3 * (size_t)n);
  if (n == 0) return out;
  const int64_t span = (n - 1) * si + 2 * sc + 1;
  std::vector<double> raw((size_t)span);
  LPM_CUDA(cudaMemcpyAsync(raw.data(), p, sizeof(double) * span, cudaMemcpyDeviceToHost, s));
  LPM_CUDA(cudaStreamSynchronize(s));
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) out[3 * i + c] = raw[(size_t)(i * si + c * sc)];
  return out;
}

void checkVec(const char* name, const void* p, int64_t n, int64_t si, int64_t sc) {
  if (n < 0) fail(LPM_ERR_INVALID_ARGUMENT, "%s: negative count", name);
  if (n > 0 && !p) fail(LPM_ERR_INVALID_ARGUMENT, "%s: null pointer with n = %lld", name, (long long)n);
  if (n > 0 && (si < 0 || sc < 0 || (si == 0 && n > 1)))
    fail(LPM_ERR_INVALID_ARGUMENT, "%s: invalid strides (%lld, %lld)", name, (long long)si, (long long)sc);
  if (n > (int64_t)INT_MAX / 4) fail(LPM_ERR_NOT_SUPPORTED, "%s: %lld points exceed the supported size", name, (long long)n);
}

HostPlan prepareHost(Mode mode, const ParticleIO& io, const uint8_t* mask, bool skipMasked, bool sort,
                     cudaStream_t s, bool symLayout, int64_t symMinLeaves) {
  std::vector<uint8_t> hmask((size_t)io.nb, 0);
  if (mask && io.nb > 0) {
    LPM_CUDA(cudaMemcpyAsync(hmask.data(), mask, (size_t)io.nb, cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaStreamSynchronize(s));
  }
  std::vector<double> ha, hb;
  if (sort) {
    if (mode != Mode::Collocated) ha = fetchPoints(io.ax.p, io.na, io.ax.si, io.ax.sc, s);
    hb = fetchPoints(io.bx.p, io.nb, io.bx.si, io.bx.sc, s);
  }
  return prepareHostFromHost(mode, io.na, io.nb, ha.empty() ? nullptr : ha.data(), hb.empty() ? nullptr : hb.data(),
                             hmask.data(), skipMasked, sort, symLayout, symMinLeaves);
}

HostPlan prepareHostFromHost(Mode mode, int64_t na, int64_t nb, const double* ha, const double* hb,
                             const uint8_t* hmaskIn, bool skipMasked, bool sort, bool symLayout,
                             int64_t symMinLeaves) {
  HostPlan H;
  H.na = na;
  H.nb = nb;
  std::vector<uint8_t>& hmask = H.hmask;
  hmask.assign((size_t)nb, 0);
  if (hmaskIn && nb > 0) std::copy(hmaskIn, hmaskIn + nb, hmask.begin());

  // Target slots: particle ids (a: id = i; face f: id = na + f).  With the symmetric layout the
  // leaves are left out here and appended in source order below.
  int64_t nleaves = 0;
  for (int64_t f = 0; f < nb; ++f) nleaves += hmask[f] ? 0 : 1;
  const bool sym = symLayout && sort && mode != Mode::Distinct && nleaves >= std::max<int64_t>(1, symMinLeaves);
  H.symWanted = symLayout;
  H.symMin = symMinLeaves;
  std::vector<int> ids;
  if (mode != Mode::Collocated)
    for (int64_t i = 0; i < na; ++i) ids.push_back((int)i);
  if (mode != Mode::Distinct)
    for (int64_t f = 0; f < nb; ++f)
      if (!(skipMasked && hmask[f]) && !(sym && !hmask[f])) ids.push_back((int)(na + f));
  std::vector<int> srcFace;
  for (int64_t f = 0; f < nb; ++f)
    if (!hmask[f]) srcFace.push_back((int)f);

  if (sort) {
    auto keyOf = [&](int id) { return id < na ? mortonKey(&ha[3 * (size_t)id]) : mortonKey(&hb[3 * (size_t)(id - na)]); };
    std::vector<std::pair<uint32_t, int>> kv(ids.size());
    for (size_t i = 0; i < ids.size(); ++i) kv[i] = {keyOf(ids[i]), ids[i]};
    std::sort(kv.begin(), kv.end());
    for (size_t i = 0; i < ids.size(); ++i) ids[i] = kv[i].second;
    H.slotKeys.resize(ids.size());
    for (size_t i = 0; i < ids.size(); ++i) H.slotKeys[i] = kv[i].first;
    std::vector<std::pair<uint32_t, int>> ks(srcFace.size());
    for (size_t i = 0; i < srcFace.size(); ++i) ks[i] = {mortonKey(&hb[3 * (size_t)srcFace[i]]), srcFace[i]};
    std::sort(ks.begin(), ks.end());
    for (size_t i = 0; i < srcFace.size(); ++i) srcFace[i] = ks[i].second;
    if (sym) {
      H.leaf0 = (int)ids.size();
      for (size_t i = 0; i < srcFace.size(); ++i) {
        ids.push_back((int)(na + srcFace[i]));
        H.slotKeys.push_back(ks[i].first);
      }
    }
  }
  const int nslots = (int)ids.size(), ns = (int)srcFace.size();
  std::vector<int> srcOf((size_t)nb, -1), slotOf((size_t)nb, -1);
  for (int i = 0; i < ns; ++i) srcOf[srcFace[i]] = i;
  std::vector<int> self((size_t)nslots, -1);
  for (int t = 0; t < nslots; ++t)
    if (ids[t] >= na) {
      const int f = (int)(ids[t] - na);
      slotOf[f] = t;
      self[t] = srcOf[f];
    }
  std::vector<int> srcSlot((size_t)ns, -1);
  for (int i = 0; i < ns; ++i) srcSlot[i] = slotOf[srcFace[i]];
  H.ids = std::move(ids);
  H.srcFace = std::move(srcFace);
  H.self = std::move(self);
  H.srcSlot = std::move(srcSlot);
  return H;
}

// Builds the per-solve device buffers for target tiles of `tileSize` from a host plan.
void buildSolve(SolvePlan& P, Mode mode, Precision prec, const ParticleIO& io, const uint8_t* mask, bool skipMasked,
                bool sort, double eps, int tileSize, const HostPlan& H, cudaStream_t s) {
  P.mode = mode;
  P.prec = prec;
  P.io = io;
  P.mask = mask;
  P.skipMasked = skipMasked;
  P.sorted = sort;
  P.eps2 = eps * eps;
  P.tileSize = tileSize;
  const int64_t na = H.na;
  const std::vector<uint8_t>& hmask = H.hmask;
  const std::vector<int>& ids = H.ids;
  const std::vector<int>& srcFace = H.srcFace;
  const std::vector<int>& self = H.self;
  const std::vector<int>& srcSlot = H.srcSlot;
  const int nslots = (int)ids.size(), ns = (int)srcFace.size();

  P.nslots = nslots;
  P.ns = ns;
  P.leaf0 = H.leaf0;
  P.symWanted = H.symWanted;
  P.symMin = H.symMin;
  // Target tiles of tileSize slots; with the symmetric layout a tile boundary falls at leaf0, so
  // no tile mixes the Morton-ordered non-leaf slots with the leaves (a mixed tile would join
  // distant parts of the sphere).
  P.tileStart.clear();
  for (int t = 0; t < nslots;) {
    P.tileStart.push_back(t);
    const int end = (H.leaf0 > 0 && t < H.leaf0) ? H.leaf0 : nslots;
    t = std::min(end, t + tileSize);
  }
  P.ntiles = (int)P.tileStart.size();
  P.tileStart.push_back(nslots);
  std::vector<int> tileOf((size_t)nslots);
  for (int t = 0; t < P.ntiles; ++t)
    for (int q = P.tileStart[t]; q < P.tileStart[t + 1]; ++q) tileOf[q] = t;
  P.tileSelfHost.assign((size_t)P.ntiles, make_int2(INT_MAX, -1));
  for (int t = 0; t < nslots; ++t)
    if (self[t] >= 0) {
      int2& r = P.tileSelfHost[tileOf[t]];
      r.x = std::min(r.x, self[t]);
      r.y = std::max(r.y, self[t]);
    }
  // Tile centres: the target nearest the middle of each tile that is not a masked face
  // (masked parents can sit on a leaf and run away; vertices and leaves stay on the sphere).
  auto centreOf = [&](int t0, int cnt) {
    const int mid = t0 + cnt / 2;
    for (int d = 0; d < cnt; ++d) {
      const int a = mid - d, b = mid + d;
      auto ok = [&](int q) { return q >= t0 && q < t0 + cnt && (ids[q] < na || !hmask[ids[q] - na]); };
      if (ok(a)) return a;
      if (ok(b)) return b;
    }
    return mid;
  };
  std::vector<int> tileCentre((size_t)P.ntiles);
  for (int t = 0; t < P.ntiles; ++t) tileCentre[t] = centreOf(P.tileStart[t], P.tileStart[t + 1] - P.tileStart[t]);
  // Tree-code tiles: the same slot order cut into runs of at most tileSize slots that never
  // cross a level-3 Morton cell (a run across a cell boundary can join distant parts of the
  // sphere, and its one bounding sphere would then accept no far field).
  std::vector<int2> treeTiles;
  std::vector<int> treeCentres;
  for (int t = 0, start = 0; t <= nslots; ++t) {
    const bool cut = t == nslots || t - start == tileSize || (t == H.leaf0 && t > start) ||
                     (!H.slotKeys.empty() && t > start && (H.slotKeys[t] >> 21) != (H.slotKeys[start] >> 21));
    if (cut && t > start) {
      treeTiles.push_back(make_int2(start, t - start));
      treeCentres.push_back(centreOf(start, t - start));
      start = t;
    }
  }
  P.nTreeTiles = (int)treeTiles.size();

  DeviceArena& M = P.mem;
  M.release();
  int* dPerm = M.alloc<int>(nslots);
  int* dSelf = M.alloc<int>(nslots);
  int2* dTileSelf = M.alloc<int2>(P.ntiles);
  int* dTileCentre = M.alloc<int>(P.ntiles);
  int* dSrcFace = M.alloc<int>(ns);
  int* dSrcSlot = M.alloc<int>(ns);
  double* dTx = M.alloc<double>(3 * (size_t)nslots);
  upload(dPerm, ids, s);
  upload(dSelf, self, s);
  upload(dTileSelf, P.tileSelfHost, s);
  upload(dTileCentre, tileCentre, s);
  P.treeTiles = M.alloc<int2>(std::max<size_t>(1, treeTiles.size()));
  P.treeCentres = M.alloc<int>(std::max<size_t>(1, treeCentres.size()));
  upload(P.treeTiles, treeTiles, s);
  upload(P.treeCentres, treeCentres, s);
  upload(dSrcFace, srcFace, s);
  upload(dSrcSlot, srcSlot, s);

  SolveStage& S = P.stage;
  S = SolveStage{};
  S.io = io;
  S.perm = dPerm;
  S.srcFace = dSrcFace;
  S.srcSlot = dSrcSlot;
  S.tx = dTx;
  if (prec == Precision::FP32C) {
    S.sp0 = M.alloc<float4>(ns);
    S.sp1 = M.alloc<float4>(ns);
  } else {
    S.sd = M.alloc<double4_32a>(ns);
  }
  if (mode == Mode::RK4) {
    for (int k = 0; k < 4; ++k) {
      S.kx[k] = M.alloc<double>(3 * (size_t)nslots);
      S.kz[k] = M.alloc<double>(nslots);
    }
  }
  S.nslots = nslots;
  S.ns = ns;
  S.leaf0 = H.leaf0;
  if (H.leaf0 >= 0 && prec == Precision::FP32C) {  // reverse sums of the symmetric leaf kernel
    S.rev = M.alloc<unsigned long long>(4 * (size_t)std::max(1, ns));
    S.revBad = M.alloc<int>(std::max(1, ns));
  }

  SolveDev& D = P.dev;
  D = SolveDev{};
  D.tx = dTx;
  D.sp0 = S.sp0;
  D.sp1 = S.sp1;
  D.sd = S.sd;
  D.self = dSelf;
  D.tileSelf = dTileSelf;
  D.tileCentre = dTileCentre;
  D.nslots = nslots;
  D.ns = ns;
  D.tileSize = tileSize;
  D.eps2 = P.eps2;
  D.leaf0 = H.leaf0;
  D.rev = S.rev;
  D.revBad = S.revBad;
}

// Source chunking of one solve.  The rule depends on the solve alone (never on the other
// solves of a batch), so a target's summation order -- and therefore its result, bit for
// bit -- is the same whether the solve runs alone, in an ensemble or inside the server.
// Up to kChunksPerTile chunks of at least kMinChunkTiles source tiles each.
constexpr int kChunksPerTile = 8;
constexpr int kMinChunkTiles = 4;

int chunkLength(int ns, int srcTile) {
  if (ns <= 0) return srcTile;
  const int minLen = kMinChunkTiles * srcTile;
  int nch = std::max(1, std::min(kChunksPerTile, (ns + minLen - 1) / minLen));
  int len = (ns + nch - 1) / nch;
  return (len + srcTile - 1) / srcTile * srcTile;
}

// Allocates partial buffers; builds items, block maps and device tables for the batch.
void finalizeBatch(Batch& B, const DeviceInfo& dev, cudaStream_t s) {
  const bool anyPsi = true;  // partial buffers sized for the stream function as well
  const int ncomp = pairNumComponents(B.prec, anyPsi);
  const int perSM = std::max(1, pairBlocksPerSM(B.prec, B.shape, false));
  const int slots = std::max(1, dev.sms * perSM);
  const int srcTile = B.shape.srcTile;
  std::vector<WorkItem> items;
  for (size_t m = 0; m < B.solves.size(); ++m) {
    SolvePlan& P = *B.solves[m];
    const int chunkLen = chunkLength(P.ns, srcTile);
    P.chunkLen = chunkLen;
    P.nchunks = P.ns > 0 ? (P.ns + chunkLen - 1) / chunkLen : 1;
    if (!P.partialReady) {
      double* partial = P.mem.alloc<double>((size_t)P.nchunks * ncomp * std::max(1, P.nslots));
      P.stage.partial = partial;
      P.dev.partial = partial;
      P.partialReady = true;
    }
    P.stage.nchunks = P.nchunks;
    P.dev.nchunks = P.nchunks;
    for (int t = 0; t < P.ntiles; ++t)
      for (int c = 0; c < P.nchunks; ++c) {
        WorkItem w{};
        w.solve = (int)m;
        w.tile = t;
        w.s0 = std::min(P.ns, c * chunkLen);
        w.s1 = std::min(P.ns, (c + 1) * chunkLen);
        w.chunk = c;
        w.tbeg = P.tileStart[t];
        w.tend = P.tileStart[t + 1];
        items.push_back(w);
      }
  }
  if (B.solves.size() > 1) {  // longest items first: the tail of the schedule is short items
    std::stable_sort(items.begin(), items.end(), [&](const WorkItem& a, const WorkItem& b) {
      const int64_t ca = (int64_t)(a.s1 - a.s0) * std::min(B.shape.tileSize(), B.solves[a.solve]->nslots);
      const int64_t cb = (int64_t)(b.s1 - b.s0) * std::min(B.shape.tileSize(), B.solves[b.solve]->nslots);
      return ca > cb;
    });
  }
  B.nitems = (int)items.size();
  B.grid = std::min(B.nitems, slots);
  B.slots = slots;
  B.itemPairs.resize(items.size());
  for (size_t i = 0; i < items.size(); ++i)
    B.itemPairs[i] = (double)(items[i].tend - items[i].tbeg) * (items[i].s1 - items[i].s0);

  // Symmetric leaf x leaf evaluation: the direct kernel keeps each solve's non-leaf target
  // tiles (vertices, masked parents; slots [0, leaf0)), the symmetric kernel takes the upper
  // triangle of its leaf tiles.  Row I (leaf tile I against tiles I..NT-1) is cut into the
  // solve's nchunks segments; segment c writes partial chunk c of tile I's slots (an empty
  // segment writes zeros), so the epilogue's fixed-order chunk sum covers every leaf slot.  The
  // cut depends on the solve alone, and the reverse sums are exact integer adds, so a solve's
  // result is the same alone, in an ensemble or in the server.
  std::vector<WorkItem> symDirect, symItems;
  if (B.sym) {
    for (const WorkItem& w : items)  // solves without the layout keep every tile here
      if (B.solves[w.solve]->leaf0 < 0 || w.tbeg < B.solves[w.solve]->leaf0) symDirect.push_back(w);
    for (size_t m = 0; m < B.solves.size(); ++m) {
      const SolvePlan& P = *B.solves[m];
      if (P.leaf0 < 0) continue;
      const int nt = (P.ns + kSymTile - 1) / kSymTile;
      for (int I = 0; I < nt; ++I) {
        const int len = nt - I;
        for (int c = 0; c < P.nchunks; ++c) {
          WorkItem w{};
          w.solve = (int)m;
          w.tile = I;
          w.s0 = I + (int)((int64_t)len * c / P.nchunks);
          w.s1 = I + (int)((int64_t)len * (c + 1) / P.nchunks);
          w.chunk = c;
          symItems.push_back(w);
        }
      }
    }
    std::stable_sort(symItems.begin(), symItems.end(),
                     [](const WorkItem& a, const WorkItem& b) { return a.s1 - a.s0 > b.s1 - b.s0; });
    B.nSymDirectItems = (int)symDirect.size();
    B.nSymItems = (int)symItems.size();
    B.symDirectGrid = std::min(B.nSymDirectItems, slots);
    B.symGrid = std::min(B.nSymItems, std::max(1, dev.sms * pairSymBlocksPerSM(false)));
    B.symGridPsi = std::min(B.nSymItems, std::max(1, dev.sms * pairSymBlocksPerSM(true)));
  }

  const int bs = stageBlockSize();
  std::vector<int4> prepMap, slotMap;
  for (size_t m = 0; m < B.solves.size(); ++m) {
    const SolvePlan& P = *B.solves[m];
    for (int i = 0; i < P.nslots; i += bs) {
      prepMap.push_back(make_int4((int)m, i, 0, 0));
      slotMap.push_back(make_int4((int)m, i, 0, 0));
    }
  }
  for (size_t m = 0; m < B.solves.size(); ++m) {
    const SolvePlan& P = *B.solves[m];
    for (int i = 0; i < P.ns; i += bs) prepMap.push_back(make_int4((int)m, i, 1, 0));
  }
  B.nPrepBlocks = (int)prepMap.size();
  B.nSlotBlocks = (int)slotMap.size();

  B.mem.release();
  B.items = B.mem.alloc<WorkItem>(items.size());
  B.solveDev = B.mem.alloc<SolveDev>(B.solves.size());
  B.stageDev = B.mem.alloc<SolveStage>(B.solves.size());
  B.prepMap = B.mem.alloc<int4>(prepMap.size());
  B.slotMap = B.mem.alloc<int4>(slotMap.size());
  B.counter = B.mem.alloc<int>(2);
  if (B.sym) {
    B.symDirectItems = B.mem.alloc<WorkItem>(symDirect.size());
    B.symItems = B.mem.alloc<WorkItem>(symItems.size());
    upload(B.symDirectItems, symDirect, s);
    upload(B.symItems, symItems, s);
  }
  upload(B.items, items, s);
  upload(B.prepMap, prepMap, s);
  upload(B.slotMap, slotMap, s);
  std::vector<SolveDev> sd;
  std::vector<SolveStage> ss;
  for (auto& p : B.solves) {
    sd.push_back(p->dev);
    ss.push_back(p->stage);
  }
  upload(B.solveDev, sd, s);
  upload(B.stageDev, ss, s);
  LPM_CUDA(cudaMemsetAsync(B.counter, 0, 2 * sizeof(int), s));
  LPM_CUDA(cudaStreamSynchronize(s));  // host vectors above go out of scope
}

// Re-uploads the per-solve parameter tables (caller pointers, dt, Omega, eps).
void refreshTables(Batch& B, cudaStream_t s) {
  std::vector<SolveDev> sd;
  std::vector<SolveStage> ss;
  for (auto& p : B.solves) {
    sd.push_back(p->dev);
    ss.push_back(p->stage);
  }
  upload(B.solveDev, sd, s);
  upload(B.stageDev, ss, s);
  LPM_CUDA(cudaStreamSynchronize(s));
}

// Side streams of a batch's tree-code evaluations (created on first use, with the priority of
// the stream the batch runs on) and the fork / join events.
constexpr int kTreeLanes = 4;
int ensureTreeLanes(Batch& B, cudaStream_t s, int want) {
  if ((int)B.treeLanes.size() < want) {
    int prio = 0;
    LPM_CUDA(cudaStreamGetPriority(s, &prio));
    if (!B.treeFork) LPM_CUDA(cudaEventCreateWithFlags(&B.treeFork, cudaEventDisableTiming));
    while ((int)B.treeLanes.size() < want) {
      cudaStream_t l = nullptr;
      cudaEvent_t e = nullptr;
      LPM_CUDA(cudaStreamCreateWithPriority(&l, cudaStreamNonBlocking, prio));
      B.treeLanes.push_back(l);
      LPM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      B.treeJoin.push_back(e);
    }
  }
  return want;
}

// One evaluation of the direct sums for every solve of the batch.
void enqueueEval(Batch& B, int prepStage, int stageOut, bool psi, bool velocity, cudaStream_t s,
                 const EvalNames* names) {
  {
    std::unique_ptr<NvtxRange> r(names ? new NvtxRange(names->prep) : nullptr);
    LPM_CUDA(launchPrep(B.stageDev, B.prepMap, B.nPrepBlocks, prepStage, B.prec, B.counter, s));
  }
  std::unique_ptr<NvtxRange> pairRange(names ? new NvtxRange(names->pair) : nullptr);
  if (B.treeMode) {  // tree code: per solve octree, lists and gathered pair kernel; one epilogue
    const size_t n = B.solves.size();
    int ntree = 0;
    for (size_t m = 0; m < n; ++m) ntree += B.treeDirect[m] ? 0 : 1;
    const int lanes = ntree > 1 ? ensureTreeLanes(B, s, std::min(ntree, kTreeLanes)) : 0;
    if (lanes > 0) {  // fork before the direct launch, so that both run side by side
      LPM_CUDA(cudaEventRecord(B.treeFork, s));
      for (int k = 0; k < lanes; ++k) LPM_CUDA(cudaStreamWaitEvent(B.treeLanes[k], B.treeFork, 0));
    }
    // solves below the size threshold: one persistent direct launch over their work items
    if (B.nDirectItems > 0)
      LPM_CUDA(launchPair(B.prec, B.shape, psi, B.precise, B.rcpApprox, B.solveDev, B.directItems, B.nDirectItems,
                          B.counter, std::min(B.nDirectItems, B.slots), s));
    for (size_t m = 0, j = 0; m < n; ++m) {
      TreeEval& T = *B.trees[m];
      if (B.treeDirect[m]) {
        T.markDirect(*B.solves[m]);
        continue;
      }
      const cudaStream_t ts = lanes > 0 ? B.treeLanes[j++ % lanes] : s;
      T.evaluate(*B.solves[m], B.treeParams, B.shape, psi, B.precise, B.rcpApprox, B.slots, B.treeGrid, B.timer, ts);
    }
    for (int k = 0; k < lanes; ++k) {
      LPM_CUDA(cudaEventRecord(B.treeJoin[k], B.treeLanes[k]));
      LPM_CUDA(cudaStreamWaitEvent(s, B.treeJoin[k], 0));
    }
    pairRange.reset();
    treeStageTable(B, s);
    std::unique_ptr<NvtxRange> epi(names ? new NvtxRange(names->epilogue) : nullptr);
    LPM_CUDA(launchEpilogue(B.treeStageDev, B.slotMap, B.nSlotBlocks, B.prec, psi, velocity, stageOut, s));
    return;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (B.timer) {
    e0 = B.timer->get();
    e1 = B.timer->get();
    LPM_CUDA(cudaEventRecord(e0, s));
  }
  // symmetric leaf x leaf evaluation (velocity, and the stream function when asked)
  const bool sym = B.sym && !B.precise;
  if (sym) {
    LPM_CUDA(launchPair(B.prec, B.shape, psi, false, B.rcpApprox, B.solveDev, B.symDirectItems, B.nSymDirectItems,
                        B.counter, B.symDirectGrid, s));
    LPM_CUDA(launchPairSym(psi, B.rcpApprox, B.solveDev, B.symItems, B.nSymItems, B.counter + 1,
                           psi ? B.symGridPsi : B.symGrid, s));
  } else {
    LPM_CUDA(launchPair(B.prec, B.shape, psi, B.precise, B.rcpApprox, B.solveDev, B.items, B.nitems, B.counter,
                        B.grid, s));
  }
  if (B.timer) {
    LPM_CUDA(cudaEventRecord(e1, s));
    B.timer->pending.emplace_back(e0, e1);
  }
  pairRange.reset();
  std::unique_ptr<NvtxRange> epi(names ? new NvtxRange(names->epilogue) : nullptr);
  LPM_CUDA(launchEpilogue(B.stageDev, B.slotMap, B.nSlotBlocks, B.prec, psi, velocity, stageOut, s, sym));
}

// The epilogue's stage table of a tree-code batch: each solve's stage with its tree partial sums.
// Uploaded only when it changes, so that a captured step holds no upload from pageable memory.
void treeStageTable(Batch& B, cudaStream_t s) {
  const size_t n = B.solves.size();
  std::vector<SolveStage> cur(n);
  for (size_t m = 0; m < n; ++m) {
    cur[m] = B.solves[m]->stage;
    const TreeEval& T = *B.trees[m];
    if (!B.treeDirect[m] && T.partial()) {
      cur[m].partial = T.partial();
      cur[m].nchunks = T.nchunks();
    }
  }
  if (B.treeStageHost.size() != n || std::memcmp(cur.data(), B.treeStageHost.data(), n * sizeof(SolveStage)) != 0) {
    B.treeStageHost = cur;
    LPM_CUDA(cudaMemcpyAsync(B.treeStageDev, B.treeStageHost.data(), n * sizeof(SolveStage), cudaMemcpyHostToDevice, s));
  }
}

// One RK4 step (src/LpmBVERK4_Impl.hpp:42-130) for every solve of the batch, its launches named
// after the reference's (:64-126; vertex and face work is fused into one launch here).
void enqueueStep(Batch& B, bool quirk, bool renorm, cudaStream_t s) {
  static const EvalNames kStage[4] = {
      {"RK4-0 positions", "RK4-0 vertex velocity + face velocity", "RK4-0 velocity out"},
      {"RK4-2 vertex and face update (x + x1/2)", "RK4-2 vertex velocity + face velocity",
       "RK4-2 vertex vorticity + face vorticity"},
      {"RK4-3 vertex and face update (x + x2/2)", "RK4-3 vertex velocity + face velocity",
       "RK4-3 vertex vorticity + face vorticity"},
      {"RK4-4 vertex and face update (x + x3)", "RK4-4 vertex velocity + face velocity",
       "RK4-4 vertex vorticity + face vorticity"}};
  enqueueEval(B, 1, 1, false, true, s, &kStage[1]);   // RK4-2: x + x_1/2
  enqueueEval(B, 2, 2, false, true, s, &kStage[2]);   // RK4-3: x + x_2/2
  enqueueEval(B, 3, 3, false, true, s, &kStage[3]);   // RK4-4: x + x_3
  {
    NvtxRange r("RK4 vertex update + face update");
    LPM_CUDA(launchCombine(B.stageDev, B.slotMap, B.nSlotBlocks, quirk, renorm, s));
  }
  enqueueEval(B, 0, 0, false, true, s, &kStage[0]);   // RK4-0: u at the new positions
}

}  // namespace lpm

// ---------------------------------------------------------------------------------------
// context and C ABI
// ---------------------------------------------------------------------------------------
struct lpm_bve_ctx {
  lpm::TreeParams treeParams;                 // tree-code parameters (lpm_bve_ctx_set_treecode)
  std::shared_ptr<lpm::TreeEval> lastTree;    // tree state of the last tree-code evaluation
  lpm::DeviceInfo dev;
  int autotune = 0, verbose = 0;
  std::string err;
  cudaStream_t capture = nullptr;  // private stream for graph capture
  // cached plans
  // the last velocity plan of each kind, [0] distinct targets, [1] collocated: BVESphere::
  // init_vorticity and every stream-function diagnostic alternate a vertex (distinct) and a face
  // (collocated) evaluation on the same sources, so both stay cached instead of being rebuilt
  // call after call
  std::unique_ptr<lpm::Batch> velPlans[2];
  int64_t symMinLeaves = lpm::kSymMinLeaves;  // lpm_bve_ctx_set_symmetric
  std::unique_ptr<lpm::Batch> rkBatch;
  std::unique_ptr<lpm::PairTimer> timer;  // set while timing is enabled
  lpm::PairShape forced{0, 0, 0, 0};       // FP32C launch shape chosen by the caller (threads 0 = none)
  std::map<std::array<int, 5>, lpm::PairShape> tuned;  // autotuner results per size bucket
  double* normScratch = nullptr;  // device: block partials + result of lpm_errnorms
  double* normHost = nullptr;     // pinned: result of lpm_errnorms
};

struct lpm_bve_ensemble {
  lpm_bve_ctx* ctx = nullptr;
  std::unique_ptr<lpm::Batch> batch;
  unsigned flags = 0;
};

namespace lpm {
namespace {

int handle(lpm_bve_ctx* ctx, const Error& e) {
  if (ctx) ctx->err = e.msg;
  return e.code;
}

void setDevice(lpm_bve_ctx* ctx) {
  int cur = -1;
  LPM_CUDA(cudaGetDevice(&cur));
  if (cur != ctx->dev.device) LPM_CUDA(cudaSetDevice(ctx->dev.device));
}

Precision precOf(unsigned flags) { return (flags & LPM_BVE_FP32C) ? Precision::FP32C : Precision::FP64; }

PairShape shapeFor(const lpm_bve_ctx* ctx, Precision p, bool tree) {
  if (p != Precision::FP32C) return kFP64Shape;
  if (tree) return kTreeShape;  // the tree kernel's shape
  return ctx && ctx->forced.threads > 0 ? ctx->forced : kDefaultFP32C;
}

bool sameVec(const DVec& a, const DVec& b) { return a.p == b.p && a.si == b.si && a.sc == b.sc; }

// True when a cached single-solve batch was built for the same geometry.
bool sameGeometry(const lpm_bve_ctx* ctx, const Batch* B, Mode mode, Precision prec, const ParticleIO& io,
                  const uint8_t* mask, bool skipMasked, bool sort, double eps, bool tree, bool sym) {
  if (!B || B->solves.size() != 1) return false;
  if (B->solves[0]->symWanted != sym || (sym && B->solves[0]->symMin != ctx->symMinLeaves)) return false;
  if (!(shapeFor(ctx, prec, tree) == B->shape)) return false;
  const SolvePlan& P = *B->solves[0];
  return P.mode == mode && P.prec == prec && P.io.na == io.na && P.io.nb == io.nb && sameVec(P.io.ax, io.ax) &&
         sameVec(P.io.bx, io.bx) && P.mask == mask && P.skipMasked == skipMasked && P.sorted == sort &&
         P.eps2 == eps * eps;
}

// Times every compiled FP32C launch shape on this problem (prep + a bounded number of pair
// work items; nothing the caller owns is written) and caches the fastest per size bucket.
PairShape autotune(lpm_bve_ctx* ctx, Mode mode, Precision prec, const ParticleIO& io, const uint8_t* mask,
                   bool skipMasked, bool sort, double eps, bool precise, const HostPlan& H, cudaStream_t s);

// A single solve's collocated / RK4 FP32C plan takes the symmetric layout unless the caller asks
// for the plain kernel (LPM_BVE_NO_SYMMETRIC), the tree code runs, or the targets keep their own
// order.
bool wantSymmetric(Mode mode, Precision prec, bool sort, bool tree, unsigned flags) {
  return mode != Mode::Distinct && prec == Precision::FP32C && sort && !tree && !(flags & LPM_BVE_NO_SYMMETRIC);
}

std::unique_ptr<Batch> makeSingle(lpm_bve_ctx* ctx, Mode mode, Precision prec, const ParticleIO& io,
                                  const uint8_t* mask, bool skipMasked, bool sort, double eps, bool precise,
                                  bool tree, cudaStream_t s, bool sym) {
  const HostPlan H = prepareHost(mode, io, mask, skipMasked, sort, s, sym, ctx->symMinLeaves);
  auto B = std::make_unique<Batch>();
  B->sym = H.leaf0 >= 0 && H.srcFace.size() > 0;  // (the layout needs enough leaves: prepareHost)
  B->prec = prec;
  B->shape = shapeFor(ctx, prec, tree);
  if (!tree && prec == Precision::FP32C && ctx->autotune && ctx->forced.threads == 0)
    B->shape = autotune(ctx, mode, prec, io, mask, skipMasked, sort, eps, precise, H, s);
  B->rk4 = (mode == Mode::RK4);
  B->precise = precise;
  B->owned.emplace_back(new SolvePlan());
  B->solves.push_back(B->owned.back().get());
  buildSolve(*B->solves[0], mode, prec, io, mask, skipMasked, sort, eps, B->shape.tileSize(), H, s);
  finalizeBatch(*B, ctx->dev, s);
  if (ctx->verbose)
    std::fprintf(stderr, "[lpm_bve] plan: mode=%d prec=%d slots=%d sources=%d tiles=%d chunks=%d items=%d grid=%d "
                 "symmetric=%d (leaf0 %d, %d + %d items)\n",
                 (int)mode, (int)prec, B->solves[0]->nslots, B->solves[0]->ns, B->solves[0]->ntiles,
                 B->solves[0]->nchunks, B->nitems, B->grid, (int)B->sym, B->solves[0]->leaf0, B->nSymDirectItems,
                 B->nSymItems);
  return B;
}

int log2Bucket(int64_t n) {
  int b = 0;
  while ((int64_t(1) << b) < n && b < 62) ++b;
  return b;
}

PairShape autotune(lpm_bve_ctx* ctx, Mode mode, Precision prec, const ParticleIO& io, const uint8_t* mask,
                   bool skipMasked, bool sort, double eps, bool precise, const HostPlan& H, cudaStream_t s) {
  const std::array<int, 5> key{(int)mode, (int)prec, precise ? 1 : 0, log2Bucket((int64_t)H.ids.size()),
                               log2Bucket((int64_t)H.srcFace.size())};
  auto it = ctx->tuned.find(key);
  if (it != ctx->tuned.end()) return it->second;
  PairShape best = kDefaultFP32C;
  double bestRate = -1.0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  LPM_CUDA(cudaEventCreate(&e0));
  LPM_CUDA(cudaEventCreate(&e1));
  try {
    for (int i = 0; i < pairShapeCount(); ++i) {
      const PairShape sh = pairShapeAt(i);
      Batch T;
      T.prec = prec;
      T.shape = sh;
      T.precise = precise;
      T.owned.emplace_back(new SolvePlan());
      T.solves.push_back(T.owned.back().get());
      buildSolve(*T.solves[0], mode, prec, io, mask, skipMasked, sort, eps, sh.tileSize(), H, s);
      finalizeBatch(T, ctx->dev, s);
      // A bounded trial: a few waves of work items are enough to rank shapes.
      const int ntrial = std::min(T.nitems, std::max(1, 4 * T.grid));
      double pairs = 0.0;
      for (int k = 0; k < ntrial; ++k) pairs += T.itemPairs[k];
      float ms = 0.f;
      for (int rep = 0; rep < 2; ++rep) {
        LPM_CUDA(launchPrep(T.stageDev, T.prepMap, T.nPrepBlocks, 0, prec, T.counter, s));
        LPM_CUDA(cudaEventRecord(e0, s));
        LPM_CUDA(launchPair(prec, sh, false, precise, false, T.solveDev, T.items, ntrial, T.counter, T.grid, s));
        LPM_CUDA(cudaEventRecord(e1, s));
        LPM_CUDA(cudaEventSynchronize(e1));
        LPM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      }
      const double rate = pairs / std::max(1e-6, (double)ms);
      if (ctx->verbose)
        std::fprintf(stderr, "[lpm_bve] autotune: shape %dx%d st=%d minb=%d: %.3f ms for %.3e pairs (%.3e pairs/s)\n",
                     sh.threads, sh.k, sh.srcTile, sh.minBlocks, ms, pairs, rate * 1e3);
      if (rate > bestRate) {
        bestRate = rate;
        best = sh;
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tuned[key] = best;
  return best;
}

// Updates the caller-facing pointers and scalars of a cached plan; re-uploads if changed.
void bindIO(Batch& B, size_t m, const ParticleIO& io, double dt, double omega, cudaStream_t s, bool& changed) {
  SolvePlan& P = *B.solves[m];
  SolveStage& S = P.stage;
  const ParticleIO& o = S.io;
  const bool diff = !(sameVec(o.au, io.au) && sameVec(o.bu, io.bu) && o.azeta == io.azeta && o.bzeta == io.bzeta &&
                      o.apsi == io.apsi && o.bpsi == io.bpsi && o.barea == io.barea && S.dt == dt && S.omega == omega);
  if (diff) {
    S.io = io;
    S.dt = dt;
    S.omega = omega;
    P.io = io;
    changed = true;
  }
  (void)s;
}

// Switches a batch (one solve or an ensemble) between the direct sum and the tree code.
void useTree(lpm_bve_ctx* ctx, Batch& B, bool tree, cudaStream_t s) {
  B.treeMode = tree;
  if (!tree) return;
  if (B.trees.empty()) {
    for (size_t m = 0; m < B.solves.size(); ++m) B.trees.push_back(std::make_shared<TreeEval>());
    B.treeStageDev = B.mem.alloc<SolveStage>(B.solves.size());
  }
  B.treeParams = ctx->treeParams;
  ctx->lastTree = B.trees.back();
  if (B.treeDirectFor == B.treeParams.minPairs) return;
  // solves too small for the tree code keep the direct sum: their work items, longest first
  B.treeDirectFor = B.treeParams.minPairs;
  B.treeDirect.assign(B.solves.size(), 0);
  std::vector<WorkItem> items;
  for (size_t m = 0; m < B.solves.size(); ++m) {
    const SolvePlan& P = *B.solves[m];
    if ((double)P.nslots * P.ns >= B.treeParams.minPairs) continue;
    B.treeDirect[m] = 1;
    for (int t = 0; t < P.ntiles; ++t)
      for (int c = 0; c < P.nchunks; ++c) {
        WorkItem w{};
        w.solve = (int)m;
        w.tile = t;
        w.s0 = std::min(P.ns, c * P.chunkLen);
        w.s1 = std::min(P.ns, (c + 1) * P.chunkLen);
        w.chunk = c;
        w.tbeg = P.tileStart[t];
        w.tend = P.tileStart[t + 1];
        items.push_back(w);
      }
  }
  std::stable_sort(items.begin(), items.end(), [&](const WorkItem& a, const WorkItem& b) {
    return (int64_t)(a.s1 - a.s0) * B.solves[a.solve]->tileSize > (int64_t)(b.s1 - b.s0) * B.solves[b.solve]->tileSize;
  });
  B.directMem.release();
  B.nDirectItems = (int)items.size();
  B.directItems = B.nDirectItems ? B.directMem.alloc<WorkItem>(items.size()) : nullptr;
  upload(B.directItems, items, s);
  LPM_CUDA(cudaStreamSynchronize(s));  // the host vector goes out of scope
}

}  // namespace

void attachTrees(Batch& B, const std::vector<std::shared_ptr<TreeEval>>& trees, const TreeParams& tp,
                 cudaStream_t s) {
  if (trees.size() != B.solves.size()) fail(LPM_ERR_INTERNAL, "tree code: one evaluator per solve");
  B.treeMode = true;
  B.trees = trees;
  if (!B.treeStageDev) B.treeStageDev = B.mem.alloc<SolveStage>(B.solves.size());
  B.treeStageHost.clear();
  B.treeParams = tp;
  B.treeDirectFor = tp.minPairs;
  B.treeDirect.assign(B.solves.size(), 0);
  B.directMem.release();
  B.directItems = nullptr;
  B.nDirectItems = 0;
  if (trees.size() > 1) ensureTreeLanes(B, s, std::min<int>((int)trees.size(), kTreeLanes));
}
}  // namespace lpm

using namespace lpm;

extern "C" {

int lpm_bve_ctx_create(lpm_bve_ctx** out, const lpm_bve_opts* opts) {
  if (!out) return LPM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto* ctx = new (std::nothrow) lpm_bve_ctx();
  if (!ctx) return LPM_ERR_OUT_OF_MEMORY;
  try {
    int dev = opts ? opts->device : -1;
    if (dev < 0) LPM_CUDA(cudaGetDevice(&dev));
    LPM_CUDA(cudaSetDevice(dev));
    ctx->dev.device = dev;
    LPM_CUDA(cudaDeviceGetAttribute(&ctx->dev.sms, cudaDevAttrMultiProcessorCount, dev));
    int major = 0, minor = 0;
    LPM_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    LPM_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3)
      fail(LPM_ERR_NOT_SUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a (GB300) only", dev, major,
           minor);
    ctx->autotune = opts ? opts->autotune : 0;
    ctx->verbose = opts ? opts->verbose : 0;
    LPM_CUDA(cudaStreamCreateWithFlags(&ctx->capture, cudaStreamNonBlocking));
  } catch (const Error& e) {
    const int code = e.code;
    std::fprintf(stderr, "lpm_bve_ctx_create: %s\n", e.msg.c_str());
    delete ctx;
    return code;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "lpm_bve_ctx_create: %s\n", e.what());
    delete ctx;
    return fromStd(e).code;
  }
  *out = ctx;
  return LPM_OK;
}

int lpm_bve_ctx_destroy(lpm_bve_ctx* ctx) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->dev.device);
  cudaDeviceSynchronize();
  for (auto& p : ctx->velPlans) p.reset();
  ctx->rkBatch.reset();
  if (ctx->capture) cudaStreamDestroy(ctx->capture);
  if (ctx->normScratch) cudaFree(ctx->normScratch);
  if (ctx->normHost) cudaFreeHost(ctx->normHost);
  delete ctx;
  return LPM_OK;
}

const char* lpm_bve_last_error(const lpm_bve_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int lpm_bve_plan_invalidate(lpm_bve_ctx* ctx) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  try {
    setDevice(ctx);
    LPM_CUDA(cudaDeviceSynchronize());
    for (auto& p : ctx->velPlans) p.reset();
    ctx->rkBatch.reset();
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_ctx_set_timing(lpm_bve_ctx* ctx, int enable) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  try {
    setDevice(ctx);
    if (enable && !ctx->timer) ctx->timer = std::make_unique<PairTimer>();
    if (!enable && ctx->timer) {
      ctx->timer->collect();
      ctx->timer.reset();
    }
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_ctx_set_shape(lpm_bve_ctx* ctx, int threads, int targets_per_thread, int source_tile, int min_blocks) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  if (threads == 0) {
    ctx->forced = PairShape{0, 0, 0, 0};
    return LPM_OK;
  }
  const PairShape sh{threads, targets_per_thread, source_tile, min_blocks};
  if (!pairShapeSupported(Precision::FP32C, sh)) {
    ctx->err = "set_shape: launch shape not compiled in";
    return LPM_ERR_NOT_SUPPORTED;
  }
  ctx->forced = sh;
  return LPM_OK;
}

int lpm_bve_ctx_shapes(int* threads, int* targets_per_thread, int* source_tile, int* min_blocks, int capacity) {
  const int n = pairShapeCount();
  for (int i = 0; i < n && i < capacity; ++i) {
    const PairShape sh = pairShapeAt(i);
    if (threads) threads[i] = sh.threads;
    if (targets_per_thread) targets_per_thread[i] = sh.k;
    if (source_tile) source_tile[i] = sh.srcTile;
    if (min_blocks) min_blocks[i] = sh.minBlocks;
  }
  return n;
}

int lpm_bve_ctx_timing(lpm_bve_ctx* ctx, double* pair_ms, int64_t* pair_launches, int reset) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  try {
    setDevice(ctx);
    double ms = 0.0;
    int64_t n = 0;
    if (ctx->timer) {
      ctx->timer->collect();
      ms = ctx->timer->totalMs;
      n = ctx->timer->launches;
      if (reset) {
        ctx->timer->totalMs = 0.0;
        ctx->timer->launches = 0;
      }
    }
    if (pair_ms) *pair_ms = ms;
    if (pair_launches) *pair_launches = n;
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_ctx_set_symmetric(lpm_bve_ctx* ctx, int64_t min_leaves) {
  if (!ctx || min_leaves < 0) return LPM_ERR_INVALID_ARGUMENT;
  ctx->symMinLeaves = min_leaves;
  return LPM_OK;
}

int lpm_bve_ctx_set_treecode(lpm_bve_ctx* ctx, int degree, double theta, int leaf_points, double min_pairs) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  if (degree < 2 || degree > 10 || !(theta > 0.0 && theta < 1.0) || leaf_points < 1 || !(min_pairs >= 0.0)) {
    ctx->err = "set_treecode: degree 2..10, theta in (0, 1), leaf_points >= 1, min_pairs >= 0";
    return LPM_ERR_INVALID_ARGUMENT;
  }
  ctx->treeParams.degree = degree;
  ctx->treeParams.theta = theta;
  ctx->treeParams.leafPoints = leaf_points;
  ctx->treeParams.minPairs = min_pairs;
  return LPM_OK;
}

int lpm_bve_ctx_tree_stats(lpm_bve_ctx* ctx, int* depth, int64_t* nodes, int64_t* far_clusters, double* pairs,
                           double* direct_pairs, double* far_pairs, double* phase_ms) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  if (!ctx->lastTree) {
    ctx->err = "tree_stats: no tree-code evaluation yet";
    return LPM_ERR_STATE;
  }
  const TreeStats& t = ctx->lastTree->stats();
  if (depth) *depth = t.depth;
  if (nodes) *nodes = t.nodes;
  if (far_clusters) *far_clusters = t.farClusters;
  if (pairs) *pairs = t.pairs;
  if (direct_pairs) *direct_pairs = t.directPairs;
  if (far_pairs) *far_pairs = t.farPairs;
  if (phase_ms) {
    phase_ms[0] = t.buildMs;
    phase_ms[1] = t.upwardMs;
    phase_ms[2] = t.listMs;
  }
  return LPM_OK;
}

int lpm_bve_velocity(lpm_bve_ctx* ctx, const lpm_points* tgt, const lpm_sources* src, double* u, int64_t u_si,
                     int64_t u_sc, double* psi, unsigned flags, double eps, lpm_stream_t stream) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  try {
    setDevice(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    if (!src) fail(LPM_ERR_INVALID_ARGUMENT, "velocity: null source set");
    const bool colloc = flags & LPM_BVE_COLLOCATED;
    const bool wantVel = !(flags & LPM_BVE_NO_VELOCITY);
    const bool wantPsi = flags & LPM_BVE_PSI;
    if (!wantVel && !wantPsi) fail(LPM_ERR_INVALID_ARGUMENT, "velocity: nothing requested (NO_VELOCITY without PSI)");
    if (!(eps >= 0.0) || !std::isfinite(eps)) fail(LPM_ERR_INVALID_ARGUMENT, "velocity: eps must be finite and >= 0");
    const lpm_points& S = src->pts;
    checkVec("sources", S.x, S.n, S.stride_i, S.stride_c);
    if (S.n > 0 && (!src->zeta || !src->area)) fail(LPM_ERR_INVALID_ARGUMENT, "velocity: null zeta/area");
    int64_t nt = S.n;
    if (!colloc) {
      if (!tgt) fail(LPM_ERR_INVALID_ARGUMENT, "velocity: null target set");
      checkVec("targets", tgt->x, tgt->n, tgt->stride_i, tgt->stride_c);
      nt = tgt->n;
    }
    if (wantVel) checkVec("u", u, nt, u_si, u_sc);
    if (wantPsi && nt > 0 && !psi) fail(LPM_ERR_INVALID_ARGUMENT, "velocity: PSI requested with null psi");
    if (nt == 0) return LPM_OK;

    ParticleIO io;
    io.nb = S.n;
    io.bx = DVec{const_cast<double*>(S.x), S.stride_i, S.stride_c};
    io.bzeta = const_cast<double*>(src->zeta);
    io.barea = src->area;
    const Mode mode = colloc ? Mode::Collocated : Mode::Distinct;
    if (colloc) {
      io.na = 0;
      io.bu = DVec{wantVel ? u : nullptr, u_si, u_sc};
      io.bpsi = wantPsi ? psi : nullptr;
    } else {
      io.na = tgt->n;
      io.ax = DVec{const_cast<double*>(tgt->x), tgt->stride_i, tgt->stride_c};
      io.au = DVec{wantVel ? u : nullptr, u_si, u_sc};
      io.apsi = wantPsi ? psi : nullptr;
    }
    const Precision prec = precOf(flags);
    const bool sort = !(flags & LPM_BVE_NO_SORT);
    const bool skip = colloc && (flags & LPM_BVE_SKIP_MASKED_TARGETS);
    const bool tree = flags & LPM_BVE_TREECODE;
    if (tree && prec != Precision::FP32C) fail(LPM_ERR_NOT_SUPPORTED, "velocity: the tree code needs LPM_BVE_FP32C");
    std::unique_ptr<Batch>& plan = ctx->velPlans[colloc ? 1 : 0];
    const bool sym = wantSymmetric(mode, prec, sort, tree, flags);
    if (!sameGeometry(ctx, plan.get(), mode, prec, io, src->mask, skip, sort, eps, tree, sym)) {
      if (plan) LPM_CUDA(cudaDeviceSynchronize());  // kernels may still read the old plan
      plan.reset();
      const bool precise = prec == Precision::FP32C && mode == Mode::Distinct && !(flags & LPM_BVE_MESH_TARGETS);
      plan = makeSingle(ctx, mode, prec, io, src->mask, skip, sort, eps, precise, tree, s, sym);
      plan->solves[0]->stage.io = ParticleIO{};  // force a table refresh below
    }
    Batch& B = *plan;
    // Distinct targets are arbitrary points unless the caller says they are mesh points.
    B.precise = prec == Precision::FP32C && mode == Mode::Distinct && !(flags & LPM_BVE_MESH_TARGETS);
    B.rcpApprox = flags & LPM_BVE_RCP_APPROX;
    useTree(ctx, B, tree, s);
    bool changed = false;
    bindIO(B, 0, io, 0.0, 0.0, s, changed);
    if (changed) refreshTables(B, s);
    B.timer = ctx->timer.get();
    // the reference's functor names: BVE{Vertex,Face}{Velocity,StreamFn,Solve}
    // (src/LpmBVEKernels.hpp:110-305)
    static const EvalNames kVel[2][3] = {
        {{"BVEVertexVelocity positions", "BVEVertexVelocity", "BVEVertexVelocity out"},
         {"BVEVertexStreamFn positions", "BVEVertexStreamFn", "BVEVertexStreamFn out"},
         {"BVEVertexSolve positions", "BVEVertexSolve", "BVEVertexSolve out"}},
        {{"BVEFaceVelocity positions", "BVEFaceVelocity", "BVEFaceVelocity out"},
         {"BVEFaceStreamFn positions", "BVEFaceStreamFn", "BVEFaceStreamFn out"},
         {"BVEFaceSolve positions", "BVEFaceSolve", "BVEFaceSolve out"}}};
    enqueueEval(B, 0, 0, wantPsi, wantVel, s, &kVel[mode == Mode::Distinct ? 0 : 1][wantPsi ? (wantVel ? 2 : 1) : 0]);
    B.timer = nullptr;
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_rk4_step(lpm_bve_ctx* ctx, const lpm_bve_state* st, double dt, double Omega, int nsteps, unsigned flags,
                     double eps, lpm_stream_t stream) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  NvtxRange region("BVERK4::advance_timestep");
  try {
    setDevice(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    if (!st) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_step: null state");
    if (nsteps < 0) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_step: negative step count");
    if (!std::isfinite(dt) || !std::isfinite(Omega)) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_step: dt/Omega not finite");
    if (!(eps >= 0.0) || !std::isfinite(eps)) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_step: eps must be finite and >= 0");
    checkVec("vx", st->vx, st->nverts, st->vx_stride_i, st->vx_stride_c);
    checkVec("vvel", st->vvel, st->nverts, st->vvel_stride_i, st->vvel_stride_c);
    checkVec("fx", st->fx, st->nfaces, st->fx_stride_i, st->fx_stride_c);
    checkVec("fvel", st->fvel, st->nfaces, st->fvel_stride_i, st->fvel_stride_c);
    if (st->nverts > 0 && !st->vzeta) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_step: null vzeta");
    if (st->nfaces > 0 && (!st->fzeta || !st->farea)) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_step: null fzeta/farea");
    if (nsteps == 0 || st->nverts + st->nfaces == 0) return LPM_OK;

    ParticleIO io;
    io.na = st->nverts;
    io.nb = st->nfaces;
    io.ax = DVec{st->vx, st->vx_stride_i, st->vx_stride_c};
    io.au = DVec{st->vvel, st->vvel_stride_i, st->vvel_stride_c};
    io.azeta = st->vzeta;
    io.bx = DVec{st->fx, st->fx_stride_i, st->fx_stride_c};
    io.bu = DVec{st->fvel, st->fvel_stride_i, st->fvel_stride_c};
    io.bzeta = st->fzeta;
    io.barea = st->farea;
    const Precision prec = precOf(flags);
    const bool sort = !(flags & LPM_BVE_NO_SORT);
    const bool skip = flags & LPM_BVE_SKIP_MASKED_TARGETS;
    const bool tree = flags & LPM_BVE_TREECODE;
    if (tree && prec != Precision::FP32C) fail(LPM_ERR_NOT_SUPPORTED, "rk4_step: the tree code needs LPM_BVE_FP32C");
    const bool sym = wantSymmetric(Mode::RK4, prec, sort, tree, flags);
    if (!sameGeometry(ctx, ctx->rkBatch.get(), Mode::RK4, prec, io, st->fmask, skip, sort, eps, tree, sym)) {
      if (ctx->rkBatch) LPM_CUDA(cudaDeviceSynchronize());
      ctx->rkBatch.reset();
      ctx->rkBatch = makeSingle(ctx, Mode::RK4, prec, io, st->fmask, skip, sort, eps, false, tree, s, sym);
      ctx->rkBatch->solves[0]->stage.io = ParticleIO{};
    }
    Batch& B = *ctx->rkBatch;
    bool changed = false;
    bindIO(B, 0, io, dt, Omega, s, changed);
    if (changed) refreshTables(B, s);
    const bool quirk = !(flags & LPM_BVE_RK4_FIX_QUIRK);
    const bool renorm = flags & LPM_BVE_RENORM;
    const bool rcp = flags & LPM_BVE_RCP_APPROX;
    B.rcpApprox = rcp;
    useTree(ctx, B, tree, s);
    // The tree code reads nothing back once its evaluations are sized (the first one), so its steps
    // are captured too; the graph is rebuilt when an evaluation's buffers or arguments change
    // (after a list overflow, reported without a synchronisation).
    bool treeReady = false;
    int treeGen = 0;
    if (tree) {
      treeReady = !B.trees.empty();
      for (auto& t : B.trees) {
        t->poll();
        treeReady = treeReady && t->ready();
        treeGen += t->generation();
      }
      if (treeReady) treeStageTable(B, s);
    }
    if ((flags & LPM_BVE_NO_GRAPH) || ctx->timer || (tree && !treeReady)) {
      B.timer = ctx->timer.get();
      for (int k = 0; k < nsteps; ++k) enqueueStep(B, quirk, renorm, s);
      B.timer = nullptr;
    } else {
      if (B.graph && (B.graphQuirk != quirk || B.graphRenorm != renorm || B.graphRcp != rcp || B.graphTree != tree ||
                      (tree && B.graphTreeGen != treeGen))) {
        cudaGraphExecDestroy(B.graph);
        B.graph = nullptr;
      }
      if (!B.graph) {
        cudaGraph_t g = nullptr;
        LPM_CUDA(cudaStreamBeginCapture(ctx->capture, cudaStreamCaptureModeThreadLocal));
        try {
          enqueueStep(B, quirk, renorm, ctx->capture);
        } catch (...) {
          cudaStreamEndCapture(ctx->capture, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        LPM_CUDA(cudaStreamEndCapture(ctx->capture, &g));
        const cudaError_t ie = cudaGraphInstantiate(&B.graph, g, 0);
        cudaGraphDestroy(g);
        LPM_CUDA(ie);
        B.graphQuirk = quirk;
        B.graphRenorm = renorm;
        B.graphRcp = rcp;
        B.graphTree = tree;
        B.graphTreeGen = 0;
        for (auto& t : B.trees) B.graphTreeGen += tree ? t->generation() : 0;
      }
      for (int k = 0; k < nsteps; ++k) LPM_CUDA(cudaGraphLaunch(B.graph, s));
    }
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_rk4_increments(lpm_bve_ctx* ctx, int stage, double* vx_inc, double* vzeta_inc, double* fx_inc,
                           double* fzeta_inc, lpm_stream_t stream) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  try {
    setDevice(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    if (stage < 0 || stage > 3) fail(LPM_ERR_INVALID_ARGUMENT, "rk4_increments: stage must be 0..3");
    if (!ctx->rkBatch) fail(LPM_ERR_STATE, "rk4_increments: no RK4 step has run on this context");
    const SolvePlan& P = *ctx->rkBatch->solves[0];
    const int n = P.nslots;
    std::vector<double> kx(3 * (size_t)n), kz((size_t)n);
    std::vector<int> perm((size_t)n);
    LPM_CUDA(cudaMemcpyAsync(kx.data(), P.stage.kx[stage], sizeof(double) * kx.size(), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(kz.data(), P.stage.kz[stage], sizeof(double) * kz.size(), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaMemcpyAsync(perm.data(), P.stage.perm, sizeof(int) * perm.size(), cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaStreamSynchronize(s));
    const int64_t na = P.io.na, nb = P.io.nb;
    if (vx_inc) std::fill(vx_inc, vx_inc + 3 * na, 0.0);
    if (vzeta_inc) std::fill(vzeta_inc, vzeta_inc + na, 0.0);
    if (fx_inc) std::fill(fx_inc, fx_inc + 3 * nb, 0.0);
    if (fzeta_inc) std::fill(fzeta_inc, fzeta_inc + nb, 0.0);
    for (int t = 0; t < n; ++t) {
      const int p = perm[t];
      double* X = p < na ? vx_inc : fx_inc;
      double* Z = p < na ? vzeta_inc : fzeta_inc;
      const int64_t q = p < na ? p : p - na;
      if (X)
        for (int c = 0; c < 3; ++c) X[3 * q + c] = kx[(size_t)c * n + t];
      if (Z) Z[q] = kz[t];
    }
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_errnorms(lpm_bve_ctx* ctx, const double* appx, int64_t a_si, int64_t a_sc, const double* exact,
                 int64_t e_si, int64_t e_sc, const double* wt, const uint8_t* skip, int64_t n, int ncomp,
                 unsigned flags, double out[3], lpm_stream_t stream) {
  if (!ctx) return LPM_ERR_INVALID_ARGUMENT;
  try {
    setDevice(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    if (!out) fail(LPM_ERR_INVALID_ARGUMENT, "errnorms: null output");
    if (ncomp != 1 && ncomp != 3) fail(LPM_ERR_INVALID_ARGUMENT, "errnorms: ncomp must be 1 or 3");
    if (ncomp == 1) a_sc = e_sc = 0;
    checkVec("appx", appx, n, a_si, ncomp == 3 ? a_sc : 0);
    checkVec("exact", exact, n, e_si, ncomp == 3 ? e_sc : 0);
    if (n == 0) fail(LPM_ERR_INVALID_ARGUMENT, "errnorms: no entries");
    const int nblocks = normBlocks(ctx->dev.sms);
    if (!ctx->normScratch) {
      void* p = nullptr;
      LPM_CUDA(cudaMalloc(&p, sizeof(double) * (6 * (size_t)nblocks + 3)));
      ctx->normScratch = static_cast<double*>(p);
    }
    if (!ctx->normHost) {
      void* p = nullptr;
      LPM_CUDA(cudaMallocHost(&p, sizeof(double) * 3));
      ctx->normHost = static_cast<double*>(p);
    }
    NormArgs a{appx, a_si, a_sc, exact, e_si, e_sc, wt, skip, n, ncomp, (flags & LPM_NORMS_ABS_LINF) ? 0 : 1};
    double* dOut = ctx->normScratch + 6 * (size_t)nblocks;
    LPM_CUDA(launchNorms(a, ctx->normScratch, nblocks, dOut, s));
    LPM_CUDA(cudaMemcpyAsync(ctx->normHost, dOut, sizeof(double) * 3, cudaMemcpyDeviceToHost, s));
    LPM_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < 3; ++k) out[k] = ctx->normHost[k];
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

// ---------------------------------------------------------------------------------------
// ensembles: many independent solves advanced by one persistent launch per RK4 evaluation
// ---------------------------------------------------------------------------------------
int lpm_bve_ensemble_create(lpm_bve_ctx* ctx, const lpm_bve_state* states, int nsolves, unsigned flags, double eps,
                            lpm_stream_t stream, lpm_bve_ensemble** out) {
  if (!ctx || !out) return LPM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  try {
    setDevice(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    if (nsolves <= 0 || !states) fail(LPM_ERR_INVALID_ARGUMENT, "ensemble_create: no solves");
    if (!(eps >= 0.0) || !std::isfinite(eps)) fail(LPM_ERR_INVALID_ARGUMENT, "ensemble_create: bad eps");
    auto E = std::make_unique<lpm_bve_ensemble>();
    E->ctx = ctx;
    E->flags = flags;
    E->batch = std::make_unique<Batch>();
    Batch& B = *E->batch;
    B.prec = precOf(flags);
    const bool tree = flags & LPM_BVE_TREECODE;
    if (tree && B.prec != Precision::FP32C) fail(LPM_ERR_NOT_SUPPORTED, "ensemble_create: the tree code needs LPM_BVE_FP32C");
    B.shape = shapeFor(ctx, B.prec, tree);
    B.rk4 = true;
    B.rcpApprox = flags & LPM_BVE_RCP_APPROX;
    const bool sort = !(flags & LPM_BVE_NO_SORT);
    const bool skip = flags & LPM_BVE_SKIP_MASKED_TARGETS;
    const bool sym = wantSymmetric(Mode::RK4, B.prec, sort, tree, flags);
    auto ioOf = [](const lpm_bve_state* st) {
      ParticleIO io;
      io.na = st->nverts;
      io.nb = st->nfaces;
      io.ax = DVec{st->vx, st->vx_stride_i, st->vx_stride_c};
      io.au = DVec{st->vvel, st->vvel_stride_i, st->vvel_stride_c};
      io.azeta = st->vzeta;
      io.bx = DVec{st->fx, st->fx_stride_i, st->fx_stride_c};
      io.bu = DVec{st->fvel, st->fvel_stride_i, st->fvel_stride_c};
      io.bzeta = st->fzeta;
      io.barea = st->farea;
      return io;
    };
    if (!tree && B.prec == Precision::FP32C && ctx->autotune && ctx->forced.threads == 0) {
      int big = 0;  // tune on the solve with the most pairs: it dominates the launch
      for (int m = 1; m < nsolves; ++m)
        if ((states[m].nverts + states[m].nfaces) * states[m].nfaces >
            (states[big].nverts + states[big].nfaces) * states[big].nfaces)
          big = m;
      const ParticleIO io = ioOf(&states[big]);
      const HostPlan H = prepareHost(Mode::RK4, io, states[big].fmask, skip, sort, s);
      B.shape = autotune(ctx, Mode::RK4, B.prec, io, states[big].fmask, skip, sort, eps, false, H, s);
    }
    for (int m = 0; m < nsolves; ++m) {
      const lpm_bve_state* st = &states[m];
      checkVec("vx", st->vx, st->nverts, st->vx_stride_i, st->vx_stride_c);
      checkVec("vvel", st->vvel, st->nverts, st->vvel_stride_i, st->vvel_stride_c);
      checkVec("fx", st->fx, st->nfaces, st->fx_stride_i, st->fx_stride_c);
      checkVec("fvel", st->fvel, st->nfaces, st->fvel_stride_i, st->fvel_stride_c);
      if (st->nverts + st->nfaces == 0) fail(LPM_ERR_INVALID_ARGUMENT, "ensemble_create: solve %d is empty", m);
      ParticleIO io;
      io.na = st->nverts;
      io.nb = st->nfaces;
      io.ax = DVec{st->vx, st->vx_stride_i, st->vx_stride_c};
      io.au = DVec{st->vvel, st->vvel_stride_i, st->vvel_stride_c};
      io.azeta = st->vzeta;
      io.bx = DVec{st->fx, st->fx_stride_i, st->fx_stride_c};
      io.bu = DVec{st->fvel, st->fvel_stride_i, st->fvel_stride_c};
      io.bzeta = st->fzeta;
      io.barea = st->farea;
      B.owned.emplace_back(new SolvePlan());
      B.solves.push_back(B.owned.back().get());
      const HostPlan H = prepareHost(Mode::RK4, io, st->fmask, skip, sort, s, sym, ctx->symMinLeaves);
      buildSolve(*B.solves.back(), Mode::RK4, B.prec, io, st->fmask, skip, sort, eps, B.shape.tileSize(), H, s);
    }
    B.sym = false;
    for (const SolvePlan* p : B.solves) B.sym = B.sym || (p->leaf0 >= 0 && p->ns > 0);
    finalizeBatch(B, ctx->dev, s);
    if (ctx->verbose)
      std::fprintf(stderr, "[lpm_bve] ensemble: %d solves, %d items, grid %d\n", nsolves, B.nitems, B.grid);
    *out = E.release();
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_ensemble_step(lpm_bve_ensemble* E, const double* dt, const double* Omega, int nsteps, lpm_stream_t stream) {
  if (!E || !E->ctx) return LPM_ERR_INVALID_ARGUMENT;
  NvtxRange region("BVERK4::advance_timestep (ensemble)");
  lpm_bve_ctx* ctx = E->ctx;
  try {
    setDevice(ctx);
    cudaStream_t s = (cudaStream_t)stream;
    if (!dt || !Omega) fail(LPM_ERR_INVALID_ARGUMENT, "ensemble_step: null dt/Omega");
    if (nsteps < 0) fail(LPM_ERR_INVALID_ARGUMENT, "ensemble_step: negative step count");
    Batch& B = *E->batch;
    bool changed = false;
    for (size_t m = 0; m < B.solves.size(); ++m) {
      if (!std::isfinite(dt[m]) || !std::isfinite(Omega[m])) fail(LPM_ERR_INVALID_ARGUMENT, "ensemble_step: bad dt");
      SolveStage& S = B.solves[m]->stage;
      if (S.dt != dt[m] || S.omega != Omega[m]) {
        S.dt = dt[m];
        S.omega = Omega[m];
        changed = true;
      }
    }
    if (changed) refreshTables(B, s);
    const bool quirk = !(E->flags & LPM_BVE_RK4_FIX_QUIRK);
    const bool renorm = E->flags & LPM_BVE_RENORM;
    const bool tree = E->flags & LPM_BVE_TREECODE;
    useTree(ctx, B, tree, s);
    // tree-code ensembles are captured once every solve's evaluation is sized (as in rk4_step)
    bool treeReady = false;
    int treeGen = 0;
    if (tree) {
      treeReady = !B.trees.empty();
      for (auto& t : B.trees) {
        t->poll();
        treeReady = treeReady && t->ready();
        treeGen += t->generation();
      }
      if (treeReady) treeStageTable(B, s);
    }
    if ((E->flags & LPM_BVE_NO_GRAPH) || ctx->timer || (tree && !treeReady)) {
      B.timer = ctx->timer.get();
      for (int k = 0; k < nsteps; ++k) enqueueStep(B, quirk, renorm, s);
      B.timer = nullptr;
    } else {
      if (B.graph && tree && B.graphTreeGen != treeGen) {
        cudaGraphExecDestroy(B.graph);
        B.graph = nullptr;
      }
      if (!B.graph) {
        cudaGraph_t g = nullptr;
        LPM_CUDA(cudaStreamBeginCapture(ctx->capture, cudaStreamCaptureModeThreadLocal));
        try {
          enqueueStep(B, quirk, renorm, ctx->capture);
        } catch (...) {
          cudaStreamEndCapture(ctx->capture, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        LPM_CUDA(cudaStreamEndCapture(ctx->capture, &g));
        const cudaError_t ie = cudaGraphInstantiate(&B.graph, g, 0);
        cudaGraphDestroy(g);
        LPM_CUDA(ie);
        B.graphTreeGen = 0;
        for (auto& t : B.trees) B.graphTreeGen += tree ? t->generation() : 0;
      }
      for (int k = 0; k < nsteps; ++k) LPM_CUDA(cudaGraphLaunch(B.graph, s));
    }
  } catch (const Error& e) {
    return handle(ctx, e);
  } catch (const std::exception& e) {
    return handle(ctx, fromStd(e));
  }
  return LPM_OK;
}

int lpm_bve_ensemble_info(const lpm_bve_ensemble* E, int* nsolves, int* nitems, int* grid, int64_t* pairs_per_eval,
                          size_t* device_bytes) {
  if (!E || !E->batch) return LPM_ERR_INVALID_ARGUMENT;
  const Batch& B = *E->batch;
  int64_t pairs = 0;
  size_t bytes = B.mem.bytes();
  for (auto& p : B.solves) {
    pairs += (int64_t)p->nslots * p->ns;
    bytes += p->mem.bytes();
  }
  if (nsolves) *nsolves = (int)B.solves.size();
  if (nitems) *nitems = B.nitems;
  if (grid) *grid = B.grid;
  if (pairs_per_eval) *pairs_per_eval = pairs;
  if (device_bytes) *device_bytes = bytes;
  return LPM_OK;
}

int lpm_bve_ensemble_destroy(lpm_bve_ensemble* E) {
  if (!E) return LPM_ERR_INVALID_ARGUMENT;
  if (E->ctx) {
    cudaSetDevice(E->ctx->dev.device);
    cudaDeviceSynchronize();
  }
  delete E;
  return LPM_OK;
}

}  // extern "C"
