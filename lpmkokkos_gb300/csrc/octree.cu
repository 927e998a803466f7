// octree.cu -- device build of the Morton octree of pbosler/lpmKokkos.
//
// The same construction as the reference (Zhou et al. 2011, listings 1-2; file:line per step
// below), organised for the GPU: one radix sort of 64-bit codes over the significant key bits
// only, scans for unique keys and sibling sets, one kernel per level bottom-up, and
// per-point kernels where the reference loops over a node's points in one thread.  All data are
// integers or exact copies of FP64 inputs, so the result equals the serial restatement bit for
// bit.  The neighbour walk reads the parent level at base_address(l-1) + index (the reference
// reads the level-local index as a global row, right only at level 1), and the neighbour tables
// come from their geometric definition (the reference's ChildLUT differs in row 0, columns
// 18-20 and 24-26, which drop the +x bit).

#include "octree.hpp"

#include <cub/cub.cuh>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <mutex>

#include "engine_core.hpp"
#include "lpm_octree.h"

namespace lpm {
namespace {

constexpr int kBlock = 256;
constexpr double kZeroTol = 1.0e-14;  // ZERO_TOL, src/LpmDefs.hpp:99

// Neighbour j = 9a + 3b + c of a node with local key i = 4x + 2y + z (offsets (a-1, b-1, c-1)
// along x, y, z): its parent is the parent's neighbour cParent[i][j], and it is that node's kid
// cChild[i][j] (src/LpmOctreeLUT.hpp:70-137 defines the same tables).
__constant__ signed char cParent[8][27];
__constant__ signed char cChild[8][27];

void makeTables(signed char tp[8][27], signed char tc[8][27]) {
  for (int i = 0; i < 8; ++i) {
    const int bit[3] = {(i >> 2) & 1, (i >> 1) & 1, i & 1};
    for (int j = 0; j < 27; ++j) {
      const int off[3] = {j / 9 - 1, (j / 3) % 3 - 1, j % 3 - 1};
      int pj = 0, cj = 0;
      for (int a = 0; a < 3; ++a) {
        const int s = bit[a] + off[a];
        const int po = s < 0 ? -1 : (s > 1 ? 1 : 0);
        pj = 3 * pj + po + 1;
        cj = 2 * cj + (s - 2 * po);
      }
      tp[i][j] = (signed char)pj;
      tc[i][j] = (signed char)cj;
    }
  }
}

// Key algebra of src/LpmOctreeUtil.hpp:83-135 (keys at max-depth resolution).
__host__ __device__ __forceinline__ uint32_t parentKey(uint32_t k, int lev, int maxDepth) {
  const int keep = 3 * (lev - 1);  // top bits kept: the ancestor at level lev-1
  return keep == 0 ? 0u : (k >> (3 * maxDepth - keep)) << (3 * maxDepth - keep);
}
__host__ __device__ __forceinline__ uint32_t localKey(uint32_t k, int lev, int maxDepth) {
  return (k >> (3 * (maxDepth - lev))) & 7u;
}
__host__ __device__ __forceinline__ uint32_t nodeKey(uint32_t pk, uint32_t lk, int lev, int maxDepth) {
  return pk + (lk << (3 * (maxDepth - lev)));
}

__device__ __forceinline__ void reduceBox(double (&v)[6], double* sh) {
  // v = {xmin, -xmax, ymin, -ymax, zmin, -zmax}; block-wide min of each
  for (int c = 0; c < 6; ++c) {
    sh[threadIdx.x] = v[c];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
      __syncthreads();
    }
    v[c] = sh[0];
    __syncthreads();
  }
}

// BoxFunctor / BBoxReducer (src/LpmBox3d.hpp:84-160): min and max per axis.
__global__ void __launch_bounds__(kBlock) boxPartial(const double* __restrict__ x, int64_t si, int64_t sc, int64_t n,
                                                     double* __restrict__ part) {
  __shared__ double sh[kBlock];
  double v[6] = {DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      const double p = x[i * si + c * sc];
      v[2 * c] = fmin(v[2 * c], p);
      v[2 * c + 1] = fmin(v[2 * c + 1], -p);
    }
  }
  reduceBox(v, sh);
  if (threadIdx.x == 0)
    for (int c = 0; c < 6; ++c) part[blockIdx.x * 6 + c] = v[c];
}

__global__ void __launch_bounds__(kBlock) boxFinal(const double* __restrict__ part, int nb, double* __restrict__ box) {
  __shared__ double sh[kBlock];
  double v[6] = {DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX, DBL_MAX};
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    for (int c = 0; c < 6; ++c) v[c] = fmin(v[c], part[b * 6 + c]);
  reduceBox(v, sh);
  if (threadIdx.x == 0) {
    box[0] = v[0]; box[1] = -v[1]; box[2] = v[2]; box[3] = -v[3]; box[4] = v[4]; box[5] = -v[5];
  }
}

// compute_key_for_point (src/LpmOctreeUtil.hpp:57-81) with box2cube (src/LpmBox3d.hpp:290-303):
// the same comparisons and centre updates, so the keys equal the reference's.
__device__ __forceinline__ uint32_t pointKey(double px, double py, double pz, int depth, const double* __restrict__ b) {
  double xmin = b[0], xmax = b[1], ymin = b[2], ymax = b[3], zmin = b[4], zmax = b[5];
  const double dx = xmax - xmin, dy = ymax - ymin, dz = zmax - zmin;
  const double lo = fmin(fmin(dx, dy), dz), hi = fmax(fmax(dx, dy), dz);
  if (fabs(hi / lo - 1.0) > kZeroTol) {
    const double h = 0.5 * hi;
    const double mx = 0.5 * (xmin + xmax), my = 0.5 * (ymin + ymax), mz = 0.5 * (zmin + zmax);
    xmin = mx - h; xmax = mx + h; ymin = my - h; ymax = my + h; zmin = mz - h; zmax = mz + h;
  }
  double cx = 0.5 * (xmin + xmax), cy = 0.5 * (ymin + ymax), cz = 0.5 * (zmin + zmax);
  double half = 0.5 * (xmax - xmin);
  uint32_t key = 0;
  for (int i = 1; i <= depth; ++i) {
    half *= 0.5;
    const int s = 3 * (depth - i);
    const bool rz = pz >= cz, ry = py >= cy, rx = px >= cx;
    key += rz ? (1u << s) : 0u;
    cz += rz ? half : -half;
    key += ry ? (2u << s) : 0u;
    cy += ry ? half : -half;
    key += rx ? (4u << s) : 0u;
    cx += rx ? half : -half;
  }
  return key;
}

// EncodeFunctor (src/LpmOctreeKernels.hpp:27-47): code = key << 32 | point id.
__global__ void codesKernel(const double* __restrict__ x, int64_t si, int64_t sc, int64_t n, int depth,
                            const double* __restrict__ box, uint64_t* __restrict__ codes) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = x + i * si;
  codes[i] = ((uint64_t)pointKey(p[0], p[sc], p[2 * sc], depth, box) << 32) | (uint64_t)i;
}

// PermuteFunctor (:49-72) and MarkDuplicates' flags (:99-128).
__global__ void permuteKernel(const uint64_t* __restrict__ codes, const double* __restrict__ x, int64_t si,
                              int64_t sc, int64_t n, double* __restrict__ sorted, int* __restrict__ orig,
                              int* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t c = codes[i];
  const int64_t id = (int64_t)(c & 0xffffffffull);
  orig[i] = (int)id;
  for (int k = 0; k < 3; ++k) sorted[3 * i + k] = x[id * si + k * sc];
  flag[i] = (i == 0 || (c >> 32) != (codes[i - 1] >> 32)) ? 1 : 0;
}

// UniqueNodeFunctor (:130-183): unique keys and the first point of each.
__global__ void uniqueKernel(const uint64_t* __restrict__ codes, const int* __restrict__ uidx, int64_t n,
                             uint32_t* __restrict__ ukeys, int* __restrict__ ustart) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i == 0 || uidx[i] != uidx[i - 1]) {
    const int u = uidx[i] - 1;
    ukeys[u] = (uint32_t)(codes[i] >> 32);
    ustart[u] = (int)i;
  }
}

// A count that is either known on the host (d == nullptr) or lives in device memory (the
// sync-free build, whose grids cover an upper bound and whose threads past the count return).
__device__ __forceinline__ int countOf(const int* d, int h) { return d ? *d : h; }

__global__ void uniqueCountKernel(const int* __restrict__ ustart, int nuHost, const int* __restrict__ nuDev, int64_t n,
                                  int* __restrict__ ucount) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  const int nu = countOf(nuDev, nuHost);
  if (u >= nu) return;
  ucount[u] = (u + 1 < nu ? ustart[u + 1] : (int)n) - ustart[u];
}

// NodeSiblingCounter's flags (:186-231): 8 where the parent at level lev-1 changes.
// (sync-free build: the grid covers `bound` entries and writes 0 past the count, so that the scan
// over the bound gives the same prefix sums)
__global__ void siblingMark(const uint32_t* __restrict__ keys, int mHost, const int* __restrict__ mDev, int div,
                            int bound, int lev, int maxDepth, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = mDev ? *mDev / div : mHost;
  if (i >= m) {
    if (mDev && i < bound) flag[i] = 0;
    return;
  }
  flag[i] = (i == 0 || parentKey(keys[i], lev, maxDepth) != parentKey(keys[i - 1], lev, maxDepth)) ? 8 : 0;
}

// NodeArrayDFunctor (:233-283): complete sibling sets at the leaf level.  The unique keys of one
// parent follow each other in ascending order, so the 8 candidate keys are matched by a merge
// walk (the reference binary-searches each; same result).
__global__ void leafNodes(const uint32_t* __restrict__ ukeys, const int* __restrict__ ustart,
                          const int* __restrict__ ucount, const int* __restrict__ sib, int nuHost,
                          const int* __restrict__ nuDev, int depth, uint32_t* __restrict__ keys, int2* __restrict__ pt,
                          int* __restrict__ parents, int* __restrict__ kids, int* __restrict__ nodeOf) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  const int nu = countOf(nuDev, nuHost);
  if (u >= nu) return;
  if (u > 0 && sib[u] == sib[u - 1]) return;
  const int kid0 = sib[u] - 8;
  const uint32_t pk = parentKey(ukeys[u], depth, depth);
  int m = u;
  for (int j = 0; j < 8; ++j) {
    const int nd = kid0 + j;
    const uint32_t key = pk + (uint32_t)j;
    keys[nd] = key;
    parents[nd] = -1;
    for (int c = 0; c < 8; ++c) kids[8 * nd + c] = -1;
    if (m < nu && ukeys[m] == key) {
      pt[nd] = make_int2(ustart[m], ucount[m]);
      nodeOf[m] = nd;
      ++m;
    } else {
      pt[nd] = make_int2(-1, 0);
    }
  }
}

__global__ void ptInLeafKernel(const int* __restrict__ uidx, const int* __restrict__ nodeOf, int64_t n,
                               int* __restrict__ ptInLeaf) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ptInLeaf[i] = nodeOf[uidx[i] - 1];
}

// ParentNodeFunctor (:285-323): one parent per complete sibling set of the lower level.
// (sync-free build: npDev points at the lower level's node count, np = count / 8)
__global__ void parentGroups(const uint32_t* __restrict__ lowKeys, const int2* __restrict__ lowPt, int npHost,
                             const int* __restrict__ lowCountDev, int lev, int maxDepth, uint32_t* __restrict__ pkeys,
                             int2* __restrict__ ppt) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = lowCountDev ? *lowCountDev / 8 : npHost;
  if (g >= np) return;
  pkeys[g] = parentKey(lowKeys[8 * g], lev + 1, maxDepth);
  int cnt = 0, start = -1;
  for (int j = 0; j < 8; ++j) {
    const int2 p = lowPt[8 * g + j];
    cnt += p.y;
    if (start == -1 && p.x != -1) start = p.x;
  }
  ppt[g] = make_int2(start, cnt);
}

// NodeArrayInternalFunctor (:325-369): complete sibling sets at level lev, kids and the lower
// level's parents.
__global__ void internalNodes(const uint32_t* __restrict__ pkeys, const int2* __restrict__ ppt,
                              const int* __restrict__ sib, int npHost, const int* __restrict__ lowCountDev, int lev,
                              int maxDepth, uint32_t* __restrict__ keys, int2* __restrict__ pt, int* __restrict__ parents,
                              int* __restrict__ kids, int* __restrict__ lowParents) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = lowCountDev ? *lowCountDev / 8 : npHost;
  if (g >= np) return;
  if (g > 0 && sib[g] == sib[g - 1]) return;
  const int kid0 = sib[g] - 8;
  const uint32_t pk = parentKey(pkeys[g], lev, maxDepth);
  int m = g;
  for (int j = 0; j < 8; ++j) {
    const int nd = kid0 + j;
    const uint32_t key = nodeKey(pk, (uint32_t)j, lev, maxDepth);
    keys[nd] = key;
    parents[nd] = -1;
    if (m < np && pkeys[m] == key) {
      pt[nd] = ppt[m];
      for (int c = 0; c < 8; ++c) {
        kids[8 * nd + c] = 8 * m + c;
        lowParents[8 * m + c] = nd;
      }
      ++m;
    } else {
      pt[nd] = make_int2(-1, 0);
      for (int c = 0; c < 8; ++c) kids[8 * nd + c] = -1;
    }
  }
}

// out = scan[len - 1] (0 for len = 0), len from the device (lenDev) or the host; with div > 1
// the length is *lenDev / div (the parents of a level's complete sibling sets).
__global__ void countFromScan(const int* __restrict__ scan, int lenHost, const int* __restrict__ lenDev, int div,
                              int* __restrict__ out) {
  const int len = lenDev ? *lenDev / div : lenHost;
  *out = len > 0 ? scan[len - 1] : 0;
}

__global__ void setInt(int* __restrict__ p, int v) { *p = v; }

// The root (src/LpmNodeArrayInternal.cpp:13-52): key 0, all points, kids 0..7.
__global__ void rootNode(const int2* __restrict__ lev1Pt, uint32_t* __restrict__ keys, int2* __restrict__ pt,
                         int* __restrict__ parents, int* __restrict__ kids, int* __restrict__ lev1Parents,
                         int* __restrict__ nbrs) {
  const int t = threadIdx.x;
  if (t < 8) {
    kids[t] = t;
    lev1Parents[t] = 0;
  }
  if (nbrs && t < 27) nbrs[t] = t == 13 ? 0 : -1;
  if (t == 0) {
    keys[0] = 0;
    parents[0] = -1;
    int cnt = 0;
    for (int j = 0; j < 8; ++j) cnt += lev1Pt[j].y;
    pt[0] = make_int2(0, cnt);
  }
}

// NeighborhoodFunctor (src/LpmOctreeKernels.hpp:371-400) at level lev, parent level arrays at
// their own base.
__global__ void neighborsKernel(const uint32_t* __restrict__ keys, const int* __restrict__ parents, int m, int lev,
                                int maxDepth, const int* __restrict__ upNbrs, const int* __restrict__ upKids,
                                int* __restrict__ nbrs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m) return;
  const int p = parents[t];
  const int i = (int)localKey(keys[t], lev, maxDepth);
  for (int j = 0; j < 27; ++j) {
    const int h = upNbrs[27 * p + cParent[i][j]];
    nbrs[27 * t + j] = h != -1 ? upKids[8 * h + cChild[i][j]] : -1;
  }
}

inline unsigned blocksFor(int64_t n) { return (unsigned)((n + kBlock - 1) / kBlock); }

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? LPM_ERR_OUT_OF_MEMORY : LPM_ERR_CUDA, "octree %s: %s", what,
         cudaGetErrorString(e));
  }
}

int readInt(const int* d, cudaStream_t s) {
  int h = 0;
  check(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s), "read-back");
  check(cudaStreamSynchronize(s), "synchronise");
  return h;
}

// __constant__ memory is per device: the tables are uploaded once on every device that builds
// an octree, with that device current.
constexpr int kMaxDevices = 64;
std::once_flag g_tablesOnce[kMaxDevices];
cudaError_t g_tablesErr[kMaxDevices];

}  // namespace

template <typename T>
T* Octree::grow(Buf& b, size_t count, cudaStream_t s) {
  const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
  if (!registered_) {
    for (Buf* p : {&bKeys, &bPt, &bPar, &bKids, &bNbrs, &bSorted, &bOrig, &bLeaf, &bBox, &bCodes, &bCodes2, &bFlag,
                   &bScan, &bUKeys, &bUStart, &bUCount, &bNodeOf, &bSib, &bTemp, &bPart, &bCount})
      all_.push_back(p);
    for (int l = 0; l <= kOctreeMaxDepth; ++l)
      for (Buf* p : {&bLevKeys[l], &bLevPt[l], &bLevPar[l], &bLevKids[l], &bLevNbrs[l]}) all_.push_back(p);
    registered_ = true;
  }
  if (b.bytes < bytes) {
    if (b.p) check(cudaFreeAsync(b.p, s), "free");
    b.p = nullptr;
    b.bytes = 0;
    const size_t want = bytes + bytes / 4;  // headroom: positions move between builds
    check(cudaMallocAsync(&b.p, want, s), "allocation");
    b.bytes = want;
  }
  return static_cast<T*>(b.p);
}

void Octree::releaseAll() {
  for (Buf* b : all_) {
    if (b->p) cudaFree(b->p);
    b->p = nullptr;
    b->bytes = 0;
  }
}

void Octree::release(cudaStream_t s) {
  for (Buf* b : all_) {
    if (b->p) cudaFreeAsync(b->p, s);
    b->p = nullptr;
    b->bytes = 0;
  }
  dcount = nullptr;
  nnodes = 0;
}

Octree::~Octree() {
  bool held = false;
  for (Buf* b : all_) held = held || b->p;
  if (!held) return;  // released in stream order: nothing to wait for
  cudaDeviceSynchronize();
  releaseAll();
}

void Octree::build(const double* x, int64_t si, int64_t sc, int64_t npts, int maxDepth, bool neighbors,
                   cudaStream_t s, bool hostBox) {
  if (maxDepth < 1 || maxDepth > kOctreeMaxDepth) fail(LPM_ERR_INVALID_ARGUMENT, "octree depth must be 1..%d", kOctreeMaxDepth);
  if (npts <= 0 || npts > INT32_MAX) fail(LPM_ERR_INVALID_ARGUMENT, "octree: 1..2^31-1 points");
  int dev = 0;
  check(cudaGetDevice(&dev), "device query");
  if (dev < 0 || dev >= kMaxDevices) fail(LPM_ERR_NOT_SUPPORTED, "octree: device ordinal %d >= %d", dev, kMaxDevices);
  std::call_once(g_tablesOnce[dev], [dev] {
    signed char tp[8][27], tc[8][27];
    makeTables(tp, tc);
    g_tablesErr[dev] = cudaMemcpyToSymbol(cParent, tp, sizeof(tp));
    if (g_tablesErr[dev] == cudaSuccess) g_tablesErr[dev] = cudaMemcpyToSymbol(cChild, tc, sizeof(tc));
  });
  check(g_tablesErr[dev], "tables");
  depth = maxDepth;
  n = npts;
  const unsigned nb = blocksFor(n);

  // 1. bounding box
  const int boxBlocks = (int)std::min<int64_t>(nb, 512);
  double* part = grow<double>(bPart, 6 * (size_t)boxBlocks, s);
  double* dbx = grow<double>(bBox, 6, s);
  boxPartial<<<boxBlocks, kBlock, 0, s>>>(x, si, sc, n, part);
  boxFinal<<<1, kBlock, 0, s>>>(part, boxBlocks, dbx);
  dbox = dbx;

  // 2-3. codes, sort, permute
  uint64_t* codes = grow<uint64_t>(bCodes, n, s);
  uint64_t* codes2 = grow<uint64_t>(bCodes2, n, s);
  codesKernel<<<nb, kBlock, 0, s>>>(x, si, sc, n, depth, dbx, codes);
  int* flag = grow<int>(bFlag, n, s);
  int* scan = grow<int>(bScan, n, s);
  size_t tsort = 0, tscan = 0;
  check(cub::DeviceRadixSort::SortKeys(nullptr, tsort, codes, codes2, (int)n, 0, 32 + 3 * depth, s), "sort size");
  check(cub::DeviceScan::InclusiveSum(nullptr, tscan, flag, scan, (int)n, s), "scan size");
  void* temp = grow<unsigned char>(bTemp, std::max(tsort, tscan), s);
  size_t tb = bTemp.bytes;
  check(cub::DeviceRadixSort::SortKeys(temp, tb, codes, codes2, (int)n, 0, 32 + 3 * depth, s), "sort");
  sorted = grow<double>(bSorted, 3 * (size_t)n, s);
  origIds = grow<int>(bOrig, n, s);
  ptInLeaf = grow<int>(bLeaf, n, s);
  permuteKernel<<<nb, kBlock, 0, s>>>(codes2, x, si, sc, n, sorted, origIds, flag);
  tb = bTemp.bytes;
  check(cub::DeviceScan::InclusiveSum(temp, tb, flag, scan, (int)n, s), "scan");
  const int nu = readInt(scan + n - 1, s);

  // 4. unique leaf keys
  uint32_t* ukeys = grow<uint32_t>(bUKeys, nu, s);
  int* ustart = grow<int>(bUStart, nu, s);
  int* ucount = grow<int>(bUCount, nu, s);
  int* nodeOf = grow<int>(bNodeOf, nu, s);
  uniqueKernel<<<nb, kBlock, 0, s>>>(codes2, scan, n, ukeys, ustart);
  uniqueCountKernel<<<blocksFor(nu), kBlock, 0, s>>>(ustart, nu, nullptr, n, ucount);

  // 5-6. leaves with full sibling sets (the point flags are free again; the point scan is kept
  // for pt_in_leaf)
  int* sib = grow<int>(bSib, nu, s);
  siblingMark<<<blocksFor(nu), kBlock, 0, s>>>(ukeys, nu, nullptr, 1, nu, depth, depth, flag);
  {
    size_t need = 0;
    check(cub::DeviceScan::InclusiveSum(nullptr, need, flag, sib, nu, s), "scan size");
    temp = grow<unsigned char>(bTemp, need, s);
    tb = bTemp.bytes;
    check(cub::DeviceScan::InclusiveSum(temp, tb, flag, sib, nu, s), "scan");
  }
  std::vector<int> cnt(depth + 1, 0);
  cnt[depth] = readInt(sib + nu - 1, s);
  {
    const int m = cnt[depth];
    uint32_t* k = grow<uint32_t>(bLevKeys[depth], m, s);
    int2* p = grow<int2>(bLevPt[depth], m, s);
    int* par = grow<int>(bLevPar[depth], m, s);
    int* kd = grow<int>(bLevKids[depth], 8 * (size_t)m, s);
    leafNodes<<<blocksFor(nu), kBlock, 0, s>>>(ukeys, ustart, ucount, sib, nu, nullptr, depth, k, p, par, kd, nodeOf);
    ptInLeafKernel<<<nb, kBlock, 0, s>>>(scan, nodeOf, n, ptInLeaf);
  }

  // 7. internal levels, bottom-up (the unique-key buffers are reused: each kernel that reads
  // them was queued before the next level rewrites them); the root last
  for (int lev = depth - 1; lev >= 1; --lev) {
    const int np = cnt[lev + 1] / 8;
    uint32_t* pk = grow<uint32_t>(bUKeys, np, s);
    int2* ppt = grow<int2>(bUStart, np, s);
    parentGroups<<<blocksFor(np), kBlock, 0, s>>>(static_cast<uint32_t*>(bLevKeys[lev + 1].p),
                                                  static_cast<int2*>(bLevPt[lev + 1].p), np, nullptr, lev, depth, pk,
                                                  ppt);
    int* f = grow<int>(bFlag, np, s);
    int* sc2 = grow<int>(bSib, np, s);
    siblingMark<<<blocksFor(np), kBlock, 0, s>>>(pk, np, nullptr, 1, np, lev, depth, f);
    size_t need = 0;
    check(cub::DeviceScan::InclusiveSum(nullptr, need, f, sc2, np, s), "scan size");
    temp = grow<unsigned char>(bTemp, need, s);
    tb = bTemp.bytes;
    check(cub::DeviceScan::InclusiveSum(temp, tb, f, sc2, np, s), "scan");
    cnt[lev] = readInt(sc2 + np - 1, s);
    const int m = cnt[lev];
    uint32_t* k = grow<uint32_t>(bLevKeys[lev], m, s);
    int2* p = grow<int2>(bLevPt[lev], m, s);
    int* par = grow<int>(bLevPar[lev], m, s);
    int* kd = grow<int>(bLevKids[lev], 8 * (size_t)m, s);
    internalNodes<<<blocksFor(np), kBlock, 0, s>>>(pk, ppt, sc2, np, nullptr, lev, depth, k, p, par, kd,
                                                   static_cast<int*>(bLevPar[lev + 1].p));
  }
  cnt[0] = 1;
  {
    uint32_t* k = grow<uint32_t>(bLevKeys[0], 1, s);
    int2* p = grow<int2>(bLevPt[0], 1, s);
    int* par = grow<int>(bLevPar[0], 1, s);
    int* kd = grow<int>(bLevKids[0], 8, s);
    int* nb0 = neighbors ? grow<int>(bLevNbrs[0], 27, s) : nullptr;
    rootNode<<<1, 32, 0, s>>>(static_cast<int2*>(bLevPt[1].p), k, p, par, kd, static_cast<int*>(bLevPar[1].p), nb0);
  }
  if (neighbors) {
    for (int lev = 1; lev <= depth; ++lev) {
      int* nbr = grow<int>(bLevNbrs[lev], 27 * (size_t)cnt[lev], s);
      neighborsKernel<<<blocksFor(cnt[lev]), kBlock, 0, s>>>(
          static_cast<uint32_t*>(bLevKeys[lev].p), static_cast<int*>(bLevPar[lev].p), cnt[lev], lev, depth,
          static_cast<int*>(bLevNbrs[lev - 1].p), static_cast<int*>(bLevKids[lev - 1].p), nbr);
    }
  }

  // 8. concatenation (Tree::initNodes, src/LpmOctree.cpp:45-75)
  nnodes = 0;
  for (int l = 0; l <= depth; ++l) {
    base[l] = (int)nnodes;
    npl[l] = cnt[l];
    nnodes += cnt[l];
  }
  keys = grow<uint32_t>(bKeys, nnodes, s);
  ptInds = grow<int2>(bPt, nnodes, s);
  parents = grow<int>(bPar, nnodes, s);
  kids = grow<int>(bKids, 8 * (size_t)nnodes, s);
  nbrs = neighbors ? grow<int>(bNbrs, 27 * (size_t)nnodes, s) : nullptr;
  for (int l = 0; l <= depth; ++l) {
    const size_t m = (size_t)cnt[l], b = (size_t)base[l];
    check(cudaMemcpyAsync(keys + b, bLevKeys[l].p, m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s), "copy");
    check(cudaMemcpyAsync(ptInds + b, bLevPt[l].p, m * sizeof(int2), cudaMemcpyDeviceToDevice, s), "copy");
    check(cudaMemcpyAsync(parents + b, bLevPar[l].p, m * sizeof(int), cudaMemcpyDeviceToDevice, s), "copy");
    check(cudaMemcpyAsync(kids + 8 * b, bLevKids[l].p, 8 * m * sizeof(int), cudaMemcpyDeviceToDevice, s), "copy");
    if (neighbors)
      check(cudaMemcpyAsync(nbrs + 27 * b, bLevNbrs[l].p, 27 * m * sizeof(int), cudaMemcpyDeviceToDevice, s), "copy");
  }
  if (hostBox) {
    check(cudaMemcpyAsync(box, dbx, sizeof(box), cudaMemcpyDeviceToHost, s), "read-back");
    check(cudaStreamSynchronize(s), "synchronise");
  }
  check(cudaGetLastError(), "launch");
}

void Octree::buildOnDevice(const double* x, int64_t si, int64_t sc, int64_t npts, int maxDepth, cudaStream_t s) {
  if (maxDepth < 1 || maxDepth > kOctreeMaxDepth) fail(LPM_ERR_INVALID_ARGUMENT, "octree depth must be 1..%d", kOctreeMaxDepth);
  if (npts <= 0 || npts > INT32_MAX / 8) fail(LPM_ERR_INVALID_ARGUMENT, "octree: 1..2^28-1 points");
  depth = maxDepth;
  n = npts;
  const unsigned nb = blocksFor(n);
  // capacities: a level holds complete sibling sets of at most 8^l nodes, and at most 8 per
  // unique leaf key below it (<= n)
  int64_t cap[kOctreeMaxDepth + 1];
  int64_t total = 0;
  for (int l = 0; l <= depth; ++l) {
    int64_t c = 1;
    for (int k = 0; k < l && c < 8 * n; ++k) c *= 8;
    cap[l] = std::min<int64_t>(c, l == 0 ? 1 : 8 * n);
    gbase[l] = (int)total;
    base[l] = (int)total;
    npl[l] = 0;  // counts live on the device (dcount)
    total += cap[l];
  }
  if (total > INT32_MAX / 8) fail(LPM_ERR_NOT_SUPPORTED, "octree: %lld nodes of fixed-level capacity", (long long)total);
  gbase[depth + 1] = (int)total;
  nnodes = total;
  keys = grow<uint32_t>(bKeys, total, s);
  ptInds = grow<int2>(bPt, total, s);
  parents = grow<int>(bPar, total, s);
  kids = grow<int>(bKids, 8 * (size_t)total, s);
  nbrs = nullptr;
  dcount = grow<int>(bCount, depth + 2, s);  // [0..depth] node counts, [depth + 1] unique leaf keys
  int* dNu = dcount + depth + 1;
  check(cudaMemsetAsync(ptInds, 0, sizeof(int2) * (size_t)total, s), "clear");  // empty past the counts

  // 1. bounding box
  const int boxBlocks = (int)std::min<int64_t>(nb, 512);
  double* part = grow<double>(bPart, 6 * (size_t)boxBlocks, s);
  double* dbx = grow<double>(bBox, 6, s);
  boxPartial<<<boxBlocks, kBlock, 0, s>>>(x, si, sc, n, part);
  boxFinal<<<1, kBlock, 0, s>>>(part, boxBlocks, dbx);
  dbox = dbx;

  // 2-3. codes, sort, permute; unique leaf keys counted on the device
  uint64_t* codes = grow<uint64_t>(bCodes, n, s);
  uint64_t* codes2 = grow<uint64_t>(bCodes2, n, s);
  codesKernel<<<nb, kBlock, 0, s>>>(x, si, sc, n, depth, dbx, codes);
  int* flag = grow<int>(bFlag, n, s);
  int* scan = grow<int>(bScan, n, s);
  size_t tsort = 0, tscan = 0;
  check(cub::DeviceRadixSort::SortKeys(nullptr, tsort, codes, codes2, (int)n, 0, 32 + 3 * depth, s), "sort size");
  check(cub::DeviceScan::InclusiveSum(nullptr, tscan, flag, scan, (int)n, s), "scan size");  // the longest scan
  void* temp = grow<unsigned char>(bTemp, std::max(tsort, tscan), s);
  size_t tb = bTemp.bytes;
  check(cub::DeviceRadixSort::SortKeys(temp, tb, codes, codes2, (int)n, 0, 32 + 3 * depth, s), "sort");
  sorted = grow<double>(bSorted, 3 * (size_t)n, s);
  origIds = grow<int>(bOrig, n, s);
  ptInLeaf = grow<int>(bLeaf, n, s);
  permuteKernel<<<nb, kBlock, 0, s>>>(codes2, x, si, sc, n, sorted, origIds, flag);
  tb = bTemp.bytes;
  check(cub::DeviceScan::InclusiveSum(temp, tb, flag, scan, (int)n, s), "scan");
  countFromScan<<<1, 1, 0, s>>>(scan, (int)n, nullptr, 1, dNu);

  // 4. unique keys (room for n of them) and the leaf level's complete sibling sets
  uint32_t* ukeys = grow<uint32_t>(bUKeys, n, s);
  int* ustart = grow<int>(bUStart, 2 * (size_t)n, s);  // later the parents' int2 point ranges
  int* ucount = grow<int>(bUCount, n, s);
  int* nodeOf = grow<int>(bNodeOf, n, s);
  int* sib = grow<int>(bSib, n, s);
  uniqueKernel<<<nb, kBlock, 0, s>>>(codes2, scan, n, ukeys, ustart);
  uniqueCountKernel<<<nb, kBlock, 0, s>>>(ustart, 0, dNu, n, ucount);
  siblingMark<<<nb, kBlock, 0, s>>>(ukeys, 0, dNu, 1, (int)n, depth, depth, flag);
  tb = bTemp.bytes;
  check(cub::DeviceScan::InclusiveSum(temp, tb, flag, sib, (int)n, s), "scan");
  countFromScan<<<1, 1, 0, s>>>(sib, 0, dNu, 1, dcount + depth);
  const int gd = gbase[depth];
  leafNodes<<<nb, kBlock, 0, s>>>(ukeys, ustart, ucount, sib, 0, dNu, depth, keys + gd, ptInds + gd, parents + gd,
                                  kids + 8 * (size_t)gd, nodeOf);
  ptInLeafKernel<<<nb, kBlock, 0, s>>>(scan, nodeOf, n, ptInLeaf);

  // 5. internal levels bottom-up, each at its fixed base (nothing to concatenate afterwards)
  for (int lev = depth - 1; lev >= 1; --lev) {
    const int npB = (int)(cap[lev + 1] / 8);  // bound on the parents of the lower level's sets
    const int gl = gbase[lev], gu = gbase[lev + 1];
    uint32_t* pk = ukeys;                          // (the leaf kernels that read ukeys ran before)
    int2* ppt = reinterpret_cast<int2*>(ustart);
    parentGroups<<<blocksFor(npB), kBlock, 0, s>>>(keys + gu, ptInds + gu, 0, dcount + lev + 1, lev, depth, pk, ppt);
    siblingMark<<<blocksFor(npB), kBlock, 0, s>>>(pk, 0, dcount + lev + 1, 8, npB, lev, depth, flag);
    tb = bTemp.bytes;
    check(cub::DeviceScan::InclusiveSum(temp, tb, flag, sib, npB, s), "scan");
    countFromScan<<<1, 1, 0, s>>>(sib, 0, dcount + lev + 1, 8, dcount + lev);
    internalNodes<<<blocksFor(npB), kBlock, 0, s>>>(pk, ppt, sib, 0, dcount + lev + 1, lev, depth, keys + gl,
                                                    ptInds + gl, parents + gl, kids + 8 * (size_t)gl, parents + gu);
  }
  rootNode<<<1, 32, 0, s>>>(ptInds + gbase[1], keys, ptInds, parents, kids, parents + gbase[1], nullptr);
  setInt<<<1, 1, 0, s>>>(dcount, 1);
  check(cudaGetLastError(), "launch");
}

}  // namespace lpm

struct lpm_octree {
  lpm::Octree tree;
  int device = 0;
  bool fixed = false;  // LPM_OCTREE_FIXED_LEVELS: counts and box still on the device
};

extern "C" {

int lpm_octree_build(const double* x, int64_t x_si, int64_t x_sc, int64_t n, int max_depth, int neighbors,
                     lpm_octree** out, lpm_stream_t stream) {
  if (!out) return LPM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!x || n <= 0 || n > INT32_MAX || x_si < 0 || x_sc < 0 || max_depth < 1 || max_depth > lpm::kOctreeMaxDepth)
    return LPM_ERR_INVALID_ARGUMENT;
  const bool fixed = neighbors & LPM_OCTREE_FIXED_LEVELS;
  if ((neighbors & ~(LPM_OCTREE_NEIGHBORS | LPM_OCTREE_FIXED_LEVELS)) ||
      (fixed && (neighbors & LPM_OCTREE_NEIGHBORS)) || (fixed && n > INT32_MAX / 8))
    return LPM_ERR_INVALID_ARGUMENT;
  lpm_octree* t = new (std::nothrow) lpm_octree();
  if (!t) return LPM_ERR_OUT_OF_MEMORY;
  try {
    lpm::check(cudaGetDevice(&t->device), "device");
    t->fixed = fixed;
    if (fixed)
      t->tree.buildOnDevice(x, x_si, x_sc, n, max_depth, (cudaStream_t)stream);
    else
      t->tree.build(x, x_si, x_sc, n, max_depth, neighbors & LPM_OCTREE_NEIGHBORS, (cudaStream_t)stream);
  } catch (const lpm::Error& e) {
    std::fprintf(stderr, "lpm_octree_build: %s\n", e.msg.c_str());
    delete t;
    return e.code;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "lpm_octree_build: %s\n", e.what());
    delete t;
    return lpm::fromStd(e).code;
  }
  *out = t;
  return LPM_OK;
}

int lpm_octree_info(const lpm_octree* t, int* max_depth, int64_t* nnodes_total, int64_t* npoints,
                    int32_t* nnodes_per_level, int32_t* base_address, double* box) {
  if (!t) return LPM_ERR_INVALID_ARGUMENT;
  lpm::Octree& T = const_cast<lpm_octree*>(t)->tree;
  if (t->fixed) {  // the sync-free build left its level counts and box on the device
    int cnt[lpm::kOctreeMaxDepth + 2] = {};
    if (cudaSetDevice(t->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(cnt, T.dcount, sizeof(int) * (T.depth + 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(T.box, T.dbox, sizeof(T.box), cudaMemcpyDeviceToHost) != cudaSuccess)
      return LPM_ERR_CUDA;
    for (int l = 0; l <= T.depth; ++l) T.npl[l] = cnt[l];
  }
  if (max_depth) *max_depth = T.depth;
  if (nnodes_total) *nnodes_total = T.nnodes;
  if (npoints) *npoints = T.n;
  for (int l = 0; l <= T.depth; ++l) {
    if (nnodes_per_level) nnodes_per_level[l] = T.npl[l];
    if (base_address) base_address[l] = T.base[l];
  }
  if (box)
    for (int c = 0; c < 6; ++c) box[c] = T.box[c];
  return LPM_OK;
}

int lpm_octree_arrays(const lpm_octree* t, const uint32_t** keys, const int32_t** pt_inds, const int32_t** parents,
                      const int32_t** kids, const int32_t** neighbors, const double** sorted_pts,
                      const int32_t** orig_ids, const int32_t** pt_in_leaf) {
  if (!t) return LPM_ERR_INVALID_ARGUMENT;
  const lpm::Octree& T = t->tree;
  if (keys) *keys = T.keys;
  if (pt_inds) *pt_inds = reinterpret_cast<const int32_t*>(T.ptInds);
  if (parents) *parents = T.parents;
  if (kids) *kids = T.kids;
  if (neighbors) *neighbors = T.nbrs;
  if (sorted_pts) *sorted_pts = T.sorted;
  if (orig_ids) *orig_ids = T.origIds;
  if (pt_in_leaf) *pt_in_leaf = T.ptInLeaf;
  return LPM_OK;
}

int lpm_octree_destroy(lpm_octree* t) {
  if (!t) return LPM_ERR_INVALID_ARGUMENT;
  cudaSetDevice(t->device);
  delete t;
  return LPM_OK;
}

}  // extern "C"
