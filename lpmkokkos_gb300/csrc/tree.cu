// tree.cu -- the tree-code evaluation (tree.hpp): source octree, upward pass (cluster centres,
// radii, gnomonic charts and proxy charges), target-tile geometry, interaction lists, and the
// host orchestration around the gathered pair kernel (pair_kernels.cu).
//
// Proxy charges use the barycentric form of Lagrange interpolation at Chebyshev points of the
// second kind, t_a = cos(pi a / n), weights (-1)^a (halved at both ends) (Berrut & Trefethen,
// "Barycentric Lagrange interpolation", SIAM Review 46(3), 2004), in the tensor-product form
// of the barycentric Lagrange tree code (Wang, Krasny & Tlupova, Commun. Comput. Phys. 28(4),
// 2020), here on a per-cluster gnomonic chart of the sphere.  All reductions run in a fixed
// order, so an evaluation is reproducible bit for bit.

#include "tree_eval.hpp"

#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <cfloat>
#include <climits>
#include <cmath>
#include <mutex>
#include <numeric>
#include <utility>
#include <vector>

namespace lpm {
namespace {

constexpr int kBlock = 256;
constexpr int kUpThreads = 128;
constexpr int kMaxDegree = 10;            // (n+1)^2 <= 121 proxies: one thread per proxy charge
constexpr int kMaxNodes1D = kMaxDegree + 1;
// A chart covers sources within ~37 degrees of its centre direction: an octant (54.7 degrees)
// stretches its gnomonic chart 3x at the edge and its degree-8 interpolant then errs by 1e-5.
constexpr double kMinChartCos = 0.8;

__device__ __forceinline__ bool sane(double x, double y, double z) {
  const double r2 = x * x + y * y + z * z;
  return r2 >= 0.25 && r2 <= 4.0;  // false for NaN
}

// Fixed-order block reductions (warp shuffles, then the warps' partials in order).
template <int NT>
__device__ __forceinline__ double blockSum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < NT / 32; ++w) t += sh[w];
  return t;
}
// FP32 versions: FP64 runs at 1/64 of the FP32 rate on GB300, and in a kernel whose work per
// block is short, FP64 reductions over every thread are a large share of the FP64 pipe.
template <int NT>
__device__ __forceinline__ float blockSumF(float v, float* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.f;
  for (int w = 0; w < NT / 32; ++w) t += sh[w];
  return t;
}
template <int NT>
__device__ __forceinline__ float blockMaxF(float v, float* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = -FLT_MAX;
  for (int w = 0; w < NT / 32; ++w) t = fmaxf(t, sh[w]);
  return t;
}
__device__ __forceinline__ void kahanAddF(float& h, float& c, float v) {
  const float y = v - c;
  const float t = h + y;
  c = (t - h) - y;
  h = t;
}
template <int NT>
__device__ __forceinline__ double blockMax(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = -DBL_MAX;
  for (int w = 0; w < NT / 32; ++w) t = fmax(t, sh[w]);
  return t;
}
__global__ void srcPositions(const float4* __restrict__ sp0, const float4* __restrict__ sp1, int ns,
                             double* __restrict__ pos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  const float4 a = sp0[i], b = sp1[i];
  pos[3 * i] = (double)a.x + (double)b.x;
  pos[3 * i + 1] = (double)a.y + (double)b.y;
  pos[3 * i + 2] = (double)a.z + (double)b.z;
}

__global__ void gatherSources(const int* __restrict__ orig, const float4* __restrict__ sp0,
                              const float4* __restrict__ sp1, const int* __restrict__ srcSlot, int ns,
                              float4* __restrict__ tsp0, float4* __restrict__ tsp1, int* __restrict__ inv,
                              int* __restrict__ tslot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ns) return;
  const int o = orig[k];
  tsp0[k] = sp0[o];
  tsp1[k] = sp1[o];
  tslot[k] = srcSlot[o];
  inv[o] = k;
}

__global__ void sortedSelf(const int* __restrict__ self, const int* __restrict__ inv, int nslots,
                           int* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nslots) return;
  const int s = self[t];
  out[t] = s >= 0 ? inv[s] : -1;
}

// Centroid and radius of each target tile over its vertices and leaf faces.  Masked parent
// faces do not shape the tile: on the icosahedral mesh a parent's centre lies within ~1e-6 of its
// middle child's, its velocity is near-singular in the reference's formula, and after a step it
// runs away (its bounding sphere would then admit no far field).  Parents are still evaluated with their tile's
// list; a cubed-sphere parent sits on its children's shared corner, inside the tile.
// One warp per tile (tiles hold at most a few hundred slots); the butterfly reductions leave the
// same value in every lane.
__device__ __forceinline__ double warpSumAll(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warpMaxAll(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

constexpr int kGeomTilesPerBlock = kBlock / 32;

__global__ void __launch_bounds__(kBlock) tileGeometry(const double* __restrict__ tx, int n,
                                                       const int2* __restrict__ tiles, int ntiles,
                                                       const int* __restrict__ perm, int64_t na,
                                                       const uint8_t* __restrict__ mask,
                                                       float4* __restrict__ geom) {
  const int lane = threadIdx.x & 31;
  const int tile = blockIdx.x * kGeomTilesPerBlock + (threadIdx.x >> 5);
  if (tile >= ntiles) return;  // the whole warp
  const int2 tr = tiles[tile];
  const int t0 = tr.x, cnt = tr.y;
  auto shapes = [&](int slot, double x, double y, double z) {
    const int id = perm[slot];
    return sane(x, y, z) && !(mask && id >= na && mask[id - na]);
  };
  double sx = 0, sy = 0, sz = 0, sc = 0;
  for (int q = lane; q < cnt; q += 32) {
    const int slot = t0 + q;
    const double x = tx[slot], y = tx[n + slot], z = tx[2 * n + slot];
    if (shapes(slot, x, y, z)) { sx += x; sy += y; sz += z; sc += 1.0; }
  }
  sx = warpSumAll(sx);
  sy = warpSumAll(sy);
  sz = warpSumAll(sz);
  sc = warpSumAll(sc);
  if (sc == 0.0) {
    if (lane == 0) geom[tile] = make_float4(0.f, 0.f, 0.f, INFINITY);
    return;
  }
  const double cx = sx / sc, cy = sy / sc, cz = sz / sc;
  double r2 = 0.0;
  for (int q = lane; q < cnt; q += 32) {
    const int slot = t0 + q;
    const double x = tx[slot], y = tx[n + slot], z = tx[2 * n + slot];
    if (shapes(slot, x, y, z)) r2 = fmax(r2, (x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz));
  }
  r2 = warpMaxAll(r2);
  // FP32 for the traversal's acceptance test; the 1e-6 margin covers the rounded centre
  if (lane == 0) geom[tile] = make_float4((float)cx, (float)cy, (float)cz, (float)(sqrt(r2) + 1e-6));
}

// Chebyshev points of the second kind t_a = cos(pi a / n) and their barycentric weights.
struct Cheb {
  double t[kMaxNodes1D];
  double w[kMaxNodes1D];
};

Cheb chebFor(int n) {
  Cheb c{};
  for (int a = 0; a <= n; ++a) {
    c.t[a] = std::cos(kPi * a / n);
    c.w[a] = ((a & 1) ? -1.0 : 1.0) * ((a == 0 || a == n) ? 0.5 : 1.0);
  }
  c.t[0] = 1.0;
  c.t[n] = -1.0;
  return c;
}

// Barycentric Lagrange basis at u in [-1, 1] (second form; forward stable at Chebyshev points,
// Higham 2004), in FP32: the proxy charges are stored as floats, and the basis needs no more.
// scale multiplies every value (the source weight for the xi factor, 1 for eta).
__device__ __forceinline__ void basisF(float u, int n, const float* t, const float* w, float scale, float* L) {
  float den = 0.f;
  int hit = -1;
  for (int a = 0; a <= n; ++a) {
    const float d = u - t[a];
    if (d == 0.f) hit = a;
    L[a] = w[a] / d;
    den += L[a];
  }
  if (hit >= 0) {
    for (int a = 0; a <= n; ++a) L[a] = a == hit ? scale : 0.f;
    return;
  }
  const float r = scale / den;
  for (int a = 0; a <= n; ++a) L[a] *= r;
}

// Upward pass, one CTA per octree node: centre and radius of the node's sources; for nodes with
// more than (n+1)^2 sources all within ~37 degrees of the centre direction, the gnomonic chart,
// the proxy charges Q_ab (one thread per proxy, sources in index order) and the proxy records
// at sp0/sp1[ns + g (n+1)^2 + ab].
__global__ void __launch_bounds__(kUpThreads) upward(const int2* __restrict__ ptInds, int degree, const Cheb C, int ns, int firstNode,
                                                     float4* __restrict__ geom, int* __restrict__ approx,
                                                     float4* __restrict__ sp0, float4* __restrict__ sp1) {
  __shared__ float shf[kUpThreads / 32];
  __shared__ float sL[kUpThreads][2 * kMaxNodes1D];
  __shared__ float sT[kMaxNodes1D], sBw[kMaxNodes1D];
  if (threadIdx.x <= degree) {
    sT[threadIdx.x] = (float)C.t[threadIdx.x];
    sBw[threadIdx.x] = (float)C.w[threadIdx.x];
  }
  const int g = blockIdx.x;
  const int2 pt = ptInds[g];
  const int n1 = degree + 1, P = n1 * n1;
  if (pt.y == 0 || g < firstNode) {
    // empty; or the root and the octants, whose sources span more than any chart allows (their
    // geometry would only ever open them, so they are opened unconditionally: infinite radius)
    if (threadIdx.x == 0) { geom[g] = make_float4(0.f, 0.f, 0.f, pt.y == 0 ? -1.f : INFINITY); approx[g] = 0; }
    return;
  }
  const int k0 = pt.x, k1 = pt.x + pt.y;
  // Every per-source loop reads the sources' FP32 hi/lo records (sp0/sp1, key order), not their
  // FP64 positions: FP64 runs at 1/64 of the FP32 rate on GB300, and with FP64 sums, differences
  // and conversions per source this pass was FP64-pipe bound.  The centroid only has to lie near
  // the cluster (the radius and chart extents are measured from it); each thread sums its hi
  // parts in FP32, the block in FP64.
  float fsx = 0.f, fsy = 0.f, fsz = 0.f;
  for (int k = k0 + threadIdx.x; k < k1; k += kUpThreads) {
    const float4 a = sp0[k];
    fsx += a.x; fsy += a.y; fsz += a.z;
  }
  const double sx = blockSumF<kUpThreads>(fsx, shf);
  const double sy = blockSumF<kUpThreads>(fsy, shf);
  const double sz = blockSumF<kUpThreads>(fsz, shf);
  const double cx = sx / pt.y, cy = sy / pt.y, cz = sz / pt.y;
  const double cn = sqrt(cx * cx + cy * cy + cz * cz);
  const bool cand = pt.y > P && cn > 1e-3;
  // chart frame: c^ and two tangent directions
  double ux = 0, uy = 0, uz = 1, e1x = 1, e1y = 0, e1z = 0, e2x = 0, e2y = 1, e2z = 0;
  if (cand) {
    ux = cx / cn; uy = cy / cn; uz = cz / cn;
    const double ax = fabs(ux) < 0.9 ? 1.0 : 0.0, ay = 1.0 - ax;  // a = x^ or y^
    e1x = uy * 0.0 - uz * ay; e1y = uz * ax - ux * 0.0; e1z = ux * ay - uy * ax;  // c^ x a
    const double e1n = sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    e1x /= e1n; e1y /= e1n; e1z /= e1n;
    e2x = uy * e1z - uz * e1y; e2y = uz * e1x - ux * e1z; e2z = ux * e1y - uy * e1x;
  }
  // Radius, chart test and chart extents in FP32 (FP64 runs at 1/64 of the FP32 rate): the radius
  // only enters the acceptance test and the extents only bound the interpolation interval, so
  // ~1e-7 absolute errors are absorbed by the margins below.  The charges take their chart
  // coordinates from each source's FP64 offset to the chart centre (below).
  const float fcx = (float)cx, fcy = (float)cy, fcz = (float)cz;
  const float fux = (float)ux, fuy = (float)uy, fuz = (float)uz;
  const float f1x = (float)e1x, f1y = (float)e1y, f1z = (float)e1z, f2x = (float)e2x, f2y = (float)e2y, f2z = (float)e2z;
  float r2 = 0.f, dmin = FLT_MAX, xmin = FLT_MAX, xmax = -FLT_MAX, ymin = FLT_MAX, ymax = -FLT_MAX;
  for (int k = k0 + threadIdx.x; k < k1; k += kUpThreads) {
    const float4 a = sp0[k];
    const float x = a.x, y = a.y, z = a.z;  // hi parts: within 6e-8 of the position
    r2 = fmaxf(r2, (x - fcx) * (x - fcx) + (y - fcy) * (y - fcy) + (z - fcz) * (z - fcz));
    if (cand) {
      const float d = x * fux + y * fuy + z * fuz;
      dmin = fminf(dmin, d);
      if (d > 0.f) {
        const float rd = __frcp_rn(d);
        const float xi = (x * f1x + y * f1y + z * f1z) * rd, eta = (x * f2x + y * f2y + z * f2z) * rd;
        xmin = fminf(xmin, xi); xmax = fmaxf(xmax, xi); ymin = fminf(ymin, eta); ymax = fmaxf(ymax, eta);
      }
    }
  }
  const double rad = sqrt((double)blockMaxF<kUpThreads>(r2, shf)) + 1e-6;  // covers the FP32 rounding
  const double dlo = -(double)blockMaxF<kUpThreads>(-dmin, shf);
  double xlo = -(double)blockMaxF<kUpThreads>(-xmin, shf);
  double xhi = blockMaxF<kUpThreads>(xmax, shf);
  double ylo = -(double)blockMaxF<kUpThreads>(-ymin, shf);
  double yhi = blockMaxF<kUpThreads>(ymax, shf);
  const bool valid = cand && dlo >= kMinChartCos && xhi > xlo && yhi > ylo;
  if (threadIdx.x == 0) {
    geom[g] = make_float4((float)cx, (float)cy, (float)cz, (float)rad);  // rad's 1e-6 margin covers the rounding
    approx[g] = valid ? 1 : 0;
  }
  if (!valid) return;
  // widen the rectangle by the FP32 error of the extents (|xi|, |eta| <= 0.75 on a valid chart)
  constexpr double kPad = 1e-6;
  xlo -= kPad; xhi += kPad; ylo -= kPad; yhi += kPad;
  const double mx = 0.5 * (xlo + xhi), hx = 0.5 * (xhi - xlo);
  const double my = 0.5 * (ylo + yhi), hy = 0.5 * (yhi - ylo);
  const float fmx = (float)mx, fmy = (float)my, fihx = (float)(1.0 / hx), fihy = (float)(1.0 / hy);
  // the chart centre c^ as FP32 hi/lo parts, for the offsets below
  const float uhx = fux, uhy = fuy, uhz = fuz;
  const float ulx = (float)(ux - (double)uhx), uly = (float)(uy - (double)uhy), ulz = (float)(uz - (double)uhz);
  const int t = threadIdx.x;
  const int ia = t / n1, ib = t % n1;
  float qh = 0.f, qc = 0.f;  // the per-chunk compensated sums, themselves added with compensation
  for (int c0 = k0; c0 < k1; c0 += kUpThreads) {
    const int k = c0 + t;
    if (k < k1) {
      // chart coordinates from the offset d = x - c^: x.c^ = 1 + d.c^ and x.e = d.e for the
      // tangent directions, so every FP32 product is of the offset's size and the coordinates
      // carry ~1e-7 of it, not of |x|.  d from hi/lo parts: the hi difference is exact when the
      // coordinates are within a factor 2 (a cluster within ~37 degrees of c^), the lo parts
      // add the rest.
      const float4 a = sp0[k], b = sp1[k];
      const float dx = (a.x - uhx) + (b.x - ulx), dy = (a.y - uhy) + (b.y - uly), dz = (a.z - uhz) + (b.z - ulz);
      const float rd = __frcp_rn(1.f + (dx * fux + dy * fuy + dz * fuz));
      const float uxi = ((dx * f1x + dy * f1y + dz * f1z) * rd - fmx) * fihx;
      const float ueta = ((dx * f2x + dy * f2y + dz * f2z) * rd - fmy) * fihy;
      basisF(uxi, degree, sT, sBw, a.w, &sL[t][0]);  // w L_a(xi): one FMA per proxy below
      basisF(ueta, degree, sT, sBw, 1.f, &sL[t][n1]);
    }
    __syncthreads();
    if (t < P) {  // Kahan-compensated FP32 over the chunk (the FP32 pipe; FP64 is 1/64 of it)
      // (two interleaved sums over even and odd sources measured slower: 1.47 against 1.25 ms per
      // level-8 pass)
      const int m = min(kUpThreads, k1 - c0);
      float h = 0.f, c = 0.f;
      for (int j = 0; j < m; ++j) {
        const float y = sL[j][ia] * sL[j][n1 + ib] - c;
        const float tt = h + y;
        c = (tt - h) - y;
        h = tt;
      }
      kahanAddF(qh, qc, h - c);
    }
    __syncthreads();
  }
  if (t < P) {
    const double q = (double)qh - (double)qc;
    const double xi = mx + hx * C.t[ia], eta = my + hy * C.t[ib];
    double px = ux + xi * e1x + eta * e2x, py = uy + xi * e1y + eta * e2y, pz = uz + xi * e1z + eta * e2z;
    const double ip = 1.0 / sqrt(px * px + py * py + pz * pz);
    px *= ip; py *= ip; pz *= ip;
    const float hx0 = __double2float_rn(px), hy0 = __double2float_rn(py), hz0 = __double2float_rn(pz);
    const int slot = ns + g * P + t;
    sp0[slot] = make_float4(hx0, hy0, hz0, __double2float_rn(q));
    sp1[slot] = make_float4(__double2float_rn(px - (double)hx0), __double2float_rn(py - (double)hy0),
                            __double2float_rn(pz - (double)hz0), __double2float_rn(1.0 - (px * px + py * py + pz * pz)));
  }
}

struct Levels {
  int base[kOctreeMaxDepth + 2];
};

constexpr int kWarpStack = 4096;  // per-warp node stack: <= 256 entries per level for depth <= 10

// Interaction lists, one warp per target tile, the tree walked 32 nodes at a time: each step
// pops up to 32 stacked nodes (one per lane), tests them, places their kids on the stack and
// their list entries in lane order (warp prefix sums), and writes each entry's index range with
// the whole warp.  The order is a function of the data alone, so the lists are reproducible.
// FILL = false: list length and far-field length per tile; FILL = true: the flattened index
// list at listOff[tile], contiguous direct ranges merged.  A stack overflow (impossible for the
// depths the tree code builds) sets *err instead of writing out of bounds.
template <bool FILL>
__global__ void __launch_bounds__(32) traverse(const float4* __restrict__ tileGeom, int ntiles,
                                               const float4* __restrict__ geom, const int* __restrict__ approx,
                                               const int2* __restrict__ ptInds, const int* __restrict__ kids,
                                               Levels lv, int depth, float theta2, int P, int ns,
                                               int64_t* __restrict__ lens, int64_t* __restrict__ farLens,
                                               const int64_t* __restrict__ listOff, int* __restrict__ list,
                                               const int* __restrict__ overflow, int* __restrict__ err) {
  __shared__ int stack[kWarpStack];
  const int tile = blockIdx.x;
  const int lane = threadIdx.x;
  if (tile >= ntiles) return;
  if (FILL && *overflow) return;  // the lists do not fit: the pair kernel sums every source instead
  const float4 tg = tileGeom[tile];
  if (lane == 0) stack[0] = 0;  // the root (level 0, global index 0)
  __syncwarp();
  int sp = 1;
  int64_t len = 0, far = 0;
  int64_t o = FILL ? listOff[tile] : 0;
  int rs = 0, rl = 0;  // pending direct range (FILL)
  while (sp > 0) {
    const int n = min(32, sp);
    const int b0 = sp - n;
    const int g = lane < n ? stack[b0 + lane] : -1;
    __syncwarp();
    sp = b0;
    int kind = 0;  // 0 nothing, 1 far, 2 direct, 3 open
    int2 pt = make_int2(0, 0);
    int lev = 0;
    if (g >= 0) {
      pt = ptInds[g];
      if (pt.y > 0) {
        // (r_tile + r_node) < theta |c_tile - c_node|, squared and in FP32 (FP64 runs at 1/64
        // of the FP32 rate; the radii carry 1e-6 margins); an infinite radius never passes
        const float4 ng = geom[g];
        const float dx = tg.x - ng.x, dy = tg.y - ng.y, dz = tg.z - ng.z;
        const float rr = tg.w + ng.w;
        const bool mac = rr * rr < theta2 * (dx * dx + dy * dy + dz * dz);
        while (lev < depth && g >= lv.base[lev + 1]) ++lev;
        if (mac && approx[g]) kind = 1;
        else if (mac && pt.y <= P) kind = 2;      // well separated but smaller than its proxy set
        else if (lev < depth) kind = 3;           // too close, or no valid chart: open the node
        else kind = 2;                            // a leaf
      }
    }
    // kids of opened nodes onto the stack (lane order, ascending child order)
    int nk = 0, kidv[8];
    if (kind == 3)
      for (int c = 0; c < 8; ++c) {
        const int k = kids[8 * g + c];
        if (k >= 0) kidv[nk++] = lv.base[lev + 1] + k;
      }
    int incl = nk;
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (sp + total > kWarpStack) {  // cannot happen for depth <= 10; never write out of bounds
      if (lane == 0) atomicExch(err, 1);
      break;
    }
    for (int c = 0; c < nk; ++c) stack[sp + incl - nk + c] = kidv[c];
    sp += total;
    __syncwarp();
    // list entries in lane order
    const unsigned emit = __ballot_sync(0xffffffffu, kind == 1 || kind == 2);
    unsigned m = emit;
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      const int kd = __shfl_sync(0xffffffffu, kind, src);
      const int st = __shfl_sync(0xffffffffu, pt.x, src);
      const int ct = __shfl_sync(0xffffffffu, pt.y, src);
      const int gg = __shfl_sync(0xffffffffu, g, src);
      if (kd == 1) {
        len += P;
        far += P;
        if (FILL) {
          for (int k = lane; k < rl; k += 32) list[o + k] = rs + k;
          o += rl;
          rl = 0;
          const int p0 = ns + gg * P;
          for (int k = lane; k < P; k += 32) list[o + k] = p0 + k;
          o += P;
        }
      } else {
        len += ct;
        if (FILL) {
          if (rl > 0 && rs + rl == st) {
            rl += ct;
          } else {
            for (int k = lane; k < rl; k += 32) list[o + k] = rs + k;
            o += rl;
            rs = st;
            rl = ct;
          }
        }
      }
    }
  }
  if (FILL) {
    for (int k = lane; k < rl; k += 32) list[o + k] = rs + k;
  } else if (lane == 0) {
    lens[tile] = len;
    farLens[tile] = far;
  }
}

// Lists that overflowed their buffer (the fill wrote nothing): every tile's list becomes the
// identity list of all sorted sources, the exact direct sum (the buffer holds at least ns).
__global__ void directFallback(const int* __restrict__ overflow, int64_t* __restrict__ off,
                               int64_t* __restrict__ lens, int ntiles, int* __restrict__ list, int ns) {
  if (!*overflow) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ntiles) {
    off[i] = 0;
    lens[i] = ns;
  }
  if (i < ns) list[i] = i;
}

// The list buffer's capacity check, before the fill: overflow = total > capacity.
__global__ void capCheck(const int64_t* __restrict__ total, int64_t cap, int* __restrict__ overflow) {
  *overflow = *total > cap ? 1 : 0;
}

// After the fill: the evaluation's report to the host, in mapped host memory (read without a
// synchronisation before a later evaluation): overflow (sticky until the host grows the
// buffer), the largest list total seen, a traversal stack overflow.
__global__ void report(const int64_t* __restrict__ total, const int* __restrict__ overflow,
                       const int* __restrict__ stackErr, TreeWatch* __restrict__ w) {
  const long long t = *total;
  if (t > w->maxTotal) w->maxTotal = t;
  if (*overflow) w->overflow = 1;
  if (*stackErr) w->stackErr = 1;
}

// Sort keys of the work order: tiles by descending list length, ties by tile index.
__global__ void orderKeys(const int64_t* __restrict__ lens, int ntiles, uint64_t* __restrict__ keys) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const uint64_t l = (uint64_t)min(lens[t], (int64_t)INT32_MAX);
  keys[t] = ((uint64_t)INT32_MAX - l) << 32 | (uint32_t)t;
}

// Work items: each tile's list in nchunks parts, tiles in key order, a tile's parts in order.
__global__ void expandOrder(const uint64_t* __restrict__ keys, int ntiles, int nchunks, int* __restrict__ order) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntiles * nchunks) return;
  const int t = (int)(uint32_t)keys[i / nchunks];
  order[i] = t * nchunks + i % nchunks;
}

// Statistics of the evaluation (fixed-order block sums): pairs, direct pairs, far (proxy) pairs,
// far clusters and the octree's nodes.  With overflowing lists every tile took every source.
__global__ void __launch_bounds__(kBlock) treeStats(const int2* __restrict__ tiles, const int64_t* __restrict__ lens,
                                                    const int64_t* __restrict__ fars, int ntiles, int P, int ns,
                                                    const int* __restrict__ overflow, const int* __restrict__ dcount,
                                                    int depth, double* __restrict__ out) {
  __shared__ double sh[kBlock / 32];
  const bool dir = *overflow != 0;
  double pairs = 0, far = 0, clusters = 0;
  for (int t = threadIdx.x; t < ntiles; t += kBlock) {
    const double tc = (double)tiles[t].y;
    pairs += tc * (double)(dir ? ns : lens[t]);
    if (!dir) {
      far += tc * (double)fars[t];
      clusters += (double)(fars[t] / max(1, P));
    }
  }
  pairs = blockSum<kBlock>(pairs, sh);
  far = blockSum<kBlock>(far, sh);
  clusters = blockSum<kBlock>(clusters, sh);
  if (threadIdx.x == 0) {
    double nodes = 0;
    if (dcount)
      for (int l = 0; l <= depth; ++l) nodes += dcount[l];
    out[0] = pairs;
    out[1] = pairs - far;
    out[2] = far;
    out[3] = clusters;
    out[4] = nodes;
  }
}

inline unsigned blocks(int64_t n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? LPM_ERR_OUT_OF_MEMORY : LPM_ERR_CUDA, "tree code %s: %s", what,
         cudaGetErrorString(e));
  }
}

}  // namespace

int treeDepthFor(int64_t n, int leafPoints) {
  int d = 1;
  while (d < kOctreeMaxDepth && 4.7 * std::pow(4.0, d) * std::max(1, leafPoints) < (double)n) ++d;
  return d;
}

template <typename T>
T* TreeEval::grow(Buf& b, size_t count, cudaStream_t s) {
  const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
  if (b.bytes < bytes) {
    if (b.p) ck(cudaFreeAsync(b.p, s), "free");
    b.p = nullptr;
    b.bytes = 0;
    const size_t want = bytes + bytes / 4;
    ck(cudaMallocAsync(&b.p, want, s), "allocation");
    b.bytes = want;
  }
  return static_cast<T*>(b.p);
}

// Report slots in mapped host memory, allocated in blocks and recycled: freeing mapped memory
// would synchronise the device, and a slot may still be written by kernels in flight when its
// evaluator goes away.  A slot returns to the pool only once the work queued before its release
// has completed (a host function on that stream) or after a device synchronisation.
class WatchPool {
 public:
  static WatchPool& get() {
    static WatchPool* p = new WatchPool();  // lives as long as the process (host functions may run late)
    return *p;
  }
  void take(TreeWatch** host, TreeWatch** dev) {
    std::lock_guard<std::mutex> lk(mu_);
    if (free_.empty()) {
      constexpr int kBlock = 64;
      void* h = nullptr;
      ck(cudaHostAlloc(&h, sizeof(TreeWatch) * kBlock, cudaHostAllocMapped | cudaHostAllocPortable),
         "host allocation");
      void* d = nullptr;
      ck(cudaHostGetDevicePointer(&d, h, 0), "mapped pointer");
      for (int i = kBlock - 1; i >= 0; --i)
        free_.emplace_back(static_cast<TreeWatch*>(h) + i, static_cast<TreeWatch*>(d) + i);
    }
    *host = free_.back().first;
    *dev = free_.back().second;
    free_.pop_back();
    std::memset(*host, 0, sizeof(TreeWatch));
  }
  void give(TreeWatch* host, TreeWatch* dev) {
    std::lock_guard<std::mutex> lk(mu_);
    free_.emplace_back(host, dev);
  }
  struct Pending {
    TreeWatch* host;
    TreeWatch* dev;
  };
  static void CUDART_CB giveLater(void* p) {  // host function: no CUDA calls
    Pending* q = static_cast<Pending*>(p);
    get().give(q->host, q->dev);
    delete q;
  }

 private:
  std::mutex mu_;
  std::vector<std::pair<TreeWatch*, TreeWatch*>> free_;
};

TreeEval::~TreeEval() {
  bool held = false;
  for (Buf* b : all_) held = held || b->p;
  if (held) {  // not released in stream order: wait for the device, then free
    cudaDeviceSynchronize();
    for (Buf* b : all_)
      if (b->p) cudaFree(b->p);
  }
  if (watch_) WatchPool::get().give(watch_, dWatch_);
}

void TreeEval::release(cudaStream_t s) {
  for (Buf* b : all_) {
    if (b->p) ck(cudaFreeAsync(b->p, s), "free");
    b->p = nullptr;
    b->bytes = 0;
  }
  tree_.release(s);
  if (watch_) {
    auto* q = new WatchPool::Pending{watch_, dWatch_};
    const cudaError_t e = cudaLaunchHostFunc(s, WatchPool::giveLater, q);
    if (e != cudaSuccess) {
      delete q;  // the slot is dropped, not reused
      ck(e, "host function");
    }
    watch_ = nullptr;
    dWatch_ = nullptr;
  }
  partial_ = nullptr;
  listCap_ = 0;
  devAt_ = nullptr;
  hDev_ = TreeDev{};
  statsOnDevice_ = false;
  ++generation_;
}

void TreeEval::ensureWatch() {
  if (watch_) return;
  WatchPool::get().take(&watch_, &dWatch_);
}

bool TreeEval::poll() {
  if (!watch_) return false;
  volatile TreeWatch* w = watch_;
  if (w->stackErr) {
    w->stackErr = 0;
    fail(LPM_ERR_INTERNAL, "tree code: traversal stack overflow (octree depth %d)", tree_.depth);
  }
  if (!w->overflow) return false;
  // an evaluation since the last poll did not fit its lists (it summed every source instead):
  // room for the largest total seen, with headroom, from the next evaluation on
  listCap_ = std::max<int64_t>(listCap_, (int64_t)(1.25 * (double)w->maxTotal) + 4096);
  w->overflow = 0;
  ++generation_;
  return true;
}

const TreeStats& TreeEval::stats() {
  if (statsOnDevice_) {
    double v[5] = {};
    ck(cudaDeviceSynchronize(), "synchronise");
    ck(cudaMemcpy(v, bStats.p, sizeof(v), cudaMemcpyDeviceToHost), "read-back");
    stats_.pairs = v[0];
    stats_.directPairs = v[1];
    stats_.farPairs = v[2];
    stats_.farClusters = (int64_t)v[3];
    stats_.nodes = (int64_t)v[4];
  }
  return stats_;
}

void TreeEval::evaluate(SolvePlan& Pl, const TreeParams& tp, const PairShape& shape, bool psi, bool precise,
                        bool rcpApprox, int slots, int grid, PairTimer* timer, cudaStream_t s) {
  if (tp.degree < 2 || tp.degree > kMaxDegree) fail(LPM_ERR_INVALID_ARGUMENT, "tree code: degree must be 2..%d", kMaxDegree);
  if (!(tp.theta > 0.0 && tp.theta < 1.0)) fail(LPM_ERR_INVALID_ARGUMENT, "tree code: theta must be in (0, 1)");
  if (!treePairShapeSupported(shape)) fail(LPM_ERR_NOT_SUPPORTED, "tree code: plan built for another launch shape");
  const int ns = Pl.ns, nslots = Pl.nslots, ntiles = Pl.nTreeTiles;
  const int P = (tp.degree + 1) * (tp.degree + 1);
  ensureWatch();
  // reports of earlier evaluations (no synchronisation); never while the stream is captured, where
  // a report arriving now would make the capture grow a buffer (callers poll before capturing)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ck(cudaStreamIsCapturing(s, &cap), "capture status");
  if (cap == cudaStreamCaptureStatusNone) poll();
  direct_ = false;
  stats_ = TreeStats{};
  statsOnDevice_ = true;
  // phase timing (with the context's timer): events at the phase boundaries, read at the end
  cudaEvent_t ev[5] = {};
  if (timer)
    for (auto& e : ev) e = timer->get();
  auto mark = [&](int i) {
    if (timer) ck(cudaEventRecord(ev[i], s), "event");
  };
  mark(0);

  const int* selfSorted = nullptr;
  int* tslot = nullptr;
  int nnodes = 0;
  float4* tsp0 = nullptr;
  float4* tsp1 = nullptr;
  float4* geom = nullptr;
  int* approx = nullptr;
  int depth = 0;
  if (ns > 0) {
    // 1-3. octree over the stage positions (fixed-level layout, counts on the device), sources in
    // key order
    double* pos = grow<double>(bPos, 3 * (size_t)ns, s);
    srcPositions<<<blocks(ns), kBlock, 0, s>>>(Pl.stage.sp0, Pl.stage.sp1, ns, pos);
    depth = treeDepthFor(ns, tp.leafPoints);
    tree_.buildOnDevice(pos, 3, 1, ns, depth, s);
    mark(1);
    nnodes = (int)tree_.nnodes;  // capacity: nodes past a level's count are empty
    stats_.depth = depth;
    const size_t nrec = (size_t)ns + (size_t)nnodes * P;
    tsp0 = grow<float4>(bSp0, nrec, s);
    tsp1 = grow<float4>(bSp1, nrec, s);
    int* inv = grow<int>(bInv, ns, s);
    tslot = grow<int>(bSlot, ns, s);
    gatherSources<<<blocks(ns), kBlock, 0, s>>>(tree_.origIds, Pl.stage.sp0, Pl.stage.sp1, Pl.stage.srcSlot, ns, tsp0,
                                                tsp1, inv, tslot);
    int* ss = grow<int>(bSelf, nslots, s);
    sortedSelf<<<blocks(nslots), kBlock, 0, s>>>(Pl.dev.self, inv, nslots, ss);
    selfSorted = ss;
    // 4. upward pass (empty nodes return at once)
    geom = grow<float4>(bGeom, nnodes, s);
    approx = grow<int>(bApprox, nnodes, s);
    upward<<<nnodes, kUpThreads, 0, s>>>(tree_.ptInds, tp.degree, chebFor(tp.degree), ns,
                                         depth >= 2 ? tree_.base[2] : nnodes, geom, approx, tsp0, tsp1);
    mark(2);
  } else {
    mark(1);
    mark(2);
    int* ss = grow<int>(bSelf, nslots, s);
    ck(cudaMemsetAsync(ss, 0xff, sizeof(int) * (size_t)nslots, s), "memset");  // -1: no sources
    selfSorted = ss;
    tsp0 = grow<float4>(bSp0, 1, s);
    tsp1 = grow<float4>(bSp1, 1, s);
    tslot = grow<int>(bSlot, 1, s);
  }
  // 5. tiles
  float4* tgeom = grow<float4>(bTileGeom, ntiles, s);
  const float theta2 = (float)(tp.theta * tp.theta);
  tileGeometry<<<(ntiles + kGeomTilesPerBlock - 1) / kGeomTilesPerBlock, kBlock, 0, s>>>(
      Pl.stage.tx, nslots, Pl.treeTiles, ntiles, Pl.stage.perm, Pl.io.na, Pl.mask, tgeom);
  // 6. interaction lists: lengths, offsets (a device scan), the work order (a device sort) and
  // the indices -- nothing read back but the very first total, which sizes the list buffer
  int64_t* lens = grow<int64_t>(bLen, ntiles, s);
  int64_t* fars = grow<int64_t>(bFar, ntiles, s);
  Levels lv{};
  for (int l = 0; l <= tree_.depth; ++l) lv.base[l] = tree_.base[l];
  lv.base[tree_.depth + 1] = nnodes;
  int* terr = grow<int>(bErr, 2, s);  // [0] stack overflow, [1] list overflow
  int* overflow = terr + 1;
  ck(cudaMemsetAsync(terr, 0, 2 * sizeof(int), s), "memset");
  if (ns > 0) {
    traverse<false><<<ntiles, 32, 0, s>>>(tgeom, ntiles, geom, approx, tree_.ptInds, tree_.kids, lv, tree_.depth,
                                          theta2, P, ns, lens, fars, nullptr, nullptr, overflow, terr);
  } else {
    ck(cudaMemsetAsync(lens, 0, sizeof(int64_t) * ntiles, s), "memset");
    ck(cudaMemsetAsync(fars, 0, sizeof(int64_t) * ntiles, s), "memset");
  }
  mark(3);
  int64_t* off = grow<int64_t>(bOff, (size_t)ntiles + 1, s);
  uint64_t* keys = grow<uint64_t>(bKey, ntiles, s);
  uint64_t* keys2 = grow<uint64_t>(bKey2, ntiles, s);
  size_t tscan = 0, tsort = 0;
  ck(cub::DeviceScan::InclusiveSum(nullptr, tscan, lens, off + 1, ntiles, s), "scan size");
  ck(cub::DeviceRadixSort::SortKeys(nullptr, tsort, keys, keys2, ntiles, 0, 64, s), "sort size");
  void* temp = grow<unsigned char>(bTemp, std::max(tscan, tsort), s);
  size_t tb = bTemp.bytes;
  ck(cudaMemsetAsync(off, 0, sizeof(int64_t), s), "memset");
  ck(cub::DeviceScan::InclusiveSum(temp, tb, lens, off + 1, ntiles, s), "scan");
  if (listCap_ == 0) {  // the first evaluation sizes the list buffer (its one synchronisation)
    int64_t total = 0;
    ck(cudaMemcpyAsync(&total, off + ntiles, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "read-back");
    ck(cudaStreamSynchronize(s), "synchronise");
    listCap_ = std::max<int64_t>((int64_t)(1.25 * (double)total) + 4096, ns);  // >= ns: the fallback
    ++generation_;
  }
  int* oldList = static_cast<int*>(bList.p);
  int* list = grow<int>(bList, (size_t)listCap_, s);
  if (list != oldList) ++generation_;
  capCheck<<<1, 1, 0, s>>>(off + ntiles, listCap_, overflow);
  // Work items: each tile's list in `nchunks` parts (enough items for ~8 waves of CTAs), each
  // part with its own partial chunk; tiles by descending list length (ties by tile index).
  const int nchunks = std::max(1, std::min(16, (8 * std::max(1, slots) + ntiles - 1) / std::max(1, ntiles)));
  const int nitems = ntiles * nchunks;
  int* order = grow<int>(bOrder, nitems, s);
  orderKeys<<<blocks(ntiles), kBlock, 0, s>>>(lens, ntiles, keys);
  tb = bTemp.bytes;
  ck(cub::DeviceRadixSort::SortKeys(temp, tb, keys, keys2, ntiles, 0, 64, s), "sort");
  expandOrder<<<blocks(nitems), kBlock, 0, s>>>(keys2, ntiles, nchunks, order);
  if (ns > 0)
    traverse<true><<<ntiles, 32, 0, s>>>(tgeom, ntiles, geom, approx, tree_.ptInds, tree_.kids, lv, tree_.depth,
                                         theta2, P, ns, nullptr, nullptr, off, list, overflow, terr);
  report<<<1, 1, 0, s>>>(off + ntiles, overflow, terr, dWatch_);
  double* dstats = grow<double>(bStats, 5, s);
  treeStats<<<1, kBlock, 0, s>>>(Pl.treeTiles, lens, fars, ntiles, P, ns, overflow, ns > 0 ? tree_.dcount : nullptr,
                                 depth, dstats);
  directFallback<<<blocks(std::max(1, std::max(ntiles, ns))), kBlock, 0, s>>>(overflow, off, lens, ntiles, list, ns);
  mark(4);
  // 7. the gathered pair kernel
  double* partial = grow<double>(bPartial, (size_t)nchunks * 5 * std::max(1, nslots), s);
  TreeDev hd;
  std::memset(&hd, 0, sizeof(hd));  // compared byte for byte with the last upload below
  hd.tx = Pl.stage.tx;
  hd.sp0 = tsp0;
  hd.sp1 = tsp1;
  hd.self = selfSorted;
  hd.tiles = Pl.treeTiles;
  hd.srcSlot = tslot;
  hd.tileCentre = Pl.treeCentres;
  hd.listOff = off;
  hd.list = list;
  hd.order = order;
  hd.partial = partial;
  hd.listLen = lens;
  hd.nslots = nslots;
  hd.ntiles = ntiles;
  hd.nchunks = nchunks;
  hd.ns = ns;
  hd.eps2 = Pl.eps2;
  TreeDev* dd = grow<TreeDev>(bDev, 1, s);
  if (dd != devAt_ || std::memcmp(&hd, &hDev_, sizeof(hd)) != 0) {  // unchanged between evaluations of a plan
    hDev_ = hd;
    devAt_ = dd;
    ck(cudaMemcpyAsync(dd, &hDev_, sizeof(hd), cudaMemcpyHostToDevice, s), "upload");
    ++generation_;
  }
  partial_ = partial;
  nchunks_ = nchunks;
  int* counter = grow<int>(bCounter, 1, s);
  ck(cudaMemsetAsync(counter, 0, sizeof(int), s), "memset");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (timer) {
    e0 = timer->get();
    e1 = timer->get();
    ck(cudaEventRecord(e0, s), "event");
  }
  ck(launchTreePair(shape, psi, precise, rcpApprox, dd, nitems, counter,
                    std::min(nitems, std::max(1, grid > 0 ? grid : slots)), s),
     "pair launch");
  if (timer) {
    ck(cudaEventRecord(e1, s), "event");
    timer->pending.emplace_back(e0, e1);
    // phases (the traversals end before the pair kernel starts)
    ck(cudaEventSynchronize(ev[4]), "event");
    float a = 0.f, b = 0.f, c = 0.f, d = 0.f;
    ck(cudaEventElapsedTime(&a, ev[0], ev[1]), "event");
    ck(cudaEventElapsedTime(&b, ev[1], ev[2]), "event");
    ck(cudaEventElapsedTime(&c, ev[2], ev[3]), "event");
    ck(cudaEventElapsedTime(&d, ev[3], ev[4]), "event");
    stats_.buildMs = a;
    stats_.upwardMs = b;
    stats_.listMs = c + d;  // tile geometry and count traversal, then offsets, order and the fill
    for (auto& e : ev) timer->pool.push_back(e);
  }
}

}  // namespace lpm
