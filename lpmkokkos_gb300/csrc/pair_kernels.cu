// pair_kernels.cu -- the O(N^2) direct sums of the BVE path for sm_103a.
//
// Two kernels evaluate the spherical Biot-Savart velocity (and optionally the stream
// function) of pbosler/lpmKokkos (src/LpmBVEKernels.hpp:21-44 greensFn / biotSavart,
// reductions :49-102 and :188-234) over work items (target tile x source chunk):
//
//  * pairFP64  -- the plain FP64 path (the GPU oracle).  Per pair it evaluates the
//    reference expression with the same operation order; multiplications and additions
//    are issued as __dmul_rn/__dadd_rn so no fused multiply-add changes a single pair's
//    rounding against the CPU.  Only the summation order differs (unpinned in Kokkos).
//
//  * pairFP32C -- the FP32-compensated path.  With d_j = x_j - x_i and
//    1 - x_i.x_j = |d|^2/2 + delta_i + delta_j (delta = (1 - |x|^2)/2, exact identity),
//      u_i = x_i x sum_j s_j d_j,   s_j = (-zeta_j A_j / 2 pi) / (|d|^2 + D_i + D_j + 2 eps^2),
//    D = 1 - |x|^2.  Coordinates are FP64 hi/lo float pairs; each CTA subtracts the centre
//    of its target tile once per staged source, so every FP32 difference is taken between
//    nearby small numbers.  Per pair: 13 FP32 FMA-pipe ops + one MUFU.RCP
//    (3 FADD d, 1 FADD + 3 FFMA for 2q, 1 FMUL + 1 FFMA + 1 FMUL for w r and the Newton
//    step, 3 FFMA accumulate), issued as paired f32x2 instructions over two targets.
//    Each 64-source sub-block is summed in FP32 and added to a Kahan-compensated FP32
//    accumulator; partials leave the kernel in FP64 and the epilogue forms the FP64 cross
//    product.  Stream function: + MUFU.LG2, 1 FFMA, 1 FADD per pair.
//
// Both kernels are persistent: each CTA takes work items from an atomic counter until
// the list is exhausted.  Self pairs (i == j, collocated face targets) are excluded by
// index only on the few source tiles that can contain them (tileSelf range), so the
// common path carries no compare.

#include "engine.hpp"
#include "tree.hpp"

#include <climits>
#include <cstdio>
#include <type_traits>

namespace lpm {
namespace {

__device__ __forceinline__ float rcpApprox(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float lg2Approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Asynchronous global -> shared copies (cp.async, cached in L1 and L2), in commit groups.
__device__ __forceinline__ void cpAsync16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpAsync4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Kahan step: add v into the compensated pair (h, c); the represented value is h - c.
__device__ __forceinline__ void kahanAdd(float& h, float& c, float v) {
  const float y = v - c;
  const float t = h + y;
  c = (t - h) - y;
  h = t;
}

// FP32 relative coordinate (x - centre) from an FP64 value split as hi + lo.
__device__ __forceinline__ float relCoord(float hi, float lo, float chi, float clo) {
  return (hi - chi) + (lo - clo);
}

constexpr int kSub = 64;  // sources per FP32 sub-block before the compensated add

// A usable tile centre lies near the unit sphere.  Masked parent faces that (nearly) coincide
// with a leaf get inf/NaN or huge velocities, as in the reference, and drift arbitrarily far.
__device__ __forceinline__ bool saneCentre(double x, double y, double z) {
  const double r2 = x * x + y * y + z * z;
  return r2 >= 0.25 && r2 <= 4.0;  // false for NaN too
}

// Centre of a target tile: the plan's centre slot (a vertex or leaf face near the middle of the
// tile) if its position is sane, else the first sane target of the tile, else the origin.
// The fallback branch is uniform across the CTA.
__device__ __forceinline__ void tileCentre(const double* __restrict__ tx, int n, int tile0, int tcount, int nth,
                                           int cs, int* sCentre, double& cx, double& cy, double& cz) {
  cx = tx[cs]; cy = tx[n + cs]; cz = tx[2 * n + cs];
  if (saneCentre(cx, cy, cz)) return;
  if (threadIdx.x == 0) *sCentre = INT_MAX;
  __syncthreads();
  for (int t = threadIdx.x; t < tcount; t += nth) {
    const int q = tile0 + t;
    if (saneCentre(tx[q], tx[n + q], tx[2 * n + q])) atomicMin(sCentre, t);
  }
  __syncthreads();
  const int c = *sCentre;
  if (c == INT_MAX) { cx = cy = cz = 0.0; return; }
  cx = tx[tile0 + c]; cy = tx[n + tile0 + c]; cz = tx[2 * n + tile0 + c];
}

// Paired FP32 arithmetic (f32x2): one instruction computes the same operation for two of a
// thread's targets, so the 13 FMA-pipe lane-ops of a pair issue as 6.5 instructions and the
// issue slots left over carry the reciprocal, the shared loads and the loop.  Each lane is
// rounded exactly as the scalar instruction would be.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Staged source tile, every value stored twice so that one shared load yields the pair operand
// (both halves hold the same source): XY = (x, x, y, y), ZW = (z, z, w, w), D = (D, D).
// Fast formulation: x, y, z relative to the tile origin; precise: hi parts, with the lo parts in
// LXY = (x_lo, x_lo, y_lo, y_lo), LZ = (z_lo, z_lo).  w = -zeta A / 2 pi, D = 1 - |x|^2.
template <bool PRECISE>
struct SourceTile;
template <>
struct SourceTile<false> {
  const float4* xy; const float4* zw; const float2* d;
};
template <>
struct SourceTile<true> {
  const float4* xy; const float4* zw; const float2* d; const float4* lxy; const float2* lz;
};

// One staged tile against the thread's K targets, held as K/2 target pairs with negated
// coordinates (nx = -x_i, so x_j + nx = x_j - x_i) and C = D_i + 2 eps^2.  Per pair:
//   d = x_j - x_i, 2q = D_j + C + |d|^2 (x, y, z in that order), r = rcp.approx(2q),
//   NEWTON:   s' = (w r) (2q r - 2) = -s   (the Newton step r (2 - 2q r), negated so that no
//             operand needs a sign flip), accumulated as v += s' d and folded with a minus sign;
//   !NEWTON:  s  = w r, folded with a plus sign.
// Each kSub-source block is summed in FP32, then added to the Kahan-compensated accumulators.
// GATHER: the staged sources are not consecutive; ids[j] holds the source index of slot j for
// the self-pair check (the tree code's index lists), else slot j is source jbase + j.
template <int K, bool PSI, bool CHECKED, bool PRECISE, bool NEWTON, bool GATHER = false>
__device__ __forceinline__ void fp32cTile(const SourceTile<PRECISE>& T, int nsrc, int jbase, const int* ids,
                                          const float2 (&nx)[K / 2], const float2 (&ny)[K / 2],
                                          const float2 (&nz)[K / 2], const float2 (&nlx)[K / 2],
                                          const float2 (&nly)[K / 2], const float2 (&nlz)[K / 2],
                                          const float2 (&C)[K / 2], const int (&self)[K],
                                          float (&hx)[K], float (&hy)[K], float (&hz)[K],
                                          float (&cx)[K], float (&cy)[K], float (&cz)[K],
                                          float (&hp)[K], float (&cp)[K], float (&hw)[K], float (&cw)[K]) {
  constexpr int P = K / 2;
  constexpr float kSign = NEWTON ? -1.f : 1.f;
  const float2 kMinusTwo = make_float2(-2.f, -2.f);
  // sources per unrolled iteration: 2 with four target pairs per thread (measured 1 % faster
  // than 4 at 128 x 8; 8 was 5 % slower), 4 otherwise
  constexpr int kUnroll = K >= 8 ? 2 : 4;
#pragma unroll 1
  for (int j0 = 0; j0 < nsrc; j0 += kSub) {
    float2 vx[P], vy[P], vz[P], vp[P], vw[P];
#pragma unroll
    for (int m = 0; m < P; ++m) {
      vx[m] = vy[m] = vz[m] = vp[m] = vw[m] = make_float2(0.f, 0.f);
    }
#pragma unroll kUnroll
    for (int j = j0; j < j0 + kSub; ++j) {
      const float4 xy = T.xy[j];
      const float4 zw = T.zw[j];
      const float2 dj = T.d[j];
      const float2 X = make_float2(xy.x, xy.y), Y = make_float2(xy.z, xy.w), Z = make_float2(zw.x, zw.y);
      const float2 W = make_float2(zw.z, zw.w);
      float2 LX, LY, LZ;
      if constexpr (PRECISE) {
        const float4 lxy = T.lxy[j];
        LX = make_float2(lxy.x, lxy.y);
        LY = make_float2(lxy.z, lxy.w);
        LZ = T.lz[j];
      }
#pragma unroll
      for (int m = 0; m < P; ++m) {
        float2 dx, dy, dz;
        if constexpr (PRECISE) {  // hi parts subtract exactly when close; lo parts restore the rest
          dx = add2(add2(X, nx[m]), add2(LX, nlx[m]));
          dy = add2(add2(Y, ny[m]), add2(LY, nly[m]));
          dz = add2(add2(Z, nz[m]), add2(LZ, nlz[m]));
        } else {
          dx = add2(X, nx[m]);
          dy = add2(Y, ny[m]);
          dz = add2(Z, nz[m]);
        }
        float2 q = add2(dj, C[m]);
        q = fma2(dx, dx, q);
        q = fma2(dy, dy, q);
        q = fma2(dz, dz, q);
        const float2 r = make_float2(rcpApprox(q.x), rcpApprox(q.y));
        float2 sp = mul2(W, r);
        if (NEWTON) sp = mul2(sp, fma2(q, r, kMinusTwo));
        float2 lg, ww;
        if (PSI) { lg = make_float2(lg2Approx(q.x), lg2Approx(q.y)); ww = W; }
        if (CHECKED) {  // a self pair has q ~ 0: drop its (inf/NaN) terms after they are formed
          const int jj = GATHER ? ids[j] : jbase + j;
          if (jj == self[2 * m]) { sp.x = 0.f; if (PSI) { lg.x = 0.f; ww.x = 0.f; } }
          if (jj == self[2 * m + 1]) { sp.y = 0.f; if (PSI) { lg.y = 0.f; ww.y = 0.f; } }
        }
        vx[m] = fma2(sp, dx, vx[m]);
        vy[m] = fma2(sp, dy, vy[m]);
        vz[m] = fma2(sp, dz, vz[m]);
        if (PSI) {
          vp[m] = fma2(W, lg, vp[m]);
          vw[m] = add2(vw[m], ww);
        }
      }
    }
#pragma unroll
    for (int m = 0; m < P; ++m) {
      kahanAdd(hx[2 * m], cx[2 * m], kSign * vx[m].x);
      kahanAdd(hx[2 * m + 1], cx[2 * m + 1], kSign * vx[m].y);
      kahanAdd(hy[2 * m], cy[2 * m], kSign * vy[m].x);
      kahanAdd(hy[2 * m + 1], cy[2 * m + 1], kSign * vy[m].y);
      kahanAdd(hz[2 * m], cz[2 * m], kSign * vz[m].x);
      kahanAdd(hz[2 * m + 1], cz[2 * m + 1], kSign * vz[m].y);
      if (PSI) {
        kahanAdd(hp[2 * m], cp[2 * m], vp[m].x);
        kahanAdd(hp[2 * m + 1], cp[2 * m + 1], vp[m].y);
        kahanAdd(hw[2 * m], cw[2 * m], vw[m].x);
        kahanAdd(hw[2 * m + 1], cw[2 * m + 1], vw[m].y);
      }
    }
  }
}

// The K targets of a thread in tile-relative FP32 form (fast) or hi/lo form (precise), as K/2
// negated pairs, with C = D_i + 2 eps^2 and each target's self index; plus the tile centre's
// hi/lo parts (fast formulation).
template <int K>
struct TileTargets {
  float2 nx[K / 2], ny[K / 2], nz[K / 2], nlx[K / 2], nly[K / 2], nlz[K / 2], C[K / 2];
  int self[K];
  float chx, chy, chz, clx, cly, clz;
};

template <int NTH, int K, bool PRECISE>
__device__ __forceinline__ void loadTileTargets(const double* __restrict__ tx, int n, int tile0, int tcount,
                                                int centreSlot, const int* __restrict__ selfIdx, double eps2,
                                                int* sCentre, TileTargets<K>& tt) {
  // Tile centre (slots are spatially sorted).  A masked parent that coincides with a leaf
  // carries inf/NaN or a runaway position (as in the reference); it must never become the
  // centre, or every target of the tile would lose its precision.
  float chx = 0.f, chy = 0.f, chz = 0.f, clx = 0.f, cly = 0.f, clz = 0.f;
  if (!PRECISE) {
    double cxd, cyd, czd;
    tileCentre(tx, n, tile0, tcount, NTH, centreSlot, sCentre, cxd, cyd, czd);
    chx = __double2float_rn(cxd); chy = __double2float_rn(cyd); chz = __double2float_rn(czd);
    clx = __double2float_rn(cxd - (double)chx);
    cly = __double2float_rn(cyd - (double)chy);
    clz = __double2float_rn(czd - (double)chz);
  }
  tt.chx = chx; tt.chy = chy; tt.chz = chz; tt.clx = clx; tt.cly = cly; tt.clz = clz;

  // Targets k = 2m, 2m+1 of this thread form pair m (slots tile0 + threadIdx.x + k NTH).
  float ax[K], ay[K], az[K], lx[K], ly[K], lz[K], Ck[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int slot = tile0 + threadIdx.x + k * NTH;
    if (threadIdx.x + k * NTH < tcount) {
      const double x = tx[slot], y = tx[n + slot], z = tx[2 * n + slot];
      const float hx = __double2float_rn(x), hy = __double2float_rn(y), hz = __double2float_rn(z);
      const float ex = __double2float_rn(x - (double)hx), ey = __double2float_rn(y - (double)hy),
                  ez = __double2float_rn(z - (double)hz);
      if (PRECISE) {
        ax[k] = hx; ay[k] = hy; az[k] = hz; lx[k] = ex; ly[k] = ey; lz[k] = ez;
      } else {
        ax[k] = relCoord(hx, ex, chx, clx);
        ay[k] = relCoord(hy, ey, chy, cly);
        az[k] = relCoord(hz, ez, chz, clz);
        lx[k] = ly[k] = lz[k] = 0.f;
      }
      Ck[k] = __double2float_rn((1.0 - (x * x + y * y + z * z)) + 2.0 * eps2);
      tt.self[k] = selfIdx[slot];
    } else {
      ax[k] = 0.f; ay[k] = 0.f; az[k] = 0.f; lx[k] = ly[k] = lz[k] = 0.f; Ck[k] = 1.f; tt.self[k] = -1;
    }
  }
#pragma unroll
  for (int m = 0; m < K / 2; ++m) {
    tt.nx[m] = make_float2(-ax[2 * m], -ax[2 * m + 1]);
    tt.ny[m] = make_float2(-ay[2 * m], -ay[2 * m + 1]);
    tt.nz[m] = make_float2(-az[2 * m], -az[2 * m + 1]);
    tt.nlx[m] = make_float2(-lx[2 * m], -lx[2 * m + 1]);
    tt.nly[m] = make_float2(-ly[2 * m], -ly[2 * m + 1]);
    tt.nlz[m] = make_float2(-lz[2 * m], -lz[2 * m + 1]);
    tt.C[m] = make_float2(Ck[2 * m], Ck[2 * m + 1]);
  }
}

// Stages one source record (p0, p1) in slot j: relative to the tile centre (fast) or as hi/lo
// parts (precise).  A dead slot gets zero weight and D = 1 at the centre / origin, so it adds
// exactly 0.
template <int K, bool PRECISE>
__device__ __forceinline__ void stageSource(int j, bool live, const float4& p0, const float4& p1,
                                            const TileTargets<K>& tt, float4* sXY, float4* sZW, float2* sD,
                                            float4* sLXY, float2* sLZ) {
  float x = 0.f, y = 0.f, z = 0.f, wj = 0.f, dj = 1.f, ux = 0.f, uy = 0.f, uz = 0.f;
  if (live) {
    if (PRECISE) {
      x = p0.x; y = p0.y; z = p0.z; ux = p1.x; uy = p1.y; uz = p1.z;
    } else {
      x = relCoord(p0.x, p1.x, tt.chx, tt.clx);
      y = relCoord(p0.y, p1.y, tt.chy, tt.cly);
      z = relCoord(p0.z, p1.z, tt.chz, tt.clz);
    }
    wj = p0.w;
    dj = p1.w;
  }
  sXY[j] = make_float4(x, x, y, y);
  sZW[j] = make_float4(z, z, wj, wj);
  sD[j] = make_float2(dj, dj);
  if (PRECISE) {
    sLXY[j] = make_float4(ux, ux, uy, uy);
    sLZ[j] = make_float2(uz, uz);
  }
}

// Writes a thread's compensated sums as FP64 partials [comp][slot] of one chunk.
template <int NTH, int K, bool PSI>
__device__ __forceinline__ void writePartials(double* __restrict__ out, int n, int tile0, int tcount,
                                              const float (&hx)[K], const float (&hy)[K], const float (&hz)[K],
                                              const float (&cx)[K], const float (&cy)[K], const float (&cz)[K],
                                              const float (&hp)[K], const float (&cp)[K], const float (&hw)[K],
                                              const float (&cw)[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int slot = tile0 + threadIdx.x + k * NTH;
    if (threadIdx.x + k * NTH < tcount) {
      out[slot] = (double)hx[k] - (double)cx[k];
      out[n + slot] = (double)hy[k] - (double)cy[k];
      out[2 * n + slot] = (double)hz[k] - (double)cz[k];
      if (PSI) {
        out[3 * n + slot] = (double)hp[k] - (double)cp[k];
        out[4 * n + slot] = (double)hw[k] - (double)cw[k];
      }
    }
  }
}

// PRECISE = false: targets are mesh points (vertices / face centres), which keep about half a
//   mesh spacing from every other source; coordinates relative to the tile centre keep the
//   FP32 differences accurate to ~1e-7 * (tile radius / spacing).  13 FMA-pipe ops per pair.
// PRECISE = true: arbitrary target points (possibly very close to a source); differences
//   are formed from hi/lo float pairs, accurate to ~1e-7 relative.  19 FMA-pipe ops per pair.
// NEWTON = false skips the Newton refinement of the hardware reciprocal (11 FMA-pipe ops per
//   pair in the fast formulation); selected by LPM_BVE_RCP_APPROX.
// MINB: minimum resident CTAs per SM the register allocation must allow (__launch_bounds__).
template <int NTH, int K, int ST, int MINB, bool PSI, bool PRECISE, bool NEWTON>
__global__ void __launch_bounds__(NTH, MINB) pairFP32C(const SolveDev* __restrict__ solves,
                                                 const WorkItem* __restrict__ items, int nitems,
                                                 int* __restrict__ counter) {
  static_assert(ST % kSub == 0, "source tile must be a multiple of the sub-block");
  static_assert(K % 2 == 0, "targets are processed in pairs");
  constexpr int P = K / 2;
  __shared__ float4 sXY[ST];
  __shared__ float4 sZW[ST];
  __shared__ float2 sD[ST];
  __shared__ float4 sLXY[PRECISE ? ST : 1];
  __shared__ float2 sLZ[PRECISE ? ST : 1];
  __shared__ int sItem;
  __shared__ int sCentre;
  SourceTile<PRECISE> T;
  T.xy = sXY; T.zw = sZW; T.d = sD;
  if constexpr (PRECISE) { T.lxy = sLXY; T.lz = sLZ; }

  for (;;) {
    if (threadIdx.x == 0) sItem = atomicAdd(counter, 1);
    __syncthreads();
    const int it = sItem;
    __syncthreads();
    if (it >= nitems) return;
    const WorkItem w = items[it];
    const SolveDev& S = solves[w.solve];
    const int n = S.nslots;
    const int tile0 = w.tbeg;
    const int tcount = min(NTH * K, w.tend - tile0);

    TileTargets<K> tt;
    loadTileTargets<NTH, K, PRECISE>(S.tx, n, tile0, tcount, S.tileCentre[w.tile], S.self, S.eps2, &sCentre, tt);
    const float2 (&nx)[P] = tt.nx;
    const float2 (&ny)[P] = tt.ny;
    const float2 (&nz)[P] = tt.nz;
    const float2 (&nlx)[P] = tt.nlx;
    const float2 (&nly)[P] = tt.nly;
    const float2 (&nlz)[P] = tt.nlz;
    const float2 (&C)[P] = tt.C;
    const int (&self)[K] = tt.self;
    float hx[K], hy[K], hz[K], cx[K], cy[K], cz[K], hp[K], cp[K], hw[K], cw[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      hx[k] = hy[k] = hz[k] = cx[k] = cy[k] = cz[k] = 0.f;
      hp[k] = cp[k] = hw[k] = cw[k] = 0.f;
    }
    const int2 ts = S.tileSelf[w.tile];

    for (int b0 = w.s0; b0 < w.s1; b0 += ST) {
      // Stage ST sources; padding (w = 0, D = 1) adds exactly 0.
      for (int j = threadIdx.x; j < ST; j += NTH) {
        const int src = b0 + j;
        const bool live = src < w.s1;
        stageSource<K, PRECISE>(j, live, live ? S.sp0[src] : float4{}, live ? S.sp1[src] : float4{}, tt, sXY, sZW,
                                sD, sLXY, sLZ);
      }
      __syncthreads();
      const bool checked = (ts.x <= b0 + ST - 1) && (ts.y >= b0);
      if (checked)
        fp32cTile<K, PSI, true, PRECISE, NEWTON>(T, ST, b0, nullptr, nx, ny, nz, nlx, nly, nlz, C, self, hx, hy, hz,
                                                 cx, cy, cz, hp, cp, hw, cw);
      else
        fp32cTile<K, PSI, false, PRECISE, NEWTON>(T, ST, b0, nullptr, nx, ny, nz, nlx, nly, nlz, C, self, hx, hy, hz,
                                                  cx, cy, cz, hp, cp, hw, cw);
      __syncthreads();
    }

    // Partials: [chunk][comp][slot], FP64.
    writePartials<NTH, K, PSI>(S.partial + (size_t)w.chunk * (PSI ? 5 : 3) * n, n, tile0, tcount, hx, hy, hz, cx,
                               cy, cz, hp, cp, hw, cw);
  }
}

// The tree code's gathered pair kernel: persistent CTAs take target tiles (longest index
// lists first); each tile walks its flattened list of sorted-source and proxy indices
// (tree.hpp), staging up to ST gathered records at a time; the gathered records of the next
// block are in flight (cp.async) while a block computes.  Only the last block of a list is
// padded (to the sub-block of 64).  The self-pair check runs only on blocks that hold the source
// of one of the tile's own targets.  One FP64 partial chunk per target.
template <int NTH, int K, int ST, int MINB, bool PSI, bool PRECISE, bool NEWTON>
__global__ void __launch_bounds__(NTH, MINB) treeFP32C(const TreeDev* __restrict__ dev, int nitems,
                                                 int* __restrict__ counter) {
  static_assert(ST % kSub == 0, "source tile must be a multiple of the sub-block");
  static_assert(ST % NTH == 0, "each thread stages ST / NTH sources");
  constexpr int P = K / 2;
  __shared__ float4 sXY[ST];
  __shared__ float4 sZW[ST];
  __shared__ float2 sD[ST];
  __shared__ float4 sLXY[PRECISE ? ST : 1];
  __shared__ float2 sLZ[PRECISE ? ST : 1];
  __shared__ int sId[ST];
  // Raw records of the next block, fetched by cp.async while the current block computes.  Slot j
  // is written and read back only by the lane that stages source j, so the lane's own wait is
  // the only synchronisation these buffers need.
  __shared__ __align__(16) float4 sRaw0[ST];
  __shared__ __align__(16) float4 sRaw1[ST];
  __shared__ int sRawSlot[ST];
  __shared__ int sRawId[ST];
  __shared__ int sItem;
  __shared__ int sCentre;
  SourceTile<PRECISE> T;
  T.xy = sXY; T.zw = sZW; T.d = sD;
  if constexpr (PRECISE) { T.lxy = sLXY; T.lz = sLZ; }
  const TreeDev& S = *dev;
  constexpr int kPer = ST / NTH;
  // Starts the copies of one block's records (ids[i]: list entry of slot threadIdx.x + i NTH,
  // INT_MIN past the end) and records the ids beside them.
  auto fetch = [&](const int (&ids)[kPer]) {
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int j = threadIdx.x + i * NTH;
      const int id = ids[i];
      sRawId[j] = id;
      if (id != INT_MIN) {
        cpAsync16(&sRaw0[j], S.sp0 + id);
        cpAsync16(&sRaw1[j], S.sp1 + id);
        if (id < S.ns) cpAsync4(&sRawSlot[j], S.srcSlot + id);
      }
    }
    cpAsyncCommit();
  };

  for (;;) {
    if (threadIdx.x == 0) sItem = atomicAdd(counter, 1);
    __syncthreads();
    const int it = sItem;
    __syncthreads();
    if (it >= nitems) return;
    const int item = S.order[it];
    const int tile = item / S.nchunks, part = item % S.nchunks;
    const int n = S.nslots;
    const int2 tr = S.tiles[tile];
    const int tile0 = tr.x, tcount = tr.y;  // tcount <= NTH * K
    TileTargets<K> tt;
    loadTileTargets<NTH, K, PRECISE>(S.tx, n, tile0, tcount, S.tileCentre[tile], S.self, S.eps2, &sCentre, tt);
    float hx[K], hy[K], hz[K], cx[K], cy[K], cz[K], hp[K], cp[K], hw[K], cw[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      hx[k] = hy[k] = hz[k] = cx[k] = cy[k] = cz[k] = 0.f;
      hp[k] = cp[k] = hw[k] = cw[k] = 0.f;
    }
    // part `part` of the tile's list: [l0, l1), cut at multiples of the sub-block.  (When the
    // evaluation's lists overflowed their buffer, every tile's list is the identity list of all
    // sorted sources: the exact direct sum.)
    const int64_t tl = S.listLen[tile];
    const int64_t l0 = tl * part / S.nchunks / kSub * kSub;
    const int64_t l1 = part + 1 == S.nchunks ? tl : tl * (part + 1) / S.nchunks / kSub * kSub;
    const int64_t off = S.listOff[tile] + l0;
    const int64_t len = l1 - l0;
    auto entry = [&](int64_t q) { return S.list[off + q]; };
    // Pipeline: the records of block b + 1 are copied (cp.async) and the list indices of block
    // b + 2 loaded into registers while block b computes; staging then reads shared memory only.
    int nextId[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int64_t q = threadIdx.x + i * NTH;
      nextId[i] = q < len ? entry(q) : INT_MIN;
    }
    fetch(nextId);
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int64_t q = ST + threadIdx.x + i * NTH;
      nextId[i] = q < len ? entry(q) : INT_MIN;
    }
    for (int64_t b0 = 0; b0 < len; b0 += ST) {
      const int nsrc = (int)min((int64_t)ST, (len - b0 + kSub - 1) / kSub * kSub);
      cpAsyncWaitAll();  // this lane's copies of block b
      int hit = 0;
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int j = threadIdx.x + i * NTH;
        if (j < nsrc) {
          const int id = sRawId[j];
          const bool live = id != INT_MIN;
          if (live && id < S.ns) {  // a source of one of this tile's own targets: check self pairs
            const int sl = sRawSlot[j];
            hit |= sl >= tile0 && sl < tile0 + tcount;
          }
          stageSource<K, PRECISE>(j, live, live ? sRaw0[j] : float4{}, live ? sRaw1[j] : float4{}, tt, sXY, sZW,
                                  sD, sLXY, sLZ);
          sId[j] = id;
        }
      }
      // (the barrier also orders this block's raw reads before the copies that refill the slots)
      const int anyHit = __syncthreads_or(hit);
      fetch(nextId);  // block b + 1 (no copies past the end of the list)
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int64_t q = b0 + 2 * ST + threadIdx.x + i * NTH;
        nextId[i] = q < len ? entry(q) : INT_MIN;
      }
      if (anyHit)
        fp32cTile<K, PSI, true, PRECISE, NEWTON, true>(T, nsrc, 0, sId, tt.nx, tt.ny, tt.nz, tt.nlx, tt.nly, tt.nlz,
                                                       tt.C, tt.self, hx, hy, hz, cx, cy, cz, hp, cp, hw, cw);
      else
        fp32cTile<K, PSI, false, PRECISE, NEWTON, true>(T, nsrc, 0, sId, tt.nx, tt.ny, tt.nz, tt.nlx, tt.nly, tt.nlz,
                                                        tt.C, tt.self, hx, hy, hz, cx, cy, cz, hp, cp, hw, cw);
      __syncthreads();
    }
    cpAsyncWaitAll();  // none are pending (the last fetch is past the list end); kept for safety
    writePartials<NTH, K, PSI>(S.partial + (size_t)part * (PSI ? 5 : 3) * n, n, tile0, tcount, hx, hy, hz, cx, cy, cz,
                               hp, cp, hw, cw);
    (void)P;
  }
}

// ---------------------------------------------------------------------------------------
// Symmetric leaf x leaf sums.  Leaf faces are targets and sources at once (collocated face
// velocity, every RK4 stage): the pair (i, j) gives source j's term on target i and source i's
// term on target j from the same d = x_j - x_i, 2q and reciprocal.  With the plan's symmetric
// layout (leaf target slot leaf0 + k is source k), an item takes leaf tile I (kSymTile targets,
// 8 per thread) against the source tiles J0..J1-1, J0 >= I:
//   * forward: source j on the thread's targets, accumulated in registers exactly as pairFP32C
//     does (FP32 sub-block sums, Kahan-compensated, one FP64 partial per chunk);
//   * reverse (J > I only): target i as the source of target j, s_r = W_i rn with the same
//     rn = r (2q r - 2) (the negated Newton reciprocal).  Each thread sums its 8 targets' terms
//     per source.  Per 32 sources a warp transposes its lanes' terms through its own shared
//     buffer (warp-synchronous, no block barrier) and lane l sums source l over the 32 lanes;
//     per 256 staged sources the four warps' sums meet once, are added in warp order and go to
//     the source's 64-bit fixed-point accumulator (kSymScale units: integer adds are exact and
//     order-free, so the result does not depend on the schedule).
//   * the diagonal tile J = I is summed in the forward direction only, with the self pair
//     (source index = the target's own) dropped.
// Per paired step (two targets, one source: four directed pairs): 17 paired FMA-pipe ops and 2
// MUFU (pairFP32C: 13 and 2 for two directed pairs), plus ~4 FP32 adds per source and thread for
// the transposed reduction.
// PSI: the stream function as well.  log2(2q) - 1 is formed once per unordered pair and serves
// both directions (3 more paired ops and 2 MUFU per step, against 4 and 4 in pairFP32C's two
// directed pairs): forward sums w_j (log2 2q - 1) Kahan-compensated in shared memory (the
// registers are spent), a fourth reverse component, and the diagonal tile through the same
// sweep with the self pair dropped.  The "- 1" folded into each term leaves the weight-sum
// partial at zero.
constexpr int kSymSt = 256;              // sources staged per step
constexpr int kSymRed = 32;              // sources per warp transpose
constexpr int kSymWarps = kSymThreads / 32;
constexpr int kSymPitch = 33;            // floats per transpose row (32 lanes + 1 skew)
// reverse components: velocity (3) and, with the stream function, sum w (log2 2q - 1)
__host__ __device__ constexpr int symComps(bool psi) { return psi ? 4 : 3; }
constexpr size_t symSmem(bool psi) {
  return sizeof(float4) * kSymSt * 2 + sizeof(float2) * kSymSt +
         sizeof(float) * kSymWarps * symComps(psi) * kSymRed * kSymPitch +
         sizeof(float) * kSymWarps * symComps(psi) * kSymSt + (psi ? sizeof(float) * 2 * kSymK * kSymThreads : 0);
}

template <bool NEWTON, bool PSI>
__global__ void __launch_bounds__(kSymThreads, 2) pairFP32CSym(const SolveDev* __restrict__ solves,
                                                             const WorkItem* __restrict__ items, int nitems,
                                                             int* __restrict__ counter) {
  constexpr int NTH = kSymThreads, K = kSymK, P = K / 2, ST = kSymSt, NC = symComps(PSI);
  static_assert(NTH == 128, "the cross-warp combine assumes four warps");
  static_assert(kSymSt % (2 * kSymRed) == 0, "compensated adds every two transpose rounds");
  extern __shared__ __align__(16) unsigned char symShared[];
  float4* sXY = reinterpret_cast<float4*>(symShared);
  float4* sZW = sXY + ST;
  float2* sD = reinterpret_cast<float2*>(sZW + ST);
  float* sWarp = reinterpret_cast<float*>(sD + ST);             // [warp][NC * 32 rows][33]
  float* sCross = sWarp + kSymWarps * NC * kSymRed * kSymPitch; // [warp][NC][ST]
  float* sPsi = sCross + kSymWarps * NC * ST;                   // PSI: [2K][NTH] forward psi sums, compensations
  __shared__ int sItem;
  __shared__ int sCentre;
  SourceTile<false> T;
  T.xy = sXY; T.zw = sZW; T.d = sD;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* myBuf = sWarp + warp * NC * kSymRed * kSymPitch;
  float* myCross = sCross + warp * NC * ST;
  const float2 kMinusTwo = make_float2(-2.f, -2.f);
  const float2 kMinusOne = make_float2(-1.f, -1.f);
  constexpr float kSign = NEWTON ? -1.f : 1.f;

  for (;;) {
    if (threadIdx.x == 0) sItem = atomicAdd(counter, 1);
    __syncthreads();
    const int it = sItem;
    __syncthreads();
    if (it >= nitems) return;
    const WorkItem w = items[it];
    const SolveDev& S = solves[w.solve];
    const int n = S.nslots, ns = S.ns;
    const int tgt0 = w.tile * kSymTile;                 // first source index of leaf tile I
    const int tcount = min(kSymTile, ns - tgt0);
    const int slot0 = S.leaf0 + tgt0;
    TileTargets<K> tt;
    loadTileTargets<NTH, K, false>(S.tx, n, slot0, tcount, slot0 + tcount / 2, S.self, S.eps2, &sCentre, tt);
    // the targets' own source weights W_i (zero for dead lanes: they then add nothing reversed)
    float2 Wt[P];
#pragma unroll
    for (int m = 0; m < P; ++m) {
      const int a = threadIdx.x + 2 * m * NTH, b = a + NTH;
      Wt[m] = make_float2(a < tcount ? S.sp0[tgt0 + a].w : 0.f, b < tcount ? S.sp0[tgt0 + b].w : 0.f);
    }
    float hx[K], hy[K], hz[K], cx[K], cy[K], cz[K], hp[K], cp[K], hw[K], cw[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      hx[k] = hy[k] = hz[k] = cx[k] = cy[k] = cz[k] = 0.f;
      hp[k] = cp[k] = hw[k] = cw[k] = 0.f;
    }
    if constexpr (PSI) {  // this thread's own slots: no barrier needed
#pragma unroll
      for (int k = 0; k < 2 * K; ++k) sPsi[k * NTH + threadIdx.x] = 0.f;
    }
    for (int J = w.s0; J < w.s1; ++J) {
      const int src0 = J * kSymTile;
      const int send = min(ns, src0 + kSymTile);
      for (int b0 = src0; b0 < send; b0 += ST) {
        for (int j = threadIdx.x; j < ST; j += NTH) {
          const int src = b0 + j;
          const bool live = src < send;
          stageSource<K, false>(j, live, live ? S.sp0[src] : float4{}, live ? S.sp1[src] : float4{}, tt, sXY, sZW, sD,
                                nullptr, nullptr);
        }
        __syncthreads();
        // One staged block.  DIAG (the tile against itself): forward terms only, the self pair
        // (source index == the target's own) dropped.  Otherwise forward and reverse terms.
        auto sweep = [&](auto diagTag) {
          constexpr bool DIAG = decltype(diagTag)::value;
          // FP32 sub-block sums over two transpose rounds (64 sources) between compensated adds;
          // one round with the stream function (whose longer-lived sums would spill)
          constexpr int kRounds = PSI ? 1 : 2;
          float2 vx[P], vy[P], vz[P], vp[P];
#pragma unroll 1
          for (int j0 = 0; j0 < ST; j0 += kSymRed) {
            if ((j0 / kSymRed) % kRounds == 0) {
#pragma unroll
              for (int m = 0; m < P; ++m) vx[m] = vy[m] = vz[m] = vp[m] = make_float2(0.f, 0.f);
            }
#pragma unroll 2
            for (int jj = 0; jj < kSymRed; ++jj) {
              const int j = j0 + jj;
              const float4 xy = sXY[j];
              const float4 zw = sZW[j];
              const float2 dj = sD[j];
              const float2 X = make_float2(xy.x, xy.y), Y = make_float2(xy.z, xy.w), Z = make_float2(zw.x, zw.y);
              const float2 W = make_float2(zw.z, zw.w);
              float2 rx = make_float2(0.f, 0.f), ry = rx, rz = rx, rp = rx;
              const int rel = b0 + j - tgt0 - (int)threadIdx.x;  // DIAG: k NTH for this thread's target k
#pragma unroll
              for (int m = 0; m < P; ++m) {
                const float2 dx = add2(X, tt.nx[m]), dy = add2(Y, tt.ny[m]), dz = add2(Z, tt.nz[m]);
                float2 q = add2(dj, tt.C[m]);
                q = fma2(dx, dx, q);
                q = fma2(dy, dy, q);
                q = fma2(dz, dz, q);
                float2 r = make_float2(rcpApprox(q.x), rcpApprox(q.y));
                if (NEWTON) r = mul2(r, fma2(q, r, kMinusTwo));  // -(Newton reciprocal)
                float2 sf = mul2(W, r);
                float2 lgm;  // log2(2q) - 1, shared by both directions
                if constexpr (PSI) lgm = add2(make_float2(lg2Approx(q.x), lg2Approx(q.y)), kMinusOne);
                if constexpr (DIAG) {
                  if (rel == 2 * m * NTH) { sf.x = 0.f; if (PSI) lgm.x = 0.f; }
                  if (rel == (2 * m + 1) * NTH) { sf.y = 0.f; if (PSI) lgm.y = 0.f; }
                }
                vx[m] = fma2(sf, dx, vx[m]);
                vy[m] = fma2(sf, dy, vy[m]);
                vz[m] = fma2(sf, dz, vz[m]);
                if constexpr (PSI) vp[m] = fma2(W, lgm, vp[m]);
                if constexpr (!DIAG) {
                  const float2 sr = mul2(Wt[m], r);
                  rx = fma2(sr, dx, rx);
                  ry = fma2(sr, dy, ry);
                  rz = fma2(sr, dz, rz);
                  if constexpr (PSI) rp = fma2(Wt[m], lgm, rp);
                }
              }
              if constexpr (!DIAG) {
                // this lane's reverse terms of source jj: row (component, jj), column = lane
                myBuf[(0 * kSymRed + jj) * kSymPitch + lane] = rx.x + rx.y;
                myBuf[(1 * kSymRed + jj) * kSymPitch + lane] = ry.x + ry.y;
                myBuf[(2 * kSymRed + jj) * kSymPitch + lane] = rz.x + rz.y;
                if constexpr (PSI) myBuf[(3 * kSymRed + jj) * kSymPitch + lane] = rp.x + rp.y;
              }
            }
            if ((j0 / kSymRed) % kRounds == kRounds - 1) {
#pragma unroll
            for (int m = 0; m < P; ++m) {
              kahanAdd(hx[2 * m], cx[2 * m], kSign * vx[m].x);
              kahanAdd(hx[2 * m + 1], cx[2 * m + 1], kSign * vx[m].y);
              kahanAdd(hy[2 * m], cy[2 * m], kSign * vy[m].x);
              kahanAdd(hy[2 * m + 1], cy[2 * m + 1], kSign * vy[m].y);
              kahanAdd(hz[2 * m], cz[2 * m], kSign * vz[m].x);
              kahanAdd(hz[2 * m + 1], cz[2 * m + 1], kSign * vz[m].y);
            }
            if constexpr (PSI) {
#pragma unroll
              for (int m = 0; m < P; ++m) {
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                  const int k = 2 * m + e;
                  float h = sPsi[k * NTH + threadIdx.x], c = sPsi[(K + k) * NTH + threadIdx.x];
                  kahanAdd(h, c, e == 0 ? vp[m].x : vp[m].y);
                  sPsi[k * NTH + threadIdx.x] = h;
                  sPsi[(K + k) * NTH + threadIdx.x] = c;
                }
              }
            }
            }
            if constexpr (!DIAG) {
              __syncwarp();
              // lane l: source j0 + l, each component summed over the warp's 32 lanes in lane order
#pragma unroll
              for (int c = 0; c < NC; ++c) {
                const float* row = myBuf + (c * kSymRed + lane) * kSymPitch;
                float2 a = make_float2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 32; k += 2) a = add2(a, make_float2(row[k], row[k + 1]));
                myCross[c * ST + j0 + lane] = a.x + a.y;
              }
              __syncwarp();  // the buffer is rewritten by the next 32 sources
            }
          }
          if constexpr (!DIAG) {
            __syncthreads();
            // the four warps' sums of each (component, source), added in warp order; the reverse
            // velocity is +sum s_r d (d_ji = -d_ij and rn = -(reciprocal) cancel), the reverse
            // stream-function sum keeps its sign
            for (int o = threadIdx.x; o < NC * ST; o += NTH) {
              const int comp = o / ST, jl = o % ST;
              const int src = b0 + jl;
              if (src >= send) continue;
              const float acc = ((sCross[0 * NC * ST + o] + sCross[1 * NC * ST + o]) + sCross[2 * NC * ST + o]) +
                                sCross[3 * NC * ST + o];
              const double v = (double)((NEWTON || comp == 3) ? acc : -acc);
              if (fabs(v) < kSymLimit) {
                atomicAdd(S.rev + (size_t)comp * ns + src, (unsigned long long)__double2ll_rn(v * kSymScale));
              } else {
                atomicExch(S.revBad + src, 1);  // inf/NaN or out of range: the source's result becomes NaN
              }
            }
          }
        };
        if constexpr (PSI) {
          if (J == w.tile)
            sweep(std::true_type{});
          else
            sweep(std::false_type{});
        } else if (J == w.tile) {  // diagonal: forward only, the self pair (source index == own) dropped
          int self[K];
#pragma unroll
          for (int k = 0; k < K; ++k) self[k] = tgt0 + threadIdx.x + k * NTH;
          fp32cTile<K, false, true, false, NEWTON>(T, ST, b0, nullptr, tt.nx, tt.ny, tt.nz, tt.nlx, tt.nly, tt.nlz,
                                                  tt.C, self, hx, hy, hz, cx, cy, cz, hp, cp, hw, cw);
        } else {
          sweep(std::false_type{});
        }
        __syncthreads();
      }
    }
    if constexpr (PSI) {  // the forward stream-function sums already hold the -1: no weight sum
#pragma unroll
      for (int k = 0; k < K; ++k) {
        hp[k] = sPsi[k * NTH + threadIdx.x];
        cp[k] = sPsi[(K + k) * NTH + threadIdx.x];
      }
    }
    writePartials<NTH, K, PSI>(S.partial + (size_t)w.chunk * (PSI ? 5 : 3) * n, n, slot0, tcount, hx, hy, hz, cx,
                               cy, cz, hp, cp, hw, cw);
  }
}

// Resident CTAs per SM of the symmetric kernel (both Newton variants get the shared-memory limit).
template <bool PSI>
int symResidency() {
  for (void* f : {(void*)pairFP32CSym<true, PSI>, (void*)pairFP32CSym<false, PSI>})
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)symSmem(PSI)) != cudaSuccess)
      return 0;
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, (void*)pairFP32CSym<true, PSI>, kSymThreads, symSmem(PSI)) !=
      cudaSuccess)
    return 0;
  return b;
}

constexpr int kFP64Threads = 128;
constexpr int kFP64Tile = 128;
constexpr double kFourPi = 4 * kPi;

template <bool PSI>
__global__ void __launch_bounds__(kFP64Threads) pairFP64(const SolveDev* __restrict__ solves,
                                                         const WorkItem* __restrict__ items, int nitems,
                                                         int* __restrict__ counter) {
  __shared__ double4_32a sS[kFP64Tile];
  __shared__ int sItem;
  for (;;) {
    if (threadIdx.x == 0) sItem = atomicAdd(counter, 1);
    __syncthreads();
    const int it = sItem;
    __syncthreads();
    if (it >= nitems) return;
    const WorkItem w = items[it];
    const SolveDev& S = solves[w.solve];
    const int n = S.nslots;
    const int slot = w.tbeg + threadIdx.x;
    const bool live = slot < w.tend;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    int self = -1;
    if (live) { tx = S.tx[slot]; ty = S.tx[n + slot]; tz = S.tx[2 * n + slot]; self = S.self[slot]; }
    const double eps2 = S.eps2;
    double u0 = 0.0, u1 = 0.0, u2 = 0.0, ps = 0.0;
    for (int b0 = w.s0; b0 < w.s1; b0 += kFP64Tile) {
      const int cnt = min(kFP64Tile, w.s1 - b0);
      if (threadIdx.x < cnt) sS[threadIdx.x] = S.sd[b0 + threadIdx.x];
      __syncthreads();
      for (int j = 0; j < cnt; ++j) {
        if (b0 + j == self) continue;
        const double4_32a s = sS[j];
        // biotSavart: cross(tgt, src) * (-zeta*A) / (4 pi (1 - dot(src, tgt)))
        const double dp = __dadd_rn(__dadd_rn(__dmul_rn(s.x, tx), __dmul_rn(s.y, ty)), __dmul_rn(s.z, tz));
        const double omd = __dadd_rn(__dsub_rn(1.0, dp), eps2);
        const double strength = s.w / __dmul_rn(kFourPi, omd);
        const double c0 = __dsub_rn(__dmul_rn(ty, s.z), __dmul_rn(tz, s.y));
        const double c1 = __dsub_rn(__dmul_rn(tz, s.x), __dmul_rn(tx, s.z));
        const double c2 = __dsub_rn(__dmul_rn(tx, s.y), __dmul_rn(ty, s.x));
        u0 = __dadd_rn(u0, __dmul_rn(c0, strength));
        u1 = __dadd_rn(u1, __dmul_rn(c1, strength));
        u2 = __dadd_rn(u2, __dmul_rn(c2, strength));
        if (PSI) ps = __dadd_rn(ps, __dmul_rn(log(omd), s.w) / kFourPi);  // greensFn
      }
      __syncthreads();
    }
    if (live) {
      double* out = S.partial + (size_t)w.chunk * (PSI ? 4 : 3) * n;
      out[slot] = u0; out[n + slot] = u1; out[2 * n + slot] = u2;
      if (PSI) out[3 * n + slot] = ps;
    }
  }
}

// Instantiated launch shapes (the autotuner chooses among these).  Variants per shape:
// [0] fast, [1] precise (hi/lo), [2] fast without the Newton step; each without / with psi.
struct ShapeFn {
  int threads, k, srcTile, minBlocks;
  void* fn[3][2];
};
#define LPM_SHAPE(T, K, S, B)                                                                                        \
  {T, K, S, B, {{(void*)pairFP32C<T, K, S, B, false, false, true>, (void*)pairFP32C<T, K, S, B, true, false, true>},   \
                {(void*)pairFP32C<T, K, S, B, false, true, true>, (void*)pairFP32C<T, K, S, B, true, true, true>},     \
                {(void*)pairFP32C<T, K, S, B, false, false, false>, (void*)pairFP32C<T, K, S, B, true, false, false>}}}
// Register use of the RK4 velocity kernel (ptxas, sm_103a, paired arithmetic) sets the
// resident CTAs per SM: 128x4 unbounded 154 regs -> 3/SM, min-blocks 4: 124 -> 4/SM;
// 128x6 min-blocks 3: 163 -> 3/SM; 128x8 233 -> 2/SM; 64x8 min-blocks 4: 233 -> 4/SM; 32x8 min-blocks 8
// -> 8/SM; 32x4 with 128-source tiles, min-blocks 12 (the tree code's shape, for the direct solves of
// a tree batch) -> 12/SM;
// 256x4 min-blocks 2: 125 -> 2/SM.  None of these spills.
const ShapeFn kShapes[] = {
  LPM_SHAPE(128, 4, 256, 1),
  LPM_SHAPE(128, 4, 256, 4),
  LPM_SHAPE(128, 6, 256, 3),
  LPM_SHAPE(128, 8, 256, 1),
  LPM_SHAPE(64, 8, 256, 4),
  LPM_SHAPE(256, 4, 256, 2),
  LPM_SHAPE(32, 8, 256, 8),
  LPM_SHAPE(32, 4, 128, 12),
};
#undef LPM_SHAPE

const ShapeFn* findShape(const PairShape& s) {
  for (const auto& e : kShapes)
    if (e.threads == s.threads && e.k == s.k && e.srcTile == s.srcTile && e.minBlocks == s.minBlocks) return &e;
  return nullptr;
}

void* kernelFor(Precision prec, const PairShape& shape, bool psi, bool precise, bool rcpApprox, int& threads) {
  if (prec == Precision::FP64) {
    threads = kFP64Threads;
    return psi ? (void*)pairFP64<true> : (void*)pairFP64<false>;
  }
  const ShapeFn* e = findShape(shape);
  if (!e) return nullptr;
  threads = e->threads;
  const int variant = precise ? 1 : (rcpApprox ? 2 : 0);
  return e->fn[variant][psi ? 1 : 0];
}

}  // namespace

int pairShapeCount() { return (int)(sizeof(kShapes) / sizeof(kShapes[0])); }

PairShape pairShapeAt(int i) {
  return PairShape{kShapes[i].threads, kShapes[i].k, kShapes[i].srcTile, kShapes[i].minBlocks};
}

bool pairShapeSupported(Precision prec, const PairShape& shape) {
  if (prec == Precision::FP64)
    return shape.threads == kFP64Threads && shape.k == 1 && shape.srcTile == kFP64Tile && shape.minBlocks == 1;
  return findShape(shape) != nullptr;
}

int pairNumComponents(Precision prec, bool psi) {
  if (prec == Precision::FP64) return psi ? 4 : 3;
  return psi ? 5 : 3;
}

bool treePairShapeSupported(const PairShape& shape) { return shape == kTreeShape; }

cudaError_t launchTreePair(const PairShape& shape, bool psi, bool precise, bool rcpApprox, const TreeDev* dev,
                           int nitems, int* counter, int grid, cudaStream_t s) {
  if (!(shape == kTreeShape)) return cudaErrorInvalidValue;
  if (nitems <= 0 || grid <= 0) return cudaSuccess;
  constexpr int T = kTreeShape.threads, K = kTreeShape.k, ST = kTreeShape.srcTile, B = kTreeShape.minBlocks;
  void* fn;
  if (precise)
    fn = psi ? (void*)treeFP32C<T, K, ST, B, true, true, true> : (void*)treeFP32C<T, K, ST, B, false, true, true>;
  else if (rcpApprox)
    fn = psi ? (void*)treeFP32C<T, K, ST, B, true, false, false> : (void*)treeFP32C<T, K, ST, B, false, false, false>;
  else
    fn = psi ? (void*)treeFP32C<T, K, ST, B, true, false, true> : (void*)treeFP32C<T, K, ST, B, false, false, true>;
  // 8 CTAs of ~22 KB static shared memory each need the shared-memory-heavy carveout (once).
  static const cudaError_t carve = [] {
    void* all[] = {(void*)treeFP32C<T, K, ST, B, true, true, true>,   (void*)treeFP32C<T, K, ST, B, false, true, true>,
                   (void*)treeFP32C<T, K, ST, B, true, false, false>, (void*)treeFP32C<T, K, ST, B, false, false, false>,
                   (void*)treeFP32C<T, K, ST, B, true, false, true>,  (void*)treeFP32C<T, K, ST, B, false, false, true>};
    for (void* f : all) {
      const cudaError_t e =
          cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }();
  if (carve != cudaSuccess) return carve;
  void* args[] = {(void*)&dev, (void*)&nitems, (void*)&counter};
  return cudaLaunchKernel(fn, dim3(grid), dim3(T), args, 0, s);
}

int pairBlocksPerSM(Precision prec, const PairShape& shape, bool psi) {
  int threads = 0;
  void* fn = kernelFor(prec, shape, psi, false, false, threads);
  if (!fn) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, 0) != cudaSuccess) return 0;
  return nb;
}

int pairSymBlocksPerSM(bool psi) {
  static const int nb[2] = {[] { return symResidency<false>(); }(), [] { return symResidency<true>(); }()};
  return nb[psi ? 1 : 0];
}

cudaError_t launchPairSym(bool psi, bool rcpApprox, const SolveDev* solves, const WorkItem* items, int nitems,
                          int* counter, int grid, cudaStream_t s) {
  if (nitems <= 0 || grid <= 0) return cudaSuccess;
  if (pairSymBlocksPerSM(psi) <= 0) return cudaErrorInvalidConfiguration;
  void* fn = psi ? (rcpApprox ? (void*)pairFP32CSym<false, true> : (void*)pairFP32CSym<true, true>)
                 : (rcpApprox ? (void*)pairFP32CSym<false, false> : (void*)pairFP32CSym<true, false>);
  void* args[] = {(void*)&solves, (void*)&items, (void*)&nitems, (void*)&counter};
  return cudaLaunchKernel(fn, dim3(grid), dim3(kSymThreads), args, symSmem(psi), s);
}

cudaError_t launchPair(Precision prec, const PairShape& shape, bool psi, bool precise, bool rcpApprox,
                       const SolveDev* solves, const WorkItem* items, int nitems, int* counter, int grid,
                       cudaStream_t s) {
  int threads = 0;
  void* fn = kernelFor(prec, shape, psi, precise, rcpApprox, threads);
  if (!fn) return cudaErrorInvalidValue;
  if (nitems <= 0 || grid <= 0) return cudaSuccess;
  void* args[] = {(void*)&solves, (void*)&items, (void*)&nitems, (void*)&counter};
  return cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, 0, s);
}

}  // namespace lpm
