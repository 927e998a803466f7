// noalloc.cu -- lpm_bve_velocity_noalloc: the FP32-compensated direct sum for callers
// that cannot allocate device memory.
//
// Some hosts own all device memory themselves: a model that hands this library its
// particle arrays from a pre-sized memory pool and forbids any later cudaMalloc (for
// example while its time loop runs inside a CUDA graph, or in a deployment that fixes
// the memory footprint at start-up).  The regular entry points allocate plans and
// workspace; this one uses only the caller's inputs and outputs plus one file-scope
// __device__ array, which the CUDA runtime places in device memory when the library is
// loaded on a device and keeps there until the process exits.
//
// Scratch (kScratchBytes, about 18 MiB per device):
//   packed sources   2 x float4 per unmasked face, up to kMaxFaces faces
//   source index     one int per face: its position in the packed list, -1 if masked
//   block counts / offsets for the deterministic mask compaction
// Limit: at most kMaxFaces faces (sources, masked or not) and kMaxTargets targets.
//
// Pipeline on `stream`: count unmasked faces per block, scan the counts (one CTA), pack
// the sources in face order, then one CTA per target tile sums over every packed source
// (the arithmetic of the pair kernel in pair_kernels.cu, unsorted targets, no source
// chunks) and writes u = x_i x V (and psi) straight to the caller's arrays.  A tile uses the
// fast formulation only when its targets are mesh points lying close together; arbitrary or
// scattered targets get the hi/lo formulation (see kFastRadius).
// The scratch is shared by every call on the device and keeps the last call's contents;
// calls whose kernels overlap on the GPU (different streams, no ordering) race on it.

#include "lpm_bve.h"

#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <mutex>

namespace {

constexpr int kMaxFaces = 1 << 19;          // 524,288 faces (icosahedral level 7 has 436,900)
constexpr int64_t kMaxTargets = INT_MAX / 4;
constexpr int kCountBlock = 1024;           // faces per compaction block
constexpr int kMaxBlocks = kMaxFaces / kCountBlock;

// Byte offsets of the scratch regions (each 256-byte aligned).
constexpr size_t kOffSp0 = 0;
constexpr size_t kOffSp1 = kOffSp0 + sizeof(float4) * kMaxFaces;
constexpr size_t kOffIdx = kOffSp1 + sizeof(float4) * kMaxFaces;
constexpr size_t kOffCnt = kOffIdx + sizeof(int) * kMaxFaces;
constexpr size_t kOffOfs = kOffCnt + sizeof(int) * kMaxBlocks;
constexpr size_t kOffLive = kOffOfs + sizeof(int) * kMaxBlocks;
constexpr size_t kScratchBytes = kOffLive + 256;

static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

constexpr int kNth = 128;   // CTA size of the pair kernel
constexpr int kK = 8;       // targets per thread (four pairs for the f32x2 arithmetic)
constexpr int kSt = 256;    // sources staged per step
constexpr int kSub = 32;    // FP32 sub-block before the compensated add
constexpr double kPi = 3.1415926535897932384626433832795027975;

struct Scratch {
  float4* sp0;
  float4* sp1;
  int* srcIdx;
  int* blockCount;
  int* blockOffset;
  int* nlive;
};

__host__ __device__ inline Scratch carve(unsigned char* base) {
  Scratch s;
  s.sp0 = reinterpret_cast<float4*>(base + kOffSp0);
  s.sp1 = reinterpret_cast<float4*>(base + kOffSp1);
  s.srcIdx = reinterpret_cast<int*>(base + kOffIdx);
  s.blockCount = reinterpret_cast<int*>(base + kOffCnt);
  s.blockOffset = reinterpret_cast<int*>(base + kOffOfs);
  s.nlive = reinterpret_cast<int*>(base + kOffLive);
  return s;
}

struct Pts {
  const double* x;
  int64_t n, si, sc;
};

__global__ void __launch_bounds__(kCountBlock) countKernel(unsigned char* base, const uint8_t* mask, int n) {
  const Scratch S = carve(base);
  const int f = blockIdx.x * kCountBlock + threadIdx.x;
  const int live = (f < n) && !(mask && mask[f]);
  const int c = __syncthreads_count(live);
  if (threadIdx.x == 0) S.blockCount[blockIdx.x] = c;
}

__global__ void __launch_bounds__(kMaxBlocks) scanKernel(unsigned char* base, int nblocks) {
  const Scratch S = carve(base);
  __shared__ int buf[kMaxBlocks];
  const int t = threadIdx.x;
  buf[t] = t < nblocks ? S.blockCount[t] : 0;
  __syncthreads();
  for (int d = 1; d < kMaxBlocks; d <<= 1) {   // inclusive Hillis-Steele scan
    const int v = t >= d ? buf[t - d] : 0;
    __syncthreads();
    buf[t] += v;
    __syncthreads();
  }
  if (t < nblocks) S.blockOffset[t] = buf[t] - S.blockCount[t];
  if (t == 0) *S.nlive = nblocks > 0 ? buf[nblocks - 1] : 0;
}

__global__ void __launch_bounds__(kCountBlock) packKernel(unsigned char* base, Pts src, const double* zeta,
                                                          const double* area, const uint8_t* mask, int n) {
  const Scratch S = carve(base);
  __shared__ int warpSum[kCountBlock / 32];
  const int f = blockIdx.x * kCountBlock + threadIdx.x;
  const int live = (f < n) && !(mask && mask[f]);
  const unsigned ballot = __ballot_sync(0xffffffffu, live);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warpSum[warp] = __popc(ballot);
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += warpSum[w];
  const int rank = before + __popc(ballot & ((1u << lane) - 1u));
  if (f >= n) return;
  if (!live) {
    S.srcIdx[f] = -1;
    return;
  }
  const int s = S.blockOffset[blockIdx.x] + rank;
  S.srcIdx[f] = s;
  const double x[3] = {src.x[f * src.si], src.x[f * src.si + src.sc], src.x[f * src.si + 2 * src.sc]};
  float hi[3], lo[3];
  for (int c = 0; c < 3; ++c) {
    hi[c] = __double2float_rn(x[c]);
    lo[c] = __double2float_rn(x[c] - (double)hi[c]);
  }
  const double circ = -zeta[f] * area[f];
  S.sp0[s] = make_float4(hi[0], hi[1], hi[2], __double2float_rn(circ * (1.0 / (2.0 * kPi))));
  S.sp1[s] = make_float4(lo[0], lo[1], lo[2], __double2float_rn(1.0 - (x[0] * x[0] + x[1] * x[1] + x[2] * x[2])));
}

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
__device__ __forceinline__ void kahanAdd(float& h, float& c, float v) {
  const float y = v - c;
  const float t = h + y;
  c = (t - h) - y;
  h = t;
}
__device__ __forceinline__ float relCoord(float hi, float lo, float chi, float clo) { return (hi - chi) + (lo - clo); }

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Targets of a tile may use the 13-op fast form (coordinates relative to a tile centre) only
// when they are mesh points -- faces summed collocated, or distinct targets the caller flags as
// mesh points, which keep about half a mesh spacing from every source -- and lie close together:
// caller order is not spatially sorted, and the fast form's FP32 differences lose accuracy in
// proportion to the tile radius over the pair distance.  Other tiles use the hi/lo form.
constexpr double kFastRadius = 0.1;

// The sum over every packed source for one tile of kNth*kK targets, epilogue fused.  Paired FP32
// (f32x2) arithmetic over a thread's target pairs, each lane rounded as the scalar instruction:
// d = x_j - x_i, 2q = D_j + C_i + |d|^2, r = rcp.approx(2q), s' = (w r)(2q r - 2) = -s (the
// Newton step without a sign flip), v += s' d, the block sums negated into the compensated
// accumulators.  The source tile stores each value twice, (x,x,y,y), (z,z,w,w), (D,D), so one
// shared load gives the pair operand.
//   PRECISE = false: x_i and x_j relative to the tile centre c (hi/lo parts of c subtracted once
//     per staged source); 13 FMA-pipe ops per pair.
//   PRECISE = true: d = (hi_j - hi_i) + (lo_j - lo_i) from the FP64 hi/lo float splits, exact
//     enough for a target arbitrarily close to a source; 19 ops per pair.
struct Stage {
  float4* xy; float4* zw; float2* d; float4* lxy; float2* lz;
};

template <bool PSI, bool PRECISE>
__device__ __forceinline__ void tileSum(const Scratch& S, int ns, const Pts& tgt, int tile0, int tcount, double cxd,
                                        double cyd, double czd, bool colloc, int lo, int hi, double eps2,
                                        const Stage& T, double* u, int64_t usi, int64_t usc, double* psi) {
  constexpr int P = kK / 2;
  float chx = 0.f, chy = 0.f, chz = 0.f, clx = 0.f, cly = 0.f, clz = 0.f;
  if (!PRECISE) {
    chx = __double2float_rn(cxd); chy = __double2float_rn(cyd); chz = __double2float_rn(czd);
    clx = __double2float_rn(cxd - (double)chx); cly = __double2float_rn(cyd - (double)chy);
    clz = __double2float_rn(czd - (double)chz);
  }
  float2 nx[P], ny[P], nz[P], nlx[P], nly[P], nlz[P], C[P];
  int self[kK];
#pragma unroll
  for (int m = 0; m < P; ++m) {
    float ax[2], ay[2], az[2], lx[2], ly[2], lz[2], ck[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 2 * m + h;
      const int i = tile0 + threadIdx.x + k * kNth;
      self[k] = -1;
      ax[h] = ay[h] = az[h] = lx[h] = ly[h] = lz[h] = 0.f; ck[h] = 1.f;
      if (threadIdx.x + k * kNth < tcount) {
        double X[3];
        for (int c = 0; c < 3; ++c) X[c] = tgt.x[(int64_t)i * tgt.si + c * tgt.sc];
        const float hx = __double2float_rn(X[0]), hy = __double2float_rn(X[1]), hz = __double2float_rn(X[2]);
        const float ex = __double2float_rn(X[0] - (double)hx), ey = __double2float_rn(X[1] - (double)hy),
                    ez = __double2float_rn(X[2] - (double)hz);
        if (PRECISE) {
          ax[h] = hx; ay[h] = hy; az[h] = hz; lx[h] = ex; ly[h] = ey; lz[h] = ez;
        } else {
          ax[h] = relCoord(hx, ex, chx, clx); ay[h] = relCoord(hy, ey, chy, cly); az[h] = relCoord(hz, ez, chz, clz);
        }
        ck[h] = __double2float_rn((1.0 - (X[0] * X[0] + X[1] * X[1] + X[2] * X[2])) + 2.0 * eps2);
        if (colloc) self[k] = S.srcIdx[i];
      }
    }
    nx[m] = make_float2(-ax[0], -ax[1]); ny[m] = make_float2(-ay[0], -ay[1]); nz[m] = make_float2(-az[0], -az[1]);
    nlx[m] = make_float2(-lx[0], -lx[1]); nly[m] = make_float2(-ly[0], -ly[1]); nlz[m] = make_float2(-lz[0], -lz[1]);
    C[m] = make_float2(ck[0], ck[1]);
  }
  float hx[kK], hy[kK], hz[kK], cx[kK], cy[kK], cz[kK], hp[kK], cp[kK], hw[kK], cw[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) hx[k] = hy[k] = hz[k] = cx[k] = cy[k] = cz[k] = hp[k] = cp[k] = hw[k] = cw[k] = 0.f;
  const float2 kMinusTwo = make_float2(-2.f, -2.f);

  for (int b0 = 0; b0 < ns; b0 += kSt) {
    __syncthreads();
    for (int j = threadIdx.x; j < kSt; j += kNth) {
      const int s = b0 + j;
      // padding: zero weight, D = 1, at the centre (fast) or the origin (precise): adds exactly 0
      float x = 0.f, y = 0.f, z = 0.f, w = 0.f, d = 1.f, ux = 0.f, uy = 0.f, uz = 0.f;
      if (s < ns) {
        const float4 p0 = S.sp0[s], p1 = S.sp1[s];
        if (PRECISE) {
          x = p0.x; y = p0.y; z = p0.z; ux = p1.x; uy = p1.y; uz = p1.z;
        } else {
          x = relCoord(p0.x, p1.x, chx, clx);
          y = relCoord(p0.y, p1.y, chy, cly);
          z = relCoord(p0.z, p1.z, chz, clz);
        }
        w = p0.w;
        d = p1.w;
      }
      T.xy[j] = make_float4(x, x, y, y);
      T.zw[j] = make_float4(z, z, w, w);
      T.d[j] = make_float2(d, d);
      if (PRECISE) {
        T.lxy[j] = make_float4(ux, ux, uy, uy);
        T.lz[j] = make_float2(uz, uz);
      }
    }
    __syncthreads();
    const bool checked = lo <= b0 + kSt - 1 && hi >= b0;
#pragma unroll 1
    for (int j0 = 0; j0 < kSt; j0 += kSub) {
      float2 vx[P], vy[P], vz[P], vp[P], vw[P];
#pragma unroll
      for (int m = 0; m < P; ++m) vx[m] = vy[m] = vz[m] = vp[m] = vw[m] = make_float2(0.f, 0.f);
#pragma unroll 2
      for (int j = j0; j < j0 + kSub; ++j) {
        const float4 xy = T.xy[j], zw = T.zw[j];
        const float2 Dj = T.d[j];
        const float2 X = make_float2(xy.x, xy.y), Y = make_float2(xy.z, xy.w), Z = make_float2(zw.x, zw.y);
        const float2 W = make_float2(zw.z, zw.w);
        float2 LX, LY, LZ;
        if (PRECISE) {
          const float4 lxy = T.lxy[j];
          LX = make_float2(lxy.x, lxy.y); LY = make_float2(lxy.z, lxy.w); LZ = T.lz[j];
        }
#pragma unroll
        for (int m = 0; m < P; ++m) {
          float2 dx, dy, dz;
          if (PRECISE) {  // hi parts subtract exactly when close; lo parts restore the rest
            dx = add2(add2(X, nx[m]), add2(LX, nlx[m]));
            dy = add2(add2(Y, ny[m]), add2(LY, nly[m]));
            dz = add2(add2(Z, nz[m]), add2(LZ, nlz[m]));
          } else {
            dx = add2(X, nx[m]); dy = add2(Y, ny[m]); dz = add2(Z, nz[m]);
          }
          float2 q = add2(Dj, C[m]);
          q = fma2(dx, dx, q);
          q = fma2(dy, dy, q);
          q = fma2(dz, dz, q);
          const float2 r = make_float2(rcpApprox(q.x), rcpApprox(q.y));
          float2 sp = mul2(mul2(W, r), fma2(q, r, kMinusTwo));
          float2 lg, ww;
          if (PSI) { lg = make_float2(lg2Approx(q.x), lg2Approx(q.y)); ww = W; }
          if (checked) {  // a self pair has q ~ 0: drop its (inf/NaN) terms after they are formed
            if (b0 + j == self[2 * m]) { sp.x = 0.f; if (PSI) { lg.x = 0.f; ww.x = 0.f; } }
            if (b0 + j == self[2 * m + 1]) { sp.y = 0.f; if (PSI) { lg.y = 0.f; ww.y = 0.f; } }
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
        kahanAdd(hx[2 * m], cx[2 * m], -vx[m].x); kahanAdd(hx[2 * m + 1], cx[2 * m + 1], -vx[m].y);
        kahanAdd(hy[2 * m], cy[2 * m], -vy[m].x); kahanAdd(hy[2 * m + 1], cy[2 * m + 1], -vy[m].y);
        kahanAdd(hz[2 * m], cz[2 * m], -vz[m].x); kahanAdd(hz[2 * m + 1], cz[2 * m + 1], -vz[m].y);
        if (PSI) {
          kahanAdd(hp[2 * m], cp[2 * m], vp[m].x); kahanAdd(hp[2 * m + 1], cp[2 * m + 1], vp[m].y);
          kahanAdd(hw[2 * m], cw[2 * m], vw[m].x); kahanAdd(hw[2 * m + 1], cw[2 * m + 1], vw[m].y);
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    const int64_t i = tile0 + threadIdx.x + k * kNth;
    if (threadIdx.x + k * kNth >= tcount) continue;
    double X[3];
    for (int c = 0; c < 3; ++c) X[c] = tgt.x[i * tgt.si + c * tgt.sc];
    const double V0 = (double)hx[k] - (double)cx[k], V1 = (double)hy[k] - (double)cy[k],
                 V2 = (double)hz[k] - (double)cz[k];
    if (u) {
      u[i * usi] = X[1] * V2 - X[2] * V1;
      u[i * usi + usc] = X[2] * V0 - X[0] * V2;
      u[i * usi + 2 * usc] = X[0] * V1 - X[1] * V0;
    }
    if (PSI && psi) psi[i] = 0.34657359027997264 * (((double)hp[k] - (double)cp[k]) - ((double)hw[k] - (double)cw[k]));
  }
}

// One CTA per tile of kNth*kK targets in caller order.  The prologue finds the tile centre (the
// middle target, or -- if its position is inf/NaN or far off the sphere, e.g. a masked parent
// that coincides with a leaf -- the first target near the sphere, or the origin), the tile radius
// about it and the range of the tile's own source indices (collocated), then picks the form.
template <bool PSI>
__global__ void __launch_bounds__(kNth) pairKernel(unsigned char* base, Pts tgt, bool colloc, bool meshTargets,
                                                   double eps2, double* u, int64_t usi, int64_t usc, double* psi) {
  const Scratch S = carve(base);
  __shared__ float4 sXY[kSt];
  __shared__ float4 sZW[kSt];
  __shared__ float2 sD[kSt];
  __shared__ float4 sLXY[kSt];
  __shared__ float2 sLZ[kSt];
  __shared__ int sLo, sHi, sCentre;
  __shared__ unsigned long long sRad;  // bits of the largest (non-negative) FP64 distance from the centre
  const int n = (int)tgt.n;
  const int ns = *S.nlive;
  const int tile0 = blockIdx.x * (kNth * kK);
  const int tcount = min(kNth * kK, n - tile0);
  int cs = tile0 + (tcount >> 1);
  double cxd = tgt.x[cs * tgt.si], cyd = tgt.x[cs * tgt.si + tgt.sc], czd = tgt.x[cs * tgt.si + 2 * tgt.sc];
  auto sane = [](double x, double y, double z) {  // near the unit sphere (false for NaN)
    const double r2 = x * x + y * y + z * z;
    return r2 >= 0.25 && r2 <= 4.0;
  };
  if (!sane(cxd, cyd, czd)) {  // uniform across the CTA
    if (threadIdx.x == 0) sCentre = INT_MAX;
    __syncthreads();
    for (int t = threadIdx.x; t < tcount; t += kNth) {
      const int64_t q = (int64_t)(tile0 + t) * tgt.si;
      if (sane(tgt.x[q], tgt.x[q + tgt.sc], tgt.x[q + 2 * tgt.sc])) atomicMin(&sCentre, t);
    }
    __syncthreads();
    cs = sCentre;
    if (cs == INT_MAX) {
      cxd = cyd = czd = 0.0;
    } else {
      const int64_t q = (int64_t)(tile0 + cs) * tgt.si;
      cxd = tgt.x[q]; cyd = tgt.x[q + tgt.sc]; czd = tgt.x[q + 2 * tgt.sc];
    }
  }
  if (threadIdx.x == 0) { sLo = INT_MAX; sHi = -1; sRad = 0ull; }
  __syncthreads();
  double rad = 0.0;
  for (int t = threadIdx.x; t < tcount; t += kNth) {
    const int64_t q = (int64_t)(tile0 + t) * tgt.si;
    const double dx = tgt.x[q] - cxd, dy = tgt.x[q + tgt.sc] - cyd, dz = tgt.x[q + 2 * tgt.sc] - czd;
    const double r2 = dx * dx + dy * dy + dz * dz;
    rad = (r2 <= 16.0) ? fmax(rad, r2) : rad;  // inf/NaN or runaway targets do not shape the tile
    if (colloc) {
      const int si = S.srcIdx[tile0 + t];
      if (si >= 0) { atomicMin(&sLo, si); atomicMax(&sHi, si); }
    }
  }
  atomicMax(&sRad, (unsigned long long)__double_as_longlong(rad));
  __syncthreads();
  const bool fast = (colloc || meshTargets) && __longlong_as_double((long long)sRad) <= kFastRadius * kFastRadius;
  const Stage T{sXY, sZW, sD, sLXY, sLZ};
  if (fast)
    tileSum<PSI, false>(S, ns, tgt, tile0, tcount, cxd, cyd, czd, colloc, sLo, sHi, eps2, T, u, usi, usc, psi);
  else
    tileSum<PSI, true>(S, ns, tgt, tile0, tcount, cxd, cyd, czd, colloc, sLo, sHi, eps2, T, u, usi, usc, psi);
}

// Device address of the scratch array, looked up once per device.
constexpr int kMaxDevices = 64;
unsigned char* g_scratchPtr[kMaxDevices];
cudaError_t g_scratchErr[kMaxDevices];
std::once_flag g_scratchOnce[kMaxDevices];

}  // namespace

extern "C" int lpm_bve_velocity_noalloc(const lpm_points* tgt, const lpm_sources* src, double* u, int64_t u_stride_i,
                                        int64_t u_stride_c, double* psi, unsigned flags, double eps,
                                        lpm_stream_t stream) {
  if (!src) return LPM_ERR_INVALID_ARGUMENT;
  const bool colloc = flags & LPM_BVE_COLLOCATED;
  const bool wantVel = !(flags & LPM_BVE_NO_VELOCITY);
  const bool wantPsi = flags & LPM_BVE_PSI;
  const bool meshTargets = flags & LPM_BVE_MESH_TARGETS;
  if (!(flags & LPM_BVE_FP32C)) {
    std::fprintf(stderr, "lpm_bve_velocity_noalloc: only the FP32C precision (LPM_BVE_FP32C) is provided\n");
    return LPM_ERR_NOT_SUPPORTED;
  }
  // Flags of lpm_bve_velocity this entry point does not implement are refused, not ignored: a
  // caller switching entry points must not silently lose the tree code, the reciprocal without
  // its Newton step or the masked-target skip.  (Targets are always taken in caller order, so
  // LPM_BVE_NO_SORT is accepted and changes nothing.)
  constexpr unsigned kAccepted = LPM_BVE_FP32C | LPM_BVE_COLLOCATED | LPM_BVE_PSI | LPM_BVE_NO_VELOCITY |
                                 LPM_BVE_NO_SORT | LPM_BVE_MESH_TARGETS;
  if (flags & ~kAccepted) {
    std::fprintf(stderr, "lpm_bve_velocity_noalloc: flags 0x%x are not supported here (accepted: FP32C, COLLOCATED, "
                 "PSI, NO_VELOCITY, NO_SORT, MESH_TARGETS); use lpm_bve_velocity\n", flags & ~kAccepted);
    return LPM_ERR_NOT_SUPPORTED;
  }
  const lpm_points& sp = src->pts;
  const lpm_points* tp = colloc ? &sp : tgt;
  if (!tp || sp.n < 0 || tp->n < 0 || !(eps >= 0.0) || (!wantVel && !wantPsi)) return LPM_ERR_INVALID_ARGUMENT;
  if (sp.n > kMaxFaces || tp->n > kMaxTargets) {
    std::fprintf(stderr,
                 "lpm_bve_velocity_noalloc: %lld sources / %lld targets exceed the static scratch limit "
                 "(%d sources, %lld targets); use lpm_bve_velocity\n",
                 (long long)sp.n, (long long)tp->n, kMaxFaces, (long long)kMaxTargets);
    return LPM_ERR_NOT_SUPPORTED;
  }
  if ((sp.n > 0 && (!sp.x || !src->zeta || !src->area)) || (tp->n > 0 && !tp->x) ||
      (wantVel && tp->n > 0 && !u) || (wantPsi && tp->n > 0 && !psi))
    return LPM_ERR_INVALID_ARGUMENT;
  if (tp->n == 0) return LPM_OK;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LPM_ERR_CUDA;
  // First call on this device: look up the array's device address (do this before any
  // stream capture; later calls only read the cached pointer).
  std::call_once(g_scratchOnce[dev], [dev]() {
    void* p = nullptr;
    g_scratchErr[dev] = cudaGetSymbolAddress(&p, g_noallocScratch);
    g_scratchPtr[dev] = static_cast<unsigned char*>(p);
  });
  if (g_scratchErr[dev] != cudaSuccess || !g_scratchPtr[dev]) {
    std::fprintf(stderr, "lpm_bve_velocity_noalloc: cudaGetSymbolAddress failed: %s\n",
                 cudaGetErrorString(g_scratchErr[dev]));
    return LPM_ERR_CUDA;
  }
  unsigned char* base = g_scratchPtr[dev];
  cudaStream_t s = (cudaStream_t)stream;
  const int nf = (int)sp.n;
  const int nblocks = (nf + kCountBlock - 1) / kCountBlock;
  const Pts S{sp.x, sp.n, sp.stride_i, sp.stride_c};
  const Pts T{tp->x, tp->n, tp->stride_i, tp->stride_c};
  if (nblocks > 0) countKernel<<<nblocks, kCountBlock, 0, s>>>(base, src->mask, nf);
  scanKernel<<<1, kMaxBlocks, 0, s>>>(base, nblocks);   // also sets the live count (0 without faces)
  if (nblocks > 0) packKernel<<<nblocks, kCountBlock, 0, s>>>(base, S, src->zeta, src->area, src->mask, nf);
  const int tiles = (int)((tp->n + kNth * kK - 1) / (kNth * kK));
  double* uo = wantVel ? u : nullptr;
  if (wantPsi)
    pairKernel<true><<<tiles, kNth, 0, s>>>(base, T, colloc, meshTargets, eps * eps, uo, u_stride_i, u_stride_c, psi);
  else
    pairKernel<false><<<tiles, kNth, 0, s>>>(base, T, colloc, meshTargets, eps * eps, uo, u_stride_i, u_stride_c, nullptr);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "lpm_bve_velocity_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return LPM_ERR_CUDA;
  }
  return LPM_OK;
}
