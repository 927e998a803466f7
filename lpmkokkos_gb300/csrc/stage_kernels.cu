// stage_kernels.cu -- O(N) kernels around the pair sums of the BVE path.
//
//  prep     : stage positions/vorticity x + c*x_k, zeta + c*zeta_k in FP64 (the
//             KokkosBlas::update calls of src/LpmBVERK4_Impl.hpp:71-107), stage-1 increments
//             from the stored velocity (KokkosBlas::scal + BVEVorticityTendency, :63-68),
//             and the packed source records read by the pair kernels.
//  epilogue : fixed-order sum of the per-chunk partials, FP64 cross product x_i x V,
//             velocity written to the caller's arrays, stage increments x_k = dt*u and
//             zeta_k = -2 Omega u_z dt (src/LpmBVEKernels.hpp:307-320) fused in.
//  combine  : BVERK4Update (src/LpmBVERK4_Impl.hpp:11-39), including the face-vorticity
//             quirk of :121, and the optional renormalisation to |x| = 1.
//
// Each kernel walks a block map {solve, first index, kind, 0} so one launch covers every
// solve of an ensemble.

#include "engine.hpp"

namespace lpm {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ double ld(const DVec& v, int64_t i, int c) { return v.p[i * v.si + c * v.sc]; }
__device__ __forceinline__ void st(const DVec& v, int64_t i, int c, double x) { v.p[i * v.si + c * v.sc] = x; }

// RK4 stage coefficient applied to the previous increment (0 for a plain evaluation).
__device__ __forceinline__ double stageCoef(int stage) { return stage == 3 ? 1.0 : 0.5; }

__global__ void __launch_bounds__(kBlock) prepKernel(const SolveStage* __restrict__ stages,
                                                     const int4* __restrict__ map, int stage, int fp32c,
                                                     int* __restrict__ counter) {
  if (blockIdx.x == 0 && threadIdx.x == 0) counter[0] = counter[1] = 0;
  const int4 m = map[blockIdx.x];
  const SolveStage& S = stages[m.x];
  const int i = m.y + threadIdx.x;
  const ParticleIO& io = S.io;
  const double dt = S.dt, omega = S.omega;
  if (m.z == 0) {                                   // target slot
    if (i >= S.nslots) return;
    const int p = S.perm[i];
    const bool isA = p < io.na;
    const int64_t q = isA ? p : p - io.na;
    const DVec& X = isA ? io.ax : io.bx;
    double x[3] = {ld(X, q, 0), ld(X, q, 1), ld(X, q, 2)};
    if (stage == 1) {                               // x_1 = dt*u (scal), zeta_1 = -2 Omega u_z dt
      const DVec& U = isA ? io.au : io.bu;
      double k[3];
      for (int c = 0; c < 3; ++c) { k[c] = dt * ld(U, q, c); S.kx[0][(size_t)c * S.nslots + i] = k[c]; }
      S.kz[0][i] = -2.0 * omega * ld(U, q, 2) * dt;
      for (int c = 0; c < 3; ++c) x[c] = x[c] + 0.5 * k[c];
    } else if (stage >= 2) {
      const double* k = S.kx[stage - 1];
      const double a = stageCoef(stage);
      for (int c = 0; c < 3; ++c) x[c] = x[c] + a * k[(size_t)c * S.nslots + i];
    }
    for (int c = 0; c < 3; ++c) S.tx[(size_t)c * S.nslots + i] = x[c];
  } else {                                          // source record
    if (i >= S.ns) return;
    const int f = S.srcFace[i];
    double x[3] = {ld(io.bx, f, 0), ld(io.bx, f, 1), ld(io.bx, f, 2)};
    double z = io.bzeta[f];
    if (stage == 1) {
      double k[3];
      for (int c = 0; c < 3; ++c) k[c] = dt * ld(io.bu, f, c);
      const double kz = -2.0 * omega * ld(io.bu, f, 2) * dt;
      for (int c = 0; c < 3; ++c) x[c] = x[c] + 0.5 * k[c];
      z = z + 0.5 * kz;
    } else if (stage >= 2) {
      const int t = S.srcSlot[i];
      const double a = stageCoef(stage);
      for (int c = 0; c < 3; ++c) x[c] = x[c] + a * S.kx[stage - 1][(size_t)c * S.nslots + t];
      z = z + a * S.kz[stage - 1][t];
    }
    const double circ = -z * io.barea[f];
    if (S.rev) {  // the symmetric leaf kernel adds into these
      for (int c = 0; c < 4; ++c) S.rev[(size_t)c * S.ns + i] = 0ull;
      S.revBad[i] = 0;
    }
    if (fp32c) {
      float hi[3], lo[3];
      for (int c = 0; c < 3; ++c) { hi[c] = __double2float_rn(x[c]); lo[c] = __double2float_rn(x[c] - (double)hi[c]); }
      const float w = __double2float_rn(circ * (1.0 / (2.0 * kPi)));
      const float D = __double2float_rn(1.0 - (x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
      S.sp0[i] = make_float4(hi[0], hi[1], hi[2], w);
      S.sp1[i] = make_float4(lo[0], lo[1], lo[2], D);
    } else {
      S.sd[i] = make_double4_32a(x[0], x[1], x[2], circ);
    }
  }
}

__global__ void __launch_bounds__(kBlock) epilogueKernel(const SolveStage* __restrict__ stages,
                                                         const int4* __restrict__ map, int fp32c, int psi,
                                                         int velocity, int stageOut, int useRev) {
  const int4 m = map[blockIdx.x];
  const SolveStage& S = stages[m.x];
  const int i = m.y + threadIdx.x;
  if (i >= S.nslots) return;
  const int n = S.nslots;
  const int ncomp = fp32c ? (psi ? 5 : 3) : (psi ? 4 : 3);
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int c = 0; c < S.nchunks; ++c) {                 // fixed order: deterministic per target
    const double* P = S.partial + (size_t)c * ncomp * n;
    for (int k = 0; k < ncomp; ++k) v[k] += P[(size_t)k * n + i];
  }
  if (useRev && S.rev && S.leaf0 >= 0 && i >= S.leaf0) {   // reverse sums of the symmetric leaf kernel
    const int k = i - S.leaf0;
    if (S.revBad[k]) {
      v[0] = v[1] = v[2] = v[3] = __longlong_as_double(0x7ff8000000000000ll);  // NaN
    } else {  // component 3: sum w (log2 2q - 1), the weight sum folded in
      const int nc = (fp32c && psi) ? 4 : 3;
      for (int c = 0; c < nc; ++c) v[c] += (double)(long long)S.rev[(size_t)c * S.ns + k] * (1.0 / kSymScale);
    }
  }
  double u[3];
  if (fp32c) {                                          // u = x_i x V
    const double x0 = S.tx[i], x1 = S.tx[n + i], x2 = S.tx[2 * n + i];
    u[0] = x1 * v[2] - x2 * v[1];
    u[1] = x2 * v[0] - x0 * v[2];
    u[2] = x0 * v[1] - x1 * v[0];
  } else {
    u[0] = v[0]; u[1] = v[1]; u[2] = v[2];
  }
  const int p = S.perm[i];
  const ParticleIO& io = S.io;
  const bool isA = p < io.na;
  const int64_t q = isA ? p : p - io.na;
  if (velocity) {
    const DVec& U = isA ? io.au : io.bu;
    for (int c = 0; c < 3; ++c) st(U, q, c, u[c]);
  }
  if (psi) {
    double* out = isA ? io.apsi : io.bpsi;
    const double ps = fp32c ? 0.34657359027997264 * (v[3] - v[4])   // (ln 2 / 2) (sum w log2(2q) - sum w)
                            : v[3];
    if (out) out[q] = ps;
  }
  if (stageOut >= 1) {
    for (int c = 0; c < 3; ++c) S.kx[stageOut][(size_t)c * n + i] = S.dt * u[c];
    S.kz[stageOut][i] = -2.0 * S.omega * u[2] * S.dt;
  }
}

__global__ void __launch_bounds__(kBlock) combineKernel(const SolveStage* __restrict__ stages,
                                                        const int4* __restrict__ map, int quirk, int renorm) {
  const int4 m = map[blockIdx.x];
  const SolveStage& S = stages[m.x];
  const int i = m.y + threadIdx.x;
  if (i >= S.nslots) return;
  const int n = S.nslots;
  const int p = S.perm[i];
  const ParticleIO& io = S.io;
  const bool isA = p < io.na;
  const int64_t q = isA ? p : p - io.na;
  const DVec& X = isA ? io.ax : io.bx;
  const double sixth = 1.0 / 6.0, third = 1.0 / 3.0;
  double x[3];
  for (int c = 0; c < 3; ++c) {
    const size_t o = (size_t)c * n + i;
    const double inc = __dadd_rn(__dmul_rn(sixth, S.kx[0][o] + S.kx[3][o]), __dmul_rn(third, S.kx[1][o] + S.kx[2][o]));
    x[c] = ld(X, q, c) + inc;
  }
  if (renorm) {
    const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    for (int c = 0; c < 3; ++c) x[c] = x[c] / r;
  }
  for (int c = 0; c < 3; ++c) st(X, q, c, x[c]);
  double* Z = isA ? io.azeta : io.bzeta;
  if (Z) {
    const double k3 = (!isA && quirk) ? S.kz[3][i] : S.kz[2][i];   // src/LpmBVERK4_Impl.hpp:121
    const double inc = __dadd_rn(__dmul_rn(sixth, S.kz[0][i] + S.kz[3][i]), __dmul_rn(third, S.kz[1][i] + k3));
    Z[q] = Z[q] + inc;
  }
}

}  // namespace

cudaError_t launchPrep(const SolveStage* st, const int4* map, int nblocks, int stage, Precision prec, int* counter,
                       cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  prepKernel<<<nblocks, kBlock, 0, s>>>(st, map, stage, prec == Precision::FP32C ? 1 : 0, counter);
  return cudaGetLastError();
}

cudaError_t launchEpilogue(const SolveStage* st, const int4* map, int nblocks, Precision prec, bool psi,
                           bool velocity, int stageOut, cudaStream_t s, bool useRev) {
  if (nblocks <= 0) return cudaSuccess;
  epilogueKernel<<<nblocks, kBlock, 0, s>>>(st, map, prec == Precision::FP32C ? 1 : 0, psi ? 1 : 0,
                                            velocity ? 1 : 0, stageOut, useRev ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launchCombine(const SolveStage* st, const int4* map, int nblocks, bool quirk, bool renorm,
                          cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  combineKernel<<<nblocks, kBlock, 0, s>>>(st, map, quirk ? 1 : 0, renorm ? 1 : 0);
  return cudaGetLastError();
}

int stageBlockSize() { return kBlock; }

}  // namespace lpm
