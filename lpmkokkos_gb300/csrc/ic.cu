// ic.cu -- initial relative vorticity on the device: the Rossby-Haurwitz wave 4 of
// src/LpmRossbyWaves.hpp:28-32 (zeta = 30 cos(4 lambda) P_5^4(z)) plus seeded Gaussian
// vortices zeta += a_g exp(-(d(x, c_g) / width)^2), d the great-circle distance.  The same
// formulas and operation order as the host functions lpm_ic_rh54 / lpm_ic_gaussians_add;
// products and sums are issued as __dmul_rn / __dadd_rn (no contraction, as the host code is
// compiled), so only cos, atan2 and exp -- CUDA's math library against the host's -- may differ,
// by a few ulps.  One thread per point; memory-bound (3 doubles in, 1 out).

#include "lpm_bve.h"

#include <cuda_runtime.h>
#include <cstdint>

namespace {

constexpr double kPiD = 3.141592653589793238462643383279502884;

struct IcParams {
  int ng;
  double width;
  double c[LPM_IC_MAX_GAUSSIANS][3];
  double a[LPM_IC_MAX_GAUSSIANS];
};

// Longitude in [0, 2 pi) with the host's branch structure.
__device__ __forceinline__ double longitudeOf(double x, double y) {
  if (x == 0.0) {
    if (y > 0.0) return 0.5 * kPiD;
    if (y < 0.0) return 1.5 * kPiD;
    return 0.0;
  }
  if (y == 0.0) return x > 0.0 ? 0.0 : kPiD;
  const double t = atan2(fabs(y), fabs(x));
  if (x > 0.0 && y > 0.0) return t;
  if (x < 0.0 && y > 0.0) return __dsub_rn(kPiD, t);
  if (x < 0.0 && y < 0.0) return __dadd_rn(kPiD, t);
  return __dsub_rn(2.0 * kPiD, t);
}

__device__ __forceinline__ double dot3(double ax, double ay, double az, double bx, double by, double bz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

__global__ void icKernel(const double* __restrict__ x, int64_t n, int64_t si, int64_t sc, IcParams p,
                         double* __restrict__ zeta) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double px = x[i * si], py = x[i * si + sc], pz = x[i * si + 2 * sc];
  const double lam = longitudeOf(px, py);
  const double zz1 = __dsub_rn(__dmul_rn(pz, pz), 1.0);
  double v = __dmul_rn(__dmul_rn(30.0, cos(__dmul_rn(4.0, lam))), __dmul_rn(__dmul_rn(pz, zz1), zz1));
  for (int g = 0; g < p.ng; ++g) {
    const double cx = p.c[g][0], cy = p.c[g][1], cz = p.c[g][2];
    // arc(a, b) = atan2(|a x b|, a . b), cross components in the host's order
    const double kx = __dsub_rn(__dmul_rn(py, cz), __dmul_rn(pz, cy));
    const double ky = __dsub_rn(__dmul_rn(pz, cx), __dmul_rn(px, cz));
    const double kz = __dsub_rn(__dmul_rn(px, cy), __dmul_rn(py, cx));
    const double d = atan2(sqrt(dot3(kx, ky, kz, kx, ky, kz)), dot3(px, py, pz, cx, cy, cz)) / p.width;
    v = __dadd_rn(v, __dmul_rn(p.a[g], exp(-__dmul_rn(d, d))));
  }
  zeta[i] = v;
}

}  // namespace

extern "C" int lpm_ic_rh54_gaussians_device(const double* x, int64_t n, int64_t si, int64_t sc, const double* centers,
                                            const double* amps, int ng, double width, double* zeta,
                                            lpm_stream_t stream) {
  if (n < 0 || ng < 0 || ng > LPM_IC_MAX_GAUSSIANS) return LPM_ERR_INVALID_ARGUMENT;
  if (n == 0) return LPM_OK;
  if (!x || !zeta || si < 0 || sc < 0 || (si == 0 && n > 1)) return LPM_ERR_INVALID_ARGUMENT;
  if (ng > 0 && (!centers || !amps || !(width > 0.0))) return LPM_ERR_INVALID_ARGUMENT;
  IcParams p{};
  p.ng = ng;
  p.width = ng > 0 ? width : 1.0;
  for (int g = 0; g < ng; ++g) {
    for (int k = 0; k < 3; ++k) p.c[g][k] = centers[3 * g + k];
    p.a[g] = amps[g];
  }
  constexpr int kBlock = 256;
  const int64_t blocks = (n + kBlock - 1) / kBlock;
  icKernel<<<(unsigned)blocks, kBlock, 0, (cudaStream_t)stream>>>(x, n, si, sc, p, zeta);
  return cudaGetLastError() == cudaSuccess ? LPM_OK : LPM_ERR_CUDA;
}
