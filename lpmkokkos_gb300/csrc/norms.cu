// norms.cu -- relative error norms of ErrNorms::compute (src/LpmErrorNorms.cpp:26-70) on
// device arrays, reduced in a fixed order so the result does not depend on scheduling.
//
// Per entry i with weight w_i (1 when no weights are given) and e_i = appx_i - exact_i:
//   vectors (3 components): m = |e_i|, x = |exact_i|
//   scalars:                m = |e_i|, x = |exact_i| for l1/l2; for linf the reference takes
//                           the largest SIGNED e_i and exact_i (src/LpmErrorNorms.cpp:62-63)
//                           unless magnitudes are asked for.
//   l1 = sum m w / sum x w,  l2 = sqrt(sum m^2 w / sum x^2 w),  linf = max m / max x.
// Pass 1: a fixed grid of blocks, each a grid-stride sum in index order per thread and a
// fixed-shape tree across the block; pass 2: one block folds the block partials in order.
// HBM-bound: 7 doubles (+ mask byte) read per vector entry.

#include "engine.hpp"
#include "lpm_bve.h"

#include <cfloat>
#include <cstdint>

namespace lpm {
namespace {

constexpr int kNormThreads = 256;

struct NormAcc {
  double l1n, l1d, l2n, l2d, linfn, linfd;
};

__device__ __forceinline__ void fold(NormAcc& a, const NormAcc& b) {
  a.l1n += b.l1n;
  a.l1d += b.l1d;
  a.l2n += b.l2n;
  a.l2d += b.l2d;
  a.linfn = fmax(a.linfn, b.linfn);
  a.linfd = fmax(a.linfd, b.linfd);
}

__device__ __forceinline__ NormAcc shuffleDown(const NormAcc& a, int off) {
  NormAcc b;
  b.l1n = __shfl_down_sync(0xffffffffu, a.l1n, off);
  b.l1d = __shfl_down_sync(0xffffffffu, a.l1d, off);
  b.l2n = __shfl_down_sync(0xffffffffu, a.l2n, off);
  b.l2d = __shfl_down_sync(0xffffffffu, a.l2d, off);
  b.linfn = __shfl_down_sync(0xffffffffu, a.linfn, off);
  b.linfd = __shfl_down_sync(0xffffffffu, a.linfd, off);
  return b;
}

// Block-wide fold in a fixed tree; the result is valid in thread 0.
__device__ NormAcc blockFold(NormAcc a) {
  __shared__ NormAcc warpAcc[kNormThreads / 32];
  for (int off = 16; off > 0; off >>= 1) fold(a, shuffleDown(a, off));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) warpAcc[warp] = a;
  __syncthreads();
  if (warp == 0) {
    a = lane < kNormThreads / 32 ? warpAcc[lane]
                                 : NormAcc{0.0, 0.0, 0.0, 0.0, -DBL_MAX, -DBL_MAX};
    for (int off = 16; off > 0; off >>= 1) fold(a, shuffleDown(a, off));
  }
  return a;
}

__global__ void __launch_bounds__(kNormThreads) normsPass1(NormArgs A, double* partial) {
  NormAcc acc{0.0, 0.0, 0.0, 0.0, -DBL_MAX, -DBL_MAX};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += stride) {
    if (A.skip && A.skip[i]) continue;
    const double w = A.wt ? A.wt[i] : 1.0;
    double m, x, mInf, xInf;
    if (A.ncomp == 3) {
      double e2 = 0.0, x2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double xe = A.exact[i * A.e_si + c * A.e_sc];
        const double e = A.appx[i * A.a_si + c * A.a_sc] - xe;
        e2 += e * e;
        x2 += xe * xe;
      }
      m = sqrt(e2);
      x = sqrt(x2);
      mInf = m;
      xInf = x;
    } else {
      const double xe = A.exact[i * A.e_si];
      const double e = A.appx[i * A.a_si] - xe;
      m = fabs(e);
      x = fabs(xe);
      mInf = A.signedLinf ? e : m;
      xInf = A.signedLinf ? xe : x;
    }
    acc.l1n += m * w;
    acc.l1d += x * w;
    acc.l2n += m * m * w;
    acc.l2d += x * x * w;
    acc.linfn = fmax(acc.linfn, mInf);
    acc.linfd = fmax(acc.linfd, xInf);
  }
  acc = blockFold(acc);
  if (threadIdx.x == 0) {
    double* p = partial + 6 * (size_t)blockIdx.x;
    p[0] = acc.l1n;
    p[1] = acc.l1d;
    p[2] = acc.l2n;
    p[3] = acc.l2d;
    p[4] = acc.linfn;
    p[5] = acc.linfd;
  }
}

__global__ void __launch_bounds__(kNormThreads) normsPass2(const double* partial, int nblocks, double* out) {
  NormAcc acc{0.0, 0.0, 0.0, 0.0, -DBL_MAX, -DBL_MAX};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double* p = partial + 6 * (size_t)b;
    fold(acc, NormAcc{p[0], p[1], p[2], p[3], p[4], p[5]});
  }
  acc = blockFold(acc);
  if (threadIdx.x == 0) {
    out[0] = acc.l1n / acc.l1d;
    out[1] = sqrt(acc.l2n / acc.l2d);
    out[2] = acc.linfn / acc.linfd;
  }
}

// u.x per point in FP64 with the reference's operation order (a0 b0 + a1 b1) + a2 b2 and no
// fused multiply-add, so each entry equals the host's bit for bit.
__global__ void __launch_bounds__(256) tangencyKernel(const double* __restrict__ x, int64_t xsi, int64_t xsc,
                                                      const double* __restrict__ u, int64_t usi, int64_t usc,
                                                      int64_t n, double* __restrict__ udotx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* xi = x + i * xsi;
  const double* ui = u + i * usi;
  const double d = __dadd_rn(__dadd_rn(__dmul_rn(xi[0], ui[0]), __dmul_rn(xi[xsc], ui[usc])),
                             __dmul_rn(xi[2 * xsc], ui[2 * usc]));
  udotx[i] = d;
}

}  // namespace

int normBlocks(int sms) { return 2 * sms; }

cudaError_t launchNorms(const NormArgs& a, double* partial, int nblocks, double* out, cudaStream_t s) {
  normsPass1<<<nblocks, kNormThreads, 0, s>>>(a, partial);
  normsPass2<<<1, kNormThreads, 0, s>>>(partial, nblocks, out);
  return cudaGetLastError();
}

}  // namespace lpm

extern "C" int lpm_sphere_tangency(const double* x, int64_t x_si, int64_t x_sc, const double* u, int64_t u_si,
                                   int64_t u_sc, int64_t n, double* udotx, lpm_stream_t stream) {
  if (n < 0) return LPM_ERR_INVALID_ARGUMENT;
  if (n == 0) return LPM_OK;
  if (!x || !u || !udotx || x_si < 0 || x_sc < 0 || u_si < 0 || u_sc < 0) return LPM_ERR_INVALID_ARGUMENT;
  constexpr int kBlock = 256;
  const int64_t blocks = (n + kBlock - 1) / kBlock;
  if (blocks > INT32_MAX) return LPM_ERR_INVALID_ARGUMENT;
  lpm::tangencyKernel<<<(unsigned)blocks, kBlock, 0, (cudaStream_t)stream>>>(x, x_si, x_sc, u, u_si, u_sc, n, udotx);
  return cudaGetLastError() == cudaSuccess ? LPM_OK : LPM_ERR_CUDA;
}
