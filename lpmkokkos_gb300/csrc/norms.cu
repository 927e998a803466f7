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

}  // namespace

int normBlocks(int sms) { return 2 * sms; }

cudaError_t launchNorms(const NormArgs& a, double* partial, int nblocks, double* out, cudaStream_t s) {
  normsPass1<<<nblocks, kNormThreads, 0, s>>>(a, partial);
  normsPass2<<<1, kNormThreads, 0, s>>>(partial, nblocks, out);
  return cudaGetLastError();
}

}  // namespace lpm
