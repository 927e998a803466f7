// probe.cu -- FP32 FMA-pipe throughput probe for the roofline of the pair kernels.
//
// The BVE pair kernels are bound by the FP32 FMA pipe (13 FMA-pipe lane-ops per velocity
// pair), a figure the HBM / bf16 peak measurements do not provide.  This kernel issues
// only independent FFMA chains (8 per thread, no loads) so its rate is the achievable
// FMA-pipe peak at the current clock.

#include "lpm_bve.h"
#include "lpm_bve_probe.h"

#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) fmaProbe(float* out, int iters, float b, float c) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains alive; never true in practice
}

// The same with paired FP32 FMAs (f32x2: two lanes' worth of FMA per issued instruction, the
// form the FP32C pair kernel uses): 8 independent float2 chains, 16 FMA lane-ops per iteration.
__global__ void __launch_bounds__(kThreads) fma2Probe(float* out, int iters, float b, float c) {
  float2 a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = make_float2((float)(threadIdx.x + k) * 1e-3f, (float)(k + 1) * 1e-3f);
  const float2 b2 = make_float2(b, b), c2 = make_float2(c, c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = __ffma2_rn(a[k], b2, c2);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k].x + a[k].y;
  if (s == 12345.678f) out[blockIdx.x] = s;
}

template <typename Kernel>
int runProbe(Kernel kernel, int lanesPerChainStep, int device, int iters, double* lane_ops_per_s, double* ms_out) {
  if (!lane_ops_per_s || iters <= 0) return LPM_ERR_INVALID_ARGUMENT;
  if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return LPM_ERR_CUDA;
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LPM_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return LPM_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kThreads, 0) != cudaSuccess) return LPM_ERR_CUDA;
  const int grid = sms * per;
  float* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = LPM_OK;
  if (cudaMalloc(&out, sizeof(float) * grid) != cudaSuccess) return LPM_ERR_OUT_OF_MEMORY;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = LPM_ERR_CUDA;
  if (rc == LPM_OK) {
    kernel<<<grid, kThreads>>>(out, iters / 10 + 1, 0.999f, 1e-3f);  // warm-up
    cudaEventRecord(e0);
    kernel<<<grid, kThreads>>>(out, iters, 0.999f, 1e-3f);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = LPM_ERR_CUDA;
  }
  if (rc == LPM_OK) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *lane_ops_per_s = (double)grid * kThreads * (double)iters * kChains * lanesPerChainStep / (ms * 1e-3);
    if (ms_out) *ms_out = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}

}  // namespace

extern "C" int lpm_probe_fp32_fma2(int device, int iters, double* lane_ops_per_s, double* ms_out) {
  return runProbe(fma2Probe, 2, device, iters, lane_ops_per_s, ms_out);
}

extern "C" int lpm_probe_fp32_fma(int device, int iters, double* lane_ops_per_s, double* ms_out) {
  return runProbe(fmaProbe, 1, device, iters, lane_ops_per_s, ms_out);
}
