/* lpm_bve_probe.h -- measurement helper for the roofline of the BVE pair kernels.
 *
 * No counterpart in pbosler/lpmKokkos (which records no timings).  The pair kernels are
 * bound by the FP32 FMA pipe; this probe measures that pipe's achievable rate with
 * independent FFMA chains, in FMA-pipe lane operations per second, over `iters`
 * iterations of 8 chains per thread on every SM.  device < 0 keeps the current device. */
#ifndef LPM_BVE_PROBE_H
#define LPM_BVE_PROBE_H

#ifdef __cplusplus
extern "C" {
#endif

int lpm_probe_fp32_fma(int device, int iters, double* lane_ops_per_s, double* ms);
/* The same with paired FP32 FMAs (f32x2, two FMA lanes per issued instruction); the rate is
 * still counted in single FMA lane operations per second. */
int lpm_probe_fp32_fma2(int device, int iters, double* lane_ops_per_s, double* ms);

#ifdef __cplusplus
}
#endif

#endif
