/* lpm_bve_ensemble.h -- batched ensembles of independent BVE solves on one GPU.
 *
 * No counterpart in pbosler/lpmKokkos, which advances one BVESphere at a time
 * (BVERK4::advance_timestep, src/LpmBVERK4_Impl.hpp:42-130).  An ensemble advances many
 * solves of uneven sizes together: every RK4 evaluation is ONE persistent pair-kernel
 * launch over a shared work list (target tile x source chunk items of all solves,
 * longest first), and a whole step is captured once as a CUDA graph and replayed.
 * Each solve's arithmetic is exactly that of lpm_bve_rk4_step on the same solve: the
 * per-target summation order is fixed by the tile/chunk layout, not by the schedule.
 */
#ifndef LPM_BVE_ENSEMBLE_H
#define LPM_BVE_ENSEMBLE_H

#include "lpm_bve.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lpm_bve_ensemble lpm_bve_ensemble;

/* Build the shared plan for `nsolves` states (device arrays stay owned by the caller and
 * must stay valid).  flags: precision and RK4 options of lpm_bve_rk4_step. */
int lpm_bve_ensemble_create(lpm_bve_ctx* ctx, const lpm_bve_state* states, int nsolves, unsigned flags, double eps,
                            lpm_stream_t stream, lpm_bve_ensemble** out);
/* Advance every solve by nsteps RK4 steps; dt[m], Omega[m] per solve (host arrays). */
int lpm_bve_ensemble_step(lpm_bve_ensemble* e, const double* dt, const double* Omega, int nsteps, lpm_stream_t stream);
/* Work-list statistics: solves, work items, persistent grid, target-source pairs per
 * evaluation (incl. masked targets), device bytes held by the plan. */
int lpm_bve_ensemble_info(const lpm_bve_ensemble* e, int* nsolves, int* nitems, int* grid, int64_t* pairs_per_eval,
                          size_t* device_bytes);
int lpm_bve_ensemble_destroy(lpm_bve_ensemble* e);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LPM_BVE_ENSEMBLE_H */
