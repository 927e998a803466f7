/* lpm_bve_server.h -- continuous-batching BVE solve server on one GPU.
 *
 * No counterpart in pbosler/lpmKokkos (one driver runs one BVESphere to completion).
 * Requests (a mesh, seeded RH54 + Gaussian-vortex initial data, dt, Omega, a step count) are
 * admitted first-come first-served while their estimated device footprint fits an HBM budget;
 * their particle state then stays on the device until they finish.  Running solves advance by
 * RK4 steps (src/LpmBVERK4_Impl.hpp:42-130); solves of similar cost share a batch whose four
 * evaluations per step are one pair-kernel launch each, on a CUDA stream whose priority falls
 * with the cost, so batches of different sizes run side by side and a small request is not held
 * behind the steps of a large one.  A request that arrives while others run joins at once and
 * leaves as soon as its own steps are done.  A solve's result does not depend on which other solves shared
 * its launches (per-solve summation order is fixed): bit-identical alone or in any mix.  Host
 * preparation (mesh, initial data, plan) runs on a separate thread.
 * With LPM_BVE_TREECODE in flags, requests of at least 1e9 target x source pairs per evaluation
 * take the tree code: two threads upload them and compute their initial velocity (which sizes
 * their interaction lists), then they step in tree classes whose steps are captured graphs,
 * side by side with the direct classes.
 */
#ifndef LPM_BVE_SERVER_H
#define LPM_BVE_SERVER_H

#include "lpm_bve.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lpm_bve_server lpm_bve_server;

typedef struct {
  int device;              /* CUDA device ordinal; -1 = current */
  size_t hbm_budget_bytes; /* admission budget for request state + plans; 0 = 80 % of free memory */
  int max_active;          /* at most this many solves run together; 0 = no limit */
  unsigned flags;          /* LPM_BVE_FP32C or LPM_BVE_FP64, plus RK4 options of lpm_bve_rk4_step */
  double eps;              /* regularisation of the kernels (0 = reference) */
  int host_ic;             /* 1: initial vorticity from the host functions (lpm_ic_rh54 +
                              lpm_ic_gaussians_add, bitwise those of a BVESphere run); 0: on the
                              GPU after the upload (lpm_ic_rh54_gaussians_device, a few ulps apart) */
} lpm_bve_server_opts;

typedef struct {
  int seed;            /* LPM_SEED_ICOS_TRI or LPM_SEED_CUBED */
  int level;           /* uniform refinement level, 0..10 */
  uint64_t ic_seed;    /* seed of the Gaussian-vortex parameters */
  int n_gaussians;     /* RH54 plus this many Gaussian vortices (<= LPM_IC_MAX_GAUSSIANS), U(-2, 2) */
  double gauss_width;  /* vortex width in radians */
  double dt, omega;    /* time step and rotation rate */
  int nsteps;          /* RK4 steps to run */
} lpm_bve_request;

enum { LPM_REQ_QUEUED = 0, LPM_REQ_PREPARING = 1, LPM_REQ_RUNNING = 2, LPM_REQ_DONE = 3,
       LPM_REQ_FAILED = -1, LPM_REQ_CANCELLED = -2 };

typedef struct {
  int64_t submitted, completed, failed, cancelled, running, queued;
  int64_t steps_run;          /* RK4 steps launched over size classes (one step of one class) */
  int64_t solve_steps;        /* sum over solves of RK4 steps taken */
  double pairs;               /* target-source pairs evaluated by the direct sum (incl. masked-parent
                                 targets); tree-code requests are not counted here */
  double busy_s;              /* wall time with at least one solve running */
  size_t reserved_bytes, budget_bytes;
  int max_running_seen;
  double tree_equiv_pairs;    /* tree-code requests: the direct-sum pairs their evaluations replace
                                 (work equivalent, not work done) */
} lpm_bve_server_counters;

int lpm_bve_server_create(const lpm_bve_server_opts* opts, lpm_bve_server** out);
/* Device bytes the server reserves for a request (state, plan and batch tables), the figure
 * admission compares with the budget.  Host-only; opts may be NULL (FP32C). */
int lpm_bve_server_estimate(const lpm_bve_server_opts* opts, const lpm_bve_request* req, size_t* bytes);
/* Non-blocking.  LPM_ERR_ADMISSION if the request can never fit the budget,
 * LPM_ERR_INVALID_ARGUMENT for a malformed request. */
int lpm_bve_server_submit(lpm_bve_server* s, const lpm_bve_request* req, int64_t* id);
/* Waits at most timeout_s (< 0: no limit) for the request to finish: LPM_OK when done,
 * LPM_ERR_TIMEOUT if it is still running, LPM_ERR_STATE if it failed or was cancelled. */
int lpm_bve_server_wait(lpm_bve_server* s, int64_t id, double timeout_s);
int lpm_bve_server_status(lpm_bve_server* s, int64_t id, int* state);
/* Cancels a request that has not started running; running requests finish normally. */
int lpm_bve_server_cancel(lpm_bve_server* s, int64_t id);
/* Final state of a finished request, host arrays (row-major n x 3 for vectors).  With all
 * array pointers NULL only the sizes are returned. */
int lpm_bve_server_result(lpm_bve_server* s, int64_t id, int64_t* nverts, int64_t* nfaces, double* vx,
                          double* vzeta, double* vvel, double* fx, double* fzeta, double* fvel);
/* Writes a finished request's final state as a snapshot file (include/lpm_bve_snapshot.h), with
 * t = nsteps * dt; lpm_bve_snapshot_read restores it into device arrays to continue the run. */
int lpm_bve_server_snapshot(lpm_bve_server* s, int64_t id, const char* path);
/* Frees the host copy of a finished (done, failed or cancelled) request and forgets its id. */
int lpm_bve_server_release(lpm_bve_server* s, int64_t id);
/* Seconds from submit to done, spent queued/preparing before the first step, and running. */
int lpm_bve_server_timing(lpm_bve_server* s, int64_t id, double* total_s, double* wait_s, double* run_s);
/* Nearest-rank quantiles q[0..nq) (each in [0, 1]) of submit-to-done latency over the completed
 * requests, in seconds.  LPM_ERR_STATE if none has completed. */
int lpm_bve_server_latency(lpm_bve_server* s, const double* q, int nq, double* out);
int lpm_bve_server_stats(lpm_bve_server* s, lpm_bve_server_counters* out);
const char* lpm_bve_server_last_error(lpm_bve_server* s);
/* Stops the server (running requests are abandoned) and frees everything. */
int lpm_bve_server_destroy(lpm_bve_server* s);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LPM_BVE_SERVER_H */
