/* lpm_bve.h -- C ABI of the GB300-native barotropic-vorticity (BVE) path.
 *
 * Drop-in replacement for the BVE hot path of pbosler/lpmKokkos: the spherical
 * Biot-Savart velocity and stream-function direct sums (src/LpmBVEKernels.hpp) and
 * the RK4 stepper that evaluates them four times per step (src/LpmBVERK4_Impl.hpp).
 * Everything below is plain C: device pointers, sizes, strides and a CUDA stream.
 *
 * Conventions
 *  - All particle arrays are DEVICE pointers owned by the caller.  A vector array is
 *    addressed as x[i*stride_i + c*stride_c] (c = 0,1,2), so both Kokkos layouts are
 *    accepted: LayoutLeft (stride_i = 1, stride_c = n, the CUDA default of
 *    View<double*[3]>) and LayoutRight (stride_i = 3, stride_c = 1).
 *  - mask arrays hold one byte per face, nonzero = masked (a divided parent panel),
 *    as Kokkos View<bool*> does.
 *  - Work is queued on `stream` and returns without synchronising, except the first
 *    call for a new problem geometry (new pointers, sizes, strides or mask), which
 *    builds a plan: it copies positions and the mask to the host, synchronising the
 *    stream once.  The plan is reused by later calls with the same geometry: a context
 *    keeps the plan of its last lpm_bve_velocity call with distinct targets, of its last
 *    collocated call (so a mesh's vertex and face evaluations both stay planned) and of
 *    its last lpm_bve_rk4_step state.
 *  - Every function returns LPM_OK (0) or a negative status; lpm_bve_last_error()
 *    gives the message.  One context per host thread / stream.
 */
#ifndef LPM_BVE_H
#define LPM_BVE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* lpm_stream_t; /* identical to cudaStream_t; NULL = legacy default stream */

/* ---- status codes ---------------------------------------------------------- */
#define LPM_OK                    0
#define LPM_ERR_INVALID_ARGUMENT (-1)
#define LPM_ERR_CUDA             (-2)
#define LPM_ERR_OUT_OF_MEMORY    (-3)
#define LPM_ERR_NOT_SUPPORTED    (-4)
#define LPM_ERR_ADMISSION        (-5) /* server: request does not fit the HBM budget */
#define LPM_ERR_STATE            (-6) /* object used in the wrong state (e.g. unknown request id) */
#define LPM_ERR_TIMEOUT          (-7) /* a bounded wait gave up */
#define LPM_ERR_INTERNAL         (-8) /* an unexpected host-side failure (message in last_error) */

/* ---- flags ------------------------------------------------------------------ */
#define LPM_BVE_FP64                0u        /* plain FP64 pair arithmetic (the GPU oracle) */
#define LPM_BVE_FP32C               (1u << 0) /* FP32 pair arithmetic, compensated sums, FP64 epilogue */
#define LPM_BVE_COLLOCATED          (1u << 1) /* velocity(): targets are the sources, i == j excluded */
#define LPM_BVE_PSI                 (1u << 2) /* also compute the stream function */
#define LPM_BVE_NO_VELOCITY         (1u << 3) /* velocity(): stream function only (u may be NULL) */
#define LPM_BVE_RK4_FIX_QUIRK       (1u << 4) /* rk4: RK4-correct face vorticity update; default
                                                 reproduces src/LpmBVERK4_Impl.hpp:121 */
#define LPM_BVE_RENORM              (1u << 5) /* rk4: project positions to |x| = 1 after each step */
#define LPM_BVE_SKIP_MASKED_TARGETS (1u << 6) /* rk4: no velocity at masked faces (their x, zeta stay fixed) */
#define LPM_BVE_NO_GRAPH            (1u << 7) /* rk4: launch kernels directly, no captured CUDA graph */
#define LPM_BVE_NO_SORT             (1u << 8) /* keep the caller's target order (no spatial sort) */
#define LPM_BVE_MESH_TARGETS        (1u << 9) /* velocity(), distinct targets: they are mesh points (e.g. the
                                                 vertices of the source mesh), each at least about half a mesh
                                                 spacing from every source.  Lets FP32C use its 13-op pair
                                                 formulation; without it arbitrary points get the hi/lo one. */
#define LPM_BVE_RCP_APPROX          (1u << 10) /* FP32C: use the hardware reciprocal without its Newton step
                                                  (11 instead of 13 FMA-pipe ops per pair, about one more
                                                  FP32 rounding per pair) */
#define LPM_BVE_TREECODE            (1u << 11) /* FP32C velocity()/rk4: tree code instead of the direct sum --
                                                 octree clusters far from a target tile act through
                                                 interpolated proxies (lpm_bve_ctx_set_treecode); an
                                                 approximation with its own tolerance, not in the reference */
#define LPM_BVE_NO_SYMMETRIC        (1u << 12) /* FP32C collocated velocity()/rk4: sum every leaf-leaf pair in
                                                 both directions with the plain direct kernel instead of once
                                                 with the symmetric leaf kernel (same sums, other rounding) */

/* ---- context ---------------------------------------------------------------- */
typedef struct lpm_bve_ctx lpm_bve_ctx;

typedef struct {
  int device;   /* CUDA device ordinal; -1 = the current device */
  int autotune; /* nonzero: time candidate launch shapes the first time a problem size is seen */
  int verbose;  /* nonzero: print plan / autotune decisions to stderr */
} lpm_bve_opts;

/* Replaces: BVERK4 construction (src/LpmBVERK4.hpp:29) and Kokkos::initialize for this path. */
int lpm_bve_ctx_create(lpm_bve_ctx** ctx, const lpm_bve_opts* opts);
int lpm_bve_ctx_destroy(lpm_bve_ctx* ctx);
const char* lpm_bve_last_error(const lpm_bve_ctx* ctx);
/* Drop cached plans (use after rewriting a mask or positions in place between unrelated problems). */
int lpm_bve_plan_invalidate(lpm_bve_ctx* ctx);

/* Timing of the O(N^2) pair kernel (the reference's Kokkos::Profiling regions around
 * advance_timestep, src/LpmBVERK4_Impl.hpp:45,129, have no per-kernel timer).  While enabled,
 * every pair-kernel launch is bracketed by CUDA events on its stream and RK4 steps are
 * launched directly instead of through the captured graph.  lpm_bve_ctx_timing synchronises
 * on the recorded events and returns the summed pair-kernel milliseconds and launch count. */
int lpm_bve_ctx_set_timing(lpm_bve_ctx* ctx, int enable);
int lpm_bve_ctx_timing(lpm_bve_ctx* ctx, double* pair_ms, int64_t* pair_launches, int reset);

/* Launch shape of the FP32C pair kernel: CTA threads x targets per thread, sources staged in
 * shared memory per step, and the resident CTAs per SM its register budget is sized for
 * (1 = compiler's choice).  lpm_bve_ctx_shapes lists the compiled shapes (returns their number,
 * fills up to `capacity`); lpm_bve_ctx_set_shape fixes one for plans built afterwards
 * (threads = 0 restores the default).  The autotuner times these same shapes. */
int lpm_bve_ctx_shapes(int* threads, int* targets_per_thread, int* source_tile, int* min_blocks, int capacity);
int lpm_bve_ctx_set_shape(lpm_bve_ctx* ctx, int threads, int targets_per_thread, int source_tile, int min_blocks);

/* ---- particle sets -------------------------------------------------------------- */
typedef struct {
  const double* x;   /* element (i, c) at x[i*stride_i + c*stride_c] */
  int64_t n;
  int64_t stride_i, stride_c;
} lpm_points;

typedef struct {
  lpm_points pts;      /* face-centre (source) positions, all faces including masked parents */
  const double* zeta;  /* relative vorticity, n */
  const double* area;  /* panel area, n */
  const uint8_t* mask; /* n bytes, nonzero = skip as a source; NULL = no face masked */
} lpm_sources;

/* Velocity (and stream function) at targets from all unmasked sources.
 *   u(x_i)   = sum_j (x_i x x_j) * (-zeta_j A_j) / (4 pi (1 - x_i.x_j + eps^2))
 *   psi(x_i) = sum_j log(1 - x_i.x_j + eps^2) * (-zeta_j A_j) / (4 pi)
 * Without LPM_BVE_COLLOCATED the targets `tgt` are a distinct set (vertices):
 *   replaces BVEVertexVelocity / BVEVertexStreamFn / BVEVertexSolve
 *   (src/LpmBVEKernels.hpp:163-186, :140-161, :110-138).
 * With LPM_BVE_COLLOCATED the targets are the sources themselves (tgt is ignored and
 * may be NULL) and the term i == j is excluded: replaces BVEFaceVelocity /
 * BVEFaceStreamFn / BVEFaceSolve (:285-305, :263-283, :236-261).
 * eps = 0 gives the reference expressions exactly.  u: (n_targets x 3) with strides;
 * psi: n_targets or NULL.  Precision: LPM_BVE_FP64 or LPM_BVE_FP32C. */
int lpm_bve_velocity(lpm_bve_ctx* ctx, const lpm_points* tgt, const lpm_sources* src,
                     double* u, int64_t u_stride_i, int64_t u_stride_c, double* psi,
                     unsigned flags, double eps, lpm_stream_t stream);

/* Same velocity / stream-function sums as lpm_bve_velocity, for callers that cannot
 * allocate device memory (no counterpart in the reference, which always allocates through
 * Kokkos).  It needs no context and never calls cudaMalloc, cudaFree or any allocating
 * library routine: besides the caller's inputs and outputs it uses one file-scope
 * __device__ scratch array (about 18 MiB) that the CUDA runtime places on every device
 * that loads this library and keeps until the process exits.
 *   - Precision: LPM_BVE_FP32C only (other precisions return LPM_ERR_NOT_SUPPORTED).
 *   - Limits: at most 524,288 source faces (masked or not) per call; larger inputs return
 *     LPM_ERR_NOT_SUPPORTED with a message on stderr.  Targets are taken in the caller's order.
 *   - The first call on a device looks up the scratch array's device address; make that
 *     first call before capturing a stream into a CUDA graph.
 *   - Every call on a device shares the one scratch array and leaves its contents behind;
 *     two calls whose kernels can run at the same time (unordered streams) race on it. */
int lpm_bve_velocity_noalloc(const lpm_points* tgt, const lpm_sources* src,
                             double* u, int64_t u_stride_i, int64_t u_stride_c, double* psi,
                             unsigned flags, double eps, lpm_stream_t stream);

/* ---- RK4 stepper ------------------------------------------------------------------ */
typedef struct {
  int64_t nverts, nfaces;                                          /* BVERK4::nverts / nfaces */
  double* vx;    int64_t vx_stride_i, vx_stride_c;                 /* vertex positions (in/out) */
  double* vzeta;                                                   /* vertex relative vorticity (in/out) */
  double* vvel;  int64_t vvel_stride_i, vvel_stride_c;             /* vertex velocity (in: u(x), out) */
  double* fx;    int64_t fx_stride_i, fx_stride_c;                 /* face positions (in/out) */
  double* fzeta;                                                   /* face relative vorticity (in/out) */
  double* fvel;  int64_t fvel_stride_i, fvel_stride_c;             /* face velocity (in: u(x), out) */
  const double* farea;                                             /* face areas (in) */
  const uint8_t* fmask;                                            /* face mask (in), NULL = none */
} lpm_bve_state;

/* Advance `nsteps` RK4 steps of the barotropic vorticity equation in place.
 * Replaces BVERK4::advance_timestep (src/LpmBVERK4.hpp:33-34, src/LpmBVERK4_Impl.hpp:42-130):
 * stage 1 uses the velocity already stored in vvel/fvel; stages 2-4 and the closing
 * re-evaluation are four velocity evaluations per step; dzeta = -2 Omega u_z dt.
 * On return vvel/fvel hold u at the new positions.  The stage workspace belongs to the
 * context (BVERK4::init, src/LpmBVERK4.cpp:5-37). */
int lpm_bve_rk4_step(lpm_bve_ctx* ctx, const lpm_bve_state* st, double dt, double Omega, int nsteps,
                     unsigned flags, double eps, lpm_stream_t stream);

/* Inspection of the last lpm_bve_rk4_step on this context: copies the increments of RK4 stage
 * `stage` (0..3: x_k = dt u_k and zeta_k = -2 Omega u_k,z dt of stages 1..4, the vertx1..4 /
 * facex1..4 and vertvort1..4 / facevort1..4 workspaces of src/LpmBVERK4.hpp:38-63) to HOST
 * arrays in particle order: vx_inc (nverts x 3, row-major), vzeta_inc (nverts), fx_inc
 * (nfaces x 3), fzeta_inc (nfaces); any may be NULL.  Synchronises the stream. */
int lpm_bve_rk4_increments(lpm_bve_ctx* ctx, int stage, double* vx_inc, double* vzeta_inc, double* fx_inc,
                           double* fzeta_inc, lpm_stream_t stream);

/* Relative error norms of ErrNorms::compute (src/LpmErrorNorms.cpp:26-70) between two DEVICE
 * arrays of n entries: ncomp = 3 for vectors (strides as above; magnitudes of the difference and
 * of `exact`), ncomp = 1 for scalars (component strides ignored).  out = {l1, l2, linf} on the
 * host: l1 = sum |e| w / sum |x| w, l2 = sqrt(sum |e|^2 w / sum |x|^2 w), linf = max |e| / max |x|.
 * wt: optional weights (e.g. face areas; NULL = 1); skip: optional byte mask, entries with
 * skip[i] != 0 are left out (e.g. masked parent faces).  For scalars the reference's linf takes
 * the largest signed error and exact value; LPM_NORMS_ABS_LINF uses magnitudes instead.  The sums
 * are reduced in a fixed order (bitwise reproducible).  Synchronises the stream. */
#define LPM_NORMS_ABS_LINF (1u << 0)
int lpm_errnorms(lpm_bve_ctx* ctx, const double* appx, int64_t a_si, int64_t a_sc, const double* exact,
                 int64_t e_si, int64_t e_sc, const double* wt, const uint8_t* skip, int64_t n, int ncomp,
                 unsigned flags, double out[3], lpm_stream_t stream);

/* Velocity tangency diagnostic of SphereVelocityTangentTestFunctor (src/LpmSphereTestKernels.hpp:11-25,
 * run by tests/LpmBVETest.cpp:61-64,160-163): udotx[i] = x_i . u_i for n points of DEVICE arrays
 * (strides as above), FP64, in the order (x0 u0 + x1 u1) + x2 u2 without fused multiply-add.
 * Zero up to rounding for velocities tangent to the sphere.  Stream-ordered; no context. */
int lpm_sphere_tangency(const double* x, int64_t x_si, int64_t x_sc, const double* u, int64_t u_si, int64_t u_sc,
                        int64_t n, double* udotx, lpm_stream_t stream);

/* Tree-code parameters of the context (LPM_BVE_TREECODE): interpolation degree n per chart
 * axis (2..10; (n+1)^2 proxies per cluster), opening parameter theta (0 < theta < 1: a cluster
 * is far from a target tile when r_tile + r_cluster < theta * distance), and the mean sources per
 * octree leaf that set the octree depth, and min_pairs: a solve whose evaluation has fewer target x
 * source pairs keeps the direct sum (the tree's fixed costs exceed its savings below ~1e9 pairs; in
 * an ensemble the small solves share one direct launch).  Defaults 8, 0.6, 512, 1e9. */
int lpm_bve_ctx_set_treecode(lpm_bve_ctx* ctx, int degree, double theta, int leaf_points, double min_pairs);
/* Symmetric leaf kernel (FP32C collocated velocity, RK4 steps, ensembles): plans built afterwards
 * compute each leaf-leaf pair once for solves with at least min_leaves leaf sources (default
 * 65,536: below that its second launch per evaluation costs more than it saves; 0 = every solve).
 * A solve's result does not depend on the batch it runs in; the server uses the default. */
int lpm_bve_ctx_set_symmetric(lpm_bve_ctx* ctx, int64_t min_leaves);
/* Statistics of the context's last tree-code evaluation: octree depth and node count, far-field
 * clusters taken over all tiles, target x source pairs evaluated (direct + proxy), and -- with
 * timing enabled (lpm_bve_ctx_set_timing) -- phase_ms[3] = milliseconds of the octree build, the
 * upward pass and the interaction lists (the pair kernel is reported by lpm_bve_ctx_timing).
 * Any pointer may be NULL. */
int lpm_bve_ctx_tree_stats(lpm_bve_ctx* ctx, int* depth, int64_t* nodes, int64_t* far_clusters, double* pairs,
                           double* direct_pairs, double* far_pairs, double* phase_ms);

/* ---- host-side mesh and initial conditions ------------------------------------------ */
#define LPM_SEED_ICOS_TRI 0 /* IcosTriSphereSeed  (src/LpmMeshSeed.hpp:134-152) */
#define LPM_SEED_CUBED    1 /* CubedSphereSeed    (src/LpmMeshSeed.hpp:113-128) */

/* Sizes of a uniformly refined tree mesh (MeshSeed::setMaxAllocations, src/LpmMeshSeed.cpp:297-305). */
int lpm_mesh_counts(int seed, int level, int64_t* nverts, int64_t* nfaces, int64_t* nleaves);
/* Build the mesh on the host (PolyMesh2d::treeInit, src/LpmPolyMesh2d.cpp:31-44) with the
 * reference's index order.  Host buffers: vx (nverts x 3, row-major), fx (nfaces x 3),
 * farea (nfaces), fmask (nfaces).  Any pointer may be NULL. */
int lpm_mesh_build(int seed, int level, double* vx, double* fx, double* farea, uint8_t* fmask);

/* Face-to-vertex connectivity of the same mesh: face_verts (nfaces x verts_per_face, row-major;
 * 3 for the icosahedral seed, 4 for the cubed sphere) in the order the divisions of
 * src/LpmFaces.cpp:115-382 give the reference's Faces::verts.  Either pointer may be NULL. */
int lpm_mesh_face_verts(int seed, int level, int32_t* face_verts, int* verts_per_face);

/* Host initial conditions on row-major (n x 3) positions.
 * RH54: zeta = 30 cos(4 lambda) P_5^4(z) (src/LpmRossbyWaves.hpp:28-32).
 * Solid body: zeta = 2*(2 pi) z (src/LpmVorticityGallery.hpp:25-40).
 * Gaussians (no reference counterpart): zeta += a_g exp(-(d(x, c_g)/width)^2). */
int lpm_ic_rh54(const double* x, int64_t n, double* zeta);
int lpm_ic_rh54_velocity(const double* x, int64_t n, double* u);
int lpm_ic_solid_body(const double* x, int64_t n, double* zeta);
int lpm_ic_gaussians_add(const double* x, int64_t n, const double* centers, const double* amps, int ng,
                         double width, double* zeta);
/* The same initial vorticity on the DEVICE: zeta[i] = RH54(x_i) + sum_g amps[g] exp(-(d(x_i,
 * c_g)/width)^2) for n device points x (strides as above), written to the device array zeta,
 * queued on `stream` with no allocation.  centers (ng x 3) and amps are HOST arrays, ng <=
 * LPM_IC_MAX_GAUSSIANS.  Products and sums are rounded as in the host functions; cos, atan2 and
 * exp come from CUDA's math library and agree with the host's to a few ulps. */
#define LPM_IC_MAX_GAUSSIANS 64
int lpm_ic_rh54_gaussians_device(const double* x, int64_t n, int64_t stride_i, int64_t stride_c,
                                 const double* centers, const double* amps, int ng, double width, double* zeta,
                                 lpm_stream_t stream);
/* Seeded Gaussian-vortex parameters: centres uniform on the sphere (normalised normal
 * vectors), amplitudes U(amp_lo, amp_hi); std::mt19937_64 with a portable 53-bit uniform. */
int lpm_ic_gaussian_params(uint64_t seed, int ng, double amp_lo, double amp_hi, double* centers, double* amps);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LPM_BVE_H */
