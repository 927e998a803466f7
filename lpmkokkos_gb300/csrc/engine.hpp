// engine.hpp -- internal data layout shared by the BVE kernels and the host engine.
//
// One evaluation of the direct sum is organised as:
//   prep      (O(N))  : stage positions x + c*k in FP64, packed source records,
//   pair      (O(N^2)): persistent CTAs pull work items (target tile x source chunk)
//                       and write one partial sum per (chunk, target),
//   epilogue  (O(N))  : fixed-order sum of the partials, FP64 cross product,
//                       velocity written to the caller's arrays, RK4 stage increments.
// Targets live in "slots": a spatially sorted permutation of the caller's vertices and
// faces, so that each target tile is compact on the sphere.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lpm {

constexpr double kPi = 3.1415926535897932384626433832795027975;

// A caller-owned FP64 vector array: element (i, c) at p[i*si + c*sc].
struct DVec {
  double* p = nullptr;
  int64_t si = 0, sc = 0;
};

// The particles of one solve as the caller sees them.  "a" particles are targets only
// (vertices, or the target points of a distinct-set call); "b" particles are faces:
// sources when unmasked, and targets too when they appear in the slot list.
struct ParticleIO {
  int64_t na = 0, nb = 0;
  DVec ax, au;                 // positions / velocity output of the a-particles
  double* azeta = nullptr;     // a-particle vorticity (RK4: integrated, not a source)
  double* apsi = nullptr;      // stream function output (a)
  DVec bx, bu;                 // positions / velocity output of the b-particles
  double* bzeta = nullptr;     // b-particle (source) vorticity
  double* bpsi = nullptr;
  const double* barea = nullptr;
};

// Pair-kernel work item: one target tile against one contiguous source chunk.  In the
// symmetric leaf kernel (pairFP32CSym) `tile` is a leaf tile I and [s0, s1) a range of leaf
// tiles J >= I.
struct WorkItem {
  int solve;     // index into the SolveDev table
  int tile;      // target tile within the solve
  int s0, s1;    // source range [s0, s1) within the solve
  int chunk;     // partial-sum slot (chunk index within the tile's row)
  int tend;      // the tile's target slots are [tbeg, min(tbeg + tile size, tend))
  int tbeg;
  int pad;
};

// Symmetric leaf x leaf evaluation: leaf tiles of kSymTile slots (128 threads x 8 targets),
// reverse sums accumulated in 64-bit fixed point with kSymScale units per 1 (exact, order-free
// integer adds; a per-source flag marks contributions that are not finite or not below
// kSymLimit, and the epilogue turns the source's result into NaN).
constexpr int kSymThreads = 128;
constexpr int kSymK = 8;
constexpr int kSymTile = kSymThreads * kSymK;
constexpr double kSymScale = 1099511627776.0;  // 2^40
constexpr double kSymLimit = 1048576.0;        // 2^20

// Device-side description of one solve for the pair kernels.
struct SolveDev {
  const double* tx;          // [3][nslots] stage positions of the target slots (SoA)
  const float4* sp0;         // [ns] FP32C: (x_hi, y_hi, z_hi, w = -zeta*A/(2 pi))
  const float4* sp1;         // [ns] FP32C: (x_lo, y_lo, z_lo, D = 1 - |x|^2)
  const double4_32a* sd;         // [ns] FP64 : (x, y, z, -zeta*A)
  const int* self;           // [nslots] source index of the same particle, -1 if none
  const int2* tileSelf;      // [ntiles] min/max self index of the tile (INT_MAX,-1 if none)
  const int* tileCentre;     // [ntiles] slot of the tile's centre target (a vertex or leaf face)
  double* partial;           // [nchunks][ncomp][nslots]
  int nslots, ns, tileSize, nchunks;
  double eps2;
  // symmetric layout: slots [leaf0, nslots) are the leaf sources 0..ns-1 in source order
  // (leaf0 = -1: no such layout); reverse sums of the symmetric leaf kernel
  int leaf0;
  unsigned long long* rev;   // [4][ns] fixed point: velocity, stream function
  int* revBad;               // [ns]
};

// Per-solve parameters for the O(N) kernels.
struct SolveStage {
  ParticleIO io;
  const int* perm;           // [nslots] slot -> particle id (id < na: a-particle, else face id - na)
  const int* srcFace;        // [ns] source -> face index
  const int* srcSlot;        // [ns] source -> slot of the same face (-1 if the face is not a target)
  double* tx;                // [3][nslots]
  float4* sp0; float4* sp1; double4_32a* sd;
  double* kx[4];             // [3][nslots] RK4 position increments x_k = dt*u
  double* kz[4];             // [nslots]    RK4 vorticity increments
  const double* partial;     // [nchunks][ncomp][nslots]
  int nslots, ns, nchunks;
  double dt, omega;
  int leaf0;                 // symmetric layout: first leaf slot (-1: none)
  unsigned long long* rev;   // [4][ns] fixed-point reverse sums (zeroed by prep), or null
  int* revBad;               // [ns]
};

// Launch-shape of the FP32C pair kernel.
struct PairShape {
  int threads;    // CTA size
  int k;          // targets per thread
  int srcTile;    // sources staged in shared memory per step
  int minBlocks;  // resident CTAs per SM the register budget is sized for (1 = compiler's choice)
  int tileSize() const { return threads * k; }
  bool operator==(const PairShape& o) const {
    return threads == o.threads && k == o.k && srcTile == o.srcTile && minBlocks == o.minBlocks;
  }
};

enum class Precision { FP64 = 0, FP32C = 1 };

// ---- kernel launchers (pair_kernels.cu / stage_kernels.cu) ----------------------------
// The O(N) kernels walk a block map of int4 {solve, first index, kind, 0}; kind 0 = target
// slots, kind 1 = source records (prep only).
// prep stage: 0 = plain evaluation at x, 1 = RK4 stage-2 inputs (x + x_1/2 with x_1 = dt*u
// from the stored velocity), 2 = stage-3 inputs (x + x_2/2), 3 = stage-4 inputs (x + x_3).
cudaError_t launchPrep(const SolveStage* st, const int4* map, int nblocks, int stage, Precision prec, int* counter,
                       cudaStream_t s);
// stageOut: 0 = no increments, 1..3 = write x_k/zeta_k of RK4 stage k+1.  useRev: add the
// symmetric kernel's reverse sums to the leaf slots.
cudaError_t launchEpilogue(const SolveStage* st, const int4* map, int nblocks, Precision prec, bool psi,
                           bool velocity, int stageOut, cudaStream_t s, bool useRev = false);
cudaError_t launchCombine(const SolveStage* st, const int4* map, int nblocks, bool quirk, bool renorm,
                          cudaStream_t s);
// precise: FP32C with hi/lo target-source differences (arbitrary distinct targets).
// rcpApprox: FP32C fast formulation without the Newton step on the reciprocal.
cudaError_t launchPair(Precision prec, const PairShape& shape, bool psi, bool precise, bool rcpApprox,
                       const SolveDev* solves, const WorkItem* items, int nitems, int* counter, int grid,
                       cudaStream_t s);
// Symmetric leaf x leaf kernel over `items` (see WorkItem), with or without the stream
// function; grid = resident CTAs.
cudaError_t launchPairSym(bool psi, bool rcpApprox, const SolveDev* solves, const WorkItem* items, int nitems,
                          int* counter, int grid, cudaStream_t s);
int pairSymBlocksPerSM(bool psi);
int pairShapeCount();              // FP32C launch shapes compiled in
PairShape pairShapeAt(int i);
int stageBlockSize();

// Relative error norms (norms.cu): appx/exact strided arrays of n entries of ncomp (1 or 3)
// components, optional weights and skip mask; out (device) = {l1, l2, linf}.
struct NormArgs {
  const double* appx;
  int64_t a_si, a_sc;
  const double* exact;
  int64_t e_si, e_sc;
  const double* wt;
  const uint8_t* skip;
  int64_t n;
  int ncomp;
  int signedLinf;
};
int normBlocks(int sms);
cudaError_t launchNorms(const NormArgs& a, double* partial, int nblocks, double* out, cudaStream_t s);
int pairBlocksPerSM(Precision prec, const PairShape& shape, bool psi);
bool pairShapeSupported(Precision prec, const PairShape& shape);
int pairNumComponents(Precision prec, bool psi);  // partial-sum components per (chunk, slot)

}  // namespace lpm
