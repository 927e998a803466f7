// nvtx.hpp -- named profiler ranges with the reference's region and kernel names.
//
// pbosler/lpmKokkos brackets BVERK4::advance_timestep with Kokkos::Profiling::pushRegion /
// popRegion and names every launch of the step ("RK4-2 vertex velocity", "RK4 face update",
// ...; src/LpmBVERK4_Impl.hpp:45-129).  The same names are pushed here as NVTX ranges around the
// host calls that enqueue the corresponding work, so a profiler timeline (nsys, or ncu with
// --nvtx filters) groups this library's kernels under them.  The ranges mark enqueue time on the
// host: a step replayed from its captured CUDA graph shows only the outer advance_timestep range
// (the per-launch ranges appear when steps launch directly: LPM_BVE_NO_GRAPH, pair timing on, or
// the tree code).  NVTX v3 is header-only; with no tool attached a range costs a branch.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace lpm {

struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// The names of one velocity evaluation's three launches: stage input (the reference's
// KokkosBlas::update of x + c x_k, zeta + c zeta_k), the fused vertex + face direct sums, and the
// fused vorticity tendency / increments (BVEVorticityTendency and KokkosBlas::scal).
struct EvalNames {
  const char* prep;
  const char* pair;
  const char* epilogue;
};

}  // namespace lpm
