// lpm_bve.hpp -- C++ drop-in for the BVE classes of pbosler/lpmKokkos over the C ABI.
//
// Keeps the host interface of the reference so a caller's time loop compiles unchanged:
//   BVERK4(dt, Omega); init(nv, nf);
//   advance_timestep(vx, vzeta, vvel, fx, fzeta, fvel, fa, fm)   (src/LpmBVERK4.hpp:13-65)
//   BVESphere<Seed>(nmaxverts, nmaxedges, nmaxfaces); treeInit(depth); set_omega(w);
//   init_vorticity(ic)                                            (src/LpmBVESphere.hpp:18-80)
// With LPM_BVE_WITH_KOKKOS defined the view types are the reference's Kokkos::View typedefs
// and only their data(), extent(0) and stride(0/1) are used.  Without Kokkos, lpm::View is
// a small reference-counted device array with the same accessors (LayoutLeft by default,
// like View<double*[3]> on CUDA).
#pragma once

#include "lpm_bve.h"

#include <cuda_runtime.h>

#include <cmath>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef LPM_BVE_WITH_KOKKOS
#include "Kokkos_Core.hpp"
#endif

namespace lpm {

typedef double Real;
typedef int Index;

inline void throwIf(int rc, const lpm_bve_ctx* ctx, const char* what) {
  if (rc != LPM_OK)
    throw std::runtime_error(std::string(what) + ": " + (ctx ? lpm_bve_last_error(ctx) : "invalid argument"));
}
inline void cudaCheck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

#ifdef LPM_BVE_WITH_KOKKOS
typedef Kokkos::View<Real*[3]> crd_view;
typedef Kokkos::View<Real*[3]> vec_view;
typedef Kokkos::View<Real*> scalar_view_type;
typedef Kokkos::View<bool*> mask_view_type;
#else
// Device array of n rows of NC components; element (i, c) at data()[i*stride(0) + c*stride(1)].
template <typename T, int NC>
class View {
 public:
  View() = default;
  explicit View(const std::string& label, int64_t n, bool layoutLeft = true) : label_(label), n_(n) {
    T* p = nullptr;
    if (n > 0) cudaCheck(cudaMalloc(&p, sizeof(T) * n * NC), "cudaMalloc");
    if (p) cudaCheck(cudaMemset(p, 0, sizeof(T) * n * NC), "cudaMemset");
    buf_ = std::shared_ptr<T>(p, [](T* q) { if (q) cudaFree(q); });
    si_ = (NC == 1 || !layoutLeft) ? NC : 1;
    sc_ = (NC == 1) ? 1 : (layoutLeft ? n : 1);
  }
  T* data() const { return buf_.get(); }
  int64_t extent(int d) const { return d == 0 ? n_ : NC; }
  int64_t stride(int d) const { return d == 0 ? si_ : sc_; }
  const std::string& label() const { return label_; }
  // Host <-> device copies of a row-major (n x NC) host array.
  void fromHost(const std::vector<T>& h) const {
    std::vector<T> tmp(n_ * NC);
    for (int64_t i = 0; i < n_; ++i)
      for (int c = 0; c < NC; ++c) tmp[i * si_ + c * sc_] = h[i * NC + c];
    if (n_) cudaCheck(cudaMemcpy(data(), tmp.data(), sizeof(T) * n_ * NC, cudaMemcpyHostToDevice), "H2D");
  }
  std::vector<T> toHost() const {
    std::vector<T> tmp(n_ * NC), h(n_ * NC);
    if (n_) cudaCheck(cudaMemcpy(tmp.data(), data(), sizeof(T) * n_ * NC, cudaMemcpyDeviceToHost), "D2H");
    for (int64_t i = 0; i < n_; ++i)
      for (int c = 0; c < NC; ++c) h[i * NC + c] = tmp[i * si_ + c * sc_];
    return h;
  }

 private:
  std::string label_;
  std::shared_ptr<T> buf_;
  int64_t n_ = 0, si_ = NC, sc_ = 1;
};
typedef View<Real, 3> crd_view;
typedef View<Real, 3> vec_view;
typedef View<Real, 1> scalar_view_type;
typedef View<bool, 1> mask_view_type;
#endif

// One context per host thread; shared by the classes below.
inline lpm_bve_ctx* defaultContext() {
  thread_local std::unique_ptr<lpm_bve_ctx, int (*)(lpm_bve_ctx*)> ctx(nullptr, lpm_bve_ctx_destroy);
  if (!ctx) {
    lpm_bve_ctx* c = nullptr;
    lpm_bve_opts o{-1, 0, 0};
    throwIf(lpm_bve_ctx_create(&c, &o), nullptr, "lpm_bve_ctx_create");
    ctx.reset(c);
  }
  return ctx.get();
}

// BVERK4 (src/LpmBVERK4.hpp:13-65).  `flags` selects precision and RK4 options
// (LPM_BVE_FP64 = the reference arithmetic; LPM_BVE_FP32C = FP32-compensated pairs).
class BVERK4 {
 public:
  crd_view vertx;
  scalar_view_type vertvort;
  vec_view vertvel;
  crd_view facex;
  scalar_view_type facevort;
  vec_view facevel;
  Real dt;
  Real Omega;
  Index nverts;
  Index nfaces;

  BVERK4(const Real& timestep, const Real& omg, unsigned flags = LPM_BVE_FP64, double eps = 0.0,
         cudaStream_t stream = nullptr)
      : dt(timestep), Omega(omg), nverts(0), nfaces(0), flags_(flags), eps_(eps), stream_(stream) {}

  // Stage workspace lives in the context and grows on first use (BVERK4::init,
  // src/LpmBVERK4.cpp:5-37); init records the sizes advance_timestep will check.
  void init(const Index& nv, const Index& nf) {
    nverts = nv;
    nfaces = nf;
  }

  void advance_timestep(crd_view& vx, scalar_view_type& vzeta, vec_view& vvel, crd_view& fx,
                        scalar_view_type& fzeta, vec_view& fvel, const scalar_view_type& fa,
                        const mask_view_type& fm) {
    if ((Index)vx.extent(0) != nverts || (Index)fx.extent(0) != nfaces)
      throw std::invalid_argument("BVERK4::advance_timestep: view sizes differ from init(nv, nf)");
    vertx = vx; vertvort = vzeta; vertvel = vvel; facex = fx; facevort = fzeta; facevel = fvel;
    lpm_bve_state st{};
    st.nverts = nverts;
    st.nfaces = nfaces;
    st.vx = vx.data(); st.vx_stride_i = vx.stride(0); st.vx_stride_c = vx.stride(1);
    st.vzeta = vzeta.data();
    st.vvel = vvel.data(); st.vvel_stride_i = vvel.stride(0); st.vvel_stride_c = vvel.stride(1);
    st.fx = fx.data(); st.fx_stride_i = fx.stride(0); st.fx_stride_c = fx.stride(1);
    st.fzeta = fzeta.data();
    st.fvel = fvel.data(); st.fvel_stride_i = fvel.stride(0); st.fvel_stride_c = fvel.stride(1);
    st.farea = fa.data();
    st.fmask = reinterpret_cast<const uint8_t*>(fm.data());
    lpm_bve_ctx* ctx = defaultContext();
    throwIf(lpm_bve_rk4_step(ctx, &st, dt, Omega, 1, flags_, eps_, (lpm_stream_t)stream_), ctx,
            "BVERK4::advance_timestep");
  }

 private:
  unsigned flags_;
  double eps_;
  cudaStream_t stream_;
};

#ifndef LPM_BVE_WITH_KOKKOS
struct IcosTriSphereSeed { static constexpr int id = LPM_SEED_ICOS_TRI; };
struct CubedSphereSeed { static constexpr int id = LPM_SEED_CUBED; };

// Relative-vorticity initial condition (VorticityInitialCondition, src/LpmVorticityGallery.hpp:13-23).
typedef std::function<Real(Real, Real, Real)> VorticityFn;

// BVESphere<Seed> (src/LpmBVESphere.hpp:18-80): the mesh (built on the host with the
// reference's index order), its particle fields on the device, and the initial solve.
template <typename SeedType>
class BVESphere {
 public:
  crd_view vertCrds, faceCrds, lagVertCrds, lagFaceCrds;
  scalar_view_type relVortVerts, absVortVerts, streamFnVerts;
  vec_view velocityVerts;
  scalar_view_type relVortFaces, absVortFaces, streamFnFaces;
  vec_view velocityFaces;
  scalar_view_type faceArea;
  mask_view_type faceMask;
  Real Omega = 2 * 3.1415926535897932384626433832795027975;
  Real t = 0;

  // Builds the uniformly refined mesh of depth `depth` (PolyMesh2d::treeInit).
  explicit BVESphere(int depth) : depth_(depth) {
    int64_t nv, nf, nl;
    throwIf(lpm_mesh_counts(SeedType::id, depth, &nv, &nf, &nl), nullptr, "lpm_mesh_counts");
    hvx_.resize(3 * nv); hfx_.resize(3 * nf); harea_.resize(nf);
    std::vector<uint8_t> hm(nf);
    throwIf(lpm_mesh_build(SeedType::id, depth, hvx_.data(), hfx_.data(), harea_.data(), hm.data()), nullptr,
            "lpm_mesh_build");
    nverts_ = nv; nfaces_ = nf; nleaves_ = nl;
    vertCrds = crd_view("vertCrds", nv); vertCrds.fromHost(hvx_);
    faceCrds = crd_view("faceCrds", nf); faceCrds.fromHost(hfx_);
    lagVertCrds = crd_view("lagVertCrds", nv); lagVertCrds.fromHost(hvx_);
    lagFaceCrds = crd_view("lagFaceCrds", nf); lagFaceCrds.fromHost(hfx_);
    relVortVerts = scalar_view_type("relVortVerts", nv); absVortVerts = scalar_view_type("absVortVerts", nv);
    streamFnVerts = scalar_view_type("streamFnVerts", nv); velocityVerts = vec_view("velocityVerts", nv);
    relVortFaces = scalar_view_type("relVortFaces", nf); absVortFaces = scalar_view_type("absVortFaces", nf);
    streamFnFaces = scalar_view_type("streamFnFaces", nf); velocityFaces = vec_view("velocityFaces", nf);
    faceArea = scalar_view_type("area", nf); faceArea.fromHost(harea_);
    faceMask = mask_view_type("mask", nf);
    static_assert(sizeof(bool) == 1, "mask views hold one byte per face");
    cudaCheck(cudaMemcpy(faceMask.data(), hm.data(), nf, cudaMemcpyHostToDevice), "mask H2D");
  }

  Index nvertsHost() const { return (Index)nverts_; }
  Index nfacesHost() const { return (Index)nfaces_; }
  Index nleavesHost() const { return (Index)nleaves_; }
  Real avg_mesh_size_radians() const { return std::sqrt(4 * 3.1415926535897932384626433832795027975 / nfaces_); }
  void set_omega(const Real& omg) { Omega = omg; }
  const std::vector<Real>& hostVertCrds() const { return hvx_; }
  const std::vector<Real>& hostFaceCrds() const { return hfx_; }

  // Host IC evaluation, then stream function and velocity at vertices and faces
  // (BVESphere::init_vorticity, src/LpmBVESphere.cpp:127-169).
  void init_vorticity(const VorticityFn& relvort, unsigned flags = LPM_BVE_FP64, double eps = 0.0) {
    std::vector<Real> zv(nverts_), av(nverts_), zf(nfaces_), af(nfaces_);
    for (int64_t i = 0; i < nverts_; ++i) {
      zv[i] = relvort(hvx_[3 * i], hvx_[3 * i + 1], hvx_[3 * i + 2]);
      av[i] = zv[i] + 2 * Omega * hvx_[3 * i + 2];
    }
    for (int64_t i = 0; i < nfaces_; ++i) {
      zf[i] = relvort(hfx_[3 * i], hfx_[3 * i + 1], hfx_[3 * i + 2]);
      af[i] = zf[i] + 2 * Omega * hfx_[3 * i + 2];
    }
    relVortVerts.fromHost(zv); absVortVerts.fromHost(av); relVortFaces.fromHost(zf); absVortFaces.fromHost(af);
    solve(flags | LPM_BVE_PSI, eps);
  }

  // Velocity (and stream function with LPM_BVE_PSI) at every vertex and face.
  void solve(unsigned flags, double eps = 0.0) {
    lpm_bve_ctx* ctx = defaultContext();
    lpm_sources src{{faceCrds.data(), nfaces_, faceCrds.stride(0), faceCrds.stride(1)}, relVortFaces.data(),
                    faceArea.data(), reinterpret_cast<const uint8_t*>(faceMask.data())};
    lpm_points tv{vertCrds.data(), nverts_, vertCrds.stride(0), vertCrds.stride(1)};
    const bool psi = flags & LPM_BVE_PSI;
    // Vertices are mesh points: they keep about half a mesh spacing from every source.
    throwIf(lpm_bve_velocity(ctx, &tv, &src, velocityVerts.data(), velocityVerts.stride(0), velocityVerts.stride(1),
                             psi ? streamFnVerts.data() : nullptr, flags | LPM_BVE_MESH_TARGETS, eps, nullptr),
            ctx, "vertex solve");
    throwIf(lpm_bve_velocity(ctx, nullptr, &src, velocityFaces.data(), velocityFaces.stride(0),
                             velocityFaces.stride(1), psi ? streamFnFaces.data() : nullptr,
                             flags | LPM_BVE_COLLOCATED, eps, nullptr), ctx, "face solve");
  }

 private:
  int depth_;
  int64_t nverts_ = 0, nfaces_ = 0, nleaves_ = 0;
  std::vector<Real> hvx_, hfx_, harea_;
};
#endif

}  // namespace lpm

// The reference's namespace, so reference-shaped driver code compiles unchanged.
namespace Lpm = lpm;
