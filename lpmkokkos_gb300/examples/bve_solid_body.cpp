// bve_solid_body.cpp -- the reference's BVE driver (tests/LpmBVETest.cpp:35-270) written
// against the drop-in classes of include/lpm_bve.hpp.
//
// Solid-body rotation on the cubed sphere: relative vorticity 2*(2 pi)*z with the
// background rotation set to 0, stepped with BVERK4(dt, 2 pi) to t = tf.  Prints the
// area-weighted velocity and position errors at the leaf faces against the exact rigid
// rotation, as the reference driver does, and optionally writes the final face positions.
//
//   bve_solid_body [-d depth] [-dt dt] [-tf tfinal] [-fp32c] [-o positions.bin]

#include "lpm_bve.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace Lpm;

int main(int argc, char* argv[]) {
  int depth = 3;
  double dt = 0.01, tfinal = 1.0;
  unsigned flags = LPM_BVE_FP64;
  std::string out;
  for (int i = 1; i < argc; ++i) {
    const std::string tok = argv[i];
    if (tok == "-d" && i + 1 < argc) depth = std::atoi(argv[++i]);
    else if (tok == "-dt" && i + 1 < argc) dt = std::atof(argv[++i]);
    else if (tok == "-tf" && i + 1 < argc) tfinal = std::atof(argv[++i]);
    else if (tok == "-o" && i + 1 < argc) out = argv[++i];
    else if (tok == "-fp32c") flags = LPM_BVE_FP32C;
  }
  try {
    const double PI = 3.1415926535897932384626433832795027975;
    const double Omega = 2 * PI;
    BVESphere<CubedSphereSeed> sphere(depth);
    sphere.set_omega(0);
    sphere.init_vorticity([&](Real, Real, Real z) { return 2 * Omega * z; }, flags);

    const int ntimesteps = (int)std::floor(tfinal / dt);
    dt = tfinal / ntimesteps;
    BVERK4 solver(dt, Omega, flags);
    solver.init(sphere.nvertsHost(), sphere.nfacesHost());
    for (int k = 0; k < ntimesteps; ++k) {
      solver.advance_timestep(sphere.vertCrds, sphere.relVortVerts, sphere.velocityVerts, sphere.faceCrds,
                              sphere.relVortFaces, sphere.velocityFaces, sphere.faceArea, sphere.faceMask);
      sphere.t = (k + 1) * dt;
    }
    cudaCheck(cudaDeviceSynchronize(), "sync");

    const std::vector<Real> x = sphere.faceCrds.toHost();
    const std::vector<Real> u = sphere.velocityFaces.toHost();
    const std::vector<Real> a = sphere.faceArea.toHost();
    const std::vector<Real>& x0 = sphere.hostFaceCrds();
    const double c = std::cos(Omega * sphere.t), s = std::sin(Omega * sphere.t);
    double un = 0, ud = 0, xn = 0, xd = 0;
    std::vector<double> leafx;
    for (int i = 0; i < sphere.nfacesHost(); ++i) {
      if (a[i] == 0.0) continue;  // masked parent
      const double ue[3] = {-Omega * x[3 * i + 1], Omega * x[3 * i], 0.0};
      const double xe[3] = {x0[3 * i] * c - x0[3 * i + 1] * s, x0[3 * i + 1] * c + x0[3 * i] * s, x0[3 * i + 2]};
      for (int k = 0; k < 3; ++k) {
        un += a[i] * (u[3 * i + k] - ue[k]) * (u[3 * i + k] - ue[k]);
        ud += a[i] * ue[k] * ue[k];
        xn += a[i] * (x[3 * i + k] - xe[k]) * (x[3 * i + k] - xe[k]);
        xd += a[i] * xe[k] * xe[k];
        leafx.push_back(x[3 * i + k]);
      }
    }
    std::printf("solid body rotation: cubed sphere depth %d, %d steps of dt %g, %s\n", depth, ntimesteps, dt,
                flags == LPM_BVE_FP32C ? "FP32C" : "FP64");
    std::printf("velocity error at t=tfinal ErrNorms: l2 = %.6e\n", std::sqrt(un / ud));
    std::printf("position error at t=tfinal ErrNorms: l2 = %.6e\n", std::sqrt(xn / xd));
    if (!out.empty()) {
      FILE* f = std::fopen(out.c_str(), "wb");
      if (!f) { std::perror("fopen"); return 2; }
      std::fwrite(leafx.data(), sizeof(double), leafx.size(), f);
      std::fclose(f);
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  std::printf("tests pass\n");
  return 0;
}
