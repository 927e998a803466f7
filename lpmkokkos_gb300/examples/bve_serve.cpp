// bve_serve.cpp -- a C++ client of the solve server (include/lpm_bve_server.hpp).
//
// Submits a stream of BVE requests -- icosahedral / cubed-sphere meshes of levels 3-5 in
// turn, RH54 plus seeded Gaussian vortices, dt at the level-4 Courant number -- a few
// milliseconds apart, so that they overlap on the GPU, waits for all of them, prints one line
// per request (id, seed, level, submit-to-result latency) and the p50 / p99 latency, and with
// -o writes each final state as a snapshot file <prefix><k>.snap.
//
//   bve_serve [-n requests] [-steps steps] [-fp64] [-o prefix]

#include "lpm_bve_server.hpp"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

int main(int argc, char* argv[]) {
  int n = 6, steps = 4;
  unsigned flags = LPM_BVE_FP32C;
  std::string prefix;
  for (int i = 1; i < argc; ++i) {
    const std::string tok = argv[i];
    if (tok == "-n" && i + 1 < argc) n = std::atoi(argv[++i]);
    else if (tok == "-steps" && i + 1 < argc) steps = std::atoi(argv[++i]);
    else if (tok == "-o" && i + 1 < argc) prefix = argv[++i];
    else if (tok == "-fp64") flags = LPM_BVE_FP64;
  }
  try {
    const double PI = 3.1415926535897932384626433832795027975;
    lpm::SolveServer server(flags);
    std::vector<lpm_bve_request> reqs;
    std::vector<int64_t> ids;
    for (int k = 0; k < n; ++k) {
      lpm_bve_request r{};
      r.seed = k % 2 == 0 ? LPM_SEED_ICOS_TRI : LPM_SEED_CUBED;
      r.level = 3 + (k / 2) % 3;
      r.ic_seed = 1000 + k;
      r.n_gaussians = 3;
      r.gauss_width = 0.1;
      r.dt = 0.01 * std::pow(2.0, 4 - r.level);
      r.omega = 2 * PI;
      r.nsteps = steps;
      reqs.push_back(r);
      ids.push_back(server.submit(r));
      std::this_thread::sleep_for(std::chrono::milliseconds(2));
    }
    for (size_t k = 0; k < ids.size(); ++k) {
      if (!server.wait(ids[k], 600.0)) throw std::runtime_error("request timed out");
      double total = 0, wait = 0, run = 0;
      server.timing(ids[k], total, wait, run);
      std::printf("request %lld seed %d level %d latency %.6f s\n", (long long)ids[k], reqs[k].seed, reqs[k].level,
                  total);
      if (!prefix.empty()) server.snapshot(ids[k], prefix + std::to_string(k) + ".snap");
    }
    const std::vector<double> q = server.latency({0.5, 0.99});
    const lpm_bve_server_counters st = server.stats();
    std::printf("p50 %.6f s p99 %.6f s completed %lld max_running %d\n", q[0], q[1], (long long)st.completed,
                st.max_running_seen);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "bve_serve: %s\n", e.what());
    return 1;
  }
  return 0;
}
