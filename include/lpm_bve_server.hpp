// lpm_bve_server.hpp -- C++ wrapper of the continuous-batching solve server
// (include/lpm_bve_server.h): RAII ownership, exceptions instead of status codes, results in
// std::vector.  Header-only; link liblpm_bve.so.
#pragma once

#include "lpm_bve_server.h"

#include <stdexcept>
#include <string>
#include <vector>

namespace lpm {

struct SolveResult {
  int64_t nverts = 0, nfaces = 0;
  std::vector<double> vx, vzeta, vvel, fx, fzeta, fvel;  // row-major, n x 3 for vectors
};

class SolveServer {
 public:
  explicit SolveServer(unsigned flags = LPM_BVE_FP32C, size_t hbmBudgetBytes = 0, int device = -1,
                       int maxActive = 0, double eps = 0.0, bool hostInitialCondition = false) {
    lpm_bve_server_opts o{};
    o.device = device;
    o.hbm_budget_bytes = hbmBudgetBytes;
    o.max_active = maxActive;
    o.flags = flags;
    o.eps = eps;
    o.host_ic = hostInitialCondition ? 1 : 0;
    const int rc = lpm_bve_server_create(&o, &s_);
    if (rc != LPM_OK) throw std::runtime_error("lpm_bve_server_create failed: status " + std::to_string(rc));
  }
  ~SolveServer() {
    if (s_) lpm_bve_server_destroy(s_);
  }
  SolveServer(const SolveServer&) = delete;
  SolveServer& operator=(const SolveServer&) = delete;

  int64_t submit(const lpm_bve_request& r) {
    int64_t id = 0;
    check(lpm_bve_server_submit(s_, &r, &id));
    return id;
  }
  // True when done, false on timeout; throws if the request failed or was cancelled.
  bool wait(int64_t id, double timeoutSeconds = -1.0) {
    const int rc = lpm_bve_server_wait(s_, id, timeoutSeconds);
    if (rc == LPM_ERR_TIMEOUT) return false;
    check(rc);
    return true;
  }
  SolveResult result(int64_t id) {
    SolveResult out;
    check(lpm_bve_server_result(s_, id, &out.nverts, &out.nfaces, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr));
    out.vx.resize(3 * out.nverts);
    out.vzeta.resize(out.nverts);
    out.vvel.resize(3 * out.nverts);
    out.fx.resize(3 * out.nfaces);
    out.fzeta.resize(out.nfaces);
    out.fvel.resize(3 * out.nfaces);
    check(lpm_bve_server_result(s_, id, nullptr, nullptr, out.vx.data(), out.vzeta.data(), out.vvel.data(),
                                out.fx.data(), out.fzeta.data(), out.fvel.data()));
    return out;
  }
  void snapshot(int64_t id, const std::string& path) { check(lpm_bve_server_snapshot(s_, id, path.c_str())); }
  void release(int64_t id) { check(lpm_bve_server_release(s_, id)); }
  // Seconds: submit to done, before the first step, running.
  void timing(int64_t id, double& total, double& wait, double& run) {
    check(lpm_bve_server_timing(s_, id, &total, &wait, &run));
  }
  std::vector<double> latency(const std::vector<double>& quantiles) {
    std::vector<double> out(quantiles.size());
    check(lpm_bve_server_latency(s_, quantiles.data(), (int)quantiles.size(), out.data()));
    return out;
  }
  lpm_bve_server_counters stats() {
    lpm_bve_server_counters c{};
    check(lpm_bve_server_stats(s_, &c));
    return c;
  }
  lpm_bve_server* handle() const { return s_; }

 private:
  void check(int rc) {
    if (rc != LPM_OK) throw std::runtime_error(std::string("lpm_bve_server: ") + lpm_bve_server_last_error(s_));
  }
  lpm_bve_server* s_ = nullptr;
};

}  // namespace lpm
