// Library-level plumbing of the C ABI: per-thread error messages, version,
// and the launch counter reported by ntg_launch_count().
#include <cstdio>
#include <string>

#include "ntg_common.cuh"

namespace ntg {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    return fail(NTG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
  return NTG_OK;
}

void note_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace ntg

extern "C" const char* ntg_last_error(void) { return ntg::g_last_error.c_str(); }

extern "C" const char* ntg_version(void) { return "nt_gb300 0.1.0 (sm_103a)"; }

extern "C" uint64_t ntg_launch_count(void) {
  return ntg::g_launches.load(std::memory_order_relaxed);
}
