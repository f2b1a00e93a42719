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

static std::atomic<int32_t> g_tune[NTG_TUNE_COUNT] = {{4}};

int32_t tune(int32_t knob) { return g_tune[knob].load(std::memory_order_relaxed); }

}  // namespace ntg

extern "C" const char* ntg_last_error(void) { return ntg::g_last_error.c_str(); }

extern "C" const char* ntg_version(void) { return "nt_gb300 0.1.0 (sm_103a)"; }

extern "C" uint64_t ntg_launch_count(void) {
  return ntg::g_launches.load(std::memory_order_relaxed);
}

extern "C" int ntg_tune_set(int32_t knob, int32_t value) {
  if (knob == NTG_TUNE_STENCIL_RING) {
    if (value != 2 && value != 3 && value != 4 && value != 6)
      return ntg::fail(NTG_ERR_INVALID_ARG, "ntg_tune_set: stencil ring must be 2, 3, 4 or 6");
  } else {
    return ntg::fail(NTG_ERR_INVALID_ARG, "ntg_tune_set: unknown knob");
  }
  ntg::g_tune[knob].store(value, std::memory_order_relaxed);
  return NTG_OK;
}

extern "C" int32_t ntg_tune_get(int32_t knob) {
  if (knob < 0 || knob >= NTG_TUNE_COUNT) return -1;
  return ntg::tune(knob);
}
