// Allocation-free variant of ntg_chol_solve.
//
// Some callers cannot allocate device memory at the point where they need the
// kernel-regression solve: an XLA FFI handler (XLA owns device memory and
// hands the handler only its operand and result buffers), a serving process that reserves
// all device memory up front, or a host runtime whose allocator is not
// reachable from the call site. ntg_chol_solve_noalloc takes the refinement
// workspace from a fixed device array owned by this library instead of a
// caller-provided buffer; the caller still passes every input and output.
#include <mutex>
#include <string>

#include "ntg_common.cuh"

namespace {

// The scratch every call shares. Each GPU that loads this library keeps it
// (NTG_NOALLOC_SCRATCH_BYTES) until the process exits.
static __device__ __align__(256) unsigned char g_solve_scratch[NTG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_solve_scratch on the current device. In host code the
// array's name only stands in for the symbol, so the address is looked up
// once per device (with that device current) and cached.
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return ntg::fail(NTG_ERR_CUDA, std::string("ntg_chol_solve_noalloc: cudaGetDevice: ") +
                                       cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return ntg::fail(NTG_ERR_UNSUPPORTED, "ntg_chol_solve_noalloc: device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_solve_scratch);
    if (e != cudaSuccess || !p)
      return ntg::fail(NTG_ERR_NO_DEVICE_SCRATCH,
                       std::string("ntg_chol_solve_noalloc: cudaGetSymbolAddress: ") +
                           cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return NTG_OK;
}

}  // namespace

extern "C" int ntg_chol_solve_noalloc(void* stream, const float* A, const float* L,
                                      const double* lambda, int64_t n, const float* B, int64_t m,
                                      float* X, int32_t refine_iters, double* final_residual) {
  NTG_REQUIRE(n > 0 && m > 0, "ntg_chol_solve_noalloc: sizes must be positive");
  // Bound n and m before any product is formed, so no size can wrap past the
  // check below: n at the factorisation's own limit, n * m at what the fixed
  // array can hold (12 bytes per entry after a 256-byte header).
  constexpr int64_t kMaxEntries = ((int64_t)NTG_NOALLOC_SCRATCH_BYTES - 256) / 12;
  if (n > 46340 || m > kMaxEntries / n)
    return ntg::fail(NTG_ERR_INVALID_ARG,
                     "ntg_chol_solve_noalloc: n * m too large for the fixed scratch (n * m "
                     "must be at most " + std::to_string(kMaxEntries) +
                     " with n <= 46340); use ntg_chol_solve with a workspace");
  const size_t need = ntg_chol_workspace_bytes(n, m);
  if (need > (size_t)NTG_NOALLOC_SCRATCH_BYTES)
    return ntg::fail(NTG_ERR_INVALID_ARG,
                     "ntg_chol_solve_noalloc: n * m too large for the fixed scratch (needs " +
                         std::to_string(need) + " bytes, the maximum is " +
                         std::to_string((size_t)NTG_NOALLOC_SCRATCH_BYTES) +
                         "); use ntg_chol_solve with a workspace");
  void* scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != NTG_OK) return rc;
  // ntg_chol_solve clears what must start at zero (the residual maximum) and
  // overwrites the rest of the workspace before reading it.
  return ntg_chol_solve(stream, A, L, lambda, n, B, m, X, refine_iters, scratch,
                        (size_t)NTG_NOALLOC_SCRATCH_BYTES, final_residual);
}
