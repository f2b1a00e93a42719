// Kernel-regression solve of predict.gradient_descent_mse (t = None):
// A = K + lambda I with lambda = diag_reg * trace(K) / n (or diag_reg),
// an FP32 blocked Cholesky A = L L^T, FP32 triangular solves, and FP64
// iterative refinement x <- x + A^{-1} (b - A x) with the residual accumulated
// in FP64 (neural_tangents/_src/predict.py:1224-1258 restated for the GPU).
#include <cstdio>

#include "ntg_common.cuh"

namespace ntg {
namespace {

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

constexpr int NB = 32;     // diagonal block of the factorisation
constexpr int TILE = 64;   // trailing-update tile

__global__ void trace_kernel(const float* __restrict__ A, int64_t n, double* __restrict__ out) {
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += (double)A[i * n + i];
  __shared__ double part[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    out[0] = t;
  }
}

// L = lower(A) + lambda I (upper part zeroed); lambda = reg * (absolute ? 1 : trace / n).
__global__ void init_factor_kernel(const float* __restrict__ A, int64_t n, double reg,
                                   int absolute, const double* __restrict__ trace,
                                   float* __restrict__ L, double* __restrict__ lambda) {
  const double lam = absolute ? reg : reg * trace[0] / (double)n;
  if (blockIdx.x == 0 && threadIdx.x == 0) lambda[0] = lam;
  const int64_t total = n * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / n, j = idx - i * n;
    float v = 0.f;
    if (j < i) v = A[idx];
    else if (j == i) v = (float)((double)A[idx] + lam);
    L[idx] = v;
  }
}

// Unblocked Cholesky of the NB x NB diagonal block at (k, k), in place.
// A non-positive pivot sets *info = global column + 1 (first one wins).
__global__ void potrf_diag_kernel(float* __restrict__ L, int64_t n, int64_t k, int* info) {
  __shared__ float a[NB][NB + 1];
  const int nb = (int)imin64(NB, n - k);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int i = ty; i < nb; i += 8)
    a[i][tx] = tx < nb ? L[(k + i) * n + k + tx] : 0.f;
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (threadIdx.x == 0) {
      float d = a[j][j];
      if (!(d > 0.f)) {
        atomicCAS(info, 0, (int)(k + j + 1));
        d = 1.f;
      }
      a[j][j] = sqrtf(d);
    }
    __syncthreads();
    const float piv = a[j][j];
    for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) a[i][j] = a[i][j] / piv;
    __syncthreads();
    for (int i = j + 1 + ty; i < nb; i += 8)
      if (tx > j && tx <= i) a[i][tx] = fmaf(-a[i][j], a[tx][j], a[i][tx]);
    __syncthreads();
  }
  for (int i = ty; i < nb; i += 8)
    if (tx < nb) L[(k + i) * n + k + tx] = tx <= i ? a[i][tx] : 0.f;
}

// Panel solve: rows r >= k + NB of block column k: L[r, k:k+nb] <- A[r, k:k+nb] L11^{-T}.
__global__ void trsm_panel_kernel(float* __restrict__ L, int64_t n, int64_t k) {
  __shared__ float l11[NB][NB + 1];
  const int nb = (int)imin64(NB, n - k);
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int i = idx / NB, j = idx % NB;
    l11[i][j] = (i < nb && j < nb) ? L[(k + i) * n + k + j] : 0.f;
  }
  __syncthreads();
  const int64_t r = k + nb + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float x[NB];
  float* row = L + r * n + k;
#pragma unroll
  for (int j = 0; j < NB; ++j) x[j] = j < nb ? row[j] : 0.f;
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    if (j < nb) {
      float s = x[j];
#pragma unroll
      for (int p = 0; p < j; ++p) s = fmaf(-x[p], l11[j][p], s);
      x[j] = s / l11[j][j];
    }
  }
#pragma unroll
  for (int j = 0; j < NB; ++j)
    if (j < nb) row[j] = x[j];
}

// Trailing update of the lower triangle: A22 -= L21 L21^T for rows/cols >= k + nb.
__global__ void __launch_bounds__(256) syrk_update_kernel(float* __restrict__ L, int64_t n,
                                                          int64_t k) {
  const int nb = (int)imin64(NB, n - k);
  const int64_t base = k + nb;
  const int64_t bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;  // lower triangle of tiles only
  const int64_t row0 = base + bi * TILE, col0 = base + bj * TILE;
  __shared__ float As[NB][TILE + 4];
  __shared__ float Bs[NB][TILE + 4];
  for (int idx = threadIdx.x; idx < NB * TILE; idx += 256) {
    const int rr = idx / NB, kk = idx % NB;
    const int64_t gi = row0 + rr, gj = col0 + rr;
    As[kk][rr] = (gi < n && kk < nb) ? L[gi * n + k + kk] : 0.f;
    Bs[kk][rr] = (gj < n && kk < nb) ? L[gj * n + k + kk] : 0.f;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4] = {};
#pragma unroll
  for (int kk = 0; kk < NB; ++kk) {
    float a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = As[kk][ty * 4 + u];
      b[u] = Bs[kk][tx * 4 + u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int64_t gi = row0 + ty * 4 + u, gj = col0 + tx * 4 + v;
      if (gi < n && gj <= gi) L[gi * n + gj] -= acc[u][v];
    }
}

// Triangular solves L y = b (forward) and L^T x = y (backward) for m right-hand
// sides, in blocks of TB rows: a single CTA solves the diagonal block (one warp
// per right-hand side), then a wide kernel applies that block to every other
// row with coalesced reads of L.
constexpr int TB = 64;

__global__ void trsv_diag_kernel(const float* __restrict__ L, int64_t n, float* __restrict__ X,
                                 int64_t m, int64_t r0, int transpose) {
  __shared__ float d[TB][TB + 1];
  const int nb = (int)imin64(TB, n - r0);
  for (int idx = threadIdx.x; idx < TB * TB; idx += blockDim.x) {
    const int i = idx / TB, j = idx % TB;
    d[i][j] = (i < nb && j < nb) ? L[(r0 + i) * n + r0 + j] : 0.f;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int64_t c = warp; c < m; c += nw) {
    float x0 = lane < nb ? X[(r0 + lane) * m + c] : 0.f;
    float x1 = lane + 32 < nb ? X[(r0 + lane + 32) * m + c] : 0.f;
    if (!transpose) {
      for (int i = 0; i < nb; ++i) {
        const float xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) / d[i][i];
        if (lane == (i & 31)) {
          if (i < 32) x0 = xi; else x1 = xi;
        }
        if (lane > i) x0 = fmaf(-d[lane][i], xi, x0);
        if (lane + 32 > i && lane + 32 < nb) x1 = fmaf(-d[lane + 32][i], xi, x1);
      }
    } else {
      for (int i = nb - 1; i >= 0; --i) {
        const float xi = __shfl_sync(0xffffffffu, i < 32 ? x0 : x1, i & 31) / d[i][i];
        if (lane == (i & 31)) {
          if (i < 32) x0 = xi; else x1 = xi;
        }
        if (lane < i) x0 = fmaf(-d[i][lane], xi, x0);
        if (lane + 32 < i) x1 = fmaf(-d[i][lane + 32], xi, x1);
      }
    }
    if (lane < nb) X[(r0 + lane) * m + c] = x0;
    if (lane + 32 < nb) X[(r0 + lane + 32) * m + c] = x1;
  }
}

// forward: rows rr >= r0 + nb:  X[rr] -= L[rr, block] X[block]   (one warp per row)
// backward: rows rr < r0:       X[rr] -= L[block, rr]^T X[block] (one thread per row)
__global__ void trsv_update_kernel(const float* __restrict__ L, int64_t n, float* __restrict__ X,
                                   int64_t m, int64_t r0, int transpose) {
  extern __shared__ float xb[];  // [TB][m] solved block
  const int nb = (int)imin64(TB, n - r0);
  for (int64_t idx = threadIdx.x; idx < (int64_t)nb * m; idx += blockDim.x)
    xb[idx] = X[(r0 + idx / m) * m + idx % m];
  __syncthreads();
  if (!transpose) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int64_t rr = r0 + nb + (int64_t)blockIdx.x * nw + warp;
    if (rr >= n) return;
    const float l0 = lane < nb ? L[rr * n + r0 + lane] : 0.f;
    const float l1 = lane + 32 < nb ? L[rr * n + r0 + lane + 32] : 0.f;
    for (int64_t c = 0; c < m; ++c) {
      float sacc = l0 * (lane < nb ? xb[lane * m + c] : 0.f);
      if (lane + 32 < nb) sacc = fmaf(l1, xb[(lane + 32) * m + c], sacc);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
      if (lane == 0) X[rr * m + c] -= sacc;
    }
  } else {
    const int64_t rr = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (rr >= r0) return;
    for (int64_t c = 0; c < m; ++c) {
      float sacc = 0.f;
      for (int i = 0; i < nb; ++i) sacc = fmaf(L[(r0 + i) * n + rr], xb[i * m + c], sacc);
      X[rr * m + c] -= sacc;
    }
  }
}

// r = b - (A + lambda I) x in FP64; one warp per row, all m columns.
__global__ void residual_kernel(const float* __restrict__ A, int64_t n, const double* lambda,
                                const float* __restrict__ B, const double* __restrict__ X,
                                int64_t m, float* __restrict__ R, double* __restrict__ rnorm) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* ar = A + row * n;
  for (int64_t c = 0; c < m; ++c) {
    double s = 0.0;
    for (int64_t j = lane; j < n; j += 32) s = fma((double)ar[j], X[j * m + c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      const double r = (double)B[row * m + c] - s - lambda[0] * X[row * m + c];
      R[row * m + c] = (float)r;
      atomicMax(reinterpret_cast<unsigned long long*>(rnorm),
                (unsigned long long)__double_as_longlong(fabs(r)));
    }
  }
}

__global__ void to_double_kernel(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

__global__ void accumulate_kernel(double* __restrict__ x, const float* __restrict__ dx,
                                  float* __restrict__ x32, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)dx[i];
    x32[i] = (float)x[i];
  }
}

__global__ void logdet_kernel(const float* __restrict__ L, int64_t n, double* __restrict__ out) {
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += log((double)L[i * n + i]);
  __shared__ double part[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    out[0] = 2.0 * t;
  }
}

// out = g (-1/2 alpha alpha^T + m/2 Kinv); trace(out) accumulated into tr[0].
__global__ void nll_grad_kernel(const float* __restrict__ kinv, const float* __restrict__ alpha,
                                int64_t n, int64_t m, float g, float* __restrict__ out,
                                double* __restrict__ tr) {
  const int64_t total = n * n;
  double ltr = 0.0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / n, j = idx - i * n;
    float aa = 0.f;
    for (int64_t c = 0; c < m; ++c) aa = fmaf(alpha[i * m + c], alpha[j * m + c], aa);
    const float v = g * (-0.5f * aa + 0.5f * (float)m * kinv[idx]);
    out[idx] = v;
    if (i == j) ltr += (double)v;
  }
  if (ltr != 0.0) atomicAdd(tr, ltr);
}

__global__ void add_diag_kernel(float* __restrict__ a, int64_t n, const double* __restrict__ tr,
                                double scale) {
  const float v = (float)(scale * tr[0]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i * n + i] += v;
}

int grid1(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

int trsv(cudaStream_t s, const float* L, int64_t n, float* X, int64_t m, int transpose) {
  const int64_t nblk = ceil_div(n, TB);
  const size_t sm = sizeof(float) * TB * m;
  for (int64_t bb = 0; bb < nblk; ++bb) {
    const int64_t blk = transpose ? nblk - 1 - bb : bb;
    const int64_t r0 = blk * TB;
    trsv_diag_kernel<<<1, 256, 0, s>>>(L, n, X, m, r0, transpose);
    const int64_t rows = transpose ? r0 : n - imin64(n, r0 + TB);
    note_launch();
    if (rows > 0) {
      const unsigned g = (unsigned)(transpose ? ceil_div(rows, 256) : ceil_div(rows, 8));
      trsv_update_kernel<<<g, 256, sm, s>>>(L, n, X, m, r0, transpose);
      note_launch();
    }
  }
  return check_launch("ntg_chol_solve trsv");
}

}  // namespace
}  // namespace ntg

using namespace ntg;

extern "C" size_t ntg_chol_workspace_bytes(int64_t n, int64_t m) {
  // trace + lambda + rnorm (3 doubles), x64 [n*m] doubles, residual [n*m] floats
  size_t b = 256 + sizeof(double) * (size_t)(n * m) + sizeof(float) * (size_t)(n * m);
  return (b + 255) & ~(size_t)255;
}

extern "C" int ntg_chol_factor(void* stream, const float* A, int64_t n, double diag_reg,
                               int32_t absolute, float* L, double* lambda, int* info) {
  NTG_REQUIRE(A && L && lambda && info, "ntg_chol_factor: null pointer");
  NTG_REQUIRE(n > 0, "ntg_chol_factor: n must be positive");
  NTG_REQUIRE(n <= 46340, "ntg_chol_factor: n too large");
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(info, 0, sizeof(int), s) != cudaSuccess)
    return check_launch("ntg_chol_factor memset");
  trace_kernel<<<1, 1024, 0, s>>>(A, n, lambda + 1);
  init_factor_kernel<<<grid1(n * n), 256, 0, s>>>(A, n, diag_reg, absolute, lambda + 1, L,
                                                   lambda);
  note_launch(2);
  for (int64_t k = 0; k < n; k += NB) {
    potrf_diag_kernel<<<1, 256, 0, s>>>(L, n, k, info);
    const int64_t rest = n - k - NB;
    note_launch();
    if (rest > 0) {
      trsm_panel_kernel<<<(unsigned)ceil_div(rest, 128), 128, 0, s>>>(L, n, k);
      const unsigned tiles = (unsigned)ceil_div(rest, TILE);
      syrk_update_kernel<<<dim3(tiles, tiles), 256, 0, s>>>(L, n, k);
      note_launch(2);
    }
  }
  return check_launch("ntg_chol_factor");
}

extern "C" int ntg_chol_solve(void* stream, const float* A, const float* L, const double* lambda,
                              int64_t n, const float* B, int64_t m, float* X,
                              int32_t refine_iters, void* workspace, size_t workspace_bytes,
                              double* final_residual) {
  NTG_REQUIRE(A && L && lambda && B && X, "ntg_chol_solve: null pointer");
  NTG_REQUIRE(n > 0 && m > 0, "ntg_chol_solve: sizes must be positive");
  NTG_REQUIRE(refine_iters >= 0 && refine_iters <= 16, "ntg_chol_solve: 0..16 refinement steps");
  NTG_REQUIRE(m <= 128, "ntg_chol_solve: at most 128 right-hand sides per call");
  cudaStream_t s = as_stream(stream);
  if (cudaMemcpyAsync(X, B, sizeof(float) * n * m, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return check_launch("ntg_chol_solve copy");
  int rc = trsv(s, L, n, X, m, 0);
  if (rc) return rc;
  rc = trsv(s, L, n, X, m, 1);
  if (rc) return rc;
  if (refine_iters == 0 && !final_residual) return NTG_OK;
  NTG_REQUIRE(workspace && workspace_bytes >= ntg_chol_workspace_bytes(n, m),
              "ntg_chol_solve: refinement needs ntg_chol_workspace_bytes(n, m) of workspace");
  char* ws = static_cast<char*>(workspace);
  double* rnorm = reinterpret_cast<double*>(ws);
  double* x64 = reinterpret_cast<double*>(ws + 256);
  float* r32 = reinterpret_cast<float*>(ws + 256 + sizeof(double) * n * m);
  to_double_kernel<<<grid1(n * m), 256, 0, s>>>(X, x64, n * m);
  note_launch();
  for (int it = 0; it <= refine_iters; ++it) {
    if (cudaMemsetAsync(rnorm, 0, sizeof(double), s) != cudaSuccess)
      return check_launch("ntg_chol_solve memset");
    residual_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(A, n, lambda, B, x64, m, r32, rnorm);
    note_launch();
    if (it == refine_iters) break;
    rc = trsv(s, L, n, r32, m, 0);
    if (rc) return rc;
    rc = trsv(s, L, n, r32, m, 1);
    if (rc) return rc;
    accumulate_kernel<<<grid1(n * m), 256, 0, s>>>(x64, r32, X, n * m);
    note_launch();
  }
  if (final_residual &&
      cudaMemcpyAsync(final_residual, rnorm, sizeof(double), cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess)
    return check_launch("ntg_chol_solve residual copy");
  return check_launch("ntg_chol_solve");
}

extern "C" int ntg_chol_logdet(void* stream, const float* L, int64_t n, double* out) {
  NTG_REQUIRE(L && out && n > 0, "ntg_chol_logdet: bad arguments");
  logdet_kernel<<<1, 1024, 0, as_stream(stream)>>>(L, n, out);
  note_launch();
  return check_launch("ntg_chol_logdet");
}

extern "C" int ntg_nll_grad(void* stream, const float* kinv, const float* alpha, int64_t n,
                            int64_t m, float g, double reg_over_n, float* out, double* tr) {
  NTG_REQUIRE(kinv && alpha && out && tr && n > 0 && m > 0, "ntg_nll_grad: bad arguments");
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(tr, 0, sizeof(double), s) != cudaSuccess) return check_launch("ntg_nll_grad");
  nll_grad_kernel<<<grid1(n * n), 256, 0, s>>>(kinv, alpha, n, m, g, out, tr);
  note_launch();
  if (reg_over_n != 0.0) {
    add_diag_kernel<<<grid1(n), 256, 0, s>>>(out, n, tr, reg_over_n);
    note_launch();
  }
  return check_launch("ntg_nll_grad");
}
