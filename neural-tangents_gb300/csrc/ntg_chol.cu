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
// sides, in blocks of TB rows: the diagonal block is solved for all columns by
// ceil(m / 32) CTAs (one warp per column), then a tiled FP32 GEMM subtracts the
// solved block from every remaining row block.
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
  const int64_t c_end = imin64(m, (int64_t)(blockIdx.x + 1) * 32);
  for (int64_t c = (int64_t)blockIdx.x * 32 + warp; c < c_end; c += nw) {
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

// X[row0 + i, j] -= sum_{k < nb} A(i, k) X[r0 + k, j] over 64 x 64 tiles of (i, j):
//   forward   A(i, k) = L[row0 + i, r0 + k]   (rows after the block)
//   transpose A(i, k) = L[r0 + k, row0 + i]   (rows before the block)
__global__ void __launch_bounds__(256)
    trsm_update_kernel(const float* __restrict__ L, int64_t n, float* __restrict__ X, int64_t m,
                       int64_t r0, int nb, int64_t row0, int64_t rows, int transpose) {
  __shared__ __align__(16) float As[TB][64 + 4];  // [k][i]
  __shared__ __align__(16) float Bs[TB][64 + 4];  // [k][j]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  for (int idx = threadIdx.x; idx < TB * 64; idx += 256) {
    if (!transpose) {
      const int i = idx / TB, k = idx % TB;
      As[k][i] = (i0 + i < rows && k < nb) ? L[(row0 + i0 + i) * n + r0 + k] : 0.f;
    } else {
      const int k = idx / 64, i = idx % 64;
      As[k][i] = (i0 + i < rows && k < nb) ? L[(r0 + k) * n + row0 + i0 + i] : 0.f;
    }
    const int k = idx / 64, j = idx % 64;
    Bs[k][j] = (k < nb && j0 + j < m) ? X[(r0 + k) * m + j0 + j] : 0.f;
  }
  __syncthreads();
  float acc[4][4] = {};
  for (int k = 0; k < nb; ++k) {
    const float4 a = *reinterpret_cast<const float4*>(&As[k][ty * 4]);
    const float4 b = *reinterpret_cast<const float4*>(&Bs[k][tx * 4]);
    const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t i = i0 + ty * 4 + u;
    if (i >= rows) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int64_t j = j0 + tx * 4 + v;
      if (j < m) X[(row0 + i) * m + j] -= acc[u][v];
    }
  }
}

// R = B - (A + lambda I) X in FP64 over 64 x 64 tiles of (row, column), X [n, m]
// in FP64; max |R| into rnorm.
__global__ void __launch_bounds__(256)
    residual_kernel(const float* __restrict__ A, int64_t n, const double* lambda,
                    const float* __restrict__ B, const double* __restrict__ X, int64_t m,
                    float* __restrict__ R, double* __restrict__ rnorm) {
  __shared__ double As[16][64 + 1];  // [k][i]
  __shared__ double Xs[16][64 + 1];  // [k][j]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  double acc[4][4] = {};
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      const int i = idx / 16, k = idx % 16;
      As[k][i] = (i0 + i < n && k0 + k < n) ? (double)A[(i0 + i) * n + k0 + k] : 0.0;
      const int kk = idx / 64, j = idx % 64;
      Xs[kk][j] = (k0 + kk < n && j0 + j < m) ? X[(k0 + kk) * m + j0 + j] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      double av[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        av[u] = As[k][ty * 4 + u];
        bv[u] = Xs[k][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(av[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
  double rmax = 0.0;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t i = i0 + ty * 4 + u;
    if (i >= n) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int64_t j = j0 + tx * 4 + v;
      if (j >= m) continue;
      const double r = (double)B[i * m + j] - acc[u][v] - lambda[0] * X[i * m + j];
      R[i * m + j] = (float)r;
      rmax = fmax(rmax, fabs(r));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  if ((threadIdx.x & 31) == 0 && rmax > 0.0)
    atomicMax(reinterpret_cast<unsigned long long*>(rnorm),
              (unsigned long long)__double_as_longlong(rmax));
}

// The same residual for few right-hand sides (m <= 16): one warp per row reads
// that row of A once and keeps the m FP64 dot products in registers.
template <int MR>
__global__ void __launch_bounds__(256)
    residual_rows_kernel(const float* __restrict__ A, int64_t n, const double* lambda,
                         const float* __restrict__ B, const double* __restrict__ X, int64_t m,
                         float* __restrict__ R, double* __restrict__ rnorm) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* ar = A + row * n;
  double acc[MR];
#pragma unroll
  for (int c = 0; c < MR; ++c) acc[c] = 0.0;
  for (int64_t j = lane; j < n; j += 32) {
    const double a = (double)ar[j];
    const double* xr = X + j * m;
#pragma unroll
    for (int c = 0; c < MR; ++c)
      if (c < m) acc[c] = fma(a, xr[c], acc[c]);
  }
  double rmax = 0.0;
#pragma unroll
  for (int c = 0; c < MR; ++c) {
    double v = acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (c < m && lane == 0) {
      const double r = (double)B[row * m + c] - v - lambda[0] * X[row * m + c];
      R[row * m + c] = (float)r;
      rmax = fmax(rmax, fabs(r));
    }
  }
  if (lane == 0 && rmax > 0.0)
    atomicMax(reinterpret_cast<unsigned long long*>(rnorm),
              (unsigned long long)__double_as_longlong(rmax));
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
  for (int64_t bb = 0; bb < nblk; ++bb) {
    const int64_t blk = transpose ? nblk - 1 - bb : bb;
    const int64_t r0 = blk * TB;
    const int nb = (int)imin64(TB, n - r0);
    trsv_diag_kernel<<<(unsigned)ceil_div(m, 32), 256, 0, s>>>(L, n, X, m, r0, transpose);
    note_launch();
    const int64_t row0 = transpose ? 0 : r0 + nb;
    const int64_t rows = transpose ? r0 : n - row0;
    if (rows > 0) {
      dim3 grid((unsigned)ceil_div(m, 64), (unsigned)ceil_div(rows, 64));
      trsm_update_kernel<<<grid, 256, 0, s>>>(L, n, X, m, r0, nb, row0, rows, transpose);
      note_launch();
    }
  }
  return check_launch("ntg_chol_solve trsv");
}

}  // namespace
}  // namespace ntg

using namespace ntg;

extern "C" size_t ntg_chol_workspace_bytes(int64_t n, int64_t m) {
  // trace + lambda + rnorm (3 doubles), x64 [n*m] doubles, residual [n*m] floats.
  // Sizes whose byte count would not fit in 63 bits report SIZE_MAX, which no
  // workspace satisfies (the product n * m itself must not wrap).
  if (n <= 0 || m <= 0) return 256;
  const uint64_t per = sizeof(double) + sizeof(float);
  if ((uint64_t)n > ((uint64_t)INT64_MAX / per) / (uint64_t)m) return SIZE_MAX;
  const uint64_t b = 256 + per * (uint64_t)n * (uint64_t)m;
  return (size_t)((b + 255) & ~(uint64_t)255);
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
  NTG_REQUIRE(ceil_div(m, 64) <= 65535 && ceil_div(m, 32) <= (1ll << 31) - 1,
              "ntg_chol_solve: too many right-hand sides");
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
  const dim3 rgrid((unsigned)ceil_div(m, 64), (unsigned)ceil_div(n, 64));
  // refine_iters residual + correction rounds, then the residual of the result
  // only when the caller asks for its norm
  for (int it = 0; it <= refine_iters; ++it) {
    if (it == refine_iters && !final_residual) break;
    if (cudaMemsetAsync(rnorm, 0, sizeof(double), s) != cudaSuccess)
      return check_launch("ntg_chol_solve memset");
    if (m <= 4)
      residual_rows_kernel<4><<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(A, n, lambda, B, x64, m,
                                                                      r32, rnorm);
    else if (m <= 16)
      residual_rows_kernel<16><<<(unsigned)ceil_div(n, 8), 256, 0, s>>>(A, n, lambda, B, x64, m,
                                                                       r32, rnorm);
    else
      residual_kernel<<<rgrid, 256, 0, s>>>(A, n, lambda, B, x64, m, r32, rnorm);
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
