// Blocked Cholesky factorisation and solves of predict.gradient_descent_mse on
// the sm_103a tensor cores (neural_tangents/_src/predict.py:1224-1258 restated
// for the GPU): A = K + lambda I = L L^T in FP32 with 128-wide panels.
//
// Per panel k:
//   diag_block_kernel   one CTA factors the 128 x 128 diagonal block (four
//                       32-wide steps, each a warp-level Cholesky + inverse in
//                       registers, then the sub-panel solve and rank-32 update in
//                       shared memory) and writes the block's inverse;
//   panel_trsm_kernel   the rows below: L21 = A21 L11^-T by forward substitution
//                       (a warp per row, backward stable);
//   gemm_tf32x3 lower   the trailing update A22 -= L21 L21^T on the tensor cores
//                       (3xTF32 products, FP32 accumulation; tiles on or below the
//                       diagonal only).
// After the panels, the explicit inverse factors L^-T (a forward block solve of
// L Y = I on the tensor cores, only the non-zero rows of each block column) and
// L^-1 (its transpose) are kept in the factor workspace: a solve is then two
// triangular products, GEMV-shaped for up to kSmallM right-hand sides (a warp
// per row, bandwidth-bound) and tensor-core GEMMs for more.
// Refinement keeps x in FP64 and accumulates every product with K in
// double-float (two FP32 words, error-free products and sums; about 44
// significant bits), which the GB300's FP32 rate makes about 6x cheaper than
// FP64: for up to kSmallM right-hand sides preconditioned conjugate gradients
// (the factor as preconditioner; converges where plain refinement stalls,
// kappa u > 1, each column stopping once its residual fell by kPcgTol), for
// more, refine_iters steps of x <- x + (L L^T)^-1 (b - A x).
#include <mutex>
#include <string>

#include "ntg_common.cuh"

namespace ntg {
int gemm_tf32x3(cudaStream_t s, const float* a, int64_t lda, const float* b, int64_t ldb,
                float* c, int64_t ldc, int64_t m, int64_t n, int64_t k, float alpha, float beta,
                int lower);

namespace {

constexpr int PB = 128;        // panel / diagonal block
constexpr int PBS = PB + 1;    // padded shared-memory row
constexpr int kSmallM = 16;    // right-hand sides of the cooperative solves

__device__ int g_chol_error = 0;

__host__ __device__ __forceinline__ int64_t mini(int64_t a, int64_t b) { return a < b ? a : b; }

// ---------------------------------------------------------------------------
// Set-up
// ---------------------------------------------------------------------------

__global__ void trace_tc_kernel(const float* __restrict__ A, int64_t n, double* __restrict__ out) {
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

// L[i, j] = A[i, j] (j < i), A[i, i] + lambda (j == i), 0 above the diagonal and in the
// padding columns n <= j < ldl.
__global__ void init_factor_ld_kernel(const float* __restrict__ A, int64_t n, int64_t ldl,
                                      double reg, int absolute, const double* __restrict__ trace,
                                      float* __restrict__ L, double* __restrict__ lambda) {
  const double lam = absolute ? reg : reg * trace[0] / (double)n;
  if (blockIdx.x == 0 && threadIdx.x == 0) lambda[0] = lam;
  const int64_t total = n * ldl;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / ldl, j = idx - i * ldl;
    float v = 0.f;
    if (j < i) v = A[i * n + j];
    else if (j == i) v = (float)((double)A[i * n + i] + lam);
    L[idx] = v;
  }
}

// ---------------------------------------------------------------------------
// Diagonal block: factor + inverse (one CTA of 512 threads)
// ---------------------------------------------------------------------------

// Warp-level Cholesky of the 32 x 32 block at (o, o) of `a` (lower part used) and the
// inverse of the factor into dinv (lower, row-major 32 x 33). Lane r holds row r in
// registers; each pivot column is broadcast through shared memory. The pivot uses the
// hardware reciprocal square root (2 ulp): L_jj = d rsqrt(d), L_rj = A_rj rsqrt(d), and
// the reciprocal pivots are kept for the inverse, which then needs no division (the
// factor is refined against the exact kernel by the solves; measured on GB300, the IEEE
// square root and divisions were 40 % of this routine).
__device__ void warp_potrf_inv32(float (*a)[PBS], int o, float (*dinv)[33], int* info,
                                 int64_t col0) {
  __shared__ float colbuf[33];
  __shared__ float rpiv[32];
  const int lane = threadIdx.x & 31;
  float v[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) v[c] = a[o + lane][o + c];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    if (lane == j) colbuf[32] = v[j];
    __syncwarp();
    float d = colbuf[32];
    if (!(d > 0.f)) {  // the same value in every lane
      if (lane == 0) atomicCAS(info, 0, (int)(col0 + o + j + 1));
      d = 1.f;
    }
    const float rs = rsqrtf(d);
    const float l = (lane == j) ? d * rs : v[j] * rs;
    v[j] = l;
    colbuf[lane] = l;
    if (lane == 0) rpiv[j] = rs;
    __syncwarp();
#pragma unroll
    for (int c = j + 1; c < 32; ++c) {
      const float lc = colbuf[c];
      if (lane >= c) v[c] = fmaf(-l, lc, v[c]);
    }
    __syncwarp();
  }
#pragma unroll
  for (int c = 0; c < 32; ++c) a[o + lane][o + c] = (c <= lane) ? v[c] : 0.f;
  __syncwarp();
  // X = L^-1, lane c computes column c: x_i = (delta_ic - sum_{p<i} L[i][p] x_p) / L[i][i]
  float x[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    float s = (i == lane) ? 1.f : 0.f;
#pragma unroll
    for (int p = 0; p < i; ++p) s = fmaf(-a[o + i][o + p], x[p], s);
    x[i] = s * rpiv[i];
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) dinv[i][lane] = x[i];
  __syncwarp();
}

// Factors L[k:k+nb, k:k+nb] in place (upper part zeroed) and writes the inverse of the
// factor, zero-padded to 128 x 128, to linv (row-major).
__global__ void __launch_bounds__(512, 1)
    diag_block_kernel(float* __restrict__ L, int64_t ldl, int64_t n, int64_t k, int* info,
                      float* __restrict__ linv) {
  extern __shared__ float sm[];
  float(*a)[PBS] = reinterpret_cast<float(*)[PBS]>(sm);
  float(*x)[PBS] = reinterpret_cast<float(*)[PBS]>(sm + PB * PBS);
  float(*t)[33] = reinterpret_cast<float(*)[33]>(sm + 2 * PB * PBS);        // 128 x 33
  float(*dinv)[32][33] = reinterpret_cast<float(*)[32][33]>(sm + 2 * PB * PBS + PB * 33);
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5;
  const int nb = (int)mini(PB, n - k);
  // padding beyond nb: identity (factors to the identity, inverse identity, cut later)
  for (int idx = tid; idx < PB * PB; idx += nth) {
    const int i = idx / PB, j = idx % PB;
    float v;
    if (i < nb && j < nb) v = (j <= i) ? L[(k + i) * ldl + k + j] : 0.f;
    else v = (i == j) ? 1.f : 0.f;
    a[i][j] = v;
  }
  __syncthreads();
  for (int sb = 0; sb < 4; ++sb) {
    const int o = sb * 32;
    if (warp == 0) warp_potrf_inv32(a, o, dinv[sb], info, k);
    __syncthreads();
    const int rows = PB - o - 32;
    if (rows > 0) {
      // sub-panel solve: L[r][o+c] = sum_{p <= c} A[r][o+p] Dinv[c][p], r >= o + 32
      for (int idx = tid; idx < rows * 32; idx += nth) {
        const int r = o + 32 + idx / 32, c = idx % 32;
        float s = 0.f;
        for (int p = 0; p <= c; ++p) s = fmaf(a[r][o + p], dinv[sb][c][p], s);
        t[r][c] = s;
      }
      __syncthreads();
      for (int idx = tid; idx < rows * 32; idx += nth) {
        const int r = o + 32 + idx / 32, c = idx % 32;
        a[r][o + c] = t[r][c];
      }
      __syncthreads();
      // trailing rank-32 update of the lower part
      for (int idx = tid; idx < rows * rows; idx += nth) {
        const int r = o + 32 + idx / rows, c = o + 32 + idx % rows;
        if (c > r) continue;
        float s = a[r][c];
#pragma unroll 8
        for (int p = 0; p < 32; ++p) s = fmaf(-a[r][o + p], a[c][o + p], s);
        a[r][c] = s;
      }
      __syncthreads();
    }
  }
  // write the factor back (lower incl. the diagonal; upper zero)
  for (int idx = tid; idx < nb * nb; idx += nth) {
    const int i = idx / nb, j = idx % nb;
    L[(k + i) * ldl + k + j] = (j <= i) ? a[i][j] : 0.f;
  }
  // inverse, 32-blocks: X_ii = Dinv_i, X_ij = -Dinv_i sum_{q=j}^{i-1} L_iq X_qj
  for (int idx = tid; idx < PB * PB; idx += nth) {
    const int i = idx / PB, j = idx % PB;
    const int bi = i >> 5, bj = j >> 5;
    x[i][j] = (bi == bj) ? dinv[bi][i & 31][j & 31] : 0.f;
  }
  __syncthreads();
  for (int bi = 1; bi < 4; ++bi) {
    // T[r][c'] over the bi blocks j < bi: T_j = sum_{q=j}^{bi-1} L_{bi,q} X_{q,j}, into t
    // (t holds 128 rows x 32: rows j*32 + r' for block j)
    for (int idx = tid; idx < bi * 1024; idx += nth) {
      const int bj = idx / 1024, r = (idx % 1024) / 32, c = idx % 32;
      float s = 0.f;
      for (int q = bj * 32; q < bi * 32; ++q) s = fmaf(a[bi * 32 + r][q], x[q][bj * 32 + c], s);
      t[bj * 32 + r][c] = s;
    }
    __syncthreads();
    for (int idx = tid; idx < bi * 1024; idx += nth) {
      const int bj = idx / 1024, r = (idx % 1024) / 32, c = idx % 32;
      float s = 0.f;
      for (int p = 0; p <= r; ++p) s = fmaf(dinv[bi][r][p], t[bj * 32 + p][c], s);
      x[bi * 32 + r][bj * 32 + c] = -s;
    }
    __syncthreads();
  }
  for (int idx = tid; idx < PB * PB; idx += nth) {
    const int i = idx / PB, j = idx % PB;
    const bool in = i < nb && j < nb;
    linv[idx] = in ? x[i][j] : 0.f;
  }
}

constexpr size_t kDiagSmem = (size_t)(2 * PB * PBS + PB * 33 + 4 * 32 * 33) * sizeof(float);

// ---------------------------------------------------------------------------
// Panel solve below the diagonal block: x L11^T = a for rows r >= k + 128, a warp per
// row; lane l holds columns l, l + 32, l + 64, l + 96.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512)
    panel_trsm_kernel(float* __restrict__ L, int64_t ldl, int64_t n, int64_t k) {
  extern __shared__ float sm[];
  float(*l11)[PBS] = reinterpret_cast<float(*)[PBS]>(sm);
  float* rdiag = sm + PB * PBS;  // 1 / L11[c][c]: a multiplication on the dependent chain
  for (int idx = threadIdx.x; idx < PB * PB; idx += blockDim.x) {
    const int i = idx / PB, j = idx % PB;
    l11[i][j] = (j <= i) ? L[(k + i) * ldl + k + j] : 0.f;
  }
  __syncthreads();
  if (threadIdx.x < PB) rdiag[threadIdx.x] = 1.f / l11[threadIdx.x][threadIdx.x];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const unsigned full = 0xffffffffu;
  for (int64_t r = k + PB + (int64_t)blockIdx.x * nw + warp; r < n; r += (int64_t)gridDim.x * nw) {
    float* row = L + r * ldl + k;
    float x[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) x[s] = row[lane + 32 * s];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
#pragma unroll 4
      for (int cc = 0; cc < 32; ++cc) {
        const int c = 32 * s + cc;
        const float xc = __shfl_sync(full, x[s], cc) * rdiag[c];
        if (lane == cc) x[s] = xc;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int p = lane + 32 * u;
          if (p > c) x[u] = fmaf(-xc, l11[p][c], x[u]);
        }
      }
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) row[lane + 32 * s] = x[s];
  }
}

constexpr size_t kPanelSmem = (size_t)(PB * PBS + PB) * sizeof(float);

// out[j, i] = in[i, j] for an [rows, cols] block (row pitches ld_in, ld_out).
__global__ void transpose_kernel(const float* __restrict__ in, int64_t ld_in, float* __restrict__ out,
                                 int64_t ld_out, int64_t rows, int64_t cols) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int i = ty; i < 32; i += 8) {
    const int64_t r = r0 + i, c = c0 + tx;
    tile[i][tx] = (r < rows && c < cols) ? in[r * ld_in + c] : 0.f;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int64_t c = c0 + i, r = r0 + tx;
    if (c < cols && r < rows) out[c * ld_out + r] = tile[tx][i];
  }
}

// ---------------------------------------------------------------------------
// Triangular products with the explicit inverse factors, for up to kSmallM
// right-hand sides: Y[i, c] = sum_{j in range(i)} M[i, j] X[j, c] with range
// j <= i (M = L^-1, lower) or j >= i (M = L^-T, upper). One warp per row.
// ---------------------------------------------------------------------------
template <int MR>
__global__ void __launch_bounds__(256)
    tri_gemv_kernel(const float* __restrict__ M, int64_t ld, int64_t n, int upper,
                    const float* __restrict__ X, int64_t m, float* __restrict__ Y,
                    const int* skip) {
  if (skip && *skip) return;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* mr = M + row * ld;
  float acc[MR];
#pragma unroll
  for (int c = 0; c < MR; ++c) acc[c] = 0.f;
  const int64_t j0 = upper ? row : 0, j1 = upper ? n : row + 1;
  for (int64_t j = j0 + lane; j < j1; j += 32) {
    const float a = mr[j];
    const float* xr = X + j * m;
#pragma unroll
    for (int c = 0; c < MR; ++c)
      if (c < m) acc[c] = fmaf(a, xr[c], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < MR; ++c) {
    if (c >= m) break;
    float v = acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) Y[row * m + c] = v;
  }
}

// I [n, ld]: ones on the diagonal, zeros elsewhere (padding columns included).
__global__ void identity_kernel(float* __restrict__ Z, int64_t n, int64_t ld) {
  const int64_t total = n * ld;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / ld, j = idx - i * ld;
    Z[idx] = (i == j) ? 1.f : 0.f;
  }
}

// ---------------------------------------------------------------------------
// Residuals R = B - (A + lambda I) X with X in FP64.
// ---------------------------------------------------------------------------

__global__ void max_abs64_kernel(const double* __restrict__ v, int64_t n, double* __restrict__ out) {
  double mx = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    mx = fmax(mx, fabs(v[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.0)
    atomicMax(reinterpret_cast<unsigned long long*>(out),
              (unsigned long long)__double_as_longlong(mx));
}

// Double-float accumulation (s_hi, s_lo) += a * (x_hi + x_lo): a * x_hi is split
// error-free (product and fused remainder), its high part added with a two-sum.
__device__ __forceinline__ void df_fma(float a, float xh, float xl, float& sh, float& sl) {
  const float ph = a * xh;
  float pl = fmaf(a, xh, -ph);
  pl = fmaf(a, xl, pl);
  const float s = sh + ph;
  const float bv = s - sh;
  const float e = (sh - (s - bv)) + (ph - bv);
  sl += e + pl;
  sh = s;
}

// Double-float residual over 64 x 64 tiles of (row, column): X (FP64) is split into
// FP32 (hi, lo) as it is staged; each thread keeps 4 x 4 double-float sums.
__global__ void __launch_bounds__(256)
    residual_df_kernel(const float* __restrict__ A, int64_t n, const double* lambda,
                       const float* __restrict__ B, const double* __restrict__ X, int64_t m,
                       float* __restrict__ R, double* __restrict__ rnorm) {
  __shared__ float As[16][64 + 1];   // [k][i]
  __shared__ float Xh[16][64 + 1];   // [k][j]
  __shared__ float Xl[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  float sh[4][4] = {}, sl[4][4] = {};
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      const int i = idx / 16, k = idx % 16;
      As[k][i] = (i0 + i < n && k0 + k < n) ? A[(i0 + i) * n + k0 + k] : 0.f;
      const int kk = idx / 64, j = idx % 64;
      const double xv = (k0 + kk < n && j0 + j < m) ? X[(k0 + kk) * m + j0 + j] : 0.0;
      const float xh = (float)xv;
      Xh[kk][j] = xh;
      Xl[kk][j] = (float)(xv - (double)xh);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      float av[4], hv[4], lv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        av[u] = As[k][ty * 4 + u];
        hv[u] = Xh[k][tx * 4 + u];
        lv[u] = Xl[k][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) df_fma(av[u], hv[v], lv[v], sh[u][v], sl[u][v]);
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
      const double ax = (double)sh[u][v] + (double)sl[u][v];
      const double r = (double)B[i * m + j] - ax - lambda[0] * X[i * m + j];
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

__global__ void to_double_tc_kernel(const float* __restrict__ a, double* __restrict__ b,
                                    int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

__global__ void accumulate_tc_kernel(double* __restrict__ x, const float* __restrict__ dx,
                                     float* __restrict__ x32, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += (double)dx[i];
    x32[i] = (float)x[i];
  }
}

// ---------------------------------------------------------------------------
// Preconditioned conjugate gradients for up to kSmallM right-hand sides: the
// FP32 factor L L^T preconditions (K + lambda I) d = r, with x, r, p, q in FP64
// and the products (K + lambda I) v accumulated in double-float. Each column
// stops (its step sizes become 0) once max |r| <= kPcgTol max |b|; when every
// column has stopped the remaining launches return at once.
// ---------------------------------------------------------------------------
constexpr double kPcgTol = 1e-10;   // residual reduction from the starting point
constexpr double kPcgFloor = 1e-15; // or residual below this times max |b|
constexpr int kPcgStall = 2;        // or no halving of the best residual for this many steps
constexpr int kDotBlocks = 128;

struct PcgState {
  double rho[2][kSmallM];   // r.z of the current / next iteration
  double bnorm[kSmallM];    // max |b_j|
  double r0norm[kSmallM];   // max |r_j| of the starting point
  double rbest[kSmallM];    // smallest max |r_j| so far
  int stall[kSmallM];       // iterations since rbest last halved
  double rmax[kSmallM];     // max |r_j| of the last residual
  int active[kSmallM];
  int all_done;
};

__device__ __forceinline__ void df_add(float& sh, float& sl, float bh, float bl) {
  const float s = sh + bh;
  const float bv = s - sh;
  const float e = (sh - (s - bv)) + (bh - bv);
  sl += e + bl;
  sh = s;
}

// X (FP64 [n, m]) as double-float pairs xs[j, c] = (hi, lo), split once per product so
// that the row kernel below runs on the FP32 pipes only.
__global__ void split_df_kernel(const double* __restrict__ X, int64_t total,
                                float2* __restrict__ xs, const PcgState* st) {
  if (st && st->all_done) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = X[i];
    const float h = (float)v;
    xs[i] = make_float2(h, (float)(v - (double)h));
  }
}

// out = B - (K + lambda I) X (subtract = 1) or (K + lambda I) X (subtract = 0) with X FP64
// [n, m] given also as its double-float split xs; one warp per row, double-float sums of
// the m <= MR products kept per lane.
template <int MR>
__global__ void __launch_bounds__(256)
    matvec_df_rows_kernel(const float* __restrict__ A, int64_t n, const double* lambda,
                          const float* __restrict__ B, const double* __restrict__ X,
                          const float2* __restrict__ xs, int64_t m, int subtract,
                          double* __restrict__ out, float* __restrict__ out32,
                          const PcgState* st) {
  if (st && st->all_done) return;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* ar = A + row * n;
  float sh[MR], sl[MR];
#pragma unroll
  for (int c = 0; c < MR; ++c) sh[c] = sl[c] = 0.f;
  for (int64_t j = lane; j < n; j += 32) {
    const float a = ar[j];
    const float2* xr = xs + j * m;
#pragma unroll
    for (int c = 0; c < MR; ++c) {
      const float2 xv = xr[c];
      df_fma(a, xv.x, xv.y, sh[c], sl[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < MR; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, sh[c], o);
      const float ol = __shfl_xor_sync(0xffffffffu, sl[c], o);
      df_add(sh[c], sl[c], oh, ol);
    }
    if (lane == 0) {
      const double v = (double)sh[c] + (double)sl[c] + lambda[0] * X[row * m + c];
      const double r = subtract ? (double)B[row * m + c] - v : v;
      out[row * m + c] = r;
      if (out32) out32[row * m + c] = (float)r;
    }
  }
}

// The row kernel instantiated for the exact number of right-hand sides (1..kSmallM), so
// no lane issues work for absent columns.
template <int MR>
void launch_matvec_t(unsigned grid, cudaStream_t s, const float* A, int64_t n,
                     const double* lambda, const float* B, const double* X, const float2* xs,
                     int64_t m, int subtract, double* out, float* out32, const PcgState* st) {
  matvec_df_rows_kernel<MR><<<grid, 256, 0, s>>>(A, n, lambda, B, X, xs, m, subtract, out,
                                                 out32, st);
}

void launch_matvec(int64_t m, unsigned grid, cudaStream_t s, const float* A, int64_t n,
                   const double* lambda, const float* B, const double* X, const float2* xs,
                   int subtract, double* out, float* out32, const PcgState* st) {
  switch (m) {
#define NTG_MV(k) \
  case k: launch_matvec_t<k>(grid, s, A, n, lambda, B, X, xs, m, subtract, out, out32, st); break;
    NTG_MV(1) NTG_MV(2) NTG_MV(3) NTG_MV(4) NTG_MV(5) NTG_MV(6) NTG_MV(7) NTG_MV(8)
    NTG_MV(9) NTG_MV(10) NTG_MV(11) NTG_MV(12) NTG_MV(13) NTG_MV(14) NTG_MV(15)
#undef NTG_MV
    default: launch_matvec_t<kSmallM>(grid, s, A, n, lambda, B, X, xs, m, subtract, out, out32, st);
  }
}

// part[blk][j] = sum over the block's rows of u[i, j] * v[i, j] (v FP64, or vf FP32).
__global__ void __launch_bounds__(256)
    col_dots_kernel(const double* __restrict__ u, const double* __restrict__ v,
                    const float* __restrict__ vf, int64_t n, int64_t m, double* __restrict__ part,
                    const PcgState* st) {
  if (st && st->all_done) return;  // st == nullptr: the set-up product, always computed
  __shared__ double red[8][kSmallM];
  double acc[kSmallM];
#pragma unroll
  for (int c = 0; c < kSmallM; ++c) acc[c] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
#pragma unroll
    for (int c = 0; c < kSmallM; ++c)
      if (c < m) acc[c] = fma(u[i * m + c], vf ? (double)vf[i * m + c] : v[i * m + c], acc[c]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < kSmallM; ++c) {
    double x = acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][c] = x;
  }
  __syncthreads();
  if (threadIdx.x < m) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w][threadIdx.x];
    part[blockIdx.x * kSmallM + threadIdx.x] = t;
  }
}

__device__ __forceinline__ double sum_parts(const double* part, int c) {
  double t = 0.0;
  for (int b = 0; b < kDotBlocks; ++b) t += part[b * kSmallM + c];
  return t;
}

// Set-up: bnorm, r0norm, rho[0] = r.z (from part), p = z, every column active.
__global__ void pcg_init_kernel(const float* __restrict__ B, const float* __restrict__ z,
                                double* __restrict__ p, const double* __restrict__ r, int64_t n,
                                int64_t m, const double* __restrict__ part, PcgState* st) {
  __shared__ double bmax[kSmallM], rmax[kSmallM];
  if (threadIdx.x < kSmallM) bmax[threadIdx.x] = rmax[threadIdx.x] = 0.0;
  __syncthreads();
  for (int64_t i = threadIdx.x; i < n * m; i += blockDim.x) {
    p[i] = (double)z[i];
    const int c = (int)(i % m);
    atomicMax(reinterpret_cast<unsigned long long*>(&bmax[c]),
              (unsigned long long)__double_as_longlong(fabs((double)B[i])));
    atomicMax(reinterpret_cast<unsigned long long*>(&rmax[c]),
              (unsigned long long)__double_as_longlong(fabs(r[i])));
  }
  __syncthreads();
  if (threadIdx.x < m) {
    const int c = threadIdx.x;
    st->bnorm[c] = bmax[c];
    st->r0norm[c] = rmax[c];
    st->rbest[c] = rmax[c];
    st->stall[c] = 0;
    st->rho[0][c] = sum_parts(part, c);
    st->rmax[c] = rmax[c];
    st->active[c] = rmax[c] > kPcgFloor * bmax[c];
  }
  if (threadIdx.x == 0) st->all_done = 0;
}

// x += alpha p, r -= alpha q (alpha_c = rho_c / p.q), r32 = (float) r; the block's
// max |r_c| into rpart.
__global__ void __launch_bounds__(256)
    pcg_step_kernel(double* __restrict__ x, double* __restrict__ r, float* __restrict__ r32,
                    const double* __restrict__ p, const double* __restrict__ q, int64_t n,
                    int64_t m, const double* __restrict__ pq_part, double* __restrict__ rpart,
                    PcgState* st, int cur) {
  if (st->all_done) return;
  __shared__ double alpha[kSmallM];
  __shared__ double rmax[kSmallM];
  if (threadIdx.x < m) {
    const int c = threadIdx.x;
    const double pq = sum_parts(pq_part, c);
    alpha[c] = (st->active[c] && pq > 0.0) ? st->rho[cur][c] / pq : 0.0;
    rmax[c] = 0.0;
  }
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * m; i += stride) {
    const int c = (int)(i % m);
    const double a = alpha[c];
    x[i] = fma(a, p[i], x[i]);
    const double rv = fma(-a, q[i], r[i]);
    r[i] = rv;
    r32[i] = (float)rv;
    atomicMax(reinterpret_cast<unsigned long long*>(&rmax[c]),
              (unsigned long long)__double_as_longlong(fabs(rv)));
  }
  __syncthreads();
  if (threadIdx.x < m) rpart[blockIdx.x * kSmallM + threadIdx.x] = rmax[threadIdx.x];
}

// Convergence: max |r_c| over the blocks' maxima; a column at or below kPcgTol max |b_c|
// stops; all_done once none is left.
__global__ void pcg_check_kernel(const double* __restrict__ rpart, int64_t m, int nblocks,
                                 PcgState* st) {
  if (st->all_done) return;
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (threadIdx.x < m) {
    const int c = threadIdx.x;
    double mx = 0.0;
    for (int b = 0; b < nblocks; ++b) mx = fmax(mx, rpart[b * kSmallM + c]);
    st->rmax[c] = mx;
    // the double-float products put a floor under the residual: a column whose best
    // residual has not halved in kPcgStall iterations has reached it and stops
    if (mx < 0.5 * st->rbest[c]) {
      st->rbest[c] = mx;
      st->stall[c] = 0;
    } else {
      ++st->stall[c];
    }
    if (st->active[c] && (mx <= kPcgTol * st->r0norm[c] || mx <= kPcgFloor * st->bnorm[c] ||
                          st->stall[c] >= kPcgStall))
      st->active[c] = 0;
    if (st->active[c]) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && !any) st->all_done = 1;
}

// beta_c = (r.z)_new / rho_c; p = z + beta p; rho[nxt] = (r.z)_new.
__global__ void __launch_bounds__(256)
    pcg_dir_kernel(double* __restrict__ p, const float* __restrict__ z, int64_t n, int64_t m,
                   const double* __restrict__ rz_part, PcgState* st, int cur) {
  if (st->all_done) return;
  __shared__ double beta[kSmallM];
  const int nxt = cur ^ 1;
  if (threadIdx.x < m) {
    const int c = threadIdx.x;
    const double rz = sum_parts(rz_part, c);
    beta[c] = st->rho[cur][c] != 0.0 ? rz / st->rho[cur][c] : 0.0;
    if (blockIdx.x == 0) st->rho[nxt][c] = rz;
  }
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * m; i += stride) {
    const int c = (int)(i % m);
    if (st->active[c]) p[i] = fma(beta[c], p[i], (double)z[i]);
  }
}

__global__ void copy_to_float_kernel(const double* __restrict__ a, float* __restrict__ b,
                                     int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void logdet_ld_kernel(const float* __restrict__ L, int64_t n, int64_t ldl,
                                 double* __restrict__ out) {
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += log((double)L[i * ldl + i]);
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

int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

int set_smem(const void* fn, size_t bytes) {
  const cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return fail(NTG_ERR_CUDA, std::string("chol: ") + cudaGetErrorString(e));
  return NTG_OK;
}

int attrs_once() {
  static std::once_flag once;
  static int rc = NTG_OK;
  std::call_once(once, [] {
    rc = set_smem((const void*)diag_block_kernel, kDiagSmem);
    if (!rc) rc = set_smem((const void*)panel_trsm_kernel, kPanelSmem);
  });
  return rc;
}

// Factor workspace layout: linv [nblk * 128 * 128] f32 (inverses of the diagonal
// blocks), uinv = L^-T [n * ldl] f32 (upper), linvf = L^-1 [n * ldl] f32 (lower).
struct FactorWs {
  float* linv;
  float* uinv;
  float* linvf;
};

size_t factor_ws_bytes(int64_t n, int64_t ldl) {
  const int64_t nblk = (n + PB - 1) / PB;
  return (size_t)(nblk * PB * PB + 2 * n * ldl) * sizeof(float) + 256;
}

FactorWs factor_ws(void* ws, int64_t n, int64_t ldl) {
  const int64_t nblk = (n + PB - 1) / PB;
  char* p = static_cast<char*>(ws);
  p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~(uintptr_t)255);
  FactorWs f;
  f.linv = reinterpret_cast<float*>(p);
  f.uinv = f.linv + nblk * PB * PB;
  f.linvf = f.uinv + n * ldl;
  return f;
}

// Solve workspace: rnorm (256 B), x64 [n m] f64, r32 [n m] f32, t32 [n m] f32, then
// for m <= kSmallM the PCG vectors r64, p64, q64 [n m] f64, three dot-product partial
// arrays [kDotBlocks * kSmallM] f64, the PcgState and the double-float split of the
// current vector [n m] float2; for more, z [m * ldl] f32 and
// y [m * ldl] f32 (the transposed right-hand sides and their half-solved form).
size_t solve_ws_bytes(int64_t n, int64_t m, int64_t ldl) {
  size_t b = 256 + (size_t)n * m * (sizeof(double) + 2 * sizeof(float)) + 256;
  if (m > kSmallM) b += 2 * (size_t)m * ldl * sizeof(float) + 512;
  else b += (size_t)3 * n * m * sizeof(double) + 3 * kDotBlocks * kSmallM * sizeof(double) +
            sizeof(PcgState) + 256 + (size_t)n * m * sizeof(float2) + 256;
  return (b + 255) & ~(size_t)255;
}

// X = (L L^T)^-1 X for up to kSmallM right-hand sides: t = L^-1 X, X = L^-T t.
int inv_apply_small(cudaStream_t s, const FactorWs& f, int64_t ldl, int64_t n, float* X, int64_t m,
                    float* t, const int* skip) {
  const unsigned g = (unsigned)ceil_div(n, 8);
  const unsigned nt = 256;
  if (m == 1) {
    tri_gemv_kernel<1><<<g, nt, 0, s>>>(f.linvf, ldl, n, 0, X, m, t, skip);
    tri_gemv_kernel<1><<<g, nt, 0, s>>>(f.uinv, ldl, n, 1, t, m, X, skip);
  } else if (m <= 4) {
    tri_gemv_kernel<4><<<g, nt, 0, s>>>(f.linvf, ldl, n, 0, X, m, t, skip);
    tri_gemv_kernel<4><<<g, nt, 0, s>>>(f.uinv, ldl, n, 1, t, m, X, skip);
  } else if (m <= 10) {
    tri_gemv_kernel<10><<<g, nt, 0, s>>>(f.linvf, ldl, n, 0, X, m, t, skip);
    tri_gemv_kernel<10><<<g, nt, 0, s>>>(f.uinv, ldl, n, 1, t, m, X, skip);
  } else {
    tri_gemv_kernel<kSmallM><<<g, nt, 0, s>>>(f.linvf, ldl, n, 0, X, m, t, skip);
    tri_gemv_kernel<kSmallM><<<g, nt, 0, s>>>(f.uinv, ldl, n, 1, t, m, X, skip);
  }
  note_launch(2);
  return check_launch("ntg_chol_solve_tc apply");
}

// X = (L L^T)^-1 X for many right-hand sides on the tensor cores, through the transposed
// right-hand sides z = X^T [m, ldl]: y = z L^-T (= (L^-1 X)^T), z = y L^-1 (= X'^T).
int inv_apply_many(cudaStream_t s, const FactorWs& f, int64_t ldl, int64_t n, float* X, int64_t m,
                   float* z, float* y) {
  {
    dim3 g((unsigned)ceil_div(m, 32), (unsigned)ceil_div(n, 32));
    transpose_kernel<<<g, 256, 0, s>>>(X, m, z, ldl, n, m);
    note_launch();
  }
  // y[c, j] = sum_i z[c, i] L^-1[j, i]: NT with B = L^-1 (row-major)
  int rc = gemm_tf32x3(s, z, ldl, f.linvf, ldl, y, ldl, m, n, n, 1.f, 0.f, 0);
  if (rc) return rc;
  // z[c, i] = sum_j y[c, j] L^-T[i, j]: NT with B = L^-T (row-major)
  rc = gemm_tf32x3(s, y, ldl, f.uinv, ldl, z, ldl, m, n, n, 1.f, 0.f, 0);
  if (rc) return rc;
  {
    dim3 g((unsigned)ceil_div(n, 32), (unsigned)ceil_div(m, 32));
    transpose_kernel<<<g, 256, 0, s>>>(z, ldl, X, m, m, n);
    note_launch();
  }
  return check_launch("ntg_chol_solve_tc apply");
}

}  // namespace

int chol_take_device_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_chol_error, sizeof(int)) != cudaSuccess) return -1;
  const int zero = 0;
  if (v != 0 && cudaMemcpyToSymbol(g_chol_error, &zero, sizeof(int)) != cudaSuccess) return -1;
  return v;
}

}  // namespace ntg

using namespace ntg;

extern "C" size_t ntg_chol_factor_tc_workspace_bytes(int64_t n, int64_t ldl) {
  if (n <= 0 || ldl < n || n > 46340 || ldl > 46340 + 128) return SIZE_MAX;
  return factor_ws_bytes(n, ldl);
}

extern "C" int ntg_chol_factor_tc(void* stream, const float* A, int64_t n, double diag_reg,
                                  int32_t absolute, float* L, int64_t ldl, double* lambda,
                                  int* info, void* workspace, size_t workspace_bytes) {
  NTG_REQUIRE(A && L && lambda && info && workspace, "ntg_chol_factor_tc: null pointer");
  NTG_REQUIRE(n > 0 && n <= 46340, "ntg_chol_factor_tc: n must be in [1, 46340]");
  NTG_REQUIRE(ldl >= n && ldl % 4 == 0 && ldl <= 46340 + 128,
              "ntg_chol_factor_tc: ldl must be >= n and a multiple of 4");
  NTG_REQUIRE((reinterpret_cast<uintptr_t>(L) & 15) == 0, "ntg_chol_factor_tc: L must be 16-byte aligned");
  NTG_REQUIRE(workspace_bytes >= factor_ws_bytes(n, ldl),
              "ntg_chol_factor_tc: workspace smaller than ntg_chol_factor_tc_workspace_bytes");
  int rc = attrs_once();
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  const FactorWs f = factor_ws(workspace, n, ldl);
  if (cudaMemsetAsync(info, 0, sizeof(int), s) != cudaSuccess)
    return check_launch("ntg_chol_factor_tc memset");
  trace_tc_kernel<<<1, 1024, 0, s>>>(A, n, lambda + 1);
  init_factor_ld_kernel<<<grid_for(n * ldl), 256, 0, s>>>(A, n, ldl, diag_reg, absolute,
                                                          lambda + 1, L, lambda);
  note_launch(2);
  const int64_t nblk = (n + PB - 1) / PB;
  for (int64_t b = 0; b < nblk; ++b) {
    const int64_t k = b * PB;
    diag_block_kernel<<<1, 512, kDiagSmem, s>>>(L, ldl, n, k, info, f.linv + b * PB * PB);
    note_launch();
    const int64_t rest = n - k - PB;
    if (rest > 0) {
      const int64_t grid = mini(ceil_div(rest, 16), 2 * 152);
      panel_trsm_kernel<<<(unsigned)grid, 512, kPanelSmem, s>>>(L, ldl, n, k);
      note_launch();
      float* l21 = L + (k + PB) * ldl + k;
      rc = gemm_tf32x3(s, l21, ldl, l21, ldl, L + (k + PB) * ldl + k + PB, ldl, rest, rest, PB,
                       -1.f, 1.f, 1);
      if (rc) return rc;
    }
  }
  // L^-T by the forward block solve of L Y = I on the transposed side, Z = Y^T: per
  // block b, Z[:, b] <- Z[:, b] Linv_b^T, then Z[:, >b] -= Z[:, b] L[>b, b]^T, where only
  // the rows [0, r0 + nb) of Z[:, b] are non-zero (Z is upper triangular)
  identity_kernel<<<grid_for(n * ldl), 256, 0, s>>>(f.uinv, n, ldl);
  note_launch();
  for (int64_t b = 0; b < nblk; ++b) {
    const int64_t r0 = b * PB, nb = mini(PB, n - r0), rows = r0 + nb;
    rc = gemm_tf32x3(s, f.uinv + r0, ldl, f.linv + b * PB * PB, PB, f.uinv + r0, ldl, rows, nb,
                     nb, 1.f, 0.f, 0);
    if (rc) return rc;
    const int64_t rest = n - rows;
    if (rest > 0) {
      rc = gemm_tf32x3(s, f.uinv + r0, ldl, L + rows * ldl + r0, ldl, f.uinv + rows, ldl, rows,
                       rest, nb, -1.f, 1.f, 0);
      if (rc) return rc;
    }
  }
  dim3 g((unsigned)ceil_div(n, 32), (unsigned)ceil_div(n, 32));
  transpose_kernel<<<g, 256, 0, s>>>(f.uinv, ldl, f.linvf, ldl, n, n);
  note_launch();
  return check_launch("ntg_chol_factor_tc");
}

extern "C" size_t ntg_chol_solve_tc_workspace_bytes(int64_t n, int64_t m, int64_t ldl) {
  if (n <= 0 || m <= 0 || ldl < n || n > 46340) return SIZE_MAX;
  const uint64_t per = sizeof(double) + sizeof(float) + sizeof(float);
  if ((uint64_t)m > ((uint64_t)INT64_MAX / per) / (uint64_t)ldl) return SIZE_MAX;
  return solve_ws_bytes(n, m, ldl);
}

extern "C" int ntg_chol_solve_tc(void* stream, const float* A, const float* L, int64_t ldl,
                                 const void* factor_workspace, const double* lambda, int64_t n,
                                 const float* B, int64_t m, float* X, int32_t refine_iters,
                                 void* workspace, size_t workspace_bytes,
                                 double* final_residual) {
  NTG_REQUIRE(A && L && factor_workspace && lambda && B && X && workspace,
              "ntg_chol_solve_tc: null pointer");
  NTG_REQUIRE(n > 0 && n <= 46340 && m > 0, "ntg_chol_solve_tc: bad sizes");
  NTG_REQUIRE(ldl >= n && ldl % 4 == 0, "ntg_chol_solve_tc: bad ldl");
  NTG_REQUIRE(refine_iters >= 0 && refine_iters <= 64, "ntg_chol_solve_tc: 0..64 refinement steps");
  NTG_REQUIRE(m <= (1ll << 31) / 64, "ntg_chol_solve_tc: too many right-hand sides");
  NTG_REQUIRE(workspace_bytes >= ntg_chol_solve_tc_workspace_bytes(n, m, ldl),
              "ntg_chol_solve_tc: workspace smaller than ntg_chol_solve_tc_workspace_bytes");
  (void)L;  // the solves use the inverse factors kept in factor_workspace
  int rc = attrs_once();
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);
  const FactorWs f = factor_ws(const_cast<void*>(factor_workspace), n, ldl);
  char* ws = static_cast<char*>(workspace);
  double* rnorm = reinterpret_cast<double*>(ws);
  double* x64 = reinterpret_cast<double*>(ws + 256);
  float* r32 = reinterpret_cast<float*>(x64 + n * m);
  float* t32 = r32 + n * m;
  char* tail = reinterpret_cast<char*>(
      (reinterpret_cast<uintptr_t>(t32 + n * m) + 255) & ~(uintptr_t)255);
  float* z = reinterpret_cast<float*>(tail);
  float* y = reinterpret_cast<float*>(
      (reinterpret_cast<uintptr_t>(z + m * ldl) + 255) & ~(uintptr_t)255);
  auto apply = [&](float* xx, const int* skip) -> int {
    if (m <= kSmallM) return inv_apply_small(s, f, ldl, n, xx, m, t32, skip);
    return inv_apply_many(s, f, ldl, n, xx, m, z, y);
  };
  if (cudaMemcpyAsync(X, B, sizeof(float) * n * m, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return check_launch("ntg_chol_solve_tc copy");
  rc = apply(X, nullptr);
  if (rc) return rc;
  if (refine_iters == 0 && !final_residual) return check_launch("ntg_chol_solve_tc");
  to_double_tc_kernel<<<grid_for(n * m), 256, 0, s>>>(X, x64, n * m);
  note_launch();
  if (m <= kSmallM) {
    // preconditioned conjugate gradients on (K + lambda I) x = b from x0 = (L L^T)^-1 b
    double* r64 = reinterpret_cast<double*>(tail);
    double* p64 = r64 + n * m;
    double* q64 = p64 + n * m;
    double* part = q64 + n * m;
    double* part_rz = part + kDotBlocks * kSmallM;
    double* part_r = part_rz + kDotBlocks * kSmallM;
    PcgState* st = reinterpret_cast<PcgState*>(part_r + kDotBlocks * kSmallM);
    float2* xs = reinterpret_cast<float2*>(
        (reinterpret_cast<uintptr_t>(st + 1) + 255) & ~(uintptr_t)255);
    const unsigned rows_grid = (unsigned)ceil_div(n, 8);
    // (K + lambda I) v for v = x64 or p64 (subtract: b - ...), through the split of v
    auto matvec = [&](const double* v, int subtract, const float* bb, double* out, float* o32,
                      const PcgState* stp) {
      split_df_kernel<<<grid_for(n * m), 256, 0, s>>>(v, n * m, xs, stp);
      launch_matvec(m, rows_grid, s, A, n, lambda, bb, v, xs, subtract, out, o32, stp);
      note_launch(2);
    };
    matvec(x64, 1, B, r64, r32, nullptr);
    if (refine_iters > 0) {
      rc = apply(r32, nullptr);  // z0
      if (rc) return rc;
      col_dots_kernel<<<kDotBlocks, 256, 0, s>>>(r64, nullptr, r32, n, m, part_rz, nullptr);
      pcg_init_kernel<<<1, 1024, 0, s>>>(B, r32, p64, r64, n, m, part_rz, st);
      note_launch(2);
      for (int it = 0; it < refine_iters; ++it) {
        const int cur = it & 1;
        matvec(p64, 0, nullptr, q64, nullptr, st);
        col_dots_kernel<<<kDotBlocks, 256, 0, s>>>(p64, q64, nullptr, n, m, part, st);
        pcg_step_kernel<<<kDotBlocks, 256, 0, s>>>(x64, r64, r32, p64, q64, n, m, part, part_r,
                                                   st, cur);
        pcg_check_kernel<<<1, 32, 0, s>>>(part_r, m, kDotBlocks, st);
        note_launch(4);
        rc = apply(r32, &st->all_done);
        if (rc) return rc;
        col_dots_kernel<<<kDotBlocks, 256, 0, s>>>(r64, nullptr, r32, n, m, part_rz, st);
        pcg_dir_kernel<<<kDotBlocks, 256, 0, s>>>(p64, r32, n, m, part_rz, st, cur);
        note_launch(2);
      }
      copy_to_float_kernel<<<grid_for(n * m), 256, 0, s>>>(x64, X, n * m);
      note_launch();
    }
    if (final_residual) {
      // the true residual of the returned solution
      matvec(x64, 1, B, r64, nullptr, nullptr);
      if (cudaMemsetAsync(rnorm, 0, sizeof(double), s) != cudaSuccess)
        return check_launch("ntg_chol_solve_tc memset");
      max_abs64_kernel<<<grid_for(n * m), 256, 0, s>>>(r64, n * m, rnorm);
      note_launch(2);
      if (cudaMemcpyAsync(final_residual, rnorm, sizeof(double), cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess)
        return check_launch("ntg_chol_solve_tc residual copy");
    }
    return check_launch("ntg_chol_solve_tc");
  }
  // many right-hand sides: refine_iters steps of iterative refinement
  for (int it = 0; it <= refine_iters; ++it) {
    if (it == refine_iters && !final_residual) break;
    if (cudaMemsetAsync(rnorm, 0, sizeof(double), s) != cudaSuccess)
      return check_launch("ntg_chol_solve_tc memset");
    residual_df_kernel<<<dim3((unsigned)ceil_div(m, 64), (unsigned)ceil_div(n, 64)), 256, 0, s>>>(
        A, n, lambda, B, x64, m, r32, rnorm);
    note_launch();
    if (it == refine_iters) break;
    rc = apply(r32, nullptr);
    if (rc) return rc;
    accumulate_tc_kernel<<<grid_for(n * m), 256, 0, s>>>(x64, r32, X, n * m);
    note_launch();
  }
  if (final_residual &&
      cudaMemcpyAsync(final_residual, rnorm, sizeof(double), cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess)
    return check_launch("ntg_chol_solve_tc residual copy");
  return check_launch("ntg_chol_solve_tc");
}

extern "C" int ntg_chol_logdet_tc(void* stream, const float* L, int64_t n, int64_t ldl,
                                  double* out) {
  NTG_REQUIRE(L && out && n > 0 && ldl >= n, "ntg_chol_logdet_tc: bad arguments");
  logdet_ld_kernel<<<1, 1024, 0, as_stream(stream)>>>(L, n, ldl, out);
  note_launch();
  return check_launch("ntg_chol_logdet_tc");
}
