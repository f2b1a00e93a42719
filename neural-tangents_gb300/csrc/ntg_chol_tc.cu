// Blocked Cholesky factorisation and solves of predict.gradient_descent_mse on
// the sm_103a tensor cores (neural_tangents/_src/predict.py:1224-1258 restated
// for the GPU): A = K + lambda I = L L^T in FP32 with 128-wide panels.
//
// Per panel k:
//   diag_block_kernel   one CTA factors the 128 x 128 diagonal block (four
//                       32-wide steps, each a warp-level Cholesky + inverse in
//                       registers overlapped with the other warps' deferred
//                       updates, then the sub-panel and the next column block as
//                       register-tiled warp products in shared memory) and writes
//                       the block's inverse L11^-1;
//   gemm_tf32x3         the rows below: L21 = A21 L11^-T as a product with that
//                       inverse (in place, one 128-wide column of tiles);
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
constexpr int XP = PB + 4;     // pitch of the p-major / 16-byte-row shared-memory tiles
constexpr int kSmallM = 16;    // right-hand sides of the cooperative solves
constexpr int kGT = 128;       // rows of a split-K product tile (one per thread)
constexpr int kGK = 32;        // columns staged in shared memory per step

__device__ int g_chol_error = 0;

__host__ __device__ __forceinline__ int64_t mini(int64_t a, int64_t b) { return a < b ? a : b; }

// Grid of a grid-stride loop over n elements, 256 threads a block.
int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g > 152 * 32 ? 152 * 32 : (g < 1 ? 1 : g));
}

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

// Warp-level Cholesky of the 32 x 32 block at (o, o) of `a` and the inverse of the
// factor. Lane r holds row r in registers; each pivot is broadcast by a shuffle and each
// finished column of L is stored to lt[j][:] (zeros above the diagonal), from where the
// rank-1 update and the inverse read it as broadcast 16-byte words. The pivot uses the
// hardware reciprocal square root (2 ulp): L_jj = d rsqrt(d), L_rj = A_rj rsqrt(d); the
// reciprocal pivots are kept for the inverse, which then needs no division (the factor
// is refined against the exact kernel by the solves). Lane c computes column c of
// X = L^-1 column-sweep style (x_p = s_p / L_pp, then s_i -= L_ip x_p for every i > p),
// so the updates of a step are independent. Writes the factor into a (upper part zero)
// and X row-major into dinv (pitch 33) and into xs at (o, o) (pitch XP).
__device__ void warp_potrf_inv32(float (*a)[PBS], int o, float (*dinv)[33], float* xs,
                                 int* info, int64_t col0) {
  __shared__ __align__(16) float lt[32][36];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  float v[32], rp[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) v[c] = a[o + lane][o + c];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    float d = __shfl_sync(full, v[j], j);
    if (!(d > 0.f)) {  // the same value in every lane
      if (lane == 0) atomicCAS(info, 0, (int)(col0 + o + j + 1));
      d = 1.f;
    }
    const float rs = rsqrtf(d);
    rp[j] = rs;
    const float l = (lane == j) ? d * rs : v[j] * rs;  // lanes < j: the unused upper part
    v[j] = l;
    lt[j][lane] = lane >= j ? l : 0.f;
    __syncwarp();
#pragma unroll
    for (int q = (j + 1) / 4; q < 8; ++q) {
      const float4 c4 = *reinterpret_cast<const float4*>(&lt[j][4 * q]);
      const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (4 * q + u > j) v[4 * q + u] = fmaf(-l, cv[u], v[4 * q + u]);
    }
  }
#pragma unroll
  for (int c = 0; c < 32; ++c) a[o + lane][o + c] = (c <= lane) ? v[c] : 0.f;
  float x[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
  for (int p = 0; p < 32; ++p) {
    const float xp = x[p] * rp[p];
    x[p] = xp;
#pragma unroll
    for (int q = (p + 1) / 4; q < 8; ++q) {
      const float4 c4 = *reinterpret_cast<const float4*>(&lt[p][4 * q]);
      const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (4 * q + u > p) x[4 * q + u] = fmaf(-cv[u], xp, x[4 * q + u]);
    }
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    dinv[i][lane] = x[i];
    xs[(o + i) * XP + o + lane] = x[i];
  }
  __syncwarp();
}

// acc[i][j] += sum_{p < 32} A(r0 + i, p) B(p, c0 + j) for the 8 x 4 piece of a 32 x 32
// tile that lane (r0 / 8) * 8 + c0 / 4 owns. AP: A is p-major (A[p * lda + r], two
// 16-byte loads per p), else row-major (A[r * lda + p]); BP: B is p-major (B[p * ldb + c],
// one 16-byte load), else transposed (B[c * ldb + p]). Row-major pitches 129 / 33 and
// p-major pitch XP keep the loads of a warp free of bank conflicts.
template <bool AP, bool BP>
__device__ __forceinline__ void warp_tile_acc(float (&acc)[8][4], const float* A, int lda,
                                              const float* B, int ldb) {
  const int lane = threadIdx.x & 31;
  const int r0 = (lane >> 3) * 8, c0 = (lane & 7) * 4;
#pragma unroll 4
  for (int p = 0; p < 32; ++p) {
    float av[8], bv[4];
    if (AP) {
      const float4 x = *reinterpret_cast<const float4*>(A + p * lda + r0);
      const float4 y = *reinterpret_cast<const float4*>(A + p * lda + r0 + 4);
      av[0] = x.x; av[1] = x.y; av[2] = x.z; av[3] = x.w;
      av[4] = y.x; av[5] = y.y; av[6] = y.z; av[7] = y.w;
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) av[i] = A[(r0 + i) * lda + p];
    }
    if (BP) {
      const float4 z = *reinterpret_cast<const float4*>(B + p * ldb + c0);
      bv[0] = z.x; bv[1] = z.y; bv[2] = z.z; bv[3] = z.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = B[(c0 + j) * ldb + p];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
  }
}

__device__ __forceinline__ void zero_acc(float (&acc)[8][4]) {
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
}

// a[32 I + r][32 J + c] -= sum_p P[32 I + r][p] P[32 J + c][p], P the panel held
// p-major in pt (one warp, one 32 x 32 tile).
__device__ __forceinline__ void warp_update_tile(float (*a)[PBS], const float* pt, int I, int J) {
  const int lane = threadIdx.x & 31;
  const int r0 = (lane >> 3) * 8, c0 = (lane & 7) * 4;
  float acc[8][4];
  zero_acc(acc);
  warp_tile_acc<true, true>(acc, pt + 32 * I, XP, pt + 32 * J, XP);
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) a[32 * I + r0 + i][32 * J + c0 + j] -= acc[i][j];
}

// Factors L[k:k+nb, k:k+nb] in place (upper part zeroed) and writes the inverse of the
// factor, zero-padded to 128 x 128, to linv (row-major). Four 32-wide steps; in step sb:
//   phase A  warp 0 factors and inverts diagonal block sb (warp_potrf_inv32) while the
//            other warps apply the previous panel's update to the column blocks beyond
//            sb + 1 (deferred: only block sb + 1 must be current for the next step) and
//            form T_j = sum_{q=j}^{sb-1} L_{sb,q} X_{q,j}, j < sb, for the inverse;
//   phase B  X_{sb,j} = -Dinv_sb T_j, and the sub-panel L_{rb,sb} = A_{rb,sb} Dinv_sb^T
//            for the row blocks rb > sb (into a and, p-major, into pt);
//   phase C  the update of column block sb + 1 by panel sb.
// Every product is a 32 x 32 x 32 warp tile (warp_tile_acc). Rows beyond nb are
// padded with the identity (which factors and inverts to itself and is cut on output).
__global__ void __launch_bounds__(512, 1)
    diag_block_kernel(float* __restrict__ L, int64_t ldl, int64_t n, int64_t k, int* info,
                      float* __restrict__ linv) {
  extern __shared__ __align__(16) float sm[];
  float(*a)[PBS] = reinterpret_cast<float(*)[PBS]>(sm);  // 128 x 129, the block
  float* pt = sm + PB * PBS;                              // 32 x XP, current panel p-major
  float* xs = pt + 32 * XP;                               // 128 x XP, X = L^-1
  float* tb = xs + PB * XP;                               // 32 x XP, T_j at columns 32 j
  float(*dinv)[32][33] = reinterpret_cast<float(*)[32][33]>(tb + 32 * XP);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = (lane >> 3) * 8, c0 = (lane & 7) * 4;
  const int nb = (int)mini(PB, n - k);
  if (nb == PB) {
    // full block (16-byte aligned: ldl % 4 == 0, k % 128 == 0): all eight 16-byte loads
    // of a thread in flight at once; entries above the diagonal are not read
    float4 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + 512 * u, i = e >> 5, j = (e & 31) * 4;
      v[u] = j <= i ? *reinterpret_cast<const float4*>(L + (k + i) * ldl + k + j)
                    : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + 512 * u, i = e >> 5, j = (e & 31) * 4;
      a[i][j] = v[u].x;
      a[i][j + 1] = j + 1 <= i ? v[u].y : 0.f;
      a[i][j + 2] = j + 2 <= i ? v[u].z : 0.f;
      a[i][j + 3] = j + 3 <= i ? v[u].w : 0.f;
    }
  } else {
    for (int idx = tid; idx < PB * PB; idx += 512) {
      const int i = idx >> 7, j = idx & (PB - 1);
      float v;
      if (i < nb && j < nb) v = (j <= i) ? L[(k + i) * ldl + k + j] : 0.f;
      else v = (i == j) ? 1.f : 0.f;
      a[i][j] = v;
    }
  }
  __syncthreads();
  for (int sb = 0; sb < 4; ++sb) {
    const int o = 32 * sb;
    // ---- phase A ----
    if (warp == 0) {
      warp_potrf_inv32(a, o, dinv[sb], xs, info, k);
    } else if (sb > 0) {
      const int u = warp - 1;
      int cnt = 0;
      for (int J = sb + 1; J < 4; ++J)
        for (int I = J; I < 4; ++I, ++cnt)
          if (cnt == u) warp_update_tile(a, pt, I, J);
      for (int j = 0; j < sb; ++j, ++cnt) {
        if (cnt != u) continue;
        float acc[8][4];
        zero_acc(acc);
        for (int q = j; q < sb; ++q)
          warp_tile_acc<false, true>(acc, &a[o][32 * q], PBS, xs + 32 * q * XP + 32 * j, XP);
#pragma unroll
        for (int i = 0; i < 8; ++i)
          *reinterpret_cast<float4*>(tb + (r0 + i) * XP + 32 * j + c0) =
              make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
      }
    }
    __syncthreads();
    // ---- phase B ----
    {
      const int u = warp;
      if (u < sb) {  // X_{sb,u} = -Dinv_sb T_u
        float acc[8][4];
        zero_acc(acc);
        warp_tile_acc<false, true>(acc, &dinv[sb][0][0], 33, tb + 32 * u, XP);
#pragma unroll
        for (int i = 0; i < 8; ++i)
          *reinterpret_cast<float4*>(xs + (o + r0 + i) * XP + 32 * u + c0) =
              make_float4(-acc[i][0], -acc[i][1], -acc[i][2], -acc[i][3]);
      } else if (u < 3) {  // sub-panel row block rb = sb + 1 + (u - sb)
        const int rb = u + 1;
        if (rb > sb) {
          float acc[8][4];
          zero_acc(acc);
          warp_tile_acc<false, false>(acc, &a[32 * rb][o], PBS, &dinv[sb][0][0], 33);
          __syncwarp();
#pragma unroll
          for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) a[32 * rb + r0 + i][o + c0 + j] = acc[i][j];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            float* d = pt + (c0 + j) * XP + 32 * rb + r0;
            *reinterpret_cast<float4*>(d) = make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
            *reinterpret_cast<float4*>(d + 4) =
                make_float4(acc[4][j], acc[5][j], acc[6][j], acc[7][j]);
          }
        }
      }
    }
    __syncthreads();
    // ---- phase C ----
    if (sb < 3) {
      const int I = sb + 1 + warp;
      if (I < 4) warp_update_tile(a, pt, I, sb + 1);
      __syncthreads();
    }
  }
  // the factor (lower incl. the diagonal; upper zero) and the inverse
  if (nb == PB) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + 512 * u, i = e >> 5, j = (e & 31) * 4;
      const float4 lv = make_float4(a[i][j], j + 1 <= i ? a[i][j + 1] : 0.f,
                                    j + 2 <= i ? a[i][j + 2] : 0.f,
                                    j + 3 <= i ? a[i][j + 3] : 0.f);
      *reinterpret_cast<float4*>(L + (k + i) * ldl + k + j) =
          j <= i ? lv : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 xv = (j >> 5) <= (i >> 5) ? *reinterpret_cast<const float4*>(xs + i * XP + j)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
      *reinterpret_cast<float4*>(linv + i * PB + j) = xv;
    }
  } else {
    for (int idx = tid; idx < nb * nb; idx += 512) {
      const int i = idx / nb, j = idx - i * nb;
      L[(k + i) * ldl + k + j] = (j <= i) ? a[i][j] : 0.f;
    }
    for (int idx = tid; idx < PB * PB; idx += 512) {
      const int i = idx >> 7, j = idx & (PB - 1);
      const bool in = i < nb && j < nb && (j >> 5) <= (i >> 5);
      linv[idx] = in ? xs[i * XP + j] : 0.f;
    }
  }
}

constexpr size_t kDiagSmem = (size_t)(PB * PBS + 32 * XP + PB * XP + 32 * XP + 4 * 32 * 33) *
                             sizeof(float);

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


__device__ __forceinline__ P2 neg2(P2 x) {
  P2 r;
  asm("xor.b64 %0, %1, 0x8000000080000000;" : "=l"(r.v) : "l"(x.v));
  return r;
}

// Double-float multiply-add on two lanes at once: (sh, sl) += a (xh + xl) with a FP32 and
// (xh, xl), (sh, sl) double-float pairs: the product a xh split exactly into ph + pl by a
// fused multiply-add, a xl added to pl, ph added to sh by the error-free two-sum (its
// rounding error to the low word), as in the accurate dot products of Ogita, Rump and
// Oishi (2005).
__device__ __forceinline__ void df_fma2(P2 a, P2 xh, P2 xl, P2& sh, P2& sl) {
  const P2 ph = mul2(a, xh);
  P2 pl = fma2(a, xh, neg2(ph));
  pl = fma2(a, xl, pl);
  const P2 sum = add2(sh, ph);
  const P2 bv = sub2(sum, sh);
  const P2 e = add2(sub2(sh, sub2(sum, bv)), sub2(ph, bv));
  sl = add2(sl, add2(e, pl));
  sh = sum;
}

// Double-float residual over 64 x 64 tiles of (row, column): R = B - (A + lambda I) X
// (B64 in place of B when given),
// the products taken with X's double-float split xs (split_df_kernel: split once, not
// once per tile). Each thread keeps 4 x 4 sums as 4 x 2 packed pairs of columns
// (df_fma2); rnorm receives max |R|.
__global__ void __launch_bounds__(256)
    residual_df_kernel(const float* __restrict__ A, int64_t n, const double* lambda,
                       const float* __restrict__ B, const double* __restrict__ B64,
                       const double* __restrict__ X,
                       const float2* __restrict__ xs, int64_t m, float* __restrict__ R,
                       double* __restrict__ rnorm) {
  __shared__ float As[16][64 + 1];   // [k][i]
  __shared__ float Xh[16][64 + 1];   // [k][j]
  __shared__ float Xl[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  P2 sh[4][2], sl[4][2];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) sh[u][v] = sl[u][v] = p2s(0.f);
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      const int i = idx / 16, k = idx % 16;
      As[k][i] = (i0 + i < n && k0 + k < n) ? A[(i0 + i) * n + k0 + k] : 0.f;
      const int kk = idx / 64, j = idx % 64;
      const float2 xv = (k0 + kk < n && j0 + j < m) ? xs[(k0 + kk) * m + j0 + j]
                                                    : make_float2(0.f, 0.f);
      Xh[kk][j] = xv.x;
      Xl[kk][j] = xv.y;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      P2 av[4], hv[2], lv[2];
#pragma unroll
      for (int u = 0; u < 4; ++u) av[u] = p2s(As[k][ty * 4 + u]);
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        hv[v] = p2(Xh[k][tx * 4 + 2 * v], Xh[k][tx * 4 + 2 * v + 1]);
        lv[v] = p2(Xl[k][tx * 4 + 2 * v], Xl[k][tx * 4 + 2 * v + 1]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) df_fma2(av[u], hv[v], lv[v], sh[u][v], sl[u][v]);
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
      float h0, h1, l0, l1;
      p2u(sh[u][v >> 1], h0, h1);
      p2u(sl[u][v >> 1], l0, l1);
      const double ax = (v & 1) ? (double)h1 + (double)l1 : (double)h0 + (double)l0;
      const double b = B64 ? B64[i * m + j] : (double)B[i * m + j];
      const double r = b - ax - lambda[0] * X[i * m + j];
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

// Columns [0, mc) of X (FP64 [n, ldx]) as double-float pairs xs[j, c] = (hi, lo) (pitch
// mc), split once per product so that the row kernel below runs on the FP32 pipes only.
__global__ void split_df_kernel(const double* __restrict__ X, int64_t ldx, int64_t n, int64_t mc,
                                float2* __restrict__ xs, const PcgState* st) {
  if (st && st->all_done) return;
  const int64_t total = n * mc;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / mc, c = i - j * mc;
    const double v = X[j * ldx + c];
    const float h = (float)v;
    xs[i] = make_float2(h, (float)(v - (double)h));
  }
}

// Skinny products with up to MR <= 16 right-hand sides, split along the columns so that
// the grid holds enough tiles to keep every SM busy: tile (rb, kb) covers rows
// [128 rb, 128 rb + 128) and columns [ks kb, ks kb + ks) of M [rows, ncols] (row pitch
// ld, ks a multiple of 32 from split_ks); one thread per row. Each 32-column step of M
// is staged in shared memory from coalesced 16-byte loads (row pitch 33: thread t reads
// its row without bank conflicts), the next step's loads already in flight in registers
// while the current one is multiplied; the matching 32 rows of x are padded to MRP = MR
// rounded up to 4 and read as broadcast 16-byte words. The tile's sums go to
// part[kb][i][c] (FP32) or part2 (double-float pairs); a reduction kernel adds a row's
// tiles in order, so the result does not depend on scheduling. tri 1 (lower: M[i, j] = 0
// for j > i) and 2 (upper: 0 for j < i) skip the tiles outside the triangle. DF: x given
// as its double-float split xs, every product accumulated in double-float (df_fma2: two
// right-hand sides per packed f32x2 instruction); else x FP32 (X) and plain FMA.
template <int MR, bool DF>
__global__ void __launch_bounds__(kGT)
    gemv_part_kernel(const float* __restrict__ M, int64_t ld, int64_t rows, int64_t ncols,
                     int64_t ks, int tri, const float* __restrict__ X,
                     const float2* __restrict__ xs, int64_t m, float* __restrict__ part,
                     float2* __restrict__ part2, const int* skip) {
  if (skip && *skip) return;
  constexpr int MRP = (MR + 3) & ~3;
  constexpr int NP = (MR + 1) / 2;           // packed column pairs (DF)
  constexpr int NL = kGT * kGK / 4 / kGT;    // 16-byte loads of M per thread and step
  const int64_t r0 = (int64_t)blockIdx.y * kGT, j0 = (int64_t)blockIdx.x * ks;
  if ((tri == 1 && j0 > r0 + kGT - 1) || (tri == 2 && j0 + ks <= r0)) return;
  __shared__ float ms[kGT][kGK + 1];
  __shared__ __align__(16) float xh[kGK][MRP];
  __shared__ __align__(16) float xl[DF ? kGK : 1][DF ? MRP : 4];
  const int t = threadIdx.x;
  // 16-byte loads of M need a pitch of a multiple of 4 floats and an aligned base
  const bool vec = (ld & 3) == 0 && (reinterpret_cast<uintptr_t>(M) & 15) == 0;
  float acc[MR];
  P2 sh2[NP], sl2[NP];
#pragma unroll
  for (int c = 0; c < MR; ++c) acc[c] = 0.f;
#pragma unroll
  for (int q = 0; q < NP; ++q) sh2[q] = sl2[q] = p2s(0.f);
  float4 pre[NL];
  // M[r0 .. r0 + 128)[jb .. jb + 32) into pre: a warp covers 4 rows of 128 bytes
  auto load_step = [&](int64_t jb) {
#pragma unroll
    for (int u = 0; u < NL; ++u) {
      const int e = t + u * kGT;
      const int64_t row = r0 + (e >> 3), col = jb + (e & 7) * 4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row < rows && col < ncols) {
        const float* src = M + row * ld + col;
        if (vec) {
          v = *reinterpret_cast<const float4*>(src);
          // columns beyond ncols (inside the row pitch) are not part of M
          if (col + 1 >= ncols) v.y = 0.f;
          if (col + 2 >= ncols) v.z = 0.f;
          if (col + 3 >= ncols) v.w = 0.f;
        } else {
          v.x = src[0];
          if (col + 1 < ncols) v.y = src[1];
          if (col + 2 < ncols) v.z = src[2];
          if (col + 3 < ncols) v.w = src[3];
        }
      }
      pre[u] = v;
    }
  };
  const int64_t jend = mini(j0 + ks, ncols);
  if (j0 < jend) load_step(j0);
  for (int64_t jb = j0; jb < jend; jb += kGK) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < NL; ++u) {
      const int e = t + u * kGT;
      const int r = e >> 3, j = (e & 7) * 4;
      ms[r][j] = pre[u].x;
      ms[r][j + 1] = pre[u].y;
      ms[r][j + 2] = pre[u].z;
      ms[r][j + 3] = pre[u].w;
    }
    for (int e = t; e < kGK * MRP; e += kGT) {
      const int j = e / MRP, c = e - j * MRP;
      const bool in = jb + j < ncols && c < m;
      if (DF) {
        const float2 v = in ? xs[(jb + j) * m + c] : make_float2(0.f, 0.f);
        xh[j][c] = v.x;
        xl[j][c] = v.y;
      } else {
        xh[j][c] = in ? X[(jb + j) * m + c] : 0.f;
      }
    }
    __syncthreads();
    if (jb + kGK < jend) load_step(jb + kGK);  // in flight during the products below
#pragma unroll 4
    for (int j = 0; j < kGK; ++j) {
      const float a = ms[t][j];
      if (DF) {
        const P2 a2 = p2s(a);
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const P2 h = p2ld(&xh[j][2 * q]), l = p2ld(&xl[j][2 * q]);
          df_fma2(a2, h, l, sh2[q], sl2[q]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < MRP / 4; ++q) {
          const float4 h = *reinterpret_cast<const float4*>(&xh[j][4 * q]);
          const float hv[4] = {h.x, h.y, h.z, h.w};
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (4 * q + u < MR) acc[4 * q + u] = fmaf(a, hv[u], acc[4 * q + u]);
        }
      }
    }
  }
  const int64_t row = r0 + t;
  if (row >= rows) return;
  const int64_t o = ((int64_t)blockIdx.x * rows + row) * m;
  if (DF) {
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      float h0, h1, l0, l1;
      p2u(sh2[q], h0, h1);
      p2u(sl2[q], l0, l1);
      if (2 * q < m) part2[o + 2 * q] = make_float2(h0, l0);
      if (2 * q + 1 < m) part2[o + 2 * q + 1] = make_float2(h1, l1);
    }
  } else {
#pragma unroll
    for (int c = 0; c < MR; ++c) {
      if (c >= m) break;
      part[o + c] = acc[c];
    }
  }
}

// Column-block width of a split-K product: about `tiles` tiles (1216 tiles of 4 warps:
// 8 resident warps per SM scheduler on 152 SMs; a triangle asks for twice as many, half
// of them lying outside it), a multiple of the 32-column step.
int64_t split_ks(int64_t rows, int64_t ncols, int64_t tiles) {
  const int64_t nrb = ceil_div(rows, kGT);
  const int64_t ks = ceil_div(ceil_div(ncols * nrb, tiles), kGK) * kGK;
  return ks < kGK ? kGK : ks;
}
constexpr int64_t kFullTiles = 1216, kTriTiles = 2432;

// The tiles of a row that gemv_part_kernel computed: [kb_lo, kb_hi).
__device__ __forceinline__ void tile_range(int64_t row, int tri, int ks, int64_t nkb,
                                           int64_t& lo, int64_t& hi) {
  lo = tri == 2 ? row / ks : 0;
  hi = tri == 1 ? row / ks + 1 : nkb;
}

// Y[i, c] = sum of the row's tiles, in tile order (FP32 products).
__global__ void gemv_reduce_kernel(const float* __restrict__ part, int64_t rows, int64_t m,
                                   int tri, int ks, int64_t nkb, float* __restrict__ Y,
                                   const int* skip) {
  if (skip && *skip) return;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < rows * m;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx / m;
    int64_t lo, hi;
    tile_range(row, tri, ks, nkb, lo, hi);
    float v = 0.f;
    for (int64_t kb = lo; kb < hi; ++kb) v += part[kb * rows * m + idx];
    Y[idx] = v;
  }
}

// Double-float products, finished: v = sum of the row's tiles (+ lambda X[i, c] when
// lambda is given: the square (K + lambda I) x), then out = v (mode 0), b - v (mode 1)
// or b + v (mode 2), b = B64 when given, else B (nullable: 0), as FP64 (out) and / or
// FP32 (out32). B, B64, X, out and out32 have row pitch ldo (the tiles' pitch is m).
__global__ void df_reduce_kernel(const float2* __restrict__ part2, int64_t rows, int64_t m,
                                 int64_t nkb, const double* lambda, const float* __restrict__ B,
                                 const double* __restrict__ B64, const double* __restrict__ X,
                                 int64_t ldo, int mode,
                                 double* __restrict__ out, float* __restrict__ out32,
                                 const int* skip) {
  if (skip && *skip) return;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < rows * m;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = idx / m, c = idx - row * m, o = row * ldo + c;
    float hi = 0.f, lo = 0.f;
    for (int64_t kb = 0; kb < nkb; ++kb) {
      const float2 p = part2[kb * rows * m + idx];
      df_add(hi, lo, p.x, p.y);
    }
    double v = (double)hi + (double)lo;
    if (lambda) v += lambda[0] * X[o];
    const double b = B64 ? B64[o] : B ? (double)B[o] : 0.0;
    const double r = mode == 1 ? b - v : mode == 2 ? b + v : v;
    if (out) out[o] = r;
    if (out32) out32[o] = (float)r;
  }
}

template <int MR>
void launch_df_part(cudaStream_t s, dim3 grid, const float* A, int64_t lda, int64_t rows,
                    int64_t ncols, int64_t ks, const float2* xs, int64_t m, float2* part2,
                    const int* skip) {
  gemv_part_kernel<MR, true><<<grid, kGT, 0, s>>>(A, lda, rows, ncols, ks, 0, nullptr, xs, m,
                                                  nullptr, part2, skip);
}

size_t tri_part_bytes(int64_t n, int64_t m) {
  return (size_t)ceil_div(n, split_ks(n, n, kTriTiles)) * n * m * sizeof(float);
}

size_t df_part_bytes(int64_t rows, int64_t ncols, int64_t m) {
  return (size_t)ceil_div(ncols, split_ks(rows, ncols, kFullTiles)) * rows * m * sizeof(float2);
}

// out = mode(B, (A + [lambda I]) x) for x [ncols, m <= kSmallM] given as its split xs:
// gemv_part_kernel in double-float, then df_reduce_kernel. part2: df_part_bytes.
void launch_matvec(cudaStream_t s, const float* A, int64_t lda, int64_t rows, int64_t ncols,
                   const double* lambda, const float* B, const double* B64, const double* X,
                   const float2* xs,
                   int64_t m, int64_t ldo, int mode, double* out, float* out32, float2* part2,
                   const PcgState* st) {
  const int* skip = st ? &st->all_done : nullptr;
  const int64_t ks = split_ks(rows, ncols, kFullTiles), nkb = ceil_div(ncols, ks);
  const dim3 grid((unsigned)nkb, (unsigned)ceil_div(rows, kGT));
  switch (m) {
#define NTG_MV(k) \
  case k: launch_df_part<k>(s, grid, A, lda, rows, ncols, ks, xs, m, part2, skip); break;
    NTG_MV(1) NTG_MV(2) NTG_MV(3) NTG_MV(4) NTG_MV(5) NTG_MV(6) NTG_MV(7) NTG_MV(8)
    NTG_MV(9) NTG_MV(10) NTG_MV(11) NTG_MV(12) NTG_MV(13) NTG_MV(14) NTG_MV(15)
#undef NTG_MV
    default: launch_df_part<kSmallM>(s, grid, A, lda, rows, ncols, ks, xs, m, part2, skip);
  }
  df_reduce_kernel<<<grid_for(rows * m), 256, 0, s>>>(part2, rows, m, nkb, lambda, B, B64, X,
                                                      ldo, mode, out, out32, skip);
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
  });
  return rc;
}

// Per-device streams and events of the factorisation: the critical chain (diagonal
// block, panel product, update of the next column block) on a high-priority stream,
// the bulk of each trailing update on a second stream one panel behind it, and the
// inverse factor L^-T, block by block as the panels become final, on a third.
struct SideStream {
  cudaStream_t hi = nullptr, trail = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, panel = nullptr, trail_done = nullptr;
  cudaEvent_t join[3] = {nullptr, nullptr, nullptr};
  // held while one factorisation enqueues its work: the events are re-recorded per panel,
  // and two host threads interleaving their records and waits would order each other's
  // launches (a wait, once enqueued, is not affected by a later record)
  std::mutex enqueue;
};

int side_stream(SideStream** out) {
  static std::mutex mu;
  static SideStream per_dev[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return fail(NTG_ERR_CUDA, "chol: no current device");
  std::lock_guard<std::mutex> lock(mu);
  SideStream& ss = per_dev[dev];
  if (!ss.hi) {
    int least = 0, greatest = 0;
    bool ok = cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess;
    ok = ok && cudaStreamCreateWithPriority(&ss.hi, cudaStreamNonBlocking, greatest) == cudaSuccess;
    ok = ok && cudaStreamCreateWithPriority(&ss.trail, cudaStreamNonBlocking, least) == cudaSuccess;
    ok = ok && cudaStreamCreateWithPriority(&ss.side, cudaStreamNonBlocking, least) == cudaSuccess;
    cudaEvent_t* evs[6] = {&ss.fork, &ss.panel, &ss.trail_done, &ss.join[0], &ss.join[1],
                           &ss.join[2]};
    for (cudaEvent_t* e : evs)
      ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      ss.hi = nullptr;
      return fail(NTG_ERR_CUDA, "chol: stream creation failed");
    }
  }
  *out = &ss;
  return NTG_OK;
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
// current vector [n m] float2, and the split-K tiles of the triangular and double-float
// products; for more, z [m * ldl] f32, y [m * ldl] f32 (the transposed right-hand sides
// and their half-solved form) and the double-float split of x [n m] float2.
size_t solve_ws_bytes(int64_t n, int64_t m, int64_t ldl) {
  size_t b = 256 + (size_t)n * m * (sizeof(double) + 2 * sizeof(float)) + 256;
  if (m > kSmallM) b += 2 * (size_t)m * ldl * sizeof(float) + 512 + (size_t)n * m * sizeof(float2);
  else b += (size_t)3 * n * m * sizeof(double) + 3 * kDotBlocks * kSmallM * sizeof(double) +
            sizeof(PcgState) + 256 + (size_t)n * m * sizeof(float2) + 256 +
            tri_part_bytes(n, m) + 256 + df_part_bytes(n, n, m) + 256;
  return (b + 255) & ~(size_t)255;
}

// X = (L L^T)^-1 X for up to kSmallM right-hand sides: t = L^-1 X, X = L^-T t, each a
// split-K triangular product (gemv_part_kernel) and its reduction; tpart holds
// tri_part_bytes(n, m).
template <int MR>
void launch_tri_part(cudaStream_t s, dim3 grid, const float* M, int64_t ld, int64_t n,
                     int64_t ks, int tri, const float* X, int64_t m, float* part,
                     const int* skip) {
  gemv_part_kernel<MR, false><<<grid, kGT, 0, s>>>(M, ld, n, n, ks, tri, X, nullptr, m, part,
                                                   nullptr, skip);
}

int inv_apply_small(cudaStream_t s, const FactorWs& f, int64_t ldl, int64_t n, float* X, int64_t m,
                    float* t, float* tpart, const int* skip) {
  const int64_t ks = split_ks(n, n, kTriTiles), nkb = ceil_div(n, ks);
  const dim3 grid((unsigned)nkb, (unsigned)ceil_div(n, kGT));
  auto tri = [&](const float* M, int tri, const float* in, float* out) {
    if (m == 1) launch_tri_part<1>(s, grid, M, ldl, n, ks, tri, in, m, tpart, skip);
    else if (m <= 4) launch_tri_part<4>(s, grid, M, ldl, n, ks, tri, in, m, tpart, skip);
    else if (m <= 10) launch_tri_part<10>(s, grid, M, ldl, n, ks, tri, in, m, tpart, skip);
    else launch_tri_part<kSmallM>(s, grid, M, ldl, n, ks, tri, in, m, tpart, skip);
    gemv_reduce_kernel<<<grid_for(n * m), 256, 0, s>>>(tpart, n, m, tri, (int)ks, nkb, out, skip);
  };
  tri(f.linvf, 1, X, t);  // L^-1: lower
  tri(f.uinv, 2, t, X);   // L^-T: upper
  note_launch(4);
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
  SideStream* ss = nullptr;
  rc = side_stream(&ss);
  if (rc) return rc;
  std::lock_guard<std::mutex> enqueue_lock(ss->enqueue);
  // L^-T by the forward block solve of L Y = I on the transposed side, Z = Y^T: per
  // block b, Z[:, b] <- Z[:, b] Linv_b^T, then Z[:, >b] -= Z[:, b] L[>b, b]^T, where only
  // the rows [0, r0 + nb) of Z[:, b] are non-zero (Z is upper triangular). Step b reads
  // panel b and Linv_b only, which no later panel changes.
  identity_kernel<<<grid_for(n * ldl), 256, 0, s>>>(f.uinv, n, ldl);
  note_launch();
  auto record_wait = [](cudaEvent_t e, cudaStream_t from, cudaStream_t to) {
    return cudaEventRecord(e, from) == cudaSuccess && cudaStreamWaitEvent(to, e, 0) == cudaSuccess;
  };
  if (!record_wait(ss->fork, s, ss->hi) || cudaStreamWaitEvent(ss->trail, ss->fork, 0) ||
      cudaStreamWaitEvent(ss->side, ss->fork, 0))
    return check_launch("ntg_chol_factor_tc fork");
  // every return after the fork joins the three streams back into s
  auto join = [&]() -> int {
    const cudaStream_t from[3] = {ss->hi, ss->trail, ss->side};
    for (int i = 0; i < 3; ++i)
      if (!record_wait(ss->join[i], from[i], s)) return check_launch("ntg_chol_factor_tc join");
    return NTG_OK;
  };
  // Step b on the high-priority stream: diagonal block, L21 = A21 L11^-T, then (after the
  // previous panel's trailing update, which also wrote it) the update of column block
  // b + 1 only, so that block b + 1 can be factored at once; the trailing update of the
  // columns beyond (rows and columns >= k + 2 PB) runs on the trailing stream meanwhile.
  const int64_t nblk = (n + PB - 1) / PB;
  for (int64_t b = 0; b < nblk; ++b) {
    const int64_t k = b * PB;
    diag_block_kernel<<<1, 512, kDiagSmem, ss->hi>>>(L, ldl, n, k, info, f.linv + b * PB * PB);
    note_launch();
    const int64_t rest = n - k - PB;
    float* l21 = L + (k + PB) * ldl + k;
    if (rest > 0) {
      // in place (n = 128 columns: each tile row is read before it is written)
      rc = gemm_tf32x3(ss->hi, l21, ldl, f.linv + b * PB * PB, PB, l21, ldl, rest, PB, PB, 1.f,
                       0.f, 0);
      if (rc) return join(), rc;
    }
    if (!record_wait(ss->panel, ss->hi, ss->side) ||
        cudaStreamWaitEvent(ss->trail, ss->panel, 0) != cudaSuccess)
      return join(), check_launch("ntg_chol_factor_tc panel event");
    {
      const int64_t r0 = k, nb = mini(PB, n - r0), rows = r0 + nb;
      rc = gemm_tf32x3(ss->side, f.uinv + r0, ldl, f.linv + b * PB * PB, PB, f.uinv + r0, ldl,
                       rows, nb, nb, 1.f, 0.f, 0);
      if (rc) return join(), rc;
      if (n - rows > 0) {
        rc = gemm_tf32x3(ss->side, f.uinv + r0, ldl, L + rows * ldl + r0, ldl, f.uinv + rows,
                         ldl, rows, n - rows, nb, -1.f, 1.f, 0);
        if (rc) return join(), rc;
      }
    }
    if (rest > 0) {
      const int64_t nb1 = mini(PB, rest), far = rest - nb1;
      if (far > 0) {
        float* l31 = l21 + nb1 * ldl;
        rc = gemm_tf32x3(ss->trail, l31, ldl, l31, ldl, L + (k + PB + nb1) * ldl + k + PB + nb1,
                         ldl, far, far, PB, -1.f, 1.f, 1);
        if (rc) return join(), rc;
      }
      // column block b + 1 after the trailing update of panel b - 1 (recorded last step)
      if (b > 0 && cudaStreamWaitEvent(ss->hi, ss->trail_done, 0) != cudaSuccess)
        return join(), check_launch("ntg_chol_factor_tc trail event");
      if (cudaEventRecord(ss->trail_done, ss->trail) != cudaSuccess)
        return join(), check_launch("ntg_chol_factor_tc trail event");
      rc = gemm_tf32x3(ss->hi, l21, ldl, l21, ldl, L + (k + PB) * ldl + k + PB, ldl, rest, nb1,
                       PB, -1.f, 1.f, 0);
      if (rc) return join(), rc;
    }
  }
  rc = join();
  if (rc) return rc;
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
                                 double* final_residual, double* x64_out, const double* B64) {
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
  auto align256 = [](const void* p) {
    return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~(uintptr_t)255);
  };
  // m <= kSmallM: the PCG vectors and the products' split-K tiles
  double* r64 = reinterpret_cast<double*>(tail);
  double* p64 = r64 + n * m;
  double* q64 = p64 + n * m;
  double* part = q64 + n * m;
  double* part_rz = part + kDotBlocks * kSmallM;
  double* part_r = part_rz + kDotBlocks * kSmallM;
  PcgState* st = reinterpret_cast<PcgState*>(part_r + kDotBlocks * kSmallM);
  float2* xs = reinterpret_cast<float2*>(align256(st + 1));
  float* tpart = reinterpret_cast<float*>(align256(xs + n * m));
  float2* dpart = reinterpret_cast<float2*>(align256(reinterpret_cast<char*>(tpart) +
                                                     tri_part_bytes(n, m)));
  auto apply = [&](float* xx, const int* skip) -> int {
    if (m <= kSmallM) return inv_apply_small(s, f, ldl, n, xx, m, t32, tpart, skip);
    return inv_apply_many(s, f, ldl, n, xx, m, z, y);
  };
  if (cudaMemcpyAsync(X, B, sizeof(float) * n * m, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return check_launch("ntg_chol_solve_tc copy");
  rc = apply(X, nullptr);
  if (rc) return rc;
  if (refine_iters == 0 && !final_residual) {
    if (x64_out) {
      to_double_tc_kernel<<<grid_for(n * m), 256, 0, s>>>(X, x64_out, n * m);
      note_launch();
    }
    return check_launch("ntg_chol_solve_tc");
  }
  to_double_tc_kernel<<<grid_for(n * m), 256, 0, s>>>(X, x64, n * m);
  note_launch();
  // the FP64 solution, for products that must keep its precision (ntg_gemm_df)
  auto copy_x64 = [&]() -> int {
    if (x64_out && cudaMemcpyAsync(x64_out, x64, sizeof(double) * n * m,
                                   cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return check_launch("ntg_chol_solve_tc solution copy");
    return NTG_OK;
  };
  if (m <= kSmallM) {
    // preconditioned conjugate gradients on (K + lambda I) x = b from x0 = (L L^T)^-1 b;
    // (K + lambda I) v for v = x64 or p64 (subtract: b - ...), through the split of v
    auto matvec = [&](const double* v, int subtract, const float* bb, double* out, float* o32,
                      const PcgState* stp) {
      split_df_kernel<<<grid_for(n * m), 256, 0, s>>>(v, m, n, m, xs, stp);
      launch_matvec(s, A, n, n, n, lambda, bb, bb ? B64 : nullptr, v, xs, m, m, subtract, out, o32,
                    dpart, stp);
      note_launch(3);
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
    rc = copy_x64();
    if (rc) return rc;
    return check_launch("ntg_chol_solve_tc");
  }
  // many right-hand sides: refine_iters steps of iterative refinement
  float2* xsplit = reinterpret_cast<float2*>(align256(y + m * ldl));
  for (int it = 0; it <= refine_iters; ++it) {
    if (it == refine_iters && !final_residual) break;
    if (cudaMemsetAsync(rnorm, 0, sizeof(double), s) != cudaSuccess)
      return check_launch("ntg_chol_solve_tc memset");
    split_df_kernel<<<grid_for(n * m), 256, 0, s>>>(x64, m, n, m, xsplit, nullptr);
    residual_df_kernel<<<dim3((unsigned)ceil_div(m, 64), (unsigned)ceil_div(n, 64)), 256, 0, s>>>(
        A, n, lambda, B, B64, x64, xsplit, m, r32, rnorm);
    note_launch(2);
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
  rc = copy_x64();
  if (rc) return rc;
  return check_launch("ntg_chol_solve_tc");
}

extern "C" size_t ntg_gemm_df_workspace_bytes(int64_t rows, int64_t n, int64_t m) {
  if (rows <= 0 || n <= 0 || m <= 0) return SIZE_MAX;
  const int64_t mc = mini(m, kSmallM);
  return (size_t)n * mc * sizeof(float2) + 256 + df_part_bytes(rows, n, mc) + 256;
}

extern "C" int ntg_gemm_df(void* stream, const float* A, int64_t lda, int64_t rows, int64_t n,
                           const double* X, int64_t m, const float* Y0, float* Y, double* Y64,
                           void* workspace, size_t workspace_bytes) {
  NTG_REQUIRE(A && X && (Y || Y64) && workspace, "ntg_gemm_df: null pointer");
  NTG_REQUIRE(rows > 0 && n > 0 && m > 0 && lda >= n, "ntg_gemm_df: bad sizes");
  NTG_REQUIRE(workspace_bytes >= ntg_gemm_df_workspace_bytes(rows, n, m),
              "ntg_gemm_df: workspace smaller than ntg_gemm_df_workspace_bytes");
  cudaStream_t s = as_stream(stream);
  float2* xs = reinterpret_cast<float2*>(
      (reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255);
  float2* dpart = reinterpret_cast<float2*>(
      (reinterpret_cast<uintptr_t>(xs + n * mini(m, kSmallM)) + 255) & ~(uintptr_t)255);
  for (int64_t c0 = 0; c0 < m; c0 += kSmallM) {
    const int64_t mc = mini(kSmallM, m - c0);
    split_df_kernel<<<grid_for(n * mc), 256, 0, s>>>(X + c0, m, n, mc, xs, nullptr);
    launch_matvec(s, A, lda, rows, n, nullptr, Y0 ? Y0 + c0 : nullptr, nullptr, nullptr, xs, mc,
                  m, 2, Y64 ? Y64 + c0 : nullptr, Y ? Y + c0 : nullptr, dpart, nullptr);
    note_launch(3);
  }
  return check_launch("ntg_gemm_df");
}

extern "C" int ntg_chol_logdet_tc(void* stream, const float* L, int64_t n, int64_t ldl,
                                  double* out) {
  NTG_REQUIRE(L && out && n > 0 && ldl >= n, "ntg_chol_logdet_tc: bad arguments");
  logdet_ld_kernel<<<1, 1024, 0, as_stream(stream)>>>(L, n, ldl, out);
  note_launch();
  return check_launch("ntg_chol_logdet_tc");
}
