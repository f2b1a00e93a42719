// Symmetric eigendecomposition for the finite-time predictions of
// predict.gradient_descent_mse and gradient_descent_mse_ensemble
// (neural_tangents/_src/predict.py:185-229, 1180-1221, where the reference calls
// eigh): two-sided block Jacobi in FP32.
//
// The matrix (padded with zeros to a multiple of 64; padded indices never couple
// to the others, so they stay exact unit vectors) is split into 32-wide blocks.
// A sweep pairs every two blocks once, in the round-robin order of a tournament
// (nb - 1 rounds of nb / 2 disjoint pairs). In a round:
//   jacobi_inner_kernel   one CTA per pair runs up to two sweeps of cyclic parallel
//                         Jacobi on the 64 x 64 matrix of its two blocks in shared
//                         memory and writes the accumulated rotation U (64 x 64);
//                         what couplings remain stay in A for the next sweeps;
//   jacobi_apply_kernel   A <- U^T A U tile by tile (a 64 x 64 tile of A couples
//                         two pairs and depends only on their rotations);
//   jacobi_apply_v_kernel V <- V U.
// After each sweep off(A) / ||A||_F is read back (one 16-byte copy) and the sweeps
// stop below the tolerance. Eigenvalues are the diagonal of the final A, not sorted.
// FP32 rounding accumulates over the rounds (about 1e-5 relative at n = 1000), so the
// pairs are then refined with double-float products (see the refinement below).
#include <cmath>
#include <string>
#include <vector>

#include "ntg_common.cuh"

namespace ntg {
namespace {

constexpr int JB = 32;        // block width
constexpr int JP = 2 * JB;    // a pair: 64 indices
constexpr int JPS = JP + 1;

__host__ __device__ __forceinline__ void rr_pair(int nplayers, int round, int k, int& a, int& b) {
  // circle method: player nplayers - 1 fixed, the others rotate
  const int m = nplayers - 1;
  if (k == 0) {
    a = m;
    b = round % m;
  } else {
    a = (round + k) % m;
    b = (round - k + m) % m;
  }
  if (a > b) {
    const int t = a;
    a = b;
    b = t;
  }
}

__device__ __forceinline__ int pair_index(int pa, int pb, int l) {
  return (l < JB ? pa : pb) * JB + (l & (JB - 1));
}

// Rotation (c, s) that zeroes s_pq of [[app, apq], [apq, aqq]] (Golub & Van Loan 8.5.1);
// (1, 0) when the coupling is negligible.
__device__ __forceinline__ void sym_schur2(float app, float aqq, float apq, float tiny, float& c,
                                          float& s) {
  if (fabsf(apq) <= tiny) {
    c = 1.f;
    s = 0.f;
    return;
  }
  const float tau = (aqq - app) / (2.f * apq);
  const float t = copysignf(1.f, tau) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.f)));
  c = 1.f / sqrtf(fmaf(t, t, 1.f));
  s = t * c;
}

// One CTA per pair of blocks: S = A[idx, idx] (64 x 64), rotated in place by cyclic
// parallel Jacobi (32 disjoint rotations per round, 63 rounds per sweep) until a sweep
// leaves no coupling above 1e-5 of its pivots or `inner_sweeps` sweeps ran; U (64 x 64,
// row-major) accumulates the rotations.
__global__ void __launch_bounds__(256)
    jacobi_inner_kernel(const float* __restrict__ A, int64_t lda, int nblk, int round,
                        int inner_sweeps, float* __restrict__ Uout, const int* done) {
  if (*done) return;
  __shared__ float S[JP][JPS];
  __shared__ float U[JP][JPS];
  __shared__ float cs[JP / 2][2];
  __shared__ int pq[JP / 2][2];
  __shared__ float smax;
  int pa, pb;
  rr_pair(nblk, round, blockIdx.x, pa, pb);
  const int tid = threadIdx.x;
  for (int idx = tid; idx < JP * JP; idx += blockDim.x) {
    const int i = idx / JP, j = idx % JP;
    S[i][j] = A[(int64_t)pair_index(pa, pb, i) * lda + pair_index(pa, pb, j)];
    U[i][j] = (i == j) ? 1.f : 0.f;
  }
  if (tid == 0) smax = 0.f;
  __syncthreads();
  if (tid < JP) atomicMax(reinterpret_cast<int*>(&smax), __float_as_int(fabsf(S[tid][tid])));
  __syncthreads();
  // couplings below this are already zero at float32 resolution of the pair's matrix
  const float tiny = 1e-9f * smax;
  for (int sw = 0; sw < inner_sweeps; ++sw) {
    int rotated = 0;  // this thread's rotations of the sweep (combined below)
    for (int r = 0; r < JP - 1; ++r) {
      if (tid < JP / 2) {
        int p, q;
        rr_pair(JP, r, tid, p, q);
        float c, s;
        const float apq = S[p][q];
        const float thr = fmaxf(tiny, 1e-7f * sqrtf(fabsf(S[p][p] * S[q][q])));
        sym_schur2(S[p][p], S[q][q], apq, thr, c, s);
        // another sweep is needed while some coupling is still above 1e-5 of its pivots
        // (the smaller ones are rotated too, but leave the rest to the outer sweeps and
        // the refinement)
        if (fabsf(apq) > 1e-5f * sqrtf(fabsf(S[p][p] * S[q][q])) && fabsf(apq) > tiny)
          rotated = 1;
        cs[tid][0] = c;
        cs[tid][1] = s;
        pq[tid][0] = p;
        pq[tid][1] = q;
      }
      __syncthreads();
      // S <- J^T S J on 2 x 2 blocks (pair a rows, pair b columns)
      for (int blk = tid; blk < (JP / 2) * (JP / 2); blk += blockDim.x) {
        const int a = blk / (JP / 2), b = blk % (JP / 2);
        const int p = pq[a][0], q = pq[a][1], r2 = pq[b][0], s2 = pq[b][1];
        const float ca = cs[a][0], sa = cs[a][1], cb = cs[b][0], sb = cs[b][1];
        const float m00 = S[p][r2], m01 = S[p][s2], m10 = S[q][r2], m11 = S[q][s2];
        // columns: (x, y) -> (c x - s y, s x + c y)
        const float n00 = cb * m00 - sb * m01, n01 = sb * m00 + cb * m01;
        const float n10 = cb * m10 - sb * m11, n11 = sb * m10 + cb * m11;
        // rows
        float o00 = ca * n00 - sa * n10, o01 = ca * n01 - sa * n11;
        float o10 = sa * n00 + ca * n10, o11 = sa * n01 + ca * n11;
        if (a == b && sa != 0.f) {
          o01 = 0.f;
          o10 = 0.f;
        }
        S[p][r2] = o00;
        S[p][s2] = o01;
        S[q][r2] = o10;
        S[q][s2] = o11;
      }
      // U <- U J
      for (int e = tid; e < JP * (JP / 2); e += blockDim.x) {
        const int i = e / (JP / 2), b = e % (JP / 2);
        const int p = pq[b][0], q = pq[b][1];
        const float c = cs[b][0], s = cs[b][1];
        const float x = U[i][p], y = U[i][q];
        U[i][p] = c * x - s * y;
        U[i][q] = s * x + c * y;
      }
      __syncthreads();
    }
    // every thread's flag, combined at a barrier (no shared flag for thread 0 to reset
    // while another warp still reads it)
    if (!__syncthreads_or(rotated)) break;
  }
  float* u = Uout + (int64_t)blockIdx.x * JP * JP;
  for (int idx = tid; idx < JP * JP; idx += blockDim.x) u[idx] = U[idx / JP][idx % JP];
}

// A[rows_i, cols_j] <- U_i^T A[rows_i, cols_j] U_j for the pair tile (i, j) = blockIdx.
__global__ void __launch_bounds__(256)
    jacobi_apply_kernel(float* __restrict__ A, int64_t lda, int nblk, int round,
                        const float* __restrict__ Uall, const int* done) {
  if (*done) return;
  __shared__ float T[JP][JPS];
  __shared__ float Ui[JP][JPS];
  __shared__ float Uj[JP][JPS];
  int ia, ib, ja, jb;
  rr_pair(nblk, round, blockIdx.y, ia, ib);
  rr_pair(nblk, round, blockIdx.x, ja, jb);
  const float* ui = Uall + (int64_t)blockIdx.y * JP * JP;
  const float* uj = Uall + (int64_t)blockIdx.x * JP * JP;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < JP * JP; idx += blockDim.x) {
    const int r = idx / JP, c = idx % JP;
    T[r][c] = A[(int64_t)pair_index(ia, ib, r) * lda + pair_index(ja, jb, c)];
    Ui[r][c] = ui[idx];
    Uj[r][c] = uj[idx];
  }
  __syncthreads();
  // thread (ty, tx): rows 4 ty .. 4 ty + 3, columns tx, tx + 16, tx + 32, tx + 48
  const int tx = tid & 15, ty = tid >> 4;
  float acc[4][4];
  // W = T U_j
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  for (int k = 0; k < JP; ++k) {
    float a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = T[4 * ty + u][k];
#pragma unroll
    for (int v = 0; v < 4; ++v) b[v] = Uj[k][tx + 16 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) T[4 * ty + u][tx + 16 * v] = acc[u][v];
  __syncthreads();
  // out = U_i^T W
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  for (int k = 0; k < JP; ++k) {
    float a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = Ui[k][4 * ty + u];
#pragma unroll
    for (int v = 0; v < 4; ++v) b[v] = T[k][tx + 16 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
  // the pair's own tile keeps what the inner sweeps left of its couplings (they need not
  // have run to convergence): the outer sweeps and the off-diagonal norm see them
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v)
      A[(int64_t)pair_index(ia, ib, 4 * ty + u) * lda + pair_index(ja, jb, tx + 16 * v)] =
          acc[u][v];
}

// V[rows, cols_j] <- V[rows, cols_j] U_j for 64 consecutive rows (blockIdx.y) and pair j.
__global__ void __launch_bounds__(256)
    jacobi_apply_v_kernel(float* __restrict__ V, int64_t ldv, int nblk, int round,
                          const float* __restrict__ Uall, const int* done) {
  if (*done) return;
  __shared__ float T[JP][JPS];
  __shared__ float Uj[JP][JPS];
  int ja, jb;
  rr_pair(nblk, round, blockIdx.x, ja, jb);
  const float* uj = Uall + (int64_t)blockIdx.x * JP * JP;
  const int64_t r0 = (int64_t)blockIdx.y * JP;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < JP * JP; idx += blockDim.x) {
    const int r = idx / JP, c = idx % JP;
    T[r][c] = V[(r0 + r) * ldv + pair_index(ja, jb, c)];
    Uj[r][c] = uj[idx];
  }
  __syncthreads();
  const int tx = tid & 15, ty = tid >> 4;
  float acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
  for (int k = 0; k < JP; ++k) {
    float a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = T[4 * ty + u][k];
#pragma unroll
    for (int v = 0; v < 4; ++v) b[v] = Uj[k][tx + 16 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v)
      V[(r0 + 4 * ty + u) * ldv + pair_index(ja, jb, tx + 16 * v)] = acc[u][v];
}

// A_work = A + shift I (padded with zeros to npad), V = I.
__global__ void eigh_init_kernel(const float* __restrict__ A, int64_t n, double shift,
                                 float* __restrict__ W, float* __restrict__ V, int64_t npad) {
  const int64_t total = npad * npad;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / npad, j = idx - i * npad;
    float a = 0.f;
    if (i < n && j < n) a = (i == j) ? (float)((double)A[i * n + j] + shift) : A[i * n + j];
    W[idx] = a;
    V[idx] = (i == j) ? 1.f : 0.f;
  }
}

// norms[0] += sum of squares off the diagonal, norms[1] += on it (FP64).
__global__ void offnorm_kernel(const float* __restrict__ W, int64_t npad, double* norms) {
  double off = 0.0, on = 0.0;
  const int64_t total = npad * npad;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / npad, j = idx - i * npad;
    const double v = W[idx];
    if (i == j) on += v * v;
    else off += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    off += __shfl_xor_sync(0xffffffffu, off, o);
    on += __shfl_xor_sync(0xffffffffu, on, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&norms[0], off);
    atomicAdd(&norms[1], on);
  }
}

__global__ void eigh_extract_kernel(const float* __restrict__ W, const float* __restrict__ V,
                                    int64_t npad, int64_t n, float* __restrict__ evals,
                                    float* __restrict__ evecs) {
  const int64_t total = n * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / n, j = idx - i * n;
    evecs[idx] = V[i * npad + j];
    if (i == j) evals[i] = W[i * npad + i];
  }
}

// Spectral weights of predict.py:1277-1294 and the ensemble's covariance terms
// (predict.py:860-1005), pos = max(lambda, 0), t already scaled by the learning rate:
//   0 expm1(-pos t / N)            1 expm1(-pos t / N) / |lambda|
//   2 pos exp(-2 pos t / N)        3 exp(-pos t / N)
//   4 -expm1(-2 pos t / N) / |lambda|
//   5 -expm1(-pos t / N)           6 -expm1(-pos t / N) / |lambda|
__device__ __forceinline__ double spectral_weight(int kind, double lam, double t, double inv_norm) {
  const double pos = lam > 0.0 ? lam : 0.0;
  const double x = pos * t * inv_norm;
  switch (kind) {
    case 0: return expm1(-x);
    case 1: return expm1(-x) / fabs(lam);
    case 2: return pos * exp(-2.0 * x);
    case 3: return exp(-x);
    case 4: return -expm1(-2.0 * x) / fabs(lam);
    case 5: return -expm1(-x);
    default: return -expm1(-x) / fabs(lam);
  }
}

// out[i, t, c] = w_kind(lambda_i, t) x[i, c] for x [n, m] and times t [nt].
__global__ void spectral_scale_kernel(const float* __restrict__ evals, const double* __restrict__ ts,
                                      int64_t nt, int kind, double inv_norm,
                                      const float* __restrict__ x, int64_t n, int64_t m,
                                      float* __restrict__ out) {
  const int64_t total = n * nt * m;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx % m;
    const int64_t t = (idx / m) % nt;
    const int64_t i = idx / (m * nt);
    out[idx] = (float)(spectral_weight(kind, (double)evals[i], ts[t], inv_norm) *
                       (double)x[i * m + c]);
  }
}

// ---------------------------------------------------------------------------
// Refinement of the Jacobi eigenpairs (Ogita & Aishima, "Iterative refinement for
// symmetric eigenvalue decomposition", Japan J. Indust. Appl. Math. 35 (2018)):
// with X the approximate eigenvectors, R = I - X^T X and S = X^T (A X) formed in
// double-float, lambda_i = S_ii / (1 - R_ii) and X <- X + X E with
// E_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i) for separated pairs,
// E_ij = R_ij / 2 for pairs whose gap is not large against that numerator or is
// below 1e-6 of the largest |lambda| (a cluster: only orthogonalised), E_ii = R_ii / 2.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void df_fma_e(float a, float xh, float xl, float& sh, float& sl) {
  const float ph = a * xh;
  float pl = fmaf(a, xh, -ph);
  pl = fmaf(a, xl, pl);
  const float s2 = sh + ph;
  const float bv = s2 - sh;
  const float e = (sh - (s2 - bv)) + (ph - bv);
  sl += e + pl;
  sh = s2;
}

// C[i, j] = sum_k P[k, i] (Qh[k, j] + Ql[k, j]) + shift (Qh[i, j] + Ql[i, j]) over 64 x 64
// tiles, double-float sums; P, Qh, Ql [n, n] row-major (Ql may be NULL). Output as
// FP64 (c64) or as a double-float pair (ch, cl).
__global__ void __launch_bounds__(256)
    df_gemm_tn_kernel(const float* __restrict__ P, const float* __restrict__ Qh,
                      const float* __restrict__ Ql, int64_t n, double shift,
                      double* __restrict__ c64, float* __restrict__ ch, float* __restrict__ cl) {
  __shared__ float Ps[16][64 + 1];
  __shared__ float Hs[16][64 + 1];
  __shared__ float Ls[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = (int64_t)blockIdx.y * 64, j0 = (int64_t)blockIdx.x * 64;
  float sh[4][4] = {}, sl[4][4] = {};
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      const int kk = idx / 64, c = idx % 64;
      const bool kin = k0 + kk < n;
      Ps[kk][c] = (kin && i0 + c < n) ? P[(k0 + kk) * n + i0 + c] : 0.f;
      Hs[kk][c] = (kin && j0 + c < n) ? Qh[(k0 + kk) * n + j0 + c] : 0.f;
      Ls[kk][c] = (Ql && kin && j0 + c < n) ? Ql[(k0 + kk) * n + j0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      float av[4], hv[4], lv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        av[u] = Ps[k][ty * 4 + u];
        hv[u] = Hs[k][tx * 4 + u];
        lv[u] = Ls[k][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) df_fma_e(av[u], hv[v], lv[v], sh[u][v], sl[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t i = i0 + ty * 4 + u;
    if (i >= n) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int64_t j = j0 + tx * 4 + v;
      if (j >= n) continue;
      double val = (double)sh[u][v] + (double)sl[u][v];
      if (shift != 0.0)
        val += shift * ((double)Qh[i * n + j] + (Ql ? (double)Ql[i * n + j] : 0.0));
      if (c64) c64[i * n + j] = val;
      if (ch) {
        const float h = (float)val;
        ch[i * n + j] = h;
        cl[i * n + j] = (float)(val - (double)h);
      }
    }
  }
}

// R <- I - R
__global__ void identity_minus_kernel(double* __restrict__ R, int64_t n) {
  const int64_t total = n * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / n, j = idx - i * n;
    R[idx] = (i == j ? 1.0 : 0.0) - R[idx];
  }
}

// lam_i = S_ii / (1 - R_ii); lam[n] receives max |lam_i| (zeroed by the caller).
__global__ void refine_lambda_kernel(const double* __restrict__ S, const double* __restrict__ R,
                                     int64_t n, double* __restrict__ lam) {
  double mx = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    lam[i] = S[i * n + i] / (1.0 - R[i * n + i]);
    mx = fmax(mx, fabs(lam[i]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.0)
    atomicMax(reinterpret_cast<unsigned long long*>(lam + n),
              (unsigned long long)__double_as_longlong(mx));
}

// E = the correction of X (see above); X1 = X (for the accumulate of X + X E).
__global__ void refine_e_kernel(const double* __restrict__ S, const double* __restrict__ R,
                                const double* __restrict__ lam, int64_t n, float* __restrict__ E) {
  const int64_t total = n * n;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / n, j = idx - i * n;
    const double r = R[idx];
    double e = 0.5 * r;
    if (i != j) {
      // separated: the gap is large against the coupling and above the resolution of the
      // float32 eigenvalues (1e-6 of the largest); closer pairs are a cluster
      const double num = S[idx] + lam[j] * r;
      const double gap = lam[j] - lam[i];
      if (fabs(gap) > 1e3 * fabs(num) && fabs(gap) > 1e-6 * lam[n]) e = num / gap;
    }
    E[idx] = (float)e;
  }
}

__global__ void lam_to_float_kernel(const double* __restrict__ lam, int64_t n,
                                    float* __restrict__ evals) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    evals[i] = (float)lam[i];
}

int egrid(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

struct EighWs {
  float* w;
  float* v;
  float* u;
  double* norms;
  int* done;
};

EighWs eigh_ws(void* ws, int64_t npad) {
  char* p = static_cast<char*>(ws);
  p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~(uintptr_t)255);
  EighWs e;
  e.w = reinterpret_cast<float*>(p);
  e.v = e.w + npad * npad;
  e.u = e.v + npad * npad;
  const int64_t npairs = npad / JP;
  e.norms = reinterpret_cast<double*>(e.u + npairs * JP * JP);
  e.done = reinterpret_cast<int*>(e.norms + 2);
  return e;
}

}  // namespace
}  // namespace ntg

using namespace ntg;

// Refinement buffers after the Jacobi ones: S, R [n n] f64, lam [n] f64, Yh, Yl, E [n n] f32.
size_t refine_bytes(int64_t n) {
  return (size_t)(2 * n * n + n + 1) * sizeof(double) + (size_t)3 * n * n * sizeof(float) + 1024;
}

extern "C" size_t ntg_eigh_workspace_bytes(int64_t n) {
  if (n <= 0 || n > 32768) return SIZE_MAX;
  const int64_t npad = (n + JP - 1) / JP * JP;
  return (size_t)(2 * npad * npad + (npad / JP) * JP * JP) * sizeof(float) + 2 * sizeof(double) +
         sizeof(int) + 512 + refine_bytes(n);
}

extern "C" int ntg_eigh(void* stream, const float* A, int64_t n, double shift, float* evals,
                        float* evecs, int32_t max_sweeps, double tol, int32_t refine_steps,
                        void* workspace, size_t workspace_bytes, int32_t* sweeps_out) {
  NTG_REQUIRE(A && evals && evecs && workspace, "ntg_eigh: null pointer");
  NTG_REQUIRE(n > 0 && n <= 32768, "ntg_eigh: n must be in [1, 32768]");
  NTG_REQUIRE(max_sweeps > 0 && max_sweeps <= 100, "ntg_eigh: max_sweeps in [1, 100]");
  NTG_REQUIRE(refine_steps >= 0 && refine_steps <= 4, "ntg_eigh: refine_steps in [0, 4]");
  NTG_REQUIRE(workspace_bytes >= ntg_eigh_workspace_bytes(n),
              "ntg_eigh: workspace smaller than ntg_eigh_workspace_bytes(n)");
  cudaStream_t s = as_stream(stream);
  const int64_t npad = (n + JP - 1) / JP * JP;
  const int nblk = (int)(npad / JB);  // even
  const int npairs = nblk / 2;
  const EighWs e = eigh_ws(workspace, npad);
  eigh_init_kernel<<<egrid(npad * npad), 256, 0, s>>>(A, n, shift, e.w, e.v, npad);
  note_launch();
  if (cudaMemsetAsync(e.done, 0, sizeof(int), s) != cudaSuccess) return check_launch("ntg_eigh");
  int sweeps = 0;
  for (int sw = 0; sw < max_sweeps; ++sw) {
    for (int r = 0; r < nblk - 1; ++r) {
      // two inner sweeps per pair and round: the outer sweeps converge as fast, and an
      // inner problem driven to convergence early on is undone by the next rounds
      jacobi_inner_kernel<<<npairs, 256, 0, s>>>(e.w, npad, nblk, r, 2, e.u, e.done);
      jacobi_apply_kernel<<<dim3(npairs, npairs), 256, 0, s>>>(e.w, npad, nblk, r, e.u, e.done);
      jacobi_apply_v_kernel<<<dim3(npairs, (unsigned)(npad / JP)), 256, 0, s>>>(
          e.v, npad, nblk, r, e.u, e.done);
      note_launch(3);
    }
    ++sweeps;
    if (cudaMemsetAsync(e.norms, 0, 2 * sizeof(double), s) != cudaSuccess)
      return check_launch("ntg_eigh");
    offnorm_kernel<<<egrid(npad * npad), 256, 0, s>>>(e.w, npad, e.norms);
    note_launch();
    double nh[2] = {0.0, 0.0};
    if (cudaMemcpyAsync(nh, e.norms, sizeof(nh), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return check_launch("ntg_eigh norms");
    const double fro2 = nh[0] + nh[1];
    if (nh[0] <= tol * tol * fro2) break;
  }
  eigh_extract_kernel<<<egrid(n * n), 256, 0, s>>>(e.w, e.v, npad, n, evals, evecs);
  note_launch();
  if (refine_steps > 0) {
    char* rp = reinterpret_cast<char*>(
        (reinterpret_cast<uintptr_t>(e.done + 1) + 255) & ~(uintptr_t)255);
    double* S = reinterpret_cast<double*>(rp);
    double* R = S + n * n;
    double* lam = R + n * n;
    float* yh = reinterpret_cast<float*>(lam + n + 1);
    float* yl = yh + n * n;
    float* E = yl + n * n;
    const dim3 g((unsigned)ceil_div(n, 64), (unsigned)ceil_div(n, 64));
    for (int it = 0; it < refine_steps; ++it) {
      // Y = (K + shift I) X (K symmetric: K^T X), S = X^T Y, R = X^T X (as -R + I below)
      df_gemm_tn_kernel<<<g, 256, 0, s>>>(A, evecs, nullptr, n, shift, nullptr, yh, yl);
      df_gemm_tn_kernel<<<g, 256, 0, s>>>(evecs, yh, yl, n, 0.0, S, nullptr, nullptr);
      df_gemm_tn_kernel<<<g, 256, 0, s>>>(evecs, evecs, nullptr, n, 0.0, R, nullptr, nullptr);
      identity_minus_kernel<<<egrid(n * n), 256, 0, s>>>(R, n);
      if (cudaMemsetAsync(lam + n, 0, sizeof(double), s) != cudaSuccess)
        return check_launch("ntg_eigh refine");
      refine_lambda_kernel<<<egrid(n), 256, 0, s>>>(S, R, n, lam);
      refine_e_kernel<<<egrid(n * n), 256, 0, s>>>(S, R, lam, n, E);
      note_launch(6);
      // X <- X + X E (the product reads a copy of X)
      if (cudaMemcpyAsync(yh, evecs, sizeof(float) * n * n, cudaMemcpyDeviceToDevice, s) !=
          cudaSuccess)
        return check_launch("ntg_eigh refine copy");
      const int rc = ntg_gemm(stream, yh, E, evecs, n, n, n, 1);
      if (rc) return rc;
    }
    lam_to_float_kernel<<<egrid(n), 256, 0, s>>>(lam, n, evals);
    note_launch();
  }
  if (sweeps_out) *sweeps_out = sweeps;
  return check_launch("ntg_eigh");
}

extern "C" int ntg_spectral_scale(void* stream, const float* evals, const double* ts, int64_t nt,
                                  int32_t kind, double norm, const float* x, int64_t n, int64_t m,
                                  float* out) {
  NTG_REQUIRE(evals && ts && x && out, "ntg_spectral_scale: null pointer");
  NTG_REQUIRE(n > 0 && m > 0 && nt > 0 && norm > 0.0, "ntg_spectral_scale: bad sizes");
  NTG_REQUIRE(kind >= 0 && kind <= 6, "ntg_spectral_scale: kind must be in [0, 6]");
  spectral_scale_kernel<<<egrid(n * nt * m), 256, 0, as_stream(stream)>>>(
      evals, ts, nt, kind, 1.0 / norm, x, n, m, out);
  note_launch();
  return check_launch("ntg_spectral_scale");
}
