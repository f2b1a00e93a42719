// Materialised layer rules of the analytic NNGP/NTK path on sm_103a:
// input covariances, the full-spatial Conv stencil (with the Dense/Conv affine
// rule and the ABRelu/Erf epilogue fused in), elementwise Dense/activation,
// pooling and the Flatten / GlobalAvgPool readouts.
#include <cstdio>
#include <string>

#include "ntg_common.cuh"
#include "ntg_vjp.cuh"

namespace ntg {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void pair_of(int64_t b, int64_t n2, int64_t& i1, int64_t& i2) {
  if (n2 > 0) {
    i1 = b / n2;
    i2 = b - i1 * n2;
  } else {
    i1 = b;
    i2 = b;
  }
}

// ---------------------------------------------------------------------------
// Flat Gram on CUDA cores: out[i, j] = sum_d x1[i, d] x2[j, d] / D, every output
// accumulated by fmaf in ascending d (the order of the per-sample variances, so that
// the diagonal of x x^T equals them bit for bit). 128 x 128 output tile per CTA, 16 x 16
// threads, 8 x 8 outputs per thread (rows 4 ty + u and 64 + 4 ty + u, columns likewise
// in tx) read from shared memory as 16-byte words. SYM (x1 == x2): the tiles on or below
// the diagonal only (blockIdx.x enumerates them row by row), each off-diagonal one also
// stored transposed: fmaf(a, b, c) == fmaf(b, a, c), so the mirror is exactly the value
// the tile (j, i) would hold.
// ---------------------------------------------------------------------------
template <bool SYM>
__global__ void __launch_bounds__(256) gram_simt_kernel(const float* __restrict__ x1,
                                                        const float* __restrict__ x2,
                                                        int64_t n1, int64_t n2, int64_t d,
                                                        float inv_d, float* __restrict__ out) {
  __shared__ __align__(16) float As[16][128 + 4];
  __shared__ __align__(16) float Bs[16][128 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  int64_t ti = blockIdx.y, tj = blockIdx.x;
  if (SYM) {  // t = i (i + 1) / 2 + j, j <= i
    const int64_t t = blockIdx.x;
    ti = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (ti * (ti + 1) / 2 > t) --ti;
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    tj = t - ti * (ti + 1) / 2;
  }
  const int64_t row0 = ti * 128, col0 = tj * 128;
  float acc[8][8];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
  for (int64_t k0 = 0; k0 < d; k0 += 16) {
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int idx = threadIdx.x + 256 * e;
      const int r = idx >> 4, kk = idx & 15;
      const int64_t gk = k0 + kk;
      const int64_t gi = row0 + r, gj = col0 + r;
      As[kk][r] = (gi < n1 && gk < d) ? __ldg(x1 + gi * d + gk) : 0.f;
      Bs[kk][r] = (gj < n2 && gk < d) ? __ldg(x2 + gj * d + gk) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][4 * ty]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][64 + 4 * ty]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][4 * tx]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][64 + 4 * tx]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], bb[v], acc[u][v]);
    }
    __syncthreads();
  }
  const bool vec = (n2 & 3) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
  const bool mirror = SYM && ti != tj;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int64_t gi = row0 + (u < 4 ? 4 * ty + u : 64 + 4 * ty + u - 4);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t gj = col0 + 64 * h + 4 * tx;
      if (gi >= n1) continue;
      if (vec && gj + 3 < n2) {
        *reinterpret_cast<float4*>(out + gi * n2 + gj) =
            make_float4(acc[u][4 * h] * inv_d, acc[u][4 * h + 1] * inv_d,
                        acc[u][4 * h + 2] * inv_d, acc[u][4 * h + 3] * inv_d);
      } else {
#pragma unroll
        for (int v = 0; v < 4; ++v)
          if (gj + v < n2) out[gi * n2 + gj + v] = acc[u][4 * h + v] * inv_d;
      }
    }
  }
  if (mirror) {  // out[gj][gi] = tile[gi][gj]
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const int64_t gj = col0 + (v < 4 ? 4 * tx + v : 64 + 4 * tx + v - 4);
      if (gj >= n1) continue;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t gi = row0 + 64 * h + 4 * ty;
        if (vec && gi + 3 < n1) {
          *reinterpret_cast<float4*>(out + gj * n2 + gi) =
              make_float4(acc[4 * h][v] * inv_d, acc[4 * h + 1][v] * inv_d,
                          acc[4 * h + 2][v] * inv_d, acc[4 * h + 3][v] * inv_d);
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (gi + u < n1) out[gj * n2 + gi + u] = acc[4 * h + u][v] * inv_d;
        }
      }
    }
  }
}

// C[M, N] = A[M, K] B[K, N] (+ C_in when accumulate): 64x64 tiles, 4x4 per thread.
__global__ void __launch_bounds__(256) gemm_nn_kernel(const float* __restrict__ A,
                                                      const float* __restrict__ B,
                                                      float* __restrict__ Cm, int64_t M, int64_t N,
                                                      int64_t K, int accumulate) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t row0 = (int64_t)blockIdx.y * 64, col0 = (int64_t)blockIdx.x * 64;
  float acc[4][4] = {};
  for (int64_t k0 = 0; k0 < K; k0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      int r = idx / 16, kk = idx % 16;
      int64_t gi = row0 + r, gk = k0 + kk;
      As[kk][r] = (gi < M && gk < K) ? __ldg(A + gi * K + gk) : 0.f;
      int kb = idx / 64, cb = idx % 64;
      int64_t gkb = k0 + kb, gj = col0 + cb;
      Bs[kb][cb] = (gkb < K && gj < N) ? __ldg(B + gkb * N + gj) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], bb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty * 4 + u];
        bb[u] = Bs[kk][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], bb[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      int64_t gi = row0 + ty * 4 + u, gj = col0 + tx * 4 + v;
      if (gi < M && gj < N) Cm[gi * N + gj] = accumulate ? Cm[gi * N + gj] + acc[u][v] : acc[u][v];
    }
}

// Per-row sum(x^2)/D, accumulated in the same order as the Gram kernel above so
// that cov[i] equals a Gram diagonal entry bit for bit.
__global__ void cov_diag_kernel(const float* __restrict__ x, int64_t n, int64_t d, float inv_d,
                                float* __restrict__ cov) {
  int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  const float* p = x + row * d;
  float s = 0.f;
  for (int64_t k = 0; k < d; ++k) {
    float v = __ldg(p + k);
    s = fmaf(v, v, s);
  }
  cov[row] = s * inv_d;
}

// ---------------------------------------------------------------------------
// Full-spatial input covariance: out[b, a, a', c, c'] = sum_k x1[a,c,k] x2[a',c',k] / K
// One CTA per (b, a) row; loops over a'.
// ---------------------------------------------------------------------------
__global__ void input_fs_kernel(const float* __restrict__ x1, const float* __restrict__ x2,
                                int64_t batch, int64_t n2, int64_t A, int64_t C, int64_t K,
                                float inv_k, float* __restrict__ out) {
  int64_t blk = blockIdx.x;
  int64_t b = blk / A, a = blk - b * A;
  if (b >= batch) return;
  int64_t i1, i2;
  pair_of(b, n2, i1, i2);
  const float* r1 = x1 + ((i1 * A + a) * C) * K;
  const float* img2 = x2 + i2 * A * C * K;
  float* o = out + ((b * A + a) * A) * C * C;
  int64_t plane = C * C;
  for (int64_t idx = threadIdx.x; idx < A * plane; idx += blockDim.x) {
    int64_t ap = idx / plane, rem = idx - ap * plane;
    int64_t c = rem / C, cp = rem - c * C;
    const float* p1 = r1 + c * K;
    const float* p2 = img2 + (ap * C + cp) * K;
    float s = 0.f;
    for (int64_t k = 0; k < K; ++k) s = fmaf(__ldg(p1 + k), __ldg(p2 + k), s);
    o[idx] = s * inv_k;
  }
}

// The same for C a power of two in [4, 32] and K <= 4 channels: the row x1[i1, a]
// and the image x2[i2] are staged in shared memory (channels padded to 4), each
// thread writes 4 consecutive entries with one vector store; the same
// multiply-add order per entry as input_fs_kernel.
__global__ void __launch_bounds__(256)
    input_fs_vec_kernel(const float* __restrict__ x1, const float* __restrict__ x2,
                        int64_t batch, int64_t n2, int A, int C, int K, float inv_k,
                        float* __restrict__ out) {
  extern __shared__ __align__(16) float xsm[];  // x1 row [C][4] | x2 image [A * C][4]
  float* r1 = xsm;
  float* im2 = xsm + 4 * C;
  const int64_t b = blockIdx.x / A;
  const int a = (int)(blockIdx.x - b * A);
  if (b >= batch) return;
  int64_t i1, i2;
  pair_of(b, n2, i1, i2);
  const float* src1 = x1 + ((i1 * A + a) * C) * K;
  const float* src2 = x2 + i2 * (int64_t)A * C * K;
  for (int e = threadIdx.x; e < 4 * C; e += blockDim.x) {
    const int c = e >> 2, k = e & 3;
    r1[e] = k < K ? __ldg(src1 + c * K + k) : 0.f;
  }
  for (int e = threadIdx.x; e < 4 * A * C; e += blockDim.x) {
    const int pos = e >> 2, k = e & 3;
    im2[e] = k < K ? __ldg(src2 + (int64_t)pos * K + k) : 0.f;
  }
  __syncthreads();
  const int lc = __ffs(C) - 1;
  float* o = out + (b * A + a) * (int64_t)A * C * C;
  const int n4 = (A * C * C) >> 2;
  for (int v = threadIdx.x; v < n4; v += blockDim.x) {
    const int idx = 4 * v;
    const int cp0 = idx & (C - 1), c = (idx >> lc) & (C - 1), ap = idx >> (2 * lc);
    const float4 u = *reinterpret_cast<const float4*>(r1 + 4 * c);
    const float ua[4] = {u.x, u.y, u.z, u.w};
    float r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float4 x = *reinterpret_cast<const float4*>(im2 + 4 * (ap * C + cp0 + j));
      const float xa[4] = {x.x, x.y, x.z, x.w};
      float sacc = 0.f;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < K) sacc = fmaf(ua[k], xa[k], sacc);
      r[j] = sacc * inv_k;
    }
    *reinterpret_cast<float4*>(o + idx) = make_float4(r[0], r[1], r[2], r[3]);
  }
}

// ---------------------------------------------------------------------------
// General full-spatial conv rule: one thread per output entry.
// ---------------------------------------------------------------------------
struct ConvGeom {
  int64_t batch, n2, A, C, Ao, Co;
  int fh, fw, sh, sw, ph, pw, circular;
};

__device__ __forceinline__ bool wrap_index(int64_t& i, int64_t n, int circular) {
  if (i >= 0 && i < n) return true;
  if (!circular) return false;
  i %= n;
  if (i < 0) i += n;
  return true;
}

__global__ void conv_fs_general_kernel(const float* __restrict__ in_q,
                                       const float* __restrict__ in_t, float* __restrict__ out_q,
                                       float* __restrict__ out_t, ConvGeom g, ntg_affine_t aff,
                                       ntg_act_t act, ntg_var_t var1, ntg_var_t var2) {
  const int64_t plane_o = g.Co * g.Co;
  const int64_t per_b = g.Ao * g.Ao * plane_o;
  const int64_t total = g.batch * per_b;
  const float inv = 1.f / (float)(g.fh * g.fw);
  const ActC ac = act_consts(act);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / per_b, r = idx - b * per_b;
    int64_t i = r / (g.Ao * plane_o);
    r -= i * g.Ao * plane_o;
    int64_t ip = r / plane_o;
    r -= ip * plane_o;
    int64_t j = r / g.Co, jp = r - j * g.Co;
    const float* bq = in_q + b * g.A * g.A * g.C * g.C;
    const float* bt = in_t ? in_t + b * g.A * g.A * g.C * g.C : nullptr;
    float sq = 0.f, st = 0.f;
    for (int d = 0; d < g.fh; ++d) {
      int64_t ia = i * g.sh + d - g.ph, iap = ip * g.sh + d - g.ph;
      if (!wrap_index(ia, g.A, g.circular) || !wrap_index(iap, g.A, g.circular)) continue;
      for (int e = 0; e < g.fw; ++e) {
        int64_t jc = j * g.sw + e - g.pw, jcp = jp * g.sw + e - g.pw;
        if (!wrap_index(jc, g.C, g.circular) || !wrap_index(jcp, g.C, g.circular)) continue;
        int64_t off = ((ia * g.A + iap) * g.C + jc) * g.C + jcp;
        sq += __ldg(bq + off);
        if (bt) st += __ldg(bt + off);
      }
    }
    float q, t = 0.f;
    apply_affine(aff, sq, st, out_t != nullptr, q, t, inv);
    if (act.kind != NTG_ACT_NONE) {
      int64_t i1, i2;
      pair_of(b, g.n2, i1, i2);
      float v1 = var_at(var1, i1, i, j), v2 = var_at(var2, i2, ip, jp);
      act_apply(ac, q, t, v1, v2);
    }
    out_q[idx] = q;
    if (out_t) out_t[idx] = t;
  }
}

// ---------------------------------------------------------------------------
// 3x3 / stride 1 / SAME / zero-padding conv rule streamed along the spatial
// diagonals of the (A, A') plane grid.  Output plane (i, i+delta) needs input
// planes (i-1, i-1+delta), (i, i+delta), (i+1, i+1+delta): every input plane
// of a diagonal line is read once, the 3-plane A-direction sum stays in
// registers, and the C-direction diagonal sum goes through a zero-haloed
// shared-memory tile.  C*C <= 1024 entries per plane, 4 per thread.
// FROM_X computes the input planes from the NHWC images (first-layer Gram).
// ---------------------------------------------------------------------------
template <bool FROM_X, bool HAS_T>
__global__ void __launch_bounds__(kThreads)
    conv3_line_kernel(const float* __restrict__ in_q, const float* __restrict__ in_t,
                      const float* __restrict__ x1, const float* __restrict__ x2, int64_t K,
                      float inv_k, float* __restrict__ out_q, float* __restrict__ out_t,
                      int64_t batch, int64_t n2, int A, int C, ntg_affine_t aff, ntg_act_t act,
                      ntg_var_t var1, ntg_var_t var2) {
  extern __shared__ float smem[];
  const int P = C + 2;                 // haloed row pitch
  float* hq[2] = {smem, smem + P * P};  // double-buffered A-sums
  float* ht[2] = {smem + 2 * P * P, smem + 3 * P * P};
  const int nlines = 2 * A - 1;
  const int64_t b = blockIdx.x / nlines;
  const int delta = (int)(blockIdx.x - b * nlines) - (A - 1);
  if (b >= batch) return;
  const int i_lo = delta < 0 ? -delta : 0;
  const int i_hi = delta < 0 ? A : A - delta;
  const int plane = C * C;
  const int64_t pair_stride = (int64_t)A * A * plane;

  for (int idx = threadIdx.x; idx < 4 * P * P; idx += blockDim.x) smem[idx] = 0.f;

  int64_t i1, i2;
  pair_of(b, n2, i1, i2);
  const ActC ac = act_consts(act);
  const int e0 = threadIdx.x * 4;
  const bool active = e0 < plane;
  const int c = active ? e0 / C : 0;
  const int cp0 = active ? e0 - c * C : 0;

  // Loads input plane at line position i (zero outside the line).
  auto load = [&](int i, float (&q)[4], float (&t)[4]) {
#pragma unroll
    for (int u = 0; u < 4; ++u) q[u] = t[u] = 0.f;
    if (!active || i < i_lo || i >= i_hi) return;
    if (FROM_X) {
      const float* p1 = x1 + (((i1 * A + i) * C + c) * K);
      const float* p2 = x2 + (((i2 * A + i + delta) * C + cp0) * K);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float s = 0.f;
        for (int64_t k = 0; k < K; ++k) s = fmaf(__ldg(p1 + k), __ldg(p2 + u * K + k), s);
        q[u] = s * inv_k;
      }
    } else {
      int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * plane + e0;
      float4 v = __ldg(reinterpret_cast<const float4*>(in_q + off));
      q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;
      if (HAS_T) {
        float4 w = __ldg(reinterpret_cast<const float4*>(in_t + off));
        t[0] = w.x; t[1] = w.y; t[2] = w.z; t[3] = w.w;
      }
    }
  };

  float qm[4], tm[4], q0[4], t0[4], qp[4], tp[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) qm[u] = tm[u] = 0.f;
  load(i_lo, q0, t0);
  __syncthreads();
  const float inv9 = 1.f / 9.f;
  int buf = 0;
  for (int i = i_lo; i < i_hi; ++i) {
    load(i + 1, qp, tp);
    if (active) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int o = (c + 1) * P + (cp0 + u + 1);
        hq[buf][o] = (qm[u] + q0[u]) + qp[u];
        if (HAS_T) ht[buf][o] = (tm[u] + t0[u]) + tp[u];
      }
    }
    __syncthreads();
    if (active) {
      float vq[4], vt[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        int o = (c + 1) * P + (cp0 + u + 1);
        float sq = (hq[buf][o - P - 1] + hq[buf][o]) + hq[buf][o + P + 1];
        float st = HAS_T ? (ht[buf][o - P - 1] + ht[buf][o]) + ht[buf][o + P + 1] : 0.f;
        float q, t = 0.f;
        apply_affine(aff, sq, st, out_t != nullptr, q, t, inv9);
        if (act.kind != NTG_ACT_NONE) {
          float v1 = var_at(var1, i1, i, c), v2 = var_at(var2, i2, i + delta, cp0 + u);
          act_apply(ac, q, t, v1, v2);
        }
        vq[u] = q;
        vt[u] = t;
      }
      int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * plane + e0;
      *reinterpret_cast<float4*>(out_q + off) = make_float4(vq[0], vq[1], vq[2], vq[3]);
      if (out_t) *reinterpret_cast<float4*>(out_t + off) = make_float4(vt[0], vt[1], vt[2], vt[3]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      qm[u] = q0[u]; tm[u] = t0[u];
      q0[u] = qp[u]; t0[u] = tp[u];
    }
    buf ^= 1;
  }
}

// ---------------------------------------------------------------------------
// Same rule with the input planes of a line streamed through a 4-stage
// shared-memory ring by bulk asynchronous copies (cp.async.bulk, completion on
// an mbarrier): one thread keeps up to 3 planes of both tensors in flight while
// the CTA works on the current one. Waits are bounded; a wait that runs out
// raises the library's device error word and the line is left unwritten.
// ---------------------------------------------------------------------------
constexpr int kRing = 4;

__device__ int g_device_error = 0;

template <bool HAS_T>
__global__ void __launch_bounds__(kThreads)
    conv3_line_bulk_kernel(const float* __restrict__ in_q, const float* __restrict__ in_t,
                           float* __restrict__ out_q, float* __restrict__ out_t, int64_t batch,
                           int64_t n2, int A, int C, ntg_affine_t aff, ntg_act_t act,
                           ntg_var_t var1, ntg_var_t var2) {
  extern __shared__ __align__(128) float smem[];
  const int plane = C * C;
  const int P = C + 2;
  float* ring_q = smem;                          // [kRing][plane]
  float* ring_t = ring_q + kRing * plane;        // [kRing][plane]
  float* hq[2] = {ring_t + kRing * plane, ring_t + kRing * plane + P * P};
  float* ht[2] = {hq[1] + P * P, hq[1] + 2 * P * P};
  uint64_t* bars = reinterpret_cast<uint64_t*>(hq[1] + 3 * P * P);
  const int nlines = 2 * A - 1;
  const int64_t b = blockIdx.x / nlines;
  const int delta = (int)(blockIdx.x - b * nlines) - (A - 1);
  if (b >= batch) return;
  const int i_lo = delta < 0 ? -delta : 0;
  const int i_hi = delta < 0 ? A : A - delta;
  const int len = i_hi - i_lo;
  const int64_t pair_stride = (int64_t)A * A * plane;
  const uint32_t bytes = (uint32_t)(plane * sizeof(float)) * (HAS_T ? 2u : 1u);

  for (int idx = threadIdx.x; idx < 4 * P * P; idx += blockDim.x) hq[0][idx] = 0.f;
  if (threadIdx.x == 0) {
    for (int sl = 0; sl < kRing; ++sl)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[sl])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto issue = [&](int j) {  // plane j of the line (0-based) into slot j % kRing
    const int i = i_lo + j;
    const int sl = j % kRing;
    const uint32_t bar = smem_addr(&bars[sl]);
    const int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * plane;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(ring_q + sl * plane)), "l"(in_q + off), "r"((uint32_t)(plane * 4)),
        "r"(bar)
        : "memory");
    if (HAS_T)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(smem_addr(ring_t + sl * plane)), "l"(in_t + off), "r"((uint32_t)(plane * 4)),
          "r"(bar)
          : "memory");
  };
  if (threadIdx.x == 0)
    for (int j = 0; j < kRing && j < len; ++j) issue(j);

  int64_t i1, i2;
  pair_of(b, n2, i1, i2);
  const ActC ac = act_consts(act);
  const int e0 = threadIdx.x * 4;
  const bool active = e0 < plane;
  const int c = active ? e0 / C : 0;
  const int cp0 = active ? e0 - c * C : 0;
  bool ok = true;

  // reads plane j (0-based) of the line from its ring slot (zero outside)
  auto take = [&](int j, float (&q)[4], float (&t)[4]) {
#pragma unroll
    for (int u = 0; u < 4; ++u) q[u] = t[u] = 0.f;
    if (j < 0 || j >= len) return;
    const int sl = j % kRing;
    if (!bar_wait(smem_addr(&bars[sl]), (uint32_t)((j / kRing) & 1))) {
      ok = false;
      return;
    }
    if (!active) return;
    const float4 v = *reinterpret_cast<const float4*>(ring_q + sl * plane + e0);
    q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;
    if (HAS_T) {
      const float4 w = *reinterpret_cast<const float4*>(ring_t + sl * plane + e0);
      t[0] = w.x; t[1] = w.y; t[2] = w.z; t[3] = w.w;
    }
  };

  float qm[4], tm[4], q0[4], t0[4], qp[4], tp[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) qm[u] = tm[u] = 0.f;
  take(0, q0, t0);
  const float inv9 = 1.f / 9.f;
  int buf = 0;
  for (int j = 0; j < len; ++j) {
    take(j + 1, qp, tp);
    const int i = i_lo + j;
    if (active) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int o = (c + 1) * P + (cp0 + u + 1);
        hq[buf][o] = (qm[u] + q0[u]) + qp[u];
        if (HAS_T) ht[buf][o] = (tm[u] + t0[u]) + tp[u];
      }
    }
    __syncthreads();
    // Plane j was read by every thread before the previous barrier, so its slot
    // takes plane j + kRing now: up to three planes stay in flight.
    if (threadIdx.x == 0 && j + kRing < len) issue(j + kRing);
    if (active && ok) {
      float sq[4], st[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int o = (c + 1) * P + (cp0 + u + 1);
        sq[u] = (hq[buf][o - P - 1] + hq[buf][o]) + hq[buf][o + P + 1];
        st[u] = HAS_T ? (ht[buf][o - P - 1] + ht[buf][o]) + ht[buf][o + P + 1] : 0.f;
      }
      // affine rule on packed pairs (same rounding as apply_affine)
      const P2 W2 = p2s(aff.w2 * inv9), B2 = p2s(aff.b2);
      const P2 TW = p2s(aff.ntk_w2 * inv9), TN = p2s(aff.ntk_nn), TC = p2s(aff.ntk_c);
      P2 q[2], t[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const P2 cq = p2(sq[2 * h], sq[2 * h + 1]), ct = p2(st[2 * h], st[2 * h + 1]);
        q[h] = fma2(W2, cq, B2);
        const P2 nn = aff.nn_scaled ? q[h] : mul2(cq, p2s(inv9));
        t[h] = fma2(TW, ct, fma2(TN, nn, TC));
      }
      if (act.kind != NTG_ACT_NONE) {
        const float v1 = var1.base[i1 * var1.s_n + (int64_t)i * var1.s_a + (int64_t)c * var1.s_c];
        const float sv1 = sqrt_var(v1);
        const float* v2r = var2.base + i2 * var2.s_n + (int64_t)(i + delta) * var2.s_a;
        float v2[4], sv2[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          v2[u] = __ldg(v2r + (int64_t)(cp0 + u) * var2.s_c);
          sv2[u] = sqrt_var(v2[u]);
        }
        if (act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f) {
#pragma unroll
          for (int h = 0; h < 2; ++h)
            abrelu2(ac, q[h], t[h], p2s(v1), p2(v2[2 * h], v2[2 * h + 1]), p2s(sv1),
                    p2(sv2[2 * h], sv2[2 * h + 1]));
        } else {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            float qa, qb, ta, tb;
            p2u(q[h], qa, qb);
            p2u(t[h], ta, tb);
            act_apply(ac, qa, ta, v1, v2[2 * h], sv1, sv2[2 * h]);
            act_apply(ac, qb, tb, v1, v2[2 * h + 1], sv1, sv2[2 * h + 1]);
            q[h] = p2(qa, qb);
            t[h] = p2(ta, tb);
          }
        }
      }
      float vq[4], vt[4];
      p2u(q[0], vq[0], vq[1]);
      p2u(q[1], vq[2], vq[3]);
      p2u(t[0], vt[0], vt[1]);
      p2u(t[1], vt[2], vt[3]);
      float* oq = out_q + b * pair_stride + ((int64_t)i * A + i + delta) * plane + e0;
      *reinterpret_cast<float4*>(oq) = make_float4(vq[0], vq[1], vq[2], vq[3]);
      if (out_t) {
        float* ot = out_t + b * pair_stride + ((int64_t)i * A + i + delta) * plane + e0;
        *reinterpret_cast<float4*>(ot) = make_float4(vt[0], vt[1], vt[2], vt[3]);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      qm[u] = q0[u]; tm[u] = t0[u];
      q0[u] = qp[u]; t0[u] = tp[u];
    }
    buf ^= 1;
  }
  if (!ok && threadIdx.x == 0) {
    atomicExch(&g_device_error, NTG_ERR_WAIT_TIMEOUT);
    // let every issued copy land (bounded) before the CTA's shared memory is released
    for (int j = 0; j < len; ++j) bar_wait(smem_addr(&bars[j % kRing]), (uint32_t)((j / kRing) & 1));
  }
}

// ---------------------------------------------------------------------------
// The same rule for 32 x 32 planes, each thread on a run of a *skewed* row:
// thread (r, w0) owns the elements (w, (w + r) mod 32) for w = w0 .. w0 + 3,
// so the w-direction stencil neighbours (w - 1, w' - 1) and (w + 1, w' + 1)
// are the row neighbours w -/+ 1 — a register, or one shuffle at the ends of
// the run — masked to zero where w' wraps around. Input planes stream in
// through the bulk-copy ring; results are written into a double-buffered
// staging plane and leave by bulk stores, so each plane costs one barrier and
// no shared-memory halo. Bank-conflict free: for a fixed element slot the 32
// lanes of a warp touch 32 distinct banks (w0 + r distinct mod 32). The sums
// run in the same order as conv3_line_kernel's, so both round alike.
// ---------------------------------------------------------------------------
constexpr int kSkewC = 32;
constexpr int kSkewPlane = kSkewC * kSkewC;
constexpr int kSkewVars = 192;  // per plane: v1[32] | sqrt v1[32] | v2[64] | sqrt v2[64]

template <int RING>
__host__ __device__ constexpr size_t skew_smem_bytes() {
  return sizeof(float) * (2 * RING * kSkewPlane + 4 * kSkewPlane + 2 * kSkewVars) +
         sizeof(uint64_t) * RING;
}

// start (bytes, 128-aligned) of the optional pre-activation staging planes
template <int RING>
__host__ __device__ constexpr size_t skew_pre_offset() {
  return (skew_smem_bytes<RING>() + 127) / 128 * 128;
}

template <int RING>
__host__ __device__ constexpr size_t skew_smem_bytes_pre() {
  return skew_pre_offset<RING>() + sizeof(float) * 4 * kSkewPlane;
}

__device__ __forceinline__ void bulk_store(float* gdst, const float* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(smem_addr(ssrc)), "r"(bytes)
               : "memory");
}

// ACTK: 1 = the ABRelu family without do_stabilize only (the other rules compiled out),
// 0 = any activation rule. HP: an AvgPool(2, 2) follows; the kernel writes hp_q / hp_t
// (window sums along w) instead of out_q / out_t.
template <bool HAS_T, int RING, int ACTK, bool HP = false>
__global__ void __launch_bounds__(kThreads)
    conv3_skew_kernel(const float* __restrict__ in_q, const float* __restrict__ in_t,
                      float* __restrict__ out_q, float* __restrict__ out_t, int64_t batch,
                      int64_t n2, int A, ntg_affine_t aff, ntg_act_t act, ntg_var_t var1,
                      ntg_var_t var2, float* __restrict__ pre_q, float* __restrict__ pre_t,
                      float* __restrict__ hp_q, float* __restrict__ hp_t) {
  extern __shared__ __align__(128) float smem[];
  __shared__ int s_err;
  float* ring_q = smem;                           // [RING][plane]
  float* ring_t = ring_q + RING * kSkewPlane;     // [RING][plane]
  float* stage_q = ring_t + RING * kSkewPlane;    // [2][plane]
  float* stage_t = stage_q + 2 * kSkewPlane;      // [2][plane]
  float* vrow = stage_t + 2 * kSkewPlane;         // [2][kSkewVars]
  uint64_t* bars = reinterpret_cast<uint64_t*>(vrow + 2 * kSkewVars);
  // with pre_q: staging of the pre-activation planes [2][plane] x 2 after the barriers
  float* stage_pq = reinterpret_cast<float*>(smem) + skew_pre_offset<RING>() / sizeof(float);
  float* stage_pt = stage_pq + 2 * kSkewPlane;
  const int nlines = 2 * A - 1;
  const int64_t b = blockIdx.x / nlines;
  const int delta = (int)(blockIdx.x - b * nlines) - (A - 1);
  if (b >= batch) return;
  const int i_lo = delta < 0 ? -delta : 0;
  const int len = (delta < 0 ? A : A - delta) - i_lo;
  const int64_t pair_stride = (int64_t)A * A * kSkewPlane;
  const uint32_t bytes = (uint32_t)(kSkewPlane * sizeof(float)) * (HAS_T ? 2u : 1u);
  const int tid = threadIdx.x, lane = tid & 31;
  const int w0 = (lane & 7) * 4;
  const int r = (tid >> 5) * 4 + (lane >> 3);
  const bool has_act = act.kind != NTG_ACT_NONE;

  int u[4];
  float mL[4], mR[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int w = w0 + k, wq = (w + r) & (kSkewC - 1);
    u[k] = w * kSkewC + wq;
    mL[k] = (w >= 1 && wq >= 1) ? 1.f : 0.f;
    mR[k] = (w <= kSkewC - 2 && wq <= kSkewC - 2) ? 1.f : 0.f;
  }
  int64_t i1, i2;
  pair_of(b, n2, i1, i2);

  // variance rows of plane j (row i = i_lo + j): v1 at (i, w), v2 at (i + delta, w')
  auto load_vars = [&](int j) {
    const int i = i_lo + j;
    float* vb = vrow + (j & 1) * kSkewVars;
    if (tid < kSkewC) {
      const float v =
          __ldg(var1.base + i1 * var1.s_n + (int64_t)i * var1.s_a + (int64_t)tid * var1.s_c);
      vb[tid] = v;
      vb[32 + tid] = sqrt_var(v);
    } else if (tid < 3 * kSkewC) {
      const int x = tid - kSkewC;
      const float v = __ldg(var2.base + i2 * var2.s_n + (int64_t)(i + delta) * var2.s_a +
                            (int64_t)(x & (kSkewC - 1)) * var2.s_c);
      vb[64 + x] = v;
      vb[128 + x] = sqrt_var(v);
    }
  };

  if (tid == 0) {
    s_err = 0;
    for (int sl = 0; sl < RING; ++sl)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[sl])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (has_act) load_vars(0);
  __syncthreads();

  auto issue = [&](int p) {  // plane p of the line into slot p % RING
    const int i = i_lo + p;
    const int sl = p % RING;
    const uint32_t bar = smem_addr(&bars[sl]);
    const int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * kSkewPlane;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(ring_q + sl * kSkewPlane)), "l"(in_q + off), "r"(kSkewPlane * 4u),
        "r"(bar)
        : "memory");
    if (HAS_T)
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(smem_addr(ring_t + sl * kSkewPlane)), "l"(in_t + off), "r"(kSkewPlane * 4u),
          "r"(bar)
          : "memory");
  };
  int next = 0;  // next plane thread 0 issues
  if (tid == 0)
    for (; next < RING && next < len; ++next) issue(next);

  // plane p of the line from its ring slot, in this thread's skewed order (zero outside)
  auto take = [&](int p, float (&q)[4], float (&t)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = t[k] = 0.f;
    if (p >= len) return;
    const int sl = p % RING;
    if (!s_err && !bar_wait(smem_addr(&bars[sl]), (uint32_t)((p / RING) & 1))) s_err = 1;
    const float* sq = ring_q + sl * kSkewPlane;
    const float* st = ring_t + sl * kSkewPlane;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      q[k] = sq[u[k]];
      if (HAS_T) t[k] = st[u[k]];
    }
  };

  const float inv9 = 1.f / 9.f;
  const ActC ac = act_consts(act);
  const P2 W2 = p2s(aff.w2 * inv9), B2 = p2s(aff.b2);
  const P2 TW = p2s(aff.ntk_w2 * inv9), TN = p2s(aff.ntk_nn), TC = p2s(aff.ntk_c);
  float qm[4], tm[4], q0[4], t0[4], qp[4], tp[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) qm[k] = tm[k] = 0.f;
  take(0, q0, t0);
  for (int j = 0; j < len; ++j) {
    take(j + 1, qp, tp);
    if (has_act && j + 1 < len) load_vars(j + 1);  // read after the next barrier
    const int i = i_lo + j;
    float hq[4], ht[4], sq[4], st[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      hq[k] = (qm[k] + q0[k]) + qp[k];
      ht[k] = HAS_T ? (tm[k] + t0[k]) + tp[k] : 0.f;
    }
    {
      const float lq = __shfl_up_sync(0xffffffffu, hq[3], 1, 8);
      const float rq = __shfl_down_sync(0xffffffffu, hq[0], 1, 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float L = k == 0 ? lq : hq[k - 1], R = k == 3 ? rq : hq[k + 1];
        sq[k] = fmaf(R, mR[k], fmaf(L, mL[k], hq[k]));
      }
    }
    if (HAS_T) {
      const float lt = __shfl_up_sync(0xffffffffu, ht[3], 1, 8);
      const float rt = __shfl_down_sync(0xffffffffu, ht[0], 1, 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float L = k == 0 ? lt : ht[k - 1], R = k == 3 ? rt : ht[k + 1];
        st[k] = fmaf(R, mR[k], fmaf(L, mL[k], ht[k]));
      }
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) st[k] = 0.f;
    }
    // affine rule on packed pairs (same rounding as apply_affine)
    P2 q[2], t[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const P2 cq = p2(sq[2 * h], sq[2 * h + 1]), ct = p2(st[2 * h], st[2 * h + 1]);
      q[h] = fma2(W2, cq, B2);
      const P2 nn = aff.nn_scaled ? q[h] : mul2(cq, p2s(inv9));
      t[h] = fma2(TW, ct, fma2(TN, nn, TC));
    }
    if (pre_q) {  // the conv output before the activation, for the activation's VJP
      float* pq = stage_pq + (j & 1) * kSkewPlane;
      float* pt = stage_pt + (j & 1) * kSkewPlane;
      float vq[4], vt[4];
      p2u(q[0], vq[0], vq[1]);
      p2u(q[1], vq[2], vq[3]);
      p2u(t[0], vt[0], vt[1]);
      p2u(t[1], vt[2], vt[3]);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        pq[u[k]] = vq[k];
        if (pre_t) pt[u[k]] = vt[k];
      }
    }
    if (has_act) {
      const float* vb = vrow + (j & 1) * kSkewVars;
      const float4 v1 = *reinterpret_cast<const float4*>(vb + w0);
      const float4 s1 = *reinterpret_cast<const float4*>(vb + 32 + w0);
      float v2[4], s2[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        v2[k] = vb[64 + w0 + r + k];
        s2[k] = vb[128 + w0 + r + k];
      }
      if (ACTK == 1 || (act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f)) {
        abrelu2(ac, q[0], t[0], p2(v1.x, v1.y), p2(v2[0], v2[1]), p2(s1.x, s1.y),
                p2(s2[0], s2[1]));
        abrelu2(ac, q[1], t[1], p2(v1.z, v1.w), p2(v2[2], v2[3]), p2(s1.z, s1.w),
                p2(s2[2], s2[3]));
      } else {
        const float a1[4] = {v1.x, v1.y, v1.z, v1.w}, b1[4] = {s1.x, s1.y, s1.z, s1.w};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float qa, qb, ta, tb;
          p2u(q[h], qa, qb);
          p2u(t[h], ta, tb);
          act_apply(ac, qa, ta, a1[2 * h], v2[2 * h], b1[2 * h], s2[2 * h]);
          act_apply(ac, qb, tb, a1[2 * h + 1], v2[2 * h + 1], b1[2 * h + 1], s2[2 * h + 1]);
          q[h] = p2(qa, qb);
          t[h] = p2(ta, tb);
        }
      }
    }
    float* gq = stage_q + (j & 1) * kSkewPlane;
    float* gt = stage_t + (j & 1) * kSkewPlane;
    {
      float vq[4], vt[4];
      p2u(q[0], vq[0], vq[1]);
      p2u(q[1], vq[2], vq[3]);
      p2u(t[0], vt[0], vt[1]);
      p2u(t[1], vt[2], vt[3]);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        gq[u[k]] = vq[k];
        if (HP ? hp_t != nullptr : out_t != nullptr) gt[u[k]] = vt[k];
      }
    }
    // staging writes -> visible to the bulk-copy engine; the store of plane j - 1
    // has finished reading its buffer before anyone writes it again (plane j + 1)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (HP) {
      // an AvgPool(2, 2) follows: instead of the activated planes, their w-direction
      // window sums (x[2j][2j'] + x[2j][2j'+1]) + (x[2j+1][2j'] + x[2j+1][2j'+1]), the
      // inner sums of pool_kernel's order; pool_planes_kernel adds the planes
      const int jj = tid >> 4, jp = tid & 15;
      const int64_t ho = b * (int64_t)A * A * (kSkewPlane / 4) +
                         ((int64_t)i * A + i + delta) * (kSkewPlane / 4) + tid;
      const float* xq = gq + (2 * jj) * kSkewC + 2 * jp;
      hp_q[ho] = (xq[0] + xq[1]) + (xq[kSkewC] + xq[kSkewC + 1]);
      if (hp_t) {
        const float* xt = gt + (2 * jj) * kSkewC + 2 * jp;
        hp_t[ho] = (xt[0] + xt[1]) + (xt[kSkewC] + xt[kSkewC + 1]);
      }
    }
    if (tid == 0) {
      const int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * kSkewPlane;
      if (!HP) {
        bulk_store(out_q + off, gq, kSkewPlane * 4u);
        if (out_t) bulk_store(out_t + off, gt, kSkewPlane * 4u);
      }
      if (pre_q) {
        bulk_store(pre_q + off, stage_pq + (j & 1) * kSkewPlane, kSkewPlane * 4u);
        if (pre_t) bulk_store(pre_t + off, stage_pt + (j & 1) * kSkewPlane, kSkewPlane * 4u);
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      // plane j + 1 has been read by every thread: its slot takes plane j + 1 + RING
      if (!s_err)
        for (; next < len && next <= j + 1 + RING; ++next) issue(next);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      qm[k] = q0[k]; tm[k] = t0[k];
      q0[k] = qp[k]; t0[k] = tp[k];
    }
  }
  if (tid == 0) {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    if (s_err) {
      atomicExch(&g_device_error, NTG_ERR_WAIT_TIMEOUT);
      // let every issued copy land (bounded) before the CTA's shared memory is released
      for (int p = next > RING ? next - RING : 0; p < next; ++p)
        bar_wait(smem_addr(&bars[p % RING]), (uint32_t)((p / RING) & 1));
    }
  }
}

// ---------------------------------------------------------------------------
// The first layer of a conv net on 32 x 32 images, in one pass per line of a
// pair: the input covariances G[h, h', w, w'] = sum_k x1[h, w, k] x2[h', w', k] / K
// (requirements.py:542-553, channels summed in the order of input_fs_vec_kernel,
// so both round alike), the 3x3 SAME conv rule on them and the activation, as
// conv3_skew_kernel does on a materialised G. The images of the pair sit in
// shared memory (planar), so G is never written to or read from HBM. The input
// NTK is zero and the rule has ntk = nngp_out + W^2 ntk_in, so the conv's NTK
// equals its NNGP bit for bit: one pre-activation plane (pre_q) serves both.
// ---------------------------------------------------------------------------
template <int K>
__host__ __device__ constexpr size_t skew_input_smem_bytes() {
  return sizeof(float) * (2 * K * kSkewPlane + 6 * kSkewPlane + 2 * kSkewVars);
}

template <int K, int ACTK>
__global__ void __launch_bounds__(kThreads)
    conv3_skew_input_kernel(const float* __restrict__ x1, const float* __restrict__ x2,
                            float* __restrict__ out_q, float* __restrict__ out_t,
                            float* __restrict__ pre_q, int64_t batch, int64_t n2,
                            ntg_affine_t aff, ntg_act_t act, ntg_var_t var1, ntg_var_t var2,
                            float inv_k) {
  extern __shared__ __align__(128) float smem[];
  constexpr int A = kSkewC;
  float* im1 = smem;                          // [K][plane] image x1[i1], planar
  float* im2 = im1 + K * kSkewPlane;          // [K][plane] image x2[i2]
  float* stage_q = im2 + K * kSkewPlane;      // [2][plane]
  float* stage_t = stage_q + 2 * kSkewPlane;  // [2][plane]
  float* stage_p = stage_t + 2 * kSkewPlane;  // [2][plane]
  float* vrow = stage_p + 2 * kSkewPlane;     // [2][kSkewVars]
  const int nlines = 2 * A - 1;
  const int64_t b = blockIdx.x / nlines;
  const int delta = (int)(blockIdx.x - b * nlines) - (A - 1);
  if (b >= batch) return;
  const int i_lo = delta < 0 ? -delta : 0;
  const int len = (delta < 0 ? A : A - delta) - i_lo;
  const int64_t pair_stride = (int64_t)A * A * kSkewPlane;
  const int tid = threadIdx.x, lane = tid & 31;
  const int w0 = (lane & 7) * 4;
  const int r = (tid >> 5) * 4 + (lane >> 3);
  const bool has_act = act.kind != NTG_ACT_NONE;

  int u[4], wq[4];
  float mL[4], mR[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int w = w0 + k;
    wq[k] = (w + r) & (kSkewC - 1);
    u[k] = w * kSkewC + wq[k];
    mL[k] = (w >= 1 && wq[k] >= 1) ? 1.f : 0.f;
    mR[k] = (w <= kSkewC - 2 && wq[k] <= kSkewC - 2) ? 1.f : 0.f;
  }
  int64_t i1, i2;
  pair_of(b, n2, i1, i2);
  {  // NHWC images -> planar [K][h * 32 + w]
    const float* s1 = x1 + i1 * (int64_t)kSkewPlane * K;
    const float* s2 = x2 + i2 * (int64_t)kSkewPlane * K;
    for (int e = tid; e < K * kSkewPlane; e += kThreads) {
      const int pos = e / K, ch = e - pos * K;
      im1[ch * kSkewPlane + pos] = __ldg(s1 + e);
      im2[ch * kSkewPlane + pos] = __ldg(s2 + e);
    }
  }
  auto load_vars = [&](int j) {
    const int i = i_lo + j;
    float* vb = vrow + (j & 1) * kSkewVars;
    if (tid < kSkewC) {
      const float v =
          __ldg(var1.base + i1 * var1.s_n + (int64_t)i * var1.s_a + (int64_t)tid * var1.s_c);
      vb[tid] = v;
      vb[32 + tid] = sqrt_var(v);
    } else if (tid < 3 * kSkewC) {
      const int x = tid - kSkewC;
      const float v = __ldg(var2.base + i2 * var2.s_n + (int64_t)(i + delta) * var2.s_a +
                            (int64_t)(x & (kSkewC - 1)) * var2.s_c);
      vb[64 + x] = v;
      vb[128 + x] = sqrt_var(v);
    }
  };
  if (has_act) load_vars(0);
  __syncthreads();

  // plane p of the line's input covariance in this thread's skewed order (zero outside)
  auto take = [&](int p, float (&q)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = 0.f;
    if (p >= len) return;
    const int h = i_lo + p, hq = h + delta;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float g = 0.f;
#pragma unroll
      for (int ch = 0; ch < K; ++ch)
        g = fmaf(im1[ch * kSkewPlane + h * kSkewC + w0 + k],
                 im2[ch * kSkewPlane + hq * kSkewC + wq[k]], g);
      q[k] = g * inv_k;
    }
  };

  const float inv9 = 1.f / 9.f;
  const ActC ac = act_consts(act);
  const P2 W2 = p2s(aff.w2 * inv9), B2 = p2s(aff.b2);
  const P2 TW = p2s(aff.ntk_w2 * inv9), TN = p2s(aff.ntk_nn), TC = p2s(aff.ntk_c);
  float qm[4], q0[4], qp[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) qm[k] = 0.f;
  take(0, q0);
  for (int j = 0; j < len; ++j) {
    take(j + 1, qp);
    if (has_act && j + 1 < len) load_vars(j + 1);  // read after the next barrier
    const int i = i_lo + j;
    float hq[4], sq[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) hq[k] = (qm[k] + q0[k]) + qp[k];
    {
      const float lq = __shfl_up_sync(0xffffffffu, hq[3], 1, 8);
      const float rq = __shfl_down_sync(0xffffffffu, hq[0], 1, 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float L = k == 0 ? lq : hq[k - 1], R = k == 3 ? rq : hq[k + 1];
        sq[k] = fmaf(R, mR[k], fmaf(L, mL[k], hq[k]));
      }
    }
    // affine rule on packed pairs, the input NTK zero (same rounding as conv3_skew_kernel)
    P2 q[2], t[2];
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const P2 cq = p2(sq[2 * hh], sq[2 * hh + 1]), ct = p2s(0.f);
      q[hh] = fma2(W2, cq, B2);
      const P2 nn = aff.nn_scaled ? q[hh] : mul2(cq, p2s(inv9));
      t[hh] = fma2(TW, ct, fma2(TN, nn, TC));
    }
    {
      float* pq = stage_p + (j & 1) * kSkewPlane;
      float vq[4];
      p2u(q[0], vq[0], vq[1]);
      p2u(q[1], vq[2], vq[3]);
#pragma unroll
      for (int k = 0; k < 4; ++k) pq[u[k]] = vq[k];
    }
    if (has_act) {
      const float* vb = vrow + (j & 1) * kSkewVars;
      const float4 v1 = *reinterpret_cast<const float4*>(vb + w0);
      const float4 s1 = *reinterpret_cast<const float4*>(vb + 32 + w0);
      float v2[4], s2[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        v2[k] = vb[64 + w0 + r + k];
        s2[k] = vb[128 + w0 + r + k];
      }
      if (ACTK == 1 || (act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f)) {
        abrelu2(ac, q[0], t[0], p2(v1.x, v1.y), p2(v2[0], v2[1]), p2(s1.x, s1.y),
                p2(s2[0], s2[1]));
        abrelu2(ac, q[1], t[1], p2(v1.z, v1.w), p2(v2[2], v2[3]), p2(s1.z, s1.w),
                p2(s2[2], s2[3]));
      } else {
        const float a1[4] = {v1.x, v1.y, v1.z, v1.w}, b1[4] = {s1.x, s1.y, s1.z, s1.w};
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          float qa, qb, ta, tb;
          p2u(q[hh], qa, qb);
          p2u(t[hh], ta, tb);
          act_apply(ac, qa, ta, a1[2 * hh], v2[2 * hh], b1[2 * hh], s2[2 * hh]);
          act_apply(ac, qb, tb, a1[2 * hh + 1], v2[2 * hh + 1], b1[2 * hh + 1], s2[2 * hh + 1]);
          q[hh] = p2(qa, qb);
          t[hh] = p2(ta, tb);
        }
      }
    }
    float* gq = stage_q + (j & 1) * kSkewPlane;
    float* gt = stage_t + (j & 1) * kSkewPlane;
    {
      float vq[4], vt[4];
      p2u(q[0], vq[0], vq[1]);
      p2u(q[1], vq[2], vq[3]);
      p2u(t[0], vt[0], vt[1]);
      p2u(t[1], vt[2], vt[3]);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        gq[u[k]] = vq[k];
        gt[u[k]] = vt[k];
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      const int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * kSkewPlane;
      bulk_store(out_q + off, gq, kSkewPlane * 4u);
      bulk_store(out_t + off, gt, kSkewPlane * 4u);
      bulk_store(pre_q + off, stage_p + (j & 1) * kSkewPlane, kSkewPlane * 4u);
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      qm[k] = q0[k];
      q0[k] = qp[k];
    }
  }
  if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Backward of a 3x3 / stride 1 / SAME conv + ABRelu (+ AvgPool(2, 2)) on 32 x 32
// pair kernels in one pass. The reverse of the pair's forward is
//   activation VJP: (g_pre_q, g_pre_t) = VJP(pre_q, pre_t, var1, var2; g_q, g_t)
//   conv transpose: g_in_t = w2/9 S(g_pre_t), g_in_q = w2/9 S(g_pre_q) + w2 S(g_pre_t)/9
// (S the 3x3 diagonal stencil sum, which a centred stride-1 window makes its own
// transpose). Separately these move 24 + 16 bytes per entry through HBM; here the
// VJP runs as each plane of a line enters the CTA (pre-activation and cotangent
// planes by bulk copy into a shared-memory ring), its results go straight into
// the stencil's 3-plane register ring, and only g_in leaves: 16 + 8 bytes per
// entry (8.5 + 8 with the pooled cotangent of AvgPool(2, 2), read at 1/16 size).
// Same thread layout, operation order and rounding as act_bwd_fs_kernel followed
// by conv3_skew_kernel with the roles of the two tensors exchanged, so g_in is
// bit-identical to the two-kernel path. The variance cotangents (sums over the
// other image's positions) are reduced per plane in shared memory and added to
// gvar1 / gvar2 ([n, 32, 32]) with one atomic per (plane, position).
// ---------------------------------------------------------------------------
constexpr int kVjpRing = 3;
constexpr int kVjpWarps = kThreads / 32;  // each keeps its own variance-cotangent partials

template <bool POOLED>
__host__ __device__ constexpr int skew_vjp_slot_floats() {
  return 2 * kSkewPlane + 2 * (POOLED ? kSkewPlane / 4 : kSkewPlane);
}

template <bool POOLED>
__host__ __device__ constexpr size_t skew_vjp_smem_bytes() {
  return sizeof(float) * (kVjpRing * skew_vjp_slot_floats<POOLED>() + 4 * kSkewPlane +
                          3 * 64 + 3 * kVjpWarps * 64) +
         sizeof(uint64_t) * kVjpRing;
}

template <bool POOLED>
__device__ __forceinline__ void skew_vjp_body(
    const float* __restrict__ pre_q, const float* __restrict__ pre_t,
    const float* __restrict__ g_q, const float* __restrict__ g_t, float* __restrict__ gin_q,
    float* __restrict__ gin_t, int64_t batch, int64_t n2, int A, float w2, ntg_act_t act,
    ntg_var_t var1, ntg_var_t var2, float* __restrict__ gvar1, float* __restrict__ gvar2) {
  extern __shared__ __align__(128) float smem[];
  __shared__ int s_err;
  constexpr int GP = POOLED ? kSkewPlane / 4 : kSkewPlane;  // floats of a cotangent plane
  constexpr int SLOT = skew_vjp_slot_floats<POOLED>();
  float* ring = smem;                                   // [ring][pre_q | pre_t | g_q | g_t]
  float* stage_q = ring + kVjpRing * SLOT;              // [2][plane]
  float* stage_t = stage_q + 2 * kSkewPlane;            // [2][plane]
  float* vrow = stage_t + 2 * kSkewPlane;               // [3][v1[32] | v2[32]]
  float* sg = vrow + 3 * 64;                            // [3][warp][g v1[32] | g v2[32]]
  uint64_t* bars = reinterpret_cast<uint64_t*>(sg + 3 * kVjpWarps * 64);  // after all of sg
  const int nlines = 2 * A - 1;
  const int64_t b = blockIdx.x / nlines;
  const int delta = (int)(blockIdx.x - b * nlines) - (A - 1);
  if (b >= batch) return;
  const int i_lo = delta < 0 ? -delta : 0;
  const int len = (delta < 0 ? A : A - delta) - i_lo;
  const int64_t pair_stride = (int64_t)A * A * kSkewPlane;
  const int Ah = A / 2;
  const int64_t gpair_stride = POOLED ? (int64_t)Ah * Ah * GP : pair_stride;
  const uint32_t bytes = (uint32_t)(2 * kSkewPlane * sizeof(float)) +
                         (uint32_t)((g_q ? 1 : 0) + (g_t ? 1 : 0)) * (uint32_t)(GP * sizeof(float));
  const int tid = threadIdx.x, lane = tid & 31;
  const int w0 = (lane & 7) * 4;
  const int r0 = (tid >> 5) * 4;  // first skewed row of this warp
  const int r = r0 + (lane >> 3);

  int u[4], gu[4], wq[4];
  float mL[4], mR[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int w = w0 + k;
    wq[k] = (w + r) & (kSkewC - 1);
    u[k] = w * kSkewC + wq[k];
    gu[k] = POOLED ? (w >> 1) * (kSkewC / 2) + (wq[k] >> 1) : u[k];
    mL[k] = (w >= 1 && wq[k] >= 1) ? 1.f : 0.f;
    mR[k] = (w <= kSkewC - 2 && wq[k] <= kSkewC - 2) ? 1.f : 0.f;
  }
  int64_t i1, i2;
  pair_of(b, n2, i1, i2);

  // variances of plane j (row i = i_lo + j): v1 at (i, w), v2 at (i + delta, w')
  auto load_vars = [&](int j) {
    const int i = i_lo + j;
    float* vb = vrow + (j % 3) * 64;
    if (tid < kSkewC)
      vb[tid] = __ldg(var1.base + i1 * var1.s_n + (int64_t)i * var1.s_a + (int64_t)tid * var1.s_c);
    else if (tid < 2 * kSkewC)
      vb[tid] = __ldg(var2.base + i2 * var2.s_n + (int64_t)(i + delta) * var2.s_a +
                      (int64_t)(tid - kSkewC) * var2.s_c);
  };
  // adds plane j's variance cotangents (the eight warps' partial sums) to gvar1 / gvar2
  auto flush = [&](int j) {
    const float* s = sg + (j % 3) * (kVjpWarps * 64);
    if (tid < 2 * kSkewC) {
      float v = 0.f;
#pragma unroll
      for (int wv = 0; wv < kVjpWarps; ++wv) v += s[wv * 64 + tid];
      const int i = i_lo + j;
      if (tid < kSkewC) {
        if (gvar1 && v != 0.f) atomicAdd(gvar1 + (i1 * A + i) * kSkewC + tid, v);
      } else {
        if (gvar2 && v != 0.f) atomicAdd(gvar2 + (i2 * A + i + delta) * kSkewC + tid - kSkewC, v);
      }
    }
  };

  if (tid == 0) {
    s_err = 0;
    for (int sl = 0; sl < kVjpRing; ++sl)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[sl])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  load_vars(0);
  if (len > 1) load_vars(1);
  __syncthreads();

  auto issue = [&](int p) {  // plane p of the line into slot p % kVjpRing
    const int i = i_lo + p;
    const int sl = p % kVjpRing;
    const uint32_t bar = smem_addr(&bars[sl]);
    float* dst = ring + sl * SLOT;
    const int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * kSkewPlane;
    const int64_t goff = POOLED ? b * gpair_stride + ((int64_t)(i >> 1) * Ah + ((i + delta) >> 1)) * GP
                                : off;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    const float* src[4] = {pre_q + off, pre_t + off, g_q ? g_q + goff : nullptr,
                           g_t ? g_t + goff : nullptr};
    const uint32_t nb[4] = {kSkewPlane * 4u, kSkewPlane * 4u, GP * 4u, GP * 4u};
    const int dofs[4] = {0, kSkewPlane, 2 * kSkewPlane, 2 * kSkewPlane + GP};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      if (!src[m]) continue;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(smem_addr(dst + dofs[m])), "l"(src[m]), "r"(nb[m]), "r"(bar)
          : "memory");
    }
  };
  int next = 0;  // next plane thread 0 issues
  if (tid == 0)
    for (; next < kVjpRing && next < len; ++next) issue(next);

  const ActC ac = act_consts(act);
  const float pool_w = 1.f / 16.f;
  // plane p's activation VJP in this thread's skewed order (zero outside the line):
  // a = g_pre_t, c = g_pre_q; variance cotangents summed into the plane's shared sums
  auto take = [&](int p, float (&a)[4], float (&c)[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = c[k] = 0.f;
    if (p >= len) return;
    const int sl = p % kVjpRing;
    if (!s_err && !bar_wait(smem_addr(&bars[sl]), (uint32_t)((p / kVjpRing) & 1))) s_err = 1;
    const float* sp = ring + sl * SLOT;
    const float* vb = vrow + (p % 3) * 64;
    float qv[4], tv[4], gqv[4], gtv[4], v1[4], v2[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      qv[k] = sp[u[k]];
      tv[k] = sp[kSkewPlane + u[k]];
      gqv[k] = g_q ? sp[2 * kSkewPlane + gu[k]] : 0.f;
      gtv[k] = g_t ? sp[2 * kSkewPlane + GP + gu[k]] : 0.f;
      if (POOLED) {
        gqv[k] *= pool_w;
        gtv[k] *= pool_w;
      }
      v1[k] = vb[w0 + k];
      v2[k] = vb[kSkewC + wq[k]];
    }
    float o1[4], o2[4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      P2 oq2, ot2, a12, a22;
      abrelu_vjp2(ac, p2(qv[2 * h], qv[2 * h + 1]), p2(tv[2 * h], tv[2 * h + 1]),
                  p2(v1[2 * h], v1[2 * h + 1]), p2(v2[2 * h], v2[2 * h + 1]),
                  p2(gqv[2 * h], gqv[2 * h + 1]), p2(gtv[2 * h], gtv[2 * h + 1]), oq2, ot2, a12,
                  a22);
      p2u(oq2, c[2 * h], c[2 * h + 1]);
      p2u(ot2, a[2 * h], a[2 * h + 1]);
      p2u(a12, o1[2 * h], o1[2 * h + 1]);
      p2u(a22, o2[2 * h], o2[2 * h + 1]);
    }
    // this warp's partial sums of the plane's variance cotangents, written without atomics:
    // var1 at w (the warp's four row groups share w), var2 at w' = w + r, gathered so that
    // lane T holds target T (for element slot k it comes from the lane with 4a + b = T - k - r0)
    float* s = sg + (p % 3) * (kVjpWarps * 64) + (tid >> 5) * 64;
    float y = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float x = o1[k];
      x += __shfl_xor_sync(0xffffffffu, x, 8);
      x += __shfl_xor_sync(0xffffffffu, x, 16);
      if (lane < 8) s[w0 + k] = x;
      const int m = (lane - k - r0) & (kSkewC - 1);
      y += __shfl_sync(0xffffffffu, o2[k], ((m & 3) << 3) | (m >> 2));
    }
    s[kSkewC + lane] = y;
  };

  const float inv9 = 1.f / 9.f;
  const P2 W2 = p2s(w2 * inv9), TW = p2s(w2 * inv9), TN = p2s(w2), Z = p2s(0.f);
  float am[4], cm[4], a0[4], c0[4], ap[4], cp[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) am[k] = cm[k] = 0.f;
  take(0, a0, c0);
  for (int j = 0; j < len; ++j) {
    if (j + 2 < len) load_vars(j + 2);  // buffer (j + 2) % 3 was last read by plane j - 1
    take(j + 1, ap, cp);
    const int i = i_lo + j;
    float ha[4], hc[4], sa[4], sc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      ha[k] = (am[k] + a0[k]) + ap[k];
      hc[k] = (cm[k] + c0[k]) + cp[k];
    }
    {
      const float la = __shfl_up_sync(0xffffffffu, ha[3], 1, 8);
      const float ra = __shfl_down_sync(0xffffffffu, ha[0], 1, 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float L = k == 0 ? la : ha[k - 1], R = k == 3 ? ra : ha[k + 1];
        sa[k] = fmaf(R, mR[k], fmaf(L, mL[k], ha[k]));
      }
    }
    {
      const float lc = __shfl_up_sync(0xffffffffu, hc[3], 1, 8);
      const float rc = __shfl_down_sync(0xffffffffu, hc[0], 1, 8);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float L = k == 0 ? lc : hc[k - 1], R = k == 3 ? rc : hc[k + 1];
        sc[k] = fmaf(R, mR[k], fmaf(L, mL[k], hc[k]));
      }
    }
    // transposed affine rule: g_in_t = W2 S(a), g_in_q = TW S(c) + TN (S(a) / 9)
    float* oq = stage_q + (j & 1) * kSkewPlane;
    float* ot = stage_t + (j & 1) * kSkewPlane;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const P2 ca = p2(sa[2 * h], sa[2 * h + 1]), cc = p2(sc[2 * h], sc[2 * h + 1]);
      const P2 gt_in = fma2(W2, ca, Z);
      const P2 gq_in = fma2(TW, cc, fma2(TN, mul2(ca, p2s(inv9)), Z));
      float x0, x1, y0, y1;
      p2u(gq_in, x0, x1);
      p2u(gt_in, y0, y1);
      oq[u[2 * h]] = x0;
      oq[u[2 * h + 1]] = x1;
      if (gin_t) {
        ot[u[2 * h]] = y0;
        ot[u[2 * h + 1]] = y1;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (j == 0) flush(0);
    if (j + 1 < len) flush(j + 1);
    if (tid == 0) {
      const int64_t off = b * pair_stride + ((int64_t)i * A + i + delta) * kSkewPlane;
      bulk_store(gin_q + off, oq, kSkewPlane * 4u);
      if (gin_t) bulk_store(gin_t + off, ot, kSkewPlane * 4u);
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      // plane j + 1 has been read by every thread: its slot takes plane j + 1 + kVjpRing
      if (!s_err)
        for (; next < len && next <= j + 1 + kVjpRing; ++next) issue(next);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      am[k] = a0[k]; cm[k] = c0[k];
      a0[k] = ap[k]; c0[k] = cp[k];
    }
  }
  if (tid == 0) {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    if (s_err) {
      atomicExch(&g_device_error, NTG_ERR_WAIT_TIMEOUT);
      // let every issued copy land (bounded) before the CTA's shared memory is released
      for (int p = next > kVjpRing ? next - kVjpRing : 0; p < next; ++p)
        bar_wait(smem_addr(&bars[p % kVjpRing]), (uint32_t)((p / kVjpRing) & 1));
    }
  }
}

template <bool POOLED>
__global__ void __launch_bounds__(kThreads)
    conv3_skew_vjp_kernel(const float* __restrict__ pre_q, const float* __restrict__ pre_t,
                          const float* __restrict__ g_q, const float* __restrict__ g_t,
                          float* __restrict__ gin_q, float* __restrict__ gin_t, int64_t batch,
                          int64_t n2, int A, float w2, ntg_act_t act, ntg_var_t var1,
                          ntg_var_t var2, float* __restrict__ gvar1, float* __restrict__ gvar2) {
  skew_vjp_body<POOLED>(pre_q, pre_t, g_q, g_t, gin_q, gin_t, batch, n2, A, w2, act, var1, var2,
                        gvar1, gvar2);
}

// ---------------------------------------------------------------------------
// Diagonal-spatial conv rule: [B, A, C] box filter (linear.py:3381-3437).
// ---------------------------------------------------------------------------
__global__ void conv_ds_kernel(const float* __restrict__ in_q, const float* __restrict__ in_t,
                               float* __restrict__ out_q, float* __restrict__ out_t, ConvGeom g,
                               ntg_affine_t aff) {
  const int64_t per_b = g.Ao * g.Co;
  const int64_t total = g.batch * per_b;
  const float inv = 1.f / (float)(g.fh * g.fw);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / per_b, r = idx - b * per_b;
    int64_t i = r / g.Co, j = r - i * g.Co;
    float sq = 0.f, st = 0.f;
    for (int d = 0; d < g.fh; ++d) {
      int64_t ia = i * g.sh + d - g.ph;
      if (!wrap_index(ia, g.A, g.circular)) continue;
      for (int e = 0; e < g.fw; ++e) {
        int64_t jc = j * g.sw + e - g.pw;
        if (!wrap_index(jc, g.C, g.circular)) continue;
        int64_t off = (b * g.A + ia) * g.C + jc;
        sq += __ldg(in_q + off);
        if (in_t) st += __ldg(in_t + off);
      }
    }
    float q, t = 0.f;
    apply_affine(aff, sq, st, out_t != nullptr, q, t, inv);
    out_q[idx] = q;
    if (out_t) out_t[idx] = t;
  }
}

// ---------------------------------------------------------------------------
// Elementwise affine + activation on [B, M].
// ---------------------------------------------------------------------------
__global__ void affine_act_kernel(const float* __restrict__ in_q, const float* __restrict__ in_t,
                                  float* __restrict__ out_q, float* __restrict__ out_t,
                                  int64_t batch, int64_t n2, int64_t A, int64_t C, int diag,
                                  int has_affine, ntg_affine_t aff, ntg_act_t act,
                                  ntg_var_t var1, ntg_var_t var2) {
  const int64_t M = diag ? A * C : A * A * C * C;
  const int64_t total = batch * M;
  const ActC ac = act_consts(act);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / M, m = idx - b * M;
    float q = in_q[idx];
    float t = in_t ? in_t[idx] : 0.f;
    if (has_affine) {
      float q2, t2 = 0.f;
      apply_affine(aff, q, t, out_t != nullptr, q2, t2);
      q = q2;
      t = t2;
    }
    if (act.kind != NTG_ACT_NONE) {
      int64_t a1, a2, c1, c2;
      if (diag) {
        a1 = a2 = m / C;
        c1 = c2 = m - a1 * C;
      } else {
        int64_t r = m;
        c2 = r % C; r /= C;
        c1 = r % C; r /= C;
        a2 = r % A;
        a1 = r / A;
      }
      int64_t i1, i2;
      pair_of(b, n2, i1, i2);
      act_apply(ac, q, t, var_at(var1, i1, a1, c1), var_at(var2, i2, a2, c2));
    }
    out_q[idx] = q;
    if (out_t) out_t[idx] = t;
  }
}

// The same rule on full-spatial [B, A, A, C, C] kernels with C a power of two in
// [4, 32] and A^2 C^2 a multiple of 1024: chunks of 1024 consecutive entries (4
// per thread, vector loads and stores); the variances a chunk needs, and their
// square roots, are staged in shared memory one chunk ahead (2 C^-1 1024 loads per
// chunk instead of 5 per thread). Same operations per entry as affine_act_kernel.
template <int ACTK>  // 1: no activation or the ABRelu family only; 0: any rule
__global__ void __launch_bounds__(kThreads)
    affine_act_fs_kernel(const float* __restrict__ in_q, const float* __restrict__ in_t,
                         float* __restrict__ out_q, float* __restrict__ out_t, int64_t batch,
                         int64_t n2, int A, int C, int has_affine, ntg_affine_t aff,
                         ntg_act_t act, ntg_var_t var1, ntg_var_t var2) {
  __shared__ __align__(16) float sv[2][4][256];  // [buffer][v1 | sqrt v1 | v2 | sqrt v2][key]
  const int64_t M = (int64_t)A * A * C * C;  // < 2^31 (checked by the host)
  const int P = (int)(M / 1024);              // chunks per pair
  const int64_t chunks = batch * P;
  const ActC ac = act_consts(act);
  const bool has_act = act.kind != NTG_ACT_NONE;
  const int tid = threadIdx.x;
  const int lc = __ffs(C) - 1;  // log2 C
  const int nkeys = 1024 >> lc;
  // keys of chunk (b, j): rows (plane, w) for var1 at (h, w); (plane, w') for var2 at (h', w')
  auto stage = [&](int64_t b, int j, int buf) {
    int64_t i1, i2;
    pair_of(b, n2, i1, i2);
    const int r0 = (j * 1024) >> lc, p0 = (j * 1024) >> (2 * lc);
    for (int k = tid; k < nkeys; k += kThreads) {
      const int rr = r0 + k, pp = p0 + (k >> lc);
      const float v1 = var_at(var1, i1, (rr >> lc) / A, rr & (C - 1));
      const float v2 = var_at(var2, i2, pp % A, k & (C - 1));
      sv[buf][0][k] = v1;
      sv[buf][1][k] = sqrt_var(v1);
      sv[buf][2][k] = v2;
      sv[buf][3][k] = sqrt_var(v2);
    }
  };
  int64_t b = blockIdx.x / P;
  int j = (int)(blockIdx.x - b * P);
  if (has_act && blockIdx.x < chunks) stage(b, j, 0);
  __syncthreads();
  const int k1 = (4 * tid) >> lc;
  const int k2 = (((4 * tid) >> (2 * lc)) << lc) + ((4 * tid) & (C - 1));
  const int step_b = (int)(gridDim.x / P), step_j = (int)(gridDim.x - (int64_t)step_b * P);
  int it = 0;
  for (int64_t ch = blockIdx.x; ch < chunks; ch += gridDim.x, ++it) {
    const int cur = it & 1;
    int64_t bn = b + step_b;
    int jn = j + step_j;
    if (jn >= P) {
      jn -= P;
      ++bn;
    }
    if (has_act && ch + gridDim.x < chunks) stage(bn, jn, cur ^ 1);  // read by the next chunk
    const int64_t e = b * M + (int64_t)j * 1024 + 4 * tid;
    b = bn;
    j = jn;
    const float4 Q = *reinterpret_cast<const float4*>(in_q + e);
    const float4 T = in_t ? *reinterpret_cast<const float4*>(in_t + e)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
    float q[4] = {Q.x, Q.y, Q.z, Q.w}, t[4] = {T.x, T.y, T.z, T.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (has_affine) {
        float q2, t2 = 0.f;
        apply_affine(aff, q[k], t[k], out_t != nullptr, q2, t2);
        q[k] = q2;
        t[k] = t2;
      }
    }
    if (has_act) {
      const float v1 = sv[cur][0][k1], s1 = sv[cur][1][k1];
      const float4 V2 = *reinterpret_cast<const float4*>(&sv[cur][2][k2]);
      const float4 S2 = *reinterpret_cast<const float4*>(&sv[cur][3][k2]);
      const float v2[4] = {V2.x, V2.y, V2.z, V2.w}, s2[4] = {S2.x, S2.y, S2.z, S2.w};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        act_apply<ACTK == 0, ACTK == 0>(ac, q[k], t[k], v1, v2[k], s1, s2[k]);
    }
    *reinterpret_cast<float4*>(out_q + e) = make_float4(q[0], q[1], q[2], q[3]);
    if (out_t) *reinterpret_cast<float4*>(out_t + e) = make_float4(t[0], t[1], t[2], t[3]);
    __syncthreads();
  }
}

__global__ void max_abs_kernel(const float* __restrict__ x, int64_t n, unsigned int* out) {
  float m = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// ---------------------------------------------------------------------------
// Pooling (reduce_window sum over the doubled window) and readouts.
// ---------------------------------------------------------------------------
struct PoolGeom {
  int64_t batch, A, C, Ao, Co;
  int wa, wc, sa, sc, pa, pc, circular, diag, average, normalize_edges, pool2;
};

// Second stage of AvgPool((2, 2), (2, 2)) after conv3_skew_kernel's half-pooled
// output hp [B, A, A, 16, 16] (w-direction window sums of each (h, h') plane):
// out[b, i, i', e] = (((hp(2i+1, 2i') + hp(2i, 2i')) + hp(2i+1, 2i'+1)) + hp(2i, 2i'+1)) / 16,
// pool_kernel's pool2 order, so both paths round alike.
__global__ void pool_planes_kernel(const float* __restrict__ hp, float* __restrict__ out,
                                   int64_t batch, int A) {
  const int Ah = A / 2;
  const int64_t total = batch * Ah * Ah * 256;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(idx & 255);
    int64_t r = idx >> 8;
    const int ip = (int)(r % Ah);
    r /= Ah;
    const int i = (int)(r % Ah);
    const int64_t b = r / Ah;
    const float* base = hp + b * (int64_t)A * A * 256 + e;
    auto plane = [&](int u, int up) {
      return __ldg(base + ((int64_t)(2 * i + u) * A + 2 * ip + up) * 256);
    };
    const float sum = ((plane(1, 0) + plane(0, 0)) + plane(1, 1)) + plane(0, 1);
    out[idx] = sum / 16.f;
  }
}

__global__ void pool_kernel(const float* __restrict__ in, float* __restrict__ out, PoolGeom g) {
  const int64_t per_b = g.diag ? g.Ao * g.Co : g.Ao * g.Ao * g.Co * g.Co;
  const int64_t in_b = g.diag ? g.A * g.C : g.A * g.A * g.C * g.C;
  const int64_t total = g.batch * per_b;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / per_b, r = idx - b * per_b;
    const float* src = in + b * in_b;
    float s = 0.f;
    int count = 0;
    if (g.diag) {
      int64_t i = r / g.Co, j = r - i * g.Co;
      for (int u = 0; u < g.wa; ++u) {
        int64_t ia = i * g.sa + u - g.pa;
        if (!wrap_index(ia, g.A, g.circular)) continue;
        for (int v = 0; v < g.wc; ++v) {
          int64_t jc = j * g.sc + v - g.pc;
          if (!wrap_index(jc, g.C, g.circular)) continue;
          s += __ldg(src + ia * g.C + jc);
          ++count;
        }
      }
    } else if (g.pool2) {
      // AvgPool(2, 2) / stride 2 / VALID: the window is summed plane by plane
      // in the order the fused chain kernel accumulates it (planes (1,0),
      // (0,0), (1,1), (0,1) of the (a, a') window), so both paths round alike.
      int64_t jp = r % g.Co; r /= g.Co;
      int64_t j = r % g.Co; r /= g.Co;
      int64_t ip = r % g.Ao;
      int64_t i = r / g.Ao;
      auto plane = [&](int u, int up) {
        const float* pl = src + (((2 * i + u) * g.A + 2 * ip + up) * g.C + 2 * j) * g.C + 2 * jp;
        return (__ldg(pl) + __ldg(pl + 1)) + (__ldg(pl + g.C) + __ldg(pl + g.C + 1));
      };
      s = ((plane(1, 0) + plane(0, 0)) + plane(1, 1)) + plane(0, 1);
      count = 16;
    } else {
      int64_t jp = r % g.Co; r /= g.Co;
      int64_t j = r % g.Co; r /= g.Co;
      int64_t ip = r % g.Ao;
      int64_t i = r / g.Ao;
      for (int u = 0; u < g.wa; ++u) {
        int64_t ia = i * g.sa + u - g.pa;
        if (!wrap_index(ia, g.A, g.circular)) continue;
        for (int up = 0; up < g.wa; ++up) {
          int64_t iap = ip * g.sa + up - g.pa;
          if (!wrap_index(iap, g.A, g.circular)) continue;
          for (int v = 0; v < g.wc; ++v) {
            int64_t jc = j * g.sc + v - g.pc;
            if (!wrap_index(jc, g.C, g.circular)) continue;
            const float* row = src + ((ia * g.A + iap) * g.C + jc) * g.C;
            for (int vp = 0; vp < g.wc; ++vp) {
              int64_t jcp = jp * g.sc + vp - g.pc;
              if (!wrap_index(jcp, g.C, g.circular)) continue;
              s += __ldg(row + jcp);
              ++count;
            }
          }
        }
      }
    }
    if (g.average) {
      float norm;
      if (g.normalize_edges) {
        norm = (float)count;
      } else {
        norm = g.diag ? (float)(g.wa * g.wc) : (float)(g.wa * g.wa * g.wc * g.wc);
      }
      s = s / norm;
      if (g.diag) s = s / norm;
    }
    out[idx] = s;
  }
}

__global__ void global_pool_kernel(const float* __restrict__ in, float* __restrict__ out,
                                   int64_t m, int average, float post_scale) {
  const float* row = in + (int64_t)blockIdx.x * m;
  float s = 0.f;
  for (int64_t k = threadIdx.x; k < m; k += blockDim.x) s += __ldg(row + k);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ float part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) {
      if (average) s = s / (float)m;
      out[blockIdx.x] = s * post_scale;
    }
  }
}

__global__ void flatten_fs_kernel(const float* __restrict__ in, float* __restrict__ out,
                                  int64_t A, int64_t C) {
  const float* src = in + (int64_t)blockIdx.x * A * A * C * C;
  float s = 0.f;
  for (int64_t k = threadIdx.x; k < A * C; k += blockDim.x) {
    int64_t a = k / C, c = k - a * C;
    s += __ldg(src + ((a * A + a) * C + c) * C + c);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ float part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[blockIdx.x] = s / (float)(A * C);
  }
}

int grid_for(int64_t total, int threads = kThreads) {
  int64_t g = ceil_div(total, threads);
  if (g > (int64_t)152 * 64) g = (int64_t)152 * 64;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace ntg

using namespace ntg;

extern "C" size_t ntg_gram_workspace_bytes(int64_t n1, int64_t n2, int64_t d) {
  return gram_tc_workspace(n1, n2, d);
}

extern "C" int ntg_gram(void* stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
                        int64_t d, float* nngp, int32_t precision, void* workspace,
                        size_t workspace_bytes) {
  NTG_REQUIRE(x1 && x2 && nngp, "ntg_gram: null pointer");
  NTG_REQUIRE(n1 > 0 && n2 > 0 && d > 0, "ntg_gram: sizes must be positive");
  if (precision == 1) {
    return gram_tc(as_stream(stream), x1, x2, n1, n2, d, nngp, workspace, workspace_bytes);
  }
  NTG_REQUIRE(precision == 0, "ntg_gram: precision must be 0 or 1");
  NTG_REQUIRE(ceil_div(n1, 128) <= 65535, "ntg_gram: n1 too large");
  const int64_t nb1 = ceil_div(n1, 128);
  if (x1 == x2 && n1 == n2) {  // the lower triangle of tiles, mirrored
    gram_simt_kernel<true><<<(unsigned)(nb1 * (nb1 + 1) / 2), 256, 0, as_stream(stream)>>>(
        x1, x2, n1, n2, d, 1.f / (float)d, nngp);
  } else {
    dim3 grid((unsigned)ceil_div(n2, 128), (unsigned)nb1);
    gram_simt_kernel<false><<<grid, 256, 0, as_stream(stream)>>>(x1, x2, n1, n2, d,
                                                                 1.f / (float)d, nngp);
  }
  note_launch();
  return check_launch("ntg_gram");
}

extern "C" int ntg_gemm(void* stream, const float* a, const float* b, float* c, int64_t m,
                        int64_t n, int64_t k, int32_t accumulate) {
  NTG_REQUIRE(a && b && c, "ntg_gemm: null pointer");
  NTG_REQUIRE(m > 0 && n > 0 && k > 0, "ntg_gemm: sizes must be positive");
  NTG_REQUIRE(ceil_div(m, 64) <= 65535, "ntg_gemm: m too large");
  dim3 grid((unsigned)ceil_div(n, 64), (unsigned)ceil_div(m, 64));
  gemm_nn_kernel<<<grid, 256, 0, as_stream(stream)>>>(a, b, c, m, n, k, accumulate);
  note_launch();
  return check_launch("ntg_gemm");
}

extern "C" int ntg_cov_diag(void* stream, const float* x, int64_t n, int64_t d, float* cov) {
  NTG_REQUIRE(x && cov, "ntg_cov_diag: null pointer");
  NTG_REQUIRE(n > 0 && d > 0, "ntg_cov_diag: sizes must be positive");
  cov_diag_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, as_stream(stream)>>>(x, n, d,
                                                                             1.f / (float)d, cov);
  note_launch();
  return check_launch("ntg_cov_diag");
}

extern "C" int ntg_input_fs(void* stream, const float* x1, const float* x2, int64_t n1,
                            int64_t n2, int64_t a, int64_t c, int64_t k, int32_t pairs,
                            float* out) {
  NTG_REQUIRE(x1 && out, "ntg_input_fs: null pointer");
  NTG_REQUIRE(n1 > 0 && a > 0 && c > 0 && k > 0, "ntg_input_fs: sizes must be positive");
  int64_t batch = pairs ? n1 * n2 : n1;
  NTG_REQUIRE(!pairs || (x2 && n2 > 0), "ntg_input_fs: pairs mode needs x2 and n2 > 0");
  const float* xb = pairs ? x2 : x1;
  int64_t blocks = batch * a;
  NTG_REQUIRE(blocks < (1ll << 31), "ntg_input_fs: grid too large");
  const size_t vec_sm = sizeof(float) * 4 * (c + a * c);
  if (c >= 4 && c <= 32 && (c & (c - 1)) == 0 && k <= 4 && vec_sm <= 48 * 1024 &&
      (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
    input_fs_vec_kernel<<<(unsigned)blocks, 256, vec_sm, as_stream(stream)>>>(
        x1, xb, batch, pairs ? n2 : 0, (int)a, (int)c, (int)k, 1.f / (float)k, out);
  } else {
    input_fs_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(
        x1, xb, batch, pairs ? n2 : 0, a, c, k, 1.f / (float)k, out);
  }
  note_launch();
  return check_launch("ntg_input_fs");
}

// Diagonal-spatial input covariances (requirements.py:641-830 with
// diagonal_spatial): out[i, j, p] = sum_k x1[i, p, k] x2[j, p, k] / K over the
// P spatial positions, or out[i, p] = sum_k x1[i, p, k]^2 / K without x2. Both
// forms sum the channels in the same order, so a self pair gives
// var1 * var2 - nngp^2 == 0 exactly.
__global__ void input_ds_kernel(const float* __restrict__ x1, const float* __restrict__ x2,
                                int64_t n2, int64_t total, int64_t P, int K, float inv_k,
                                float* __restrict__ out) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = idx % P, b = idx / P;
    const int64_t i = n2 > 0 ? b / n2 : b, j = n2 > 0 ? b - i * n2 : b;
    const float* a = x1 + (i * P + p) * K;
    const float* c = (n2 > 0 ? x2 : x1) + (j * P + p) * K;
    float g = 0.f;
    for (int k = 0; k < K; ++k) g = fmaf(a[k], c[k], g);
    out[idx] = g * inv_k;
  }
}

extern "C" int ntg_input_ds(void* stream, const float* x1, const float* x2, int64_t n1,
                            int64_t n2, int64_t p, int64_t k, float* out) {
  NTG_REQUIRE(x1 && out, "ntg_input_ds: null pointer");
  NTG_REQUIRE(n1 > 0 && p > 0 && k > 0 && k < (1 << 30), "ntg_input_ds: sizes must be positive");
  NTG_REQUIRE(!x2 == (n2 == 0) && n2 >= 0, "ntg_input_ds: x2 and n2 > 0 go together");
  const int64_t total = (n2 > 0 ? n1 * n2 : n1) * p;
  input_ds_kernel<<<grid_for(total), 256, 0, as_stream(stream)>>>(x1, x2, n2, total, p, (int)k,
                                                                  1.f / (float)k, out);
  note_launch();
  return check_launch("ntg_input_ds");
}

template <bool HAS_T, int RING, int ACTK, bool HP = false>
cudaError_t launch_skew_k(cudaStream_t s, int64_t blocks, size_t sm, const float* in_q,
                          const float* in_t, float* out_q, float* out_t, int64_t batch,
                          int64_t n2, int64_t a, ntg_affine_t aff, ntg_act_t act, ntg_var_t var1,
                          ntg_var_t var2, float* pre_q, float* pre_t, float* hp_q,
                          float* hp_t) {
  cudaError_t e = cudaFuncSetAttribute(conv3_skew_kernel<HAS_T, RING, ACTK, HP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)skew_smem_bytes_pre<RING>());
  if (e == cudaSuccess)
    conv3_skew_kernel<HAS_T, RING, ACTK, HP><<<(unsigned)blocks, kThreads, sm, s>>>(
        in_q, in_t, out_q, out_t, batch, n2, (int)a, aff, act, var1, var2, pre_q, pre_t, hp_q,
        hp_t);
  return e;
}

template <int RING>
cudaError_t launch_skew(cudaStream_t s, int64_t blocks, const float* in_q, const float* in_t,
                        float* out_q, float* out_t, int64_t batch, int64_t n2, int64_t a,
                        ntg_affine_t aff, ntg_act_t act, ntg_var_t var1, ntg_var_t var2,
                        float* pre_q = nullptr, float* pre_t = nullptr) {
  const size_t sm = pre_q ? skew_smem_bytes_pre<RING>() : skew_smem_bytes<RING>();
  const bool relu = act.kind == NTG_ACT_NONE ||
                    (act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f);
  if (in_t)
    return relu ? launch_skew_k<true, RING, 1>(s, blocks, sm, in_q, in_t, out_q, out_t, batch, n2,
                                               a, aff, act, var1, var2, pre_q, pre_t, nullptr,
                                               nullptr)
                : launch_skew_k<true, RING, 0>(s, blocks, sm, in_q, in_t, out_q, out_t, batch, n2,
                                               a, aff, act, var1, var2, pre_q, pre_t, nullptr,
                                               nullptr);
  return relu ? launch_skew_k<false, RING, 1>(s, blocks, sm, in_q, nullptr, out_q, out_t, batch,
                                              n2, a, aff, act, var1, var2, pre_q, pre_t, nullptr,
                                              nullptr)
              : launch_skew_k<false, RING, 0>(s, blocks, sm, in_q, nullptr, out_q, out_t, batch,
                                              n2, a, aff, act, var1, var2, pre_q, pre_t, nullptr,
                                              nullptr);
}

// The conv + activation kernel with the half-pooled output (ring depth 4).
cudaError_t launch_skew_pool(cudaStream_t s, int64_t blocks, const float* in_q,
                             const float* in_t, int64_t batch, int64_t n2, int64_t a,
                             ntg_affine_t aff, ntg_act_t act, ntg_var_t var1, ntg_var_t var2,
                             float* pre_q, float* pre_t, float* hp_q, float* hp_t) {
  const size_t sm = skew_smem_bytes_pre<4>();
  const bool relu = act.kind == NTG_ACT_NONE ||
                    (act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f);
  if (in_t)
    return relu ? launch_skew_k<true, 4, 1, true>(s, blocks, sm, in_q, in_t, nullptr, nullptr,
                                                  batch, n2, a, aff, act, var1, var2, pre_q,
                                                  pre_t, hp_q, hp_t)
                : launch_skew_k<true, 4, 0, true>(s, blocks, sm, in_q, in_t, nullptr, nullptr,
                                                  batch, n2, a, aff, act, var1, var2, pre_q,
                                                  pre_t, hp_q, hp_t);
  return relu ? launch_skew_k<false, 4, 1, true>(s, blocks, sm, in_q, nullptr, nullptr, nullptr,
                                                 batch, n2, a, aff, act, var1, var2, pre_q,
                                                 pre_t, hp_q, hp_t)
              : launch_skew_k<false, 4, 0, true>(s, blocks, sm, in_q, nullptr, nullptr, nullptr,
                                                 batch, n2, a, aff, act, var1, var2, pre_q,
                                                 pre_t, hp_q, hp_t);
}

extern "C" int ntg_conv_fs(void* stream, const float* in_q, const float* in_t, float* out_q,
                           float* out_t, int64_t batch, int64_t n2, int64_t a, int64_t c,
                           int32_t fh, int32_t fw, int32_t sh, int32_t sw, int32_t ph, int32_t pw,
                           int64_t ao, int64_t co, int32_t pad_mode, ntg_affine_t aff,
                           ntg_act_t act, ntg_var_t var1, ntg_var_t var2) {
  NTG_REQUIRE(in_q && out_q, "ntg_conv_fs: null pointer");
  NTG_REQUIRE(batch > 0 && a > 0 && c > 0 && ao > 0 && co > 0, "ntg_conv_fs: bad sizes");
  NTG_REQUIRE(fh > 0 && fw > 0 && sh > 0 && sw > 0 && ph >= 0 && pw >= 0,
              "ntg_conv_fs: bad filter geometry");
  NTG_REQUIRE(act.kind == NTG_ACT_NONE || (var1.base && var2.base),
              "ntg_conv_fs: activation needs var1/var2");
  cudaStream_t s = as_stream(stream);
  const bool line_ok = fh == 3 && fw == 3 && sh == 1 && sw == 1 && ph == 1 && pw == 1 &&
                       ao == a && co == c && pad_mode == NTG_PAD_ZERO && c % 4 == 0 &&
                       c * c <= 4 * kThreads && a <= 4096;
  const bool aligned = ((reinterpret_cast<uintptr_t>(in_q) | reinterpret_cast<uintptr_t>(in_t) |
                         reinterpret_cast<uintptr_t>(out_q) | reinterpret_cast<uintptr_t>(out_t)) &
                        15) == 0;
  if (line_ok && aligned && c == kSkewC) {
    int64_t blocks = batch * (2 * a - 1);
    NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_fs: grid too large");
    cudaError_t e;
    switch (tune(NTG_TUNE_STENCIL_RING)) {
      case 2: e = launch_skew<2>(s, blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2); break;
      case 3: e = launch_skew<3>(s, blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2); break;
      case 6: e = launch_skew<6>(s, blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2); break;
      default: e = launch_skew<4>(s, blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2); break;
    }
    if (e != cudaSuccess) return fail(NTG_ERR_CUDA, std::string("ntg_conv_fs: ") + cudaGetErrorString(e));
  } else if (line_ok && aligned) {
    int64_t blocks = batch * (2 * a - 1);
    NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_fs: grid too large");
    const size_t sm = sizeof(float) * (2 * kRing * c * c + 4 * (c + 2) * (c + 2)) +
                      sizeof(uint64_t) * kRing;
    cudaError_t e;
    if (in_t) {
      e = cudaFuncSetAttribute(conv3_line_bulk_kernel<true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e == cudaSuccess)
        conv3_line_bulk_kernel<true><<<(unsigned)blocks, kThreads, sm, s>>>(
            in_q, in_t, out_q, out_t, batch, n2, (int)a, (int)c, aff, act, var1, var2);
    } else {
      e = cudaFuncSetAttribute(conv3_line_bulk_kernel<false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e == cudaSuccess)
        conv3_line_bulk_kernel<false><<<(unsigned)blocks, kThreads, sm, s>>>(
            in_q, nullptr, out_q, out_t, batch, n2, (int)a, (int)c, aff, act, var1, var2);
    }
    if (e != cudaSuccess) return fail(NTG_ERR_CUDA, std::string("ntg_conv_fs: ") + cudaGetErrorString(e));
  } else if (line_ok) {
    int64_t blocks = batch * (2 * a - 1);
    NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_fs: grid too large");
    size_t sm = sizeof(float) * 4 * (c + 2) * (c + 2);
    if (in_t)
      conv3_line_kernel<false, true><<<(unsigned)blocks, kThreads, sm, s>>>(
          in_q, in_t, nullptr, nullptr, 0, 0.f, out_q, out_t, batch, n2, (int)a, (int)c, aff, act,
          var1, var2);
    else
      conv3_line_kernel<false, false><<<(unsigned)blocks, kThreads, sm, s>>>(
          in_q, nullptr, nullptr, nullptr, 0, 0.f, out_q, out_t, batch, n2, (int)a, (int)c, aff,
          act, var1, var2);
  } else {
    ConvGeom g{batch, n2, a, c, ao, co, fh, fw, sh, sw, ph, pw, pad_mode == NTG_PAD_CIRCULAR};
    int64_t total = batch * ao * ao * co * co;
    conv_fs_general_kernel<<<grid_for(total), kThreads, 0, s>>>(in_q, in_t, out_q, out_t, g, aff,
                                                                 act, var1, var2);
  }
  note_launch();
  return check_launch("ntg_conv_fs");
}

extern "C" int ntg_conv_act_fs(void* stream, const float* in_q, const float* in_t,
                               float* out_q, float* out_t, float* pre_q, float* pre_t,
                               int64_t batch, int64_t n2, int64_t a, int64_t c, ntg_affine_t aff,
                               ntg_act_t act, ntg_var_t var1, ntg_var_t var2) {
  NTG_REQUIRE(in_q && out_q && pre_q, "ntg_conv_act_fs: null pointer");
  NTG_REQUIRE(!out_t == !pre_t, "ntg_conv_act_fs: out_t and pre_t go together");
  NTG_REQUIRE(batch > 0 && a > 0 && a <= 4096, "ntg_conv_act_fs: bad sizes");
  NTG_REQUIRE(act.kind == NTG_ACT_NONE || (var1.base && var2.base),
              "ntg_conv_act_fs: activation needs var1/var2");
  const bool aligned = ((reinterpret_cast<uintptr_t>(in_q) | reinterpret_cast<uintptr_t>(in_t) |
                         reinterpret_cast<uintptr_t>(out_q) | reinterpret_cast<uintptr_t>(out_t) |
                         reinterpret_cast<uintptr_t>(pre_q) | reinterpret_cast<uintptr_t>(pre_t)) &
                        15) == 0;
  if (c != kSkewC || !aligned)
    return fail(NTG_ERR_UNSUPPORTED,
                "ntg_conv_act_fs: needs 32 x 32 planes and 16-byte aligned buffers");
  const int64_t blocks = batch * (2 * a - 1);
  NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_act_fs: grid too large");
  cudaError_t e;
  switch (tune(NTG_TUNE_STENCIL_RING)) {
    case 2: e = launch_skew<2>(as_stream(stream), blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2, pre_q, pre_t); break;
    case 3: e = launch_skew<3>(as_stream(stream), blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2, pre_q, pre_t); break;
    case 6: e = launch_skew<6>(as_stream(stream), blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2, pre_q, pre_t); break;
    default: e = launch_skew<4>(as_stream(stream), blocks, in_q, in_t, out_q, out_t, batch, n2, a, aff, act, var1, var2, pre_q, pre_t); break;
  }
  if (e != cudaSuccess) return fail(NTG_ERR_CUDA, std::string("ntg_conv_act_fs: ") + cudaGetErrorString(e));
  note_launch();
  return check_launch("ntg_conv_act_fs");
}

template <int K, int ACTK>
cudaError_t launch_skew_input_k(cudaStream_t s, int64_t blocks, const float* x1,
                                const float* x2, float* out_q, float* out_t, float* pre_q,
                                int64_t batch, int64_t n2, ntg_affine_t aff, ntg_act_t act,
                                ntg_var_t var1, ntg_var_t var2) {
  constexpr size_t sm = skew_input_smem_bytes<K>();
  cudaError_t e = cudaFuncSetAttribute(conv3_skew_input_kernel<K, ACTK>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess)
    conv3_skew_input_kernel<K, ACTK><<<(unsigned)blocks, kThreads, sm, s>>>(
        x1, x2, out_q, out_t, pre_q, batch, n2, aff, act, var1, var2, 1.f / (float)K);
  return e;
}

template <int K>
cudaError_t launch_skew_input(bool relu, cudaStream_t s, int64_t blocks, const float* x1,
                              const float* x2, float* out_q, float* out_t, float* pre_q,
                              int64_t batch, int64_t n2, ntg_affine_t aff, ntg_act_t act,
                              ntg_var_t var1, ntg_var_t var2) {
  return relu ? launch_skew_input_k<K, 1>(s, blocks, x1, x2, out_q, out_t, pre_q, batch, n2, aff,
                                          act, var1, var2)
              : launch_skew_input_k<K, 0>(s, blocks, x1, x2, out_q, out_t, pre_q, batch, n2, aff,
                                          act, var1, var2);
}

extern "C" int ntg_input_conv_act_fs(void* stream, const float* x1, const float* x2, int64_t n1,
                                     int64_t n2, int64_t k, float* out_q, float* out_t,
                                     float* pre_q, ntg_affine_t aff, ntg_act_t act,
                                     ntg_var_t var1, ntg_var_t var2) {
  NTG_REQUIRE(x1 && x2 && out_q && out_t && pre_q && var1.base && var2.base,
              "ntg_input_conv_act_fs: null pointer");
  NTG_REQUIRE(n1 > 0 && n2 > 0 && k >= 1 && k <= 4, "ntg_input_conv_act_fs: bad sizes");
  NTG_REQUIRE(aff.ntk_nn == 1.f && aff.ntk_c == 0.f && aff.nn_scaled,
              "ntg_input_conv_act_fs: needs the NTK rule ntk = nngp_out + W^2 ntk_in");
  NTG_REQUIRE(act.kind != NTG_ACT_NONE, "ntg_input_conv_act_fs: needs an activation");
  const bool aligned = ((reinterpret_cast<uintptr_t>(out_q) | reinterpret_cast<uintptr_t>(out_t) |
                         reinterpret_cast<uintptr_t>(pre_q)) & 15) == 0;
  NTG_REQUIRE(aligned, "ntg_input_conv_act_fs: outputs must be 16-byte aligned");
  const int64_t batch = n1 * n2;
  const int64_t blocks = batch * (2 * kSkewC - 1);
  NTG_REQUIRE(blocks < (1ll << 31), "ntg_input_conv_act_fs: grid too large");
  const bool relu = act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f;
  cudaStream_t s = as_stream(stream);
  cudaError_t e;
  switch (k) {
    case 1: e = launch_skew_input<1>(relu, s, blocks, x1, x2, out_q, out_t, pre_q, batch, n2, aff, act, var1, var2); break;
    case 2: e = launch_skew_input<2>(relu, s, blocks, x1, x2, out_q, out_t, pre_q, batch, n2, aff, act, var1, var2); break;
    case 3: e = launch_skew_input<3>(relu, s, blocks, x1, x2, out_q, out_t, pre_q, batch, n2, aff, act, var1, var2); break;
    default: e = launch_skew_input<4>(relu, s, blocks, x1, x2, out_q, out_t, pre_q, batch, n2, aff, act, var1, var2); break;
  }
  if (e != cudaSuccess)
    return fail(NTG_ERR_CUDA, std::string("ntg_input_conv_act_fs: ") + cudaGetErrorString(e));
  note_launch();
  return check_launch("ntg_input_conv_act_fs");
}

template <bool POOLED>
cudaError_t launch_skew_vjp(cudaStream_t s, int64_t blocks, const float* pre_q, const float* pre_t,
                            const float* g_q, const float* g_t, float* gin_q, float* gin_t,
                            int64_t batch, int64_t n2, int64_t a, float w2, ntg_act_t act,
                            ntg_var_t var1, ntg_var_t var2, float* gvar1, float* gvar2) {
  constexpr size_t sm = skew_vjp_smem_bytes<POOLED>();
  cudaError_t e = cudaFuncSetAttribute(conv3_skew_vjp_kernel<POOLED>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  // all of the unified L1 / shared memory as shared memory: the resident CTAs' rings
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(conv3_skew_vjp_kernel<POOLED>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e == cudaSuccess)
    conv3_skew_vjp_kernel<POOLED><<<(unsigned)blocks, kThreads, sm, s>>>(
        pre_q, pre_t, g_q, g_t, gin_q, gin_t, batch, n2, (int)a, w2, act, var1, var2, gvar1,
        gvar2);
  return e;
}

extern "C" int ntg_conv_act_bwd(void* stream, const float* pre_q, const float* pre_t,
                                const float* g_q, const float* g_t, int32_t pooled, float* gin_q,
                                float* gin_t, int64_t batch, int64_t n2, int64_t a, float w2,
                                ntg_act_t act, ntg_var_t var1, ntg_var_t var2, float* gvar1,
                                float* gvar2) {
  NTG_REQUIRE(pre_q && pre_t && gin_q && var1.base && var2.base,
              "ntg_conv_act_bwd: null pointer");
  NTG_REQUIRE(batch > 0 && a == kSkewC, "ntg_conv_act_bwd: needs [B, 32, 32, 32, 32] kernels");
  NTG_REQUIRE(act.kind == NTG_ACT_ABRELU && act.stabilize <= 0.f,
              "ntg_conv_act_bwd: fuses the ABRelu rule (without do_stabilize) only");
  const bool aligned =
      ((reinterpret_cast<uintptr_t>(pre_q) | reinterpret_cast<uintptr_t>(pre_t) |
        reinterpret_cast<uintptr_t>(g_q) | reinterpret_cast<uintptr_t>(g_t) |
        reinterpret_cast<uintptr_t>(gin_q) | reinterpret_cast<uintptr_t>(gin_t)) & 15) == 0;
  NTG_REQUIRE(aligned, "ntg_conv_act_bwd: buffers must be 16-byte aligned");
  const int64_t blocks = batch * (2 * a - 1);
  NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_act_bwd: grid too large");
  const cudaError_t e =
      pooled ? launch_skew_vjp<true>(as_stream(stream), blocks, pre_q, pre_t, g_q, g_t, gin_q,
                                     gin_t, batch, n2, a, w2, act, var1, var2, gvar1, gvar2)
             : launch_skew_vjp<false>(as_stream(stream), blocks, pre_q, pre_t, g_q, g_t, gin_q,
                                      gin_t, batch, n2, a, w2, act, var1, var2, gvar1, gvar2);
  if (e != cudaSuccess)
    return fail(NTG_ERR_CUDA, std::string("ntg_conv_act_bwd: ") + cudaGetErrorString(e));
  note_launch();
  return check_launch("ntg_conv_act_bwd");
}

extern "C" int ntg_conv_act_pool_fs(void* stream, const float* in_q, const float* in_t,
                                    float* out_q, float* out_t, float* pre_q, float* pre_t,
                                    float* hp_q, float* hp_t, int64_t batch, int64_t n2,
                                    int64_t a, ntg_affine_t aff, ntg_act_t act, ntg_var_t var1,
                                    ntg_var_t var2) {
  NTG_REQUIRE(in_q && out_q && pre_q && hp_q, "ntg_conv_act_pool_fs: null pointer");
  NTG_REQUIRE(!out_t == !pre_t && !out_t == !hp_t,
              "ntg_conv_act_pool_fs: out_t, pre_t and hp_t go together");
  NTG_REQUIRE(batch > 0 && a == kSkewC, "ntg_conv_act_pool_fs: needs [B, 32, 32, 32, 32] kernels");
  NTG_REQUIRE(act.kind == NTG_ACT_NONE || (var1.base && var2.base),
              "ntg_conv_act_pool_fs: activation needs var1/var2");
  const bool aligned = ((reinterpret_cast<uintptr_t>(in_q) | reinterpret_cast<uintptr_t>(in_t) |
                         reinterpret_cast<uintptr_t>(pre_q) | reinterpret_cast<uintptr_t>(pre_t)) &
                        15) == 0;
  NTG_REQUIRE(aligned, "ntg_conv_act_pool_fs: buffers must be 16-byte aligned");
  const int64_t blocks = batch * (2 * a - 1);
  NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_act_pool_fs: grid too large");
  cudaStream_t s = as_stream(stream);
  const cudaError_t e = launch_skew_pool(s, blocks, in_q, in_t, batch, n2, a, aff, act, var1,
                                         var2, pre_q, pre_t, hp_q, hp_t);
  if (e != cudaSuccess)
    return fail(NTG_ERR_CUDA, std::string("ntg_conv_act_pool_fs: ") + cudaGetErrorString(e));
  note_launch();
  const int64_t total = batch * (a / 2) * (a / 2) * 256;
  pool_planes_kernel<<<grid_for(total), kThreads, 0, s>>>(hp_q, out_q, batch, (int)a);
  note_launch();
  if (out_t) {
    pool_planes_kernel<<<grid_for(total), kThreads, 0, s>>>(hp_t, out_t, batch, (int)a);
    note_launch();
  }
  return check_launch("ntg_conv_act_pool_fs");
}

extern "C" int ntg_conv_input_fs(void* stream, const float* x1, const float* x2, int64_t n1,
                                 int64_t n2, int64_t a, int64_t c, int64_t k, float* out_q,
                                 float* out_t, ntg_affine_t aff, ntg_act_t act, ntg_var_t var1,
                                 ntg_var_t var2) {
  NTG_REQUIRE(x1 && x2 && out_q, "ntg_conv_input_fs: null pointer");
  NTG_REQUIRE(n1 > 0 && n2 > 0 && a > 0 && c > 0 && k > 0, "ntg_conv_input_fs: bad sizes");
  NTG_REQUIRE(c % 4 == 0 && c * c <= 4 * kThreads, "ntg_conv_input_fs: needs C % 4 == 0, C <= 32");
  NTG_REQUIRE(act.kind == NTG_ACT_NONE || (var1.base && var2.base),
              "ntg_conv_input_fs: activation needs var1/var2");
  int64_t batch = n1 * n2;
  int64_t blocks = batch * (2 * a - 1);
  NTG_REQUIRE(blocks < (1ll << 31), "ntg_conv_input_fs: grid too large");
  size_t sm = sizeof(float) * 4 * (c + 2) * (c + 2);
  conv3_line_kernel<true, false><<<(unsigned)blocks, kThreads, sm, as_stream(stream)>>>(
      nullptr, nullptr, x1, x2, k, 1.f / (float)k, out_q, out_t, batch, n2, (int)a, (int)c, aff,
      act, var1, var2);
  note_launch();
  return check_launch("ntg_conv_input_fs");
}

extern "C" int ntg_conv_ds(void* stream, const float* in_q, const float* in_t, float* out_q,
                           float* out_t, int64_t batch, int64_t a, int64_t c, int32_t fh,
                           int32_t fw, int32_t sh, int32_t sw, int32_t ph, int32_t pw, int64_t ao,
                           int64_t co, int32_t pad_mode, ntg_affine_t aff) {
  NTG_REQUIRE(in_q && out_q, "ntg_conv_ds: null pointer");
  NTG_REQUIRE(batch > 0 && a > 0 && c > 0 && ao > 0 && co > 0, "ntg_conv_ds: bad sizes");
  ConvGeom g{batch, 0, a, c, ao, co, fh, fw, sh, sw, ph, pw, pad_mode == NTG_PAD_CIRCULAR};
  conv_ds_kernel<<<grid_for(batch * ao * co), kThreads, 0, as_stream(stream)>>>(in_q, in_t, out_q,
                                                                              out_t, g, aff);
  note_launch();
  return check_launch("ntg_conv_ds");
}

extern "C" int ntg_affine_act(void* stream, const float* in_q, const float* in_t, float* out_q,
                              float* out_t, int64_t batch, int64_t n2, int64_t a, int64_t c,
                              int32_t diag_spatial, int32_t has_affine, ntg_affine_t aff,
                              ntg_act_t act, ntg_var_t var1, ntg_var_t var2) {
  NTG_REQUIRE(in_q && out_q, "ntg_affine_act: null pointer");
  NTG_REQUIRE(batch > 0 && a > 0 && c > 0, "ntg_affine_act: bad sizes");
  NTG_REQUIRE(act.kind == NTG_ACT_NONE || (var1.base && var2.base),
              "ntg_affine_act: activation needs var1/var2");
  int64_t m = diag_spatial ? a * c : a * a * c * c;
  const bool pow2 = c >= 4 && c <= 32 && (c & (c - 1)) == 0;
  const bool aligned = ((reinterpret_cast<uintptr_t>(in_q) | reinterpret_cast<uintptr_t>(in_t) |
                         reinterpret_cast<uintptr_t>(out_q) | reinterpret_cast<uintptr_t>(out_t)) &
                        15) == 0;
  if (!diag_spatial && pow2 && m % 1024 == 0 && aligned && m < (1ll << 31)) {
    const int64_t chunks = batch * (m / 1024);
    const int grid = (int)(chunks < 152 * 8 ? chunks : 152 * 8);
    const bool relu = act.kind == NTG_ACT_NONE || act.kind == NTG_ACT_ABRELU;
    if (relu)
      affine_act_fs_kernel<1><<<grid, kThreads, 0, as_stream(stream)>>>(
          in_q, in_t, out_q, out_t, batch, n2, (int)a, (int)c, has_affine, aff, act, var1, var2);
    else
      affine_act_fs_kernel<0><<<grid, kThreads, 0, as_stream(stream)>>>(
        in_q, in_t, out_q, out_t, batch, n2, (int)a, (int)c, has_affine, aff, act, var1, var2);
  } else {
    affine_act_kernel<<<grid_for(batch * m), kThreads, 0, as_stream(stream)>>>(
        in_q, in_t, out_q, out_t, batch, n2, a, c, diag_spatial, has_affine, aff, act, var1,
        var2);
  }
  note_launch();
  return check_launch("ntg_affine_act");
}

extern "C" int ntg_max_abs(void* stream, const float* x, int64_t n, float* out) {
  NTG_REQUIRE(x && out && n > 0, "ntg_max_abs: bad arguments");
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out, 0, sizeof(float), s) != cudaSuccess)
    return check_launch("ntg_max_abs memset");
  max_abs_kernel<<<grid_for(n), kThreads, 0, s>>>(x, n, reinterpret_cast<unsigned int*>(out));
  note_launch();
  return check_launch("ntg_max_abs");
}

extern "C" int ntg_pool(void* stream, const float* in, float* out, int64_t batch, int64_t a,
                        int64_t c, int32_t wa, int32_t wc, int32_t sa, int32_t sc, int32_t pa,
                        int32_t pc, int64_t ao, int64_t co, int32_t pad_mode,
                        int32_t diag_spatial, int32_t average, int32_t normalize_edges) {
  NTG_REQUIRE(in && out, "ntg_pool: null pointer");
  NTG_REQUIRE(batch > 0 && a > 0 && c > 0 && ao > 0 && co > 0, "ntg_pool: bad sizes");
  NTG_REQUIRE(wa > 0 && wc > 0 && sa > 0 && sc > 0 && pa >= 0 && pc >= 0, "ntg_pool: bad window");
  const int pool2 = !diag_spatial && wa == 2 && wc == 2 && sa == 2 && sc == 2 && pa == 0 &&
                    pc == 0 && 2 * ao <= a && 2 * co <= c;
  PoolGeom g{batch, a, c, ao, co, wa, wc, sa, sc, pa, pc, pad_mode == NTG_PAD_CIRCULAR,
             diag_spatial, average, normalize_edges, pool2};
  int64_t total = diag_spatial ? batch * ao * co : batch * ao * ao * co * co;
  pool_kernel<<<grid_for(total), kThreads, 0, as_stream(stream)>>>(in, out, g);
  note_launch();
  return check_launch("ntg_pool");
}

extern "C" int ntg_global_pool(void* stream, const float* in, float* out, int64_t batch,
                               int64_t m, int32_t average, float post_scale) {
  NTG_REQUIRE(in && out && batch > 0 && m > 0, "ntg_global_pool: bad arguments");
  NTG_REQUIRE(batch < (1ll << 31), "ntg_global_pool: batch too large");
  global_pool_kernel<<<(unsigned)batch, kThreads, 0, as_stream(stream)>>>(in, out, m, average,
                                                                          post_scale);
  note_launch();
  return check_launch("ntg_global_pool");
}

extern "C" int ntg_flatten_fs(void* stream, const float* in, float* out, int64_t batch,
                              int64_t a, int64_t c) {
  NTG_REQUIRE(in && out && batch > 0 && a > 0 && c > 0, "ntg_flatten_fs: bad arguments");
  NTG_REQUIRE(batch < (1ll << 31), "ntg_flatten_fs: batch too large");
  flatten_fs_kernel<<<(unsigned)batch, kThreads, 0, as_stream(stream)>>>(in, out, a, c);
  note_launch();
  return check_launch("ntg_flatten_fs");
}

extern "C" int ntg_device_status(void) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_device_error, sizeof(int)) != cudaSuccess)
    return check_launch("ntg_device_status");
  const int zero = 0;
  if (v != 0 && cudaMemcpyToSymbol(g_device_error, &zero, sizeof(int)) != cudaSuccess)
    return check_launch("ntg_device_status");
  // every word is read and cleared, so one timeout is reported once
  const int others[4] = {bwd_take_device_error(), gram_take_device_error(),
                         gemm_take_device_error(), chol_take_device_error()};
  for (int o : others) {
    if (o < 0) return check_launch("ntg_device_status");
    if (v == 0) v = o;
  }
  if (v != 0) return fail(v, "a bounded device wait ran out in a streamed kernel");
  return NTG_OK;
}
