// Adjoints (vector-Jacobian products) of the layer rules, for reverse-mode
// differentiation of kernel_fn with respect to its inputs and to W_std / b_std.
// The derivative conventions follow the reference's custom JVPs:
// _sqrt (elementwise.py:1278-1290) has derivative 0 where its argument is
// <= 1e-30, and _arctan2 (:1293-1310) divides by max(x^2 + y^2, 1e-30).
#include <cstdio>

#include "ntg_common.cuh"
#include "ntg_vjp.cuh"

namespace ntg {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ void pair_of(int64_t b, int64_t n2, int64_t& i1, int64_t& i2) {
  if (n2 > 0) {
    i1 = b / n2;
    i2 = b - i1 * n2;
  } else {
    i1 = b;
    i2 = b;
  }
}

struct VarGrad {
  float* base;
  int64_t s_n, s_a, s_c;
};

__device__ __forceinline__ void vg_add(const VarGrad& g, int64_t n, int64_t a, int64_t c, float v) {
  if (g.base && v != 0.f) atomicAdd(g.base + n * g.s_n + a * g.s_a + c * g.s_c, v);
}

// VJP of the activation rule at one entry: given the pre-activation (q, t) and
// variances (v1, v2) and the output cotangents (gq, gt), returns the
// cotangents of q, t, v1, v2.
__device__ __forceinline__ void act_vjp(const ntg_act_t& act, float q, float t, float v1,
                                        float v2, float gq, float gt, float& oq, float& ot,
                                        float& ov1, float& ov2) {
  const float tol = 1e-30f;
  if (act.kind == NTG_ACT_ABRELU) {
    const float a = act.a, b = act.b;
    const float factor = (a - b) * (a - b) / (2.f * kPi);
    const float half = 0.5f * (a * a + b * b);
    // rounded like the forward rule, so that a self pair (q == v1 == v2) has d == 0 exactly
    const float d = prod_minus_sq(v1, v2, q, act.compensated);
    const float s = sqrtf(fmaxf(d, 0.f));
    const float th = (s == 0.f && q == 0.f) ? 0.5f * kPi : atan2f(s, q);
    const float dot = half - factor * th;
    // q' = factor s + dot q ; t' = t dot ; dot = half - factor th
    const float g_dot = q * gq + t * gt;
    float g_s = factor * gq;
    float g_q = dot * gq;
    ot = dot * gt;
    const float g_th = -factor * g_dot;
    const float den = fmaxf(s * s + q * q, tol);
    g_s += g_th * (q / den);
    g_q -= g_th * (s / den);
    const float g_d = (d > tol) ? g_s / (2.f * sqrtf(fmaxf(d, tol))) : 0.f;
    g_q -= 2.f * q * g_d;
    ov1 = g_d * v2;
    ov2 = g_d * v1;
    oq = g_q;
  } else if (act.kind == NTG_ACT_ERF) {
    const float a2 = act.a * act.a, b2 = act.b * act.b;
    const float qb = b2 * q, tb = b2 * t;
    const float d1 = 1.f + 2.f * b2 * v1, d2 = 1.f + 2.f * b2 * v2;
    const float y = 2.f * qb;
    const float dd = prod_minus_sq(d1, d2, y, act.compensated);
    const float s = sqrtf(fmaxf(dd, 0.f));
    const float gq2 = a2 * gq, gt2 = a2 * gt;
    const float dot = (4.f / kPi) / s;
    const float g_tb = dot * gt2;
    const float g_dot = tb * gt2;
    float g_s = -(4.f / kPi) / (s * s) * g_dot;
    const float g_phi = (2.f / kPi) * gq2;
    const float den = s * s + y * y;  // jnp.arctan2 derivative
    const float g_y = den > 0.f ? g_phi * s / den : 0.f;
    g_s += den > 0.f ? -g_phi * y / den : 0.f;
    float g_qb = 2.f * g_y;
    const float g_dd = (dd > tol) ? g_s / (2.f * sqrtf(fmaxf(dd, tol))) : 0.f;
    g_qb -= 2.f * y * g_dd * 2.f;  // d(y^2)/dqb = 2 y * 2
    const float g_d1 = g_dd * d2, g_d2 = g_dd * d1;
    oq = b2 * g_qb;
    ot = b2 * g_tb;
    ov1 = b2 * 2.f * g_d1;
    ov2 = b2 * 2.f * g_d2;
  } else if (act_is_rare(act.kind)) {
    act_vjp_rare(act_consts(act), q, t, v1, v2, gq, gt, oq, ot, ov1, ov2);
  } else {
    oq = gq;
    ot = gt;
    ov1 = ov2 = 0.f;
  }
}

// Activation VJP over [B, M] kernels; variance cotangents are accumulated
// atomically into gvar1 / gvar2 (same addressing as var1 / var2).
__global__ void act_bwd_kernel(const float* __restrict__ q, const float* __restrict__ t,
                               const float* __restrict__ gq, const float* __restrict__ gt,
                               float* __restrict__ oq, float* __restrict__ ot, int64_t batch,
                               int64_t n2, int64_t A, int64_t C, int diag, ntg_act_t act,
                               ntg_var_t var1, ntg_var_t var2, VarGrad gv1, VarGrad gv2) {
  const int64_t M = diag ? A * C : A * A * C * C;
  const int64_t total = batch * M;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = idx / M, m = idx - b * M;
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
    const float v1 = var_at(var1, i1, a1, c1), v2 = var_at(var2, i2, a2, c2);
    float rq, rt, rv1, rv2;
    act_vjp(act, q[idx], t ? t[idx] : 0.f, v1, v2, gq ? gq[idx] : 0.f, gt ? gt[idx] : 0.f, rq,
            rt, rv1, rv2);
    oq[idx] = rq;
    if (ot) ot[idx] = rt;
    vg_add(gv1, i1, a1, c1, rv1);
    vg_add(gv2, i2, a2, c2, rv2);
  }
}

// Activation VJP on flat pair kernels [N1, N2] (no spatial axes: the Dense layers of a
// fully-connected network): a CTA takes 32 rows x 256 columns, a thread one column. The
// column's variance cotangent is summed over the 32 rows in a register and the rows' by
// shuffles and shared memory, so each key receives one global atomic per tile instead of
// one per entry (4096 per key on a 4096 x 4096 kernel).
constexpr int kFlatRows = 32;
__global__ void __launch_bounds__(256)
    act_bwd_flat_kernel(const float* __restrict__ q, const float* __restrict__ t,
                        const float* __restrict__ gq, const float* __restrict__ gt,
                        float* __restrict__ oq, float* __restrict__ ot, int64_t n1, int64_t n2,
                        ntg_act_t act, ntg_var_t var1, ntg_var_t var2, VarGrad gv1,
                        VarGrad gv2) {
  __shared__ float rowpart[kFlatRows][8];
  const int64_t j = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.y * kFlatRows;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool col_ok = j < n2;
  const float v2 = col_ok ? var_at(var2, j, 0, 0) : 0.f;
  float g2 = 0.f;
  for (int r = 0; r < kFlatRows; ++r) {
    const int64_t i1 = i0 + r;
    float rv1 = 0.f;
    if (col_ok && i1 < n1) {
      const int64_t idx = i1 * n2 + j;
      float rq, rt, rv2;
      act_vjp(act, q[idx], t ? t[idx] : 0.f, var_at(var1, i1, 0, 0), v2, gq ? gq[idx] : 0.f,
              gt ? gt[idx] : 0.f, rq, rt, rv1, rv2);
      oq[idx] = rq;
      if (ot) ot[idx] = rt;
      g2 += rv2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rv1 += __shfl_xor_sync(0xffffffffu, rv1, o);
    if (lane == 0) rowpart[r][warp] = rv1;
  }
  vg_add(gv2, col_ok ? j : 0, 0, 0, col_ok ? g2 : 0.f);
  __syncthreads();
  if (threadIdx.x < kFlatRows && i0 + threadIdx.x < n1) {
    float sum = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) sum += rowpart[threadIdx.x][w];
    vg_add(gv1, i0 + threadIdx.x, 0, 0, sum);
  }
}

// Activation VJP on full-spatial [B, A, A, C, C] kernels with C a power of two
// in [4, 32] and A^2 C^2 a multiple of 1024: a CTA takes chunks of 1024
// consecutive entries (one pair; 4 entries per thread, vector loads). The
// variances a chunk reads are staged in shared memory one chunk ahead; its
// variance cotangents are summed by warp shuffles and shared-memory atomics per
// (plane, row) for var1 and per (plane, column) for var2 and leave with one
// global atomic per key instead of one per entry. Double-buffered shared arrays
// leave one barrier per chunk. RELU: the ABRelu rule only (the Erf VJP compiled
// out); POOLED: the cotangent is that of the AvgPool(2, 2) output (pooled != 0);
// RARE: the Sin / Rbf / Gelu VJPs compiled in.
template <bool RELU, bool POOLED, bool RARE = false>
__global__ void __launch_bounds__(kT)
    act_bwd_fs_kernel(const float* __restrict__ q, const float* __restrict__ t,
                      const float* __restrict__ gq, const float* __restrict__ gt,
                      float* __restrict__ oq, float* __restrict__ ot, int64_t batch, int64_t n2,
                      int A, int C, ntg_act_t act, ntg_var_t var1, ntg_var_t var2, VarGrad gv1,
                      VarGrad gv2, int pooled, float pool_w) {
  __shared__ __align__(16) float sv[2][2][256];  // [buffer][v1 | v2][key]
  __shared__ float sg[2][2][256];                // [buffer][g v1 | g v2][key]
  const int64_t M = (int64_t)A * A * C * C;  // < 2^31 (checked by the host)
  const int P = (int)(M / 1024);              // chunks per pair
  const int64_t chunks = batch * P;
  const ActC ac = act_consts(act);
  const int tid = threadIdx.x, lane = tid & 31;
  const int lc = __ffs(C) - 1;                       // log2 C
  const int nkeys = 1024 >> lc;
  const int seg = C / 4;                             // lanes per row
  const int pseg = C * C / 4 < 32 ? C * C / 4 : 32;  // lanes per plane within a warp
  // chunk ch = b * P + j: pair b, entries [1024 j, 1024 j + 1024) of that pair
  auto stage = [&](int64_t b, int j, int buf) {
    int64_t i1, i2;
    pair_of(b, n2, i1, i2);
    const int r0 = (j * 1024) >> lc, p0 = (j * 1024) >> (2 * lc);
    for (int k = tid; k < nkeys; k += kT) {
      const int rr = r0 + k, pp = p0 + (k >> lc);
      sv[buf][0][k] = var_at(var1, i1, (rr >> lc) / A, rr & (C - 1));
      sv[buf][1][k] = var_at(var2, i2, pp % A, k & (C - 1));
    }
  };
  for (int k = tid; k < 2 * 2 * 256; k += kT) (&sg[0][0][0])[k] = 0.f;
  int64_t b = blockIdx.x / P;
  int j = (int)(blockIdx.x - b * P);
  if (blockIdx.x < chunks) stage(b, j, 0);
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
    if (ch + gridDim.x < chunks) stage(bn, jn, cur ^ 1);
    const int64_t e = b * M + (int64_t)j * 1024 + 4 * tid;
    const float4 Q = *reinterpret_cast<const float4*>(q + e);
    const float4 T = t ? *reinterpret_cast<const float4*>(t + e) : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 GQ, GT;
    if (!POOLED) {
      GQ = gq ? *reinterpret_cast<const float4*>(gq + e) : make_float4(0.f, 0.f, 0.f, 0.f);
      GT = gt ? *reinterpret_cast<const float4*>(gt + e) : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      // cotangent of the AvgPool(2, 2) output, taken at the window of each entry
      const int m = j * 1024 + 4 * tid;
      const int row = m >> lc, pl = row >> lc;
      const int wq = m & (C - 1), w = row & (C - 1), hq = pl % A, h = pl / A;
      const int Ao = A >> 1, Co = C >> 1;
      const int64_t o = b * ((int64_t)Ao * Ao * Co * Co) +
                        ((int64_t)((h >> 1) * Ao + (hq >> 1)) * Co + (w >> 1)) * Co + (wq >> 1);
      const float a0 = gq ? __ldg(gq + o) * pool_w : 0.f, a1 = gq ? __ldg(gq + o + 1) * pool_w : 0.f;
      const float c0 = gt ? __ldg(gt + o) * pool_w : 0.f, c1 = gt ? __ldg(gt + o + 1) * pool_w : 0.f;
      GQ = make_float4(a0, a0, a1, a1);
      GT = make_float4(c0, c0, c1, c1);
    }
    const float qa[4] = {Q.x, Q.y, Q.z, Q.w}, ta[4] = {T.x, T.y, T.z, T.w};
    const float ga[4] = {GQ.x, GQ.y, GQ.z, GQ.w}, gb[4] = {GT.x, GT.y, GT.z, GT.w};
    const float v1 = sv[cur][0][k1];
    const float4 V2 = *reinterpret_cast<const float4*>(&sv[cur][1][k2]);
    const float v2[4] = {V2.x, V2.y, V2.z, V2.w};
    float rq[4], rt[4], r2[4], r1 = 0.f;
    if (RELU || act.kind == NTG_ACT_ABRELU) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        P2 oq2, ot2, o12, o22;
        abrelu_vjp2(ac, p2(qa[2 * h], qa[2 * h + 1]), p2(ta[2 * h], ta[2 * h + 1]), p2s(v1),
                    p2(v2[2 * h], v2[2 * h + 1]), p2(ga[2 * h], ga[2 * h + 1]),
                    p2(gb[2 * h], gb[2 * h + 1]), oq2, ot2, o12, o22);
        float a0, a1;
        p2u(oq2, rq[2 * h], rq[2 * h + 1]);
        p2u(ot2, rt[2 * h], rt[2 * h + 1]);
        p2u(o12, a0, a1);
        p2u(o22, r2[2 * h], r2[2 * h + 1]);
        r1 += a0 + a1;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float o1;
        act_vjp_fast<RARE>(act, ac, qa[k], ta[k], v1, v2[k], ga[k], gb[k], rq[k], rt[k], o1,
                           r2[k]);
        r1 += o1;
      }
    }
    *reinterpret_cast<float4*>(oq + e) = make_float4(rq[0], rq[1], rq[2], rq[3]);
    if (ot) *reinterpret_cast<float4*>(ot + e) = make_float4(rt[0], rt[1], rt[2], rt[3]);
    for (int o = 1; o < seg; o <<= 1) r1 += __shfl_xor_sync(0xffffffffu, r1, o);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      for (int o = seg; o < pseg; o <<= 1) r2[k] += __shfl_xor_sync(0xffffffffu, r2[k], o);
    if ((lane & (seg - 1)) == 0) atomicAdd(&sg[cur][0][k1], r1);
    if ((lane & (pseg - 1)) < seg) {
#pragma unroll
      for (int k = 0; k < 4; ++k) atomicAdd(&sg[cur][1][k2 + k], r2[k]);
    }
    __syncthreads();
    // flush this chunk's sums; the buffer is accumulated again two chunks later
    int64_t i1, i2;
    pair_of(b, n2, i1, i2);
    const int r0 = (j * 1024) >> lc, p0 = (j * 1024) >> (2 * lc);
    for (int k = tid; k < nkeys; k += kT) {
      const float a1 = sg[cur][0][k], a2 = sg[cur][1][k];
      sg[cur][0][k] = 0.f;
      sg[cur][1][k] = 0.f;
      const int rr = r0 + k, pp = p0 + (k >> lc);
      if (gv1.base && a1 != 0.f)
        atomicAdd(gv1.base + i1 * gv1.s_n + (int64_t)((rr >> lc) / A) * gv1.s_a +
                      (int64_t)(rr & (C - 1)) * gv1.s_c, a1);
      if (gv2.base && a2 != 0.f)
        atomicAdd(gv2.base + i2 * gv2.s_n + (int64_t)(pp % A) * gv2.s_a +
                      (int64_t)(k & (C - 1)) * gv2.s_c, a2);
    }
    b = bn;
    j = jn;
  }
}

// Transpose of a pooling rule with full, non-overlapping windows (stride ==
// window, no padding, A and C multiples of the window): every input entry
// takes its window's cotangent times the forward's weight (1 / window size for
// the average, 1 for the sum). Four entries per thread, vector stores.
__global__ void __launch_bounds__(kT)
    pool_t_block_kernel(const float* __restrict__ gout, float* __restrict__ gin, int64_t batch,
                        int A, int C, int wa, int wc, float weight) {
  const int Ao = A / wa, Co = C / wc;
  const int per_b = A * A * C * C;  // < 2^31 (checked by the host)
  const int n4 = per_b / 4;
  for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
    const float* gb = gout + b * (int64_t)Ao * Ao * Co * Co;
    float* ib = gin + b * (int64_t)per_b;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n4; v += gridDim.x * blockDim.x) {
      const int idx = 4 * v;
      int r = idx;
      const int cp = r % C;
      r /= C;
      const int c = r % C;
      r /= C;
      const int ap = r % A;
      const int a = r / A;
      const float* g = gb + (((a / wa) * Ao + ap / wa) * Co + c / wc) * Co;
      float o[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) o[k] = __ldg(g + (cp + k) / wc) * weight;
      *reinterpret_cast<float4*>(ib + idx) = make_float4(o[0], o[1], o[2], o[3]);
    }
  }
}

// Cotangent of the unscaled stencil sums of a conv/dense affine rule:
//   q = w2 s U + b2,  t = tw2 s Ut + nn_w (nn_scaled ? q : s U) + c
// gives  gU = s (w2 (gq + [nn_scaled] nn_w gt) + [!nn_scaled] nn_w gt),  gUt = tw2 s gt.
__global__ void affine_bwd_kernel(const float* __restrict__ gq, const float* __restrict__ gt,
                                  float* __restrict__ gu, float* __restrict__ gut, int64_t n,
                                  ntg_affine_t f, float scale) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float a = gq ? gq[i] : 0.f, b = gt ? gt[i] : 0.f;
    const float gqq = a + (f.nn_scaled ? f.ntk_nn * b : 0.f);
    gu[i] = scale * (f.w2 * gqq + (f.nn_scaled ? 0.f : f.ntk_nn * b));
    if (gut) gut[i] = scale * f.ntk_w2 * b;
  }
}

// Sums for the W^2 / b^2 cotangents of an NTK-parameterised affine rule from
// its outputs: q = W^2 X + b^2, t = W^2 Y + q  =>  dq/dW^2 = X = (q - b^2) / W^2,
// dt/dW^2 = Y + X = (t - b^2) / W^2, dq/db^2 = dt/db^2 = 1.
// out[0] += sum(gq X + gt (t - b^2)/W^2), out[1] += sum(gq + gt).
__global__ void affine_hyper_kernel(const float* __restrict__ q, const float* __restrict__ t,
                                    const float* __restrict__ gq, const float* __restrict__ gt,
                                    int64_t n, float w2, float b2, double* __restrict__ out) {
  // FP32 partial sums per thread (a few hundred terms each), FP64 across threads
  float fw = 0.f, fb = 0.f;
  const float inv = w2 != 0.f ? 1.f / w2 : 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float g1 = gq ? gq[i] : 0.f;
    const float g2 = (gt && t) ? gt[i] : 0.f;
    fw = fmaf(g1, (q[i] - b2) * inv, fw);
    if (g2 != 0.f) fw = fmaf(g2, (t[i] - b2) * inv, fw);
    fb += g1 + g2;
  }
  double sw = fw, sb = fb;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sw += __shfl_xor_sync(0xffffffffu, sw, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, sw);
    atomicAdd(out + 1, sb);
  }
}

// Outputs i in [0, no) whose window offset `off` lands on input x:
// i*s + off - p == x (zero padding) or == x mod n (circular). At most 3.
__device__ __forceinline__ int candidates(int64_t x, int off, int s, int p, int64_t n, int64_t no,
                                          int circular, int64_t out[3]) {
  int cnt = 0;
  const int k0 = circular ? -1 : 0, k1 = circular ? 1 : 0;
  for (int k = k0; k <= k1; ++k) {
    const int64_t pp = x + p + k * n - off;  // = i * s
    if (pp < 0 || pp % s) continue;
    const int64_t i = pp / s;
    if (i < no) out[cnt++] = i;
  }
  return cnt;
}

// Transpose of the full-spatial stencil sum U[o] = sum_{d,e} in[o*s + d - p]:
// gin[a, a', c, c'] = sum of gU over every output whose window holds (a, a', c, c')
// (the same offset d on both A axes and e on both C axes).
__global__ void stencil_t_kernel(const float* __restrict__ gu, float* __restrict__ gin,
                                 int64_t batch, int64_t A, int64_t C, int64_t Ao, int64_t Co,
                                 int fh, int fw, int sh, int sw, int ph, int pw, int circular) {
  const int64_t per_b = A * A * C * C;
  const int64_t total = batch * per_b;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / per_b, r = idx - b * per_b;
    const int64_t cp = r % C; r /= C;
    const int64_t c = r % C; r /= C;
    const int64_t ap = r % A;
    const int64_t a = r / A;
    const float* g = gu + b * Ao * Ao * Co * Co;
    float s = 0.f;
    int64_t ia[3], iap[3], jc[3], jcp[3];
    for (int d = 0; d < fh; ++d) {
      const int na = candidates(a, d, sh, ph, A, Ao, circular, ia);
      const int nap = candidates(ap, d, sh, ph, A, Ao, circular, iap);
      for (int x = 0; x < na; ++x)
        for (int y = 0; y < nap; ++y)
          for (int e = 0; e < fw; ++e) {
            const int nc = candidates(c, e, sw, pw, C, Co, circular, jc);
            const int ncp = candidates(cp, e, sw, pw, C, Co, circular, jcp);
            for (int u = 0; u < nc; ++u)
              for (int v = 0; v < ncp; ++v)
                s += g[((ia[x] * Ao + iap[y]) * Co + jc[u]) * Co + jcp[v]];
          }
    }
    gin[idx] = s;
  }
}

// Same for a 3x3 / stride 1 / SAME / zero-padded stencil: its transpose is the
// same 3x3 diagonal box sum.
__global__ void stencil3_t_kernel(const float* __restrict__ gu, float* __restrict__ gin,
                                  int64_t batch, int64_t A, int64_t C) {
  const int64_t per_b = A * A * C * C;
  const int64_t total = batch * per_b;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / per_b, r = idx - b * per_b;
    const int64_t cp = r % C; r /= C;
    const int64_t c = r % C; r /= C;
    const int64_t ap = r % A;
    const int64_t a = r / A;
    const float* g = gu + b * per_b;
    float s = 0.f;
    for (int d = -1; d <= 1; ++d) {
      const int64_t ia = a + d, iap = ap + d;
      if (ia < 0 || ia >= A || iap < 0 || iap >= A) continue;
      for (int e = -1; e <= 1; ++e) {
        const int64_t jc = c + e, jcp = cp + e;
        if (jc < 0 || jc >= C || jcp < 0 || jcp >= C) continue;
        s += g[((ia * A + iap) * C + jc) * C + jcp];
      }
    }
    gin[idx] = s;
  }
}

// Diagonal-spatial stencil transpose on [B, A, C].
__global__ void stencil_ds_t_kernel(const float* __restrict__ gu, float* __restrict__ gin,
                                    int64_t batch, int64_t A, int64_t C, int64_t Ao, int64_t Co,
                                    int fh, int fw, int sh, int sw, int ph, int pw,
                                    int circular) {
  const int64_t total = batch * A * C;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = idx / (A * C), r = idx - b * A * C;
    const int64_t a = r / C, c = r - a * C;
    float s = 0.f;
    int64_t ia[3], jc[3];
    for (int d = 0; d < fh; ++d) {
      const int na = candidates(a, d, sh, ph, A, Ao, circular, ia);
      for (int x = 0; x < na; ++x)
        for (int e = 0; e < fw; ++e) {
          const int nc = candidates(c, e, sw, pw, C, Co, circular, jc);
          for (int u = 0; u < nc; ++u) s += gu[(b * Ao + ia[x]) * Co + jc[u]];
        }
    }
    gin[idx] = s;
  }
}

__device__ __forceinline__ int inbounds(int64_t o, int w, int s, int p, int64_t n) {
  int cnt = 0;
  for (int u = 0; u < w; ++u) {
    const int64_t x = o * s + u - p;
    if (x >= 0 && x < n) ++cnt;
  }
  return cnt;
}

// Transpose of the pooling rule: every input entry collects the cotangents of
// the outputs whose window holds it, scaled as in the forward (window offsets
// are independent on each of the four axes).
__global__ void pool_t_kernel(const float* __restrict__ gout, float* __restrict__ gin,
                              int64_t batch, int64_t A, int64_t C, int64_t Ao, int64_t Co, int wa,
                              int wc, int sa, int sc, int pa, int pc, int circular, int diag,
                              int average, int normalize_edges) {
  const int64_t per_b = diag ? A * C : A * A * C * C;
  const int64_t total = batch * per_b;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t b = idx / per_b, r = idx - b * per_b;
    int64_t a, ap, c, cp;
    if (diag) {
      a = ap = r / C;
      c = cp = r - a * C;
    } else {
      cp = r % C; r /= C;
      c = r % C; r /= C;
      ap = r % A;
      a = r / A;
    }
    // candidate output indices per axis (over all window offsets)
    int64_t ca[8], cap[8], cc[8], ccp[8];
    int na = 0, nap = 0, nc = 0, ncp = 0;
    int64_t tmp[3];
    for (int u = 0; u < wa && na < 6; ++u) {
      int k = candidates(a, u, sa, pa, A, Ao, circular, tmp);
      for (int x = 0; x < k && na < 8; ++x) ca[na++] = tmp[x];
    }
    for (int v = 0; v < wc && nc < 6; ++v) {
      int k = candidates(c, v, sc, pc, C, Co, circular, tmp);
      for (int x = 0; x < k && nc < 8; ++x) cc[nc++] = tmp[x];
    }
    if (!diag) {
      for (int u = 0; u < wa && nap < 6; ++u) {
        int k = candidates(ap, u, sa, pa, A, Ao, circular, tmp);
        for (int x = 0; x < k && nap < 8; ++x) cap[nap++] = tmp[x];
      }
      for (int v = 0; v < wc && ncp < 6; ++v) {
        int k = candidates(cp, v, sc, pc, C, Co, circular, tmp);
        for (int x = 0; x < k && ncp < 8; ++x) ccp[ncp++] = tmp[x];
      }
    } else {
      nap = ncp = 1;
      cap[0] = ccp[0] = 0;
    }
    float s = 0.f;
    const int64_t ob = diag ? b * Ao * Co : b * Ao * Ao * Co * Co;
    const float full = diag ? (float)(wa * wc) : (float)(wa * wa * wc * wc);
    for (int x = 0; x < na; ++x)
      for (int y = 0; y < nap; ++y)
        for (int u = 0; u < nc; ++u)
          for (int v = 0; v < ncp; ++v) {
            const int64_t i = ca[x], ip = cap[y], j = cc[u], jp = ccp[v];
            float g = diag ? gout[ob + i * Co + j] : gout[ob + ((i * Ao + ip) * Co + j) * Co + jp];
            if (average) {
              float norm = full;
              if (normalize_edges) {
                int cnt = inbounds(i, wa, sa, pa, A) * inbounds(j, wc, sc, pc, C);
                if (!diag) cnt *= inbounds(ip, wa, sa, pa, A) * inbounds(jp, wc, sc, pc, C);
                norm = (float)cnt;
              }
              g = g / norm;
              if (diag) g = g / norm;
            }
            s += g;
          }
    gin[idx] = s;
  }
}

// Broadcast of a readout cotangent: gin[b, m] = gout[b] * scale (mean or sum),
// or, for Flatten on a full-spatial kernel, only on the spatial diagonal.
__global__ void readout_t_kernel(const float* __restrict__ gout, float* __restrict__ gin,
                                 int64_t batch, int64_t A, int64_t C, int flatten_fs,
                                 int64_t m, float scale) {
  const int64_t total = batch * m;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = idx / m, r = idx - b * m;
    float v = gout[b] * scale;
    if (flatten_fs) {
      const int64_t cp = r % C, c = (r / C) % C, ap = (r / (C * C)) % A, a = r / (A * C * C);
      if (a != ap || c != cp) v = 0.f;
    }
    gin[idx] = v;
  }
}

// Cotangent of the image inputs through the full-spatial input covariance
// G[b, h, h', w, w'] = sum_k x1[i1, h, w, k] x2[i2, h', w', k] / K:
//   side 0: gx1[i1, h, w, k] += sum_{pairs with i1, h', w'} G'[..] x2[i2, h', w', k] / K
//   side 1: gx2[i2, h', w', k] += sum_{pairs with i2, h, w} G'[..] x1[i1, h, w, k] / K
// One CTA per (sample, row); n2 == 0 means per-sample pairs (i, i).
__global__ void input_fs_t_kernel(const float* __restrict__ g, const float* __restrict__ xo,
                                  float* __restrict__ gx, int64_t nself, int64_t nother,
                                  int64_t n2, int64_t A, int64_t C, int64_t K, int side,
                                  float inv_k) {
  const int64_t i = blockIdx.x / A, h = blockIdx.x % A;
  if (i >= nself) return;
  extern __shared__ float acc[];  // [C][K]
  for (int64_t e = threadIdx.x; e < C * K; e += blockDim.x) acc[e] = 0.f;
  __syncthreads();
  const int64_t plane = C * C;
  const int64_t partners = n2 > 0 ? nother : 1;
  for (int64_t pj = 0; pj < partners; ++pj) {
    const int64_t j = n2 > 0 ? pj : i;
    const int64_t b = n2 > 0 ? (side == 0 ? i * n2 + j : j * n2 + i) : i;
    for (int64_t hp = 0; hp < A; ++hp) {
      const float* pl = side == 0 ? g + ((b * A + h) * A + hp) * plane
                                  : g + ((b * A + hp) * A + h) * plane;
      const float* xr = xo + ((j * A + hp) * C) * K;
      for (int64_t e = threadIdx.x; e < C * K; e += blockDim.x) {
        const int64_t w = e / K, k = e - w * K;
        float s = 0.f;
        for (int64_t wp = 0; wp < C; ++wp) {
          const float gv = side == 0 ? pl[w * C + wp] : pl[wp * C + w];
          s = fmaf(gv, __ldg(xr + wp * K + k), s);
        }
        acc[e] += s;
      }
    }
  }
  __syncthreads();
  for (int64_t e = threadIdx.x; e < C * K; e += blockDim.x) {
    const int64_t w = e / K, k = e - w * K;
    atomicAdd(gx + ((i * A + h) * C + w) * K + k, acc[e] * inv_k);
  }
}

// Image cotangents of the full-spatial input covariance, 32 x 32 planes and
// K <= 4 channels (requirements.py:542-553, differentiated):
//   gx1[i1, h, w, k]   += sum_{i2, h', w'} G[i1, i2, h, h', w, w'] x2[i2, h', w', k] / K
//   gx2[i2, h', w', k] += sum_{i1, h, w}   G[i1, i2, h, h', w, w'] x1[i1, h, w, k] / K
constexpr int kIfC = 32;

__device__ int g_bwd_error = 0;

constexpr int kIfRing = 4;

// Two-pass form of the input-covariance adjoint, each pass a pure stream over G
// with per-thread accumulators and one owner per output row (no atomics):
//   rows (COLS = false): CTA (i1, h) streams the planes (i2, h') of its rows,
//     gx1[i1, h, w, k] += sum_{i2, h', w'} G[i1, i2, h, h', w, w'] x2[i2, h', w', k] / K;
//   cols (COLS = true): CTA (i2, h') streams the planes (i1, h) of its columns,
//     gx2[i2, h', w', k] += sum_{i1, h, w} G[i1, i2, h, h', w, w'] x1[i1, h, w, k] / K.
// With n2 == 0 (the per-sample covariances of x1) both passes run over G[i, h, h']
// and add into gx1. G planes and the matching image rows come through a bulk-copy
// ring (one thread issues, completion on an mbarrier, every wait bounded).
template <int K, bool COLS>
__global__ void __launch_bounds__(256)
    input_fs_pass_kernel(const float* __restrict__ g, const float* __restrict__ x1,
                         const float* __restrict__ x2, float* __restrict__ gx, int64_t n1,
                         int64_t n2, int A, float inv_k) {
  constexpr int C = kIfC;
  constexpr int XF = C * K;
  __shared__ __align__(128) float gs[kIfRing][C * C];
  __shared__ __align__(16) float xs[kIfRing][XF];
  __shared__ float red[8][C * K];
  __shared__ __align__(8) uint64_t bars[kIfRing];
  __shared__ int s_err;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool self = n2 == 0;
  const int64_t nown = COLS ? (self ? n1 : n2) : n1;  // images owning the output rows
  const int64_t own = blockIdx.x / A;                 // i1 (rows) or i2 (cols)
  const int hown = (int)(blockIdx.x % A);             // h (rows) or h' (cols)
  if (own >= nown) return;
  const int64_t nother = self ? 1 : (COLS ? n1 : n2);
  const int64_t np = nother * A;
  // rows read x2 rows (x1's own rows when self); cols read x1 rows
  const float* xo = COLS ? x1 : (self ? x1 : x2);
  const int w = tid >> 3, wq0 = (tid & 7) * 4;
  float acc[4][K];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int k = 0; k < K; ++k) acc[j][k] = 0.f;
  int64_t issued = 0;
  auto issue = [&]() {
    const int sl = (int)(issued % kIfRing);
    const int64_t o = self ? own : issued / A;  // the other image
    const int hq = (int)(issued % A);           // the other position row
    const uint32_t bar = smem_addr(&bars[sl]);
    int64_t plane;
    if (!COLS)
      plane = self ? (own * A + hown) * A + hq : ((own * n2 + o) * A + hown) * A + hq;
    else
      plane = self ? (own * A + hq) * A + hown : ((o * n2 + own) * A + hq) * A + hown;
    const float* gsrc = g + plane * (int64_t)(C * C);
    const float* xsrc = xo + ((o * A + hq) * C) * K;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"((uint32_t)((C * C + XF) * sizeof(float)))
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(&gs[sl][0])), "l"(gsrc), "r"((uint32_t)(C * C * sizeof(float))), "r"(bar)
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(&xs[sl][0])), "l"(xsrc), "r"((uint32_t)(XF * sizeof(float))), "r"(bar)
        : "memory");
    ++issued;
  };
  if (tid == 0) {
    s_err = 0;
    for (int sl = 0; sl < kIfRing; ++sl)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[sl])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0)
    while (issued < kIfRing && issued < np) issue();
  for (int64_t p = 0; p < np; ++p) {
    const int sl = (int)(p % kIfRing);
    if (!s_err && !bar_wait(smem_addr(&bars[sl]), (uint32_t)((p / kIfRing) & 1))) s_err = 1;
    const float4 G = *reinterpret_cast<const float4*>(&gs[sl][w * C + wq0]);
    const float ga[4] = {G.x, G.y, G.z, G.w};
    if (!COLS) {
      // acc[0][k]: sum over the row's columns w' of G[w, w'] x[w', k]
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[0][k] = fmaf(ga[j], xs[sl][(wq0 + j) * K + k], acc[0][k]);
    } else {
      // acc[j][k]: column w' = wq0 + j, summed over rows w of G[w, w'] x[w, k]
      float xv[K];
#pragma unroll
      for (int k = 0; k < K; ++k) xv[k] = xs[sl][w * K + k];
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < K; ++k) acc[j][k] = fmaf(ga[j], xv[k], acc[j][k]);
    }
    __syncthreads();
    // every thread has read slot sl: it takes plane p + kIfRing
    if (tid == 0 && !s_err && issued < np) issue();
  }
  float* out;
  if (!COLS) {
    // the 8 threads of a row w hold the row's partial sums over disjoint columns
#pragma unroll
    for (int k = 0; k < K; ++k) {
      acc[0][k] += __shfl_xor_sync(0xffffffffu, acc[0][k], 1);
      acc[0][k] += __shfl_xor_sync(0xffffffffu, acc[0][k], 2);
      acc[0][k] += __shfl_xor_sync(0xffffffffu, acc[0][k], 4);
    }
    out = gx + ((own * A + hown) * C + w) * K;
    if ((lane & 7) == 0) {
#pragma unroll
      for (int k = 0; k < K; ++k) out[k] += acc[0][k] * inv_k;
    }
  } else {
    // sums over the 4 rows of the warp (lanes 8 apart), then over the 8 warps
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int k = 0; k < K; ++k) {
        acc[j][k] += __shfl_xor_sync(0xffffffffu, acc[j][k], 8);
        acc[j][k] += __shfl_xor_sync(0xffffffffu, acc[j][k], 16);
      }
    if (lane < 8) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < K; ++k) red[warp][(wq0 + j) * K + k] = acc[j][k];
    }
    __syncthreads();
    out = gx + ((own * A + hown) * C) * K;
    if (tid < C * K) {
      float v = 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u) v += red[u][tid];
      out[tid] += v * inv_k;
    }
  }
  if (tid == 0 && s_err) {
    atomicExch(&g_bwd_error, NTG_ERR_WAIT_TIMEOUT);
    for (int64_t p = issued > kIfRing ? issued - kIfRing : 0; p < issued; ++p)
      bar_wait(smem_addr(&bars[p % kIfRing]), (uint32_t)((p / kIfRing) & 1));
  }
}

// C[m, n] (+)= alpha * op(A) B with op(A) = A [m, k] or A^T (A stored [k, m]).
__global__ void __launch_bounds__(256) gemm_ex_kernel(const float* __restrict__ A,
                                                      const float* __restrict__ B,
                                                      float* __restrict__ Cm, int64_t M, int64_t N,
                                                      int64_t K, int trans_a, float alpha,
                                                      int accumulate) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t row0 = (int64_t)blockIdx.y * 64, col0 = (int64_t)blockIdx.x * 64;
  float acc[4][4] = {};
  for (int64_t k0 = 0; k0 < K; k0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * 64; idx += 256) {
      if (trans_a) {
        const int kk = idx / 64, r = idx % 64;
        const int64_t gk = k0 + kk, gi = row0 + r;
        As[kk][r] = (gi < M && gk < K) ? __ldg(A + gk * M + gi) : 0.f;
      } else {
        const int r = idx / 16, kk = idx % 16;
        const int64_t gi = row0 + r, gk = k0 + kk;
        As[kk][r] = (gi < M && gk < K) ? __ldg(A + gi * K + gk) : 0.f;
      }
      const int kb = idx / 64, cb = idx % 64;
      const int64_t gkb = k0 + kb, gj = col0 + cb;
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
      const int64_t gi = row0 + ty * 4 + u, gj = col0 + tx * 4 + v;
      if (gi < M && gj < N) {
        const float r = alpha * acc[u][v];
        Cm[gi * N + gj] = accumulate ? Cm[gi * N + gj] + r : r;
      }
    }
}

// gx[i, :] += 2 gcov[i] x[i, :] / D (adjoint of cov_i = |x_i|^2 / D).
__global__ void cov_diag_t_kernel(const float* __restrict__ gcov, const float* __restrict__ x,
                                  float* __restrict__ gx, int64_t n, int64_t d, float two_over_d) {
  const int64_t total = n * d;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    gx[idx] += two_over_d * gcov[idx / d] * x[idx];
}

// dst[n, a, a, c, c] (strided diagonal view) += src[n, a, c].
__global__ void diag_add_kernel(const float* __restrict__ src, float* __restrict__ dst, int64_t n,
                                int64_t A, int64_t C, int64_t s_n, int64_t s_a, int64_t s_c) {
  const int64_t total = n * A * C;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / (A * C), r = idx - i * A * C, a = r / C, c = r - a * C;
    dst[i * s_n + a * s_a + c * s_c] += src[idx];
  }
}

int grid_for(int64_t n) {
  int64_t g = (n + kT - 1) / kT;
  if (g > 152 * 64) g = 152 * 64;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace ntg

using namespace ntg;

extern "C" int ntg_act_bwd(void* stream, const float* q, const float* t, const float* gq,
                           const float* gt, float* oq, float* ot, int64_t batch, int64_t n2,
                           int64_t a, int64_t c, int32_t diag_spatial, ntg_act_t act,
                           ntg_var_t var1, ntg_var_t var2, float* gvar1, float* gvar2) {
  NTG_REQUIRE(q && oq && var1.base && var2.base, "ntg_act_bwd: null pointer");
  NTG_REQUIRE(batch > 0 && a > 0 && c > 0, "ntg_act_bwd: bad sizes");
  NTG_REQUIRE(act.kind != NTG_ACT_ABRELU || act.stabilize <= 0.f,
              "ntg_act_bwd: do_stabilize is not differentiable here");
  if (act.kind < NTG_ACT_NONE || act.kind > NTG_ACT_GELU)
    return fail(NTG_ERR_UNSUPPORTED, "ntg_act_bwd: unknown activation kind");
  const bool rare = act.kind >= NTG_ACT_SIN;
  // variance cotangents are compact [n, A, C] arrays
  VarGrad g1{gvar1, a * c, c, 1}, g2{gvar2, a * c, c, 1};
  const int64_t m = diag_spatial ? a * c : a * a * c * c;
  const bool pow2 = c >= 4 && c <= 32 && (c & (c - 1)) == 0;
  const bool aligned = ((reinterpret_cast<uintptr_t>(q) | reinterpret_cast<uintptr_t>(t) |
                         reinterpret_cast<uintptr_t>(gq) | reinterpret_cast<uintptr_t>(gt) |
                         reinterpret_cast<uintptr_t>(oq) | reinterpret_cast<uintptr_t>(ot)) &
                        15) == 0;
  if (!diag_spatial && pow2 && m % 1024 == 0 && aligned && m < (1ll << 31)) {
    const int64_t chunks = batch * (m / 1024);
    const int grid = (int)(chunks < 152 * 8 ? chunks : 152 * 8);
    if (act.kind == NTG_ACT_ABRELU)
      act_bwd_fs_kernel<true, false><<<grid, kT, 0, as_stream(stream)>>>(
          q, t, gq, gt, oq, ot, batch, n2, (int)a, (int)c, act, var1, var2, g1, g2, 0, 0.f);
    else if (rare)
      act_bwd_fs_kernel<false, false, true><<<grid, kT, 0, as_stream(stream)>>>(
          q, t, gq, gt, oq, ot, batch, n2, (int)a, (int)c, act, var1, var2, g1, g2, 0, 0.f);
    else
      act_bwd_fs_kernel<false, false><<<grid, kT, 0, as_stream(stream)>>>(
          q, t, gq, gt, oq, ot, batch, n2, (int)a, (int)c, act, var1, var2, g1, g2, 0, 0.f);
  } else if (a == 1 && c == 1 && n2 > 0 && batch % n2 == 0 && batch / n2 < 65535ll * kFlatRows) {
    const int64_t n1 = batch / n2;
    const dim3 grid((unsigned)ceil_div(n2, 256), (unsigned)ceil_div(n1, kFlatRows));
    act_bwd_flat_kernel<<<grid, 256, 0, as_stream(stream)>>>(q, t, gq, gt, oq, ot, n1, n2, act,
                                                             var1, var2, g1, g2);
  } else {
    act_bwd_kernel<<<grid_for(batch * m), kT, 0, as_stream(stream)>>>(
        q, t, gq, gt, oq, ot, batch, n2, a, c, diag_spatial, act, var1, var2, g1, g2);
  }
  note_launch();
  return check_launch("ntg_act_bwd");
}

extern "C" int ntg_act_pool_bwd(void* stream, const float* q, const float* t,
                                const float* gq_pooled, const float* gt_pooled, float* oq,
                                float* ot, int64_t batch, int64_t n2, int64_t a, int64_t c,
                                ntg_act_t act, ntg_var_t var1, ntg_var_t var2, float* gvar1,
                                float* gvar2) {
  NTG_REQUIRE(q && oq && var1.base && var2.base, "ntg_act_pool_bwd: null pointer");
  NTG_REQUIRE(batch > 0 && a > 0 && c > 0, "ntg_act_pool_bwd: bad sizes");
  NTG_REQUIRE(act.kind != NTG_ACT_ABRELU || act.stabilize <= 0.f,
              "ntg_act_pool_bwd: do_stabilize is not differentiable here");
  if (act.kind < NTG_ACT_NONE || act.kind > NTG_ACT_GELU)
    return fail(NTG_ERR_UNSUPPORTED, "ntg_act_pool_bwd: unknown activation kind");
  const int64_t m = a * a * c * c;
  const bool pow2 = c >= 4 && c <= 32 && (c & (c - 1)) == 0;
  const bool aligned = ((reinterpret_cast<uintptr_t>(q) | reinterpret_cast<uintptr_t>(t) |
                         reinterpret_cast<uintptr_t>(oq) | reinterpret_cast<uintptr_t>(ot)) &
                        15) == 0;
  NTG_REQUIRE(pow2 && a % 2 == 0 && m % 1024 == 0 && aligned && m < (1ll << 31),
              "ntg_act_pool_bwd: needs C a power of two in [4, 32], even A, 16-byte aligned "
              "buffers and A^2 C^2 a multiple of 1024");
  VarGrad g1{gvar1, a * c, c, 1}, g2{gvar2, a * c, c, 1};
  const int64_t chunks = batch * (m / 1024);
  const int grid = (int)(chunks < 152 * 8 ? chunks : 152 * 8);
  if (act.kind == NTG_ACT_ABRELU)
    act_bwd_fs_kernel<true, true><<<grid, kT, 0, as_stream(stream)>>>(
        q, t, gq_pooled, gt_pooled, oq, ot, batch, n2, (int)a, (int)c, act, var1, var2, g1, g2, 1,
        1.f / 16.f);
  else if (act.kind >= NTG_ACT_SIN)
    act_bwd_fs_kernel<false, true, true><<<grid, kT, 0, as_stream(stream)>>>(
        q, t, gq_pooled, gt_pooled, oq, ot, batch, n2, (int)a, (int)c, act, var1, var2, g1, g2, 1,
        1.f / 16.f);
  else
    act_bwd_fs_kernel<false, true><<<grid, kT, 0, as_stream(stream)>>>(
        q, t, gq_pooled, gt_pooled, oq, ot, batch, n2, (int)a, (int)c, act, var1, var2, g1, g2, 1,
        1.f / 16.f);
  note_launch();
  return check_launch("ntg_act_pool_bwd");
}

extern "C" int ntg_affine_bwd(void* stream, const float* gq, const float* gt, float* gu,
                              float* gut, int64_t n, ntg_affine_t aff, float scale) {
  NTG_REQUIRE(gu && n > 0, "ntg_affine_bwd: bad arguments");
  affine_bwd_kernel<<<grid_for(n), kT, 0, as_stream(stream)>>>(gq, gt, gu, gut, n, aff, scale);
  note_launch();
  return check_launch("ntg_affine_bwd");
}

extern "C" int ntg_affine_hyper_bwd(void* stream, const float* q, const float* t,
                                    const float* gq, const float* gt, int64_t n, float w2,
                                    float b2, double* out) {
  NTG_REQUIRE(q && out && n > 0, "ntg_affine_hyper_bwd: bad arguments");
  affine_hyper_kernel<<<grid_for(n), kT, 0, as_stream(stream)>>>(q, t, gq, gt, n, w2, b2, out);
  note_launch();
  return check_launch("ntg_affine_hyper_bwd");
}

extern "C" int ntg_stencil_bwd(void* stream, const float* gu, float* gin, int64_t batch, int64_t a,
                               int64_t c, int32_t fh, int32_t fw, int32_t sh, int32_t sw,
                               int32_t ph, int32_t pw, int64_t ao, int64_t co, int32_t pad_mode,
                               int32_t diag_spatial) {
  NTG_REQUIRE(gu && gin && batch > 0 && a > 0 && c > 0, "ntg_stencil_bwd: bad arguments");
  cudaStream_t s = as_stream(stream);
  if (diag_spatial) {
    stencil_ds_t_kernel<<<grid_for(batch * a * c), kT, 0, s>>>(
        gu, gin, batch, a, c, ao, co, fh, fw, sh, sw, ph, pw, pad_mode == NTG_PAD_CIRCULAR);
  } else if (fh == 3 && fw == 3 && sh == 1 && sw == 1 && ph == 1 && pw == 1 && ao == a &&
             co == c && pad_mode == NTG_PAD_ZERO) {
    stencil3_t_kernel<<<grid_for(batch * a * a * c * c), kT, 0, s>>>(gu, gin, batch, a, c);
  } else {
    stencil_t_kernel<<<grid_for(batch * a * a * c * c), kT, 0, s>>>(
        gu, gin, batch, a, c, ao, co, fh, fw, sh, sw, ph, pw, pad_mode == NTG_PAD_CIRCULAR);
  }
  note_launch();
  return check_launch("ntg_stencil_bwd");
}

extern "C" int ntg_pool_bwd(void* stream, const float* gout, float* gin, int64_t batch, int64_t a,
                            int64_t c, int32_t wa, int32_t wc, int32_t sa, int32_t sc, int32_t pa,
                            int32_t pc, int64_t ao, int64_t co, int32_t pad_mode,
                            int32_t diag_spatial, int32_t average, int32_t normalize_edges) {
  NTG_REQUIRE(gout && gin && batch > 0, "ntg_pool_bwd: bad arguments");
  NTG_REQUIRE(wa <= 6 && wc <= 6, "ntg_pool_bwd: windows up to 6 per axis");
  const int64_t total = diag_spatial ? batch * a * c : batch * a * a * c * c;
  const bool blocks = !diag_spatial && pa == 0 && pc == 0 && sa == wa && sc == wc &&
                      a % wa == 0 && c % wc == 0 && ao == a / wa && co == c / wc && c % 4 == 0 &&
                      a * a * c * c < (1ll << 31) &&
                      ((reinterpret_cast<uintptr_t>(gin) & 15) == 0);
  if (blocks) {
    const float weight = average ? 1.f / (float)(wa * wa * wc * wc) : 1.f;
    const int64_t n4 = a * a * c * c / 4;
    int64_t gx = ceil_div(n4, kT);
    const int64_t gy = batch < 65535 ? batch : 65535;
    while (gx * gy > 152 * 64 && gx > 1) gx = ceil_div(gx, 2);
    pool_t_block_kernel<<<dim3((unsigned)gx, (unsigned)gy), kT, 0, as_stream(stream)>>>(
        gout, gin, batch, (int)a, (int)c, wa, wc, weight);
    note_launch();
    return check_launch("ntg_pool_bwd");
  }
  pool_t_kernel<<<grid_for(total), kT, 0, as_stream(stream)>>>(
      gout, gin, batch, a, c, ao, co, wa, wc, sa, sc, pa, pc, pad_mode == NTG_PAD_CIRCULAR,
      diag_spatial, average, normalize_edges);
  note_launch();
  return check_launch("ntg_pool_bwd");
}

extern "C" int ntg_readout_bwd(void* stream, const float* gout, float* gin, int64_t batch,
                               int64_t a, int64_t c, int32_t flatten_fs, int64_t m, float scale) {
  NTG_REQUIRE(gout && gin && batch > 0 && m > 0, "ntg_readout_bwd: bad arguments");
  readout_t_kernel<<<grid_for(batch * m), kT, 0, as_stream(stream)>>>(gout, gin, batch, a, c,
                                                                      flatten_fs, m, scale);
  note_launch();
  return check_launch("ntg_readout_bwd");
}

extern "C" int ntg_input_fs_bwd(void* stream, const float* g, const float* x_other, float* gx,
                                int64_t nself, int64_t nother, int64_t n2, int64_t a, int64_t c,
                                int64_t k, int32_t side) {
  NTG_REQUIRE(g && x_other && gx && nself > 0 && a > 0 && c > 0 && k > 0,
              "ntg_input_fs_bwd: bad arguments");
  const size_t sm = sizeof(float) * c * k;
  NTG_REQUIRE(sm <= 48 * 1024, "ntg_input_fs_bwd: C * K too large");
  input_fs_t_kernel<<<(unsigned)(nself * a), 128, sm, as_stream(stream)>>>(
      g, x_other, gx, nself, nother, n2, a, c, k, side, 1.f / (float)k);
  note_launch();
  return check_launch("ntg_input_fs_bwd");
}

extern "C" int ntg_input_fs_bwd2(void* stream, const float* g, const float* x1,
                                 const float* x2, float* gx1, float* gx2, int64_t n1, int64_t n2,
                                 int64_t a, int64_t c, int64_t k) {
  NTG_REQUIRE(g && x1 && gx1 && n1 > 0 && n2 >= 0 && a > 0 && c > 0 && k > 0,
              "ntg_input_fs_bwd2: bad arguments");
  NTG_REQUIRE(n2 == 0 || (x2 && gx2), "ntg_input_fs_bwd2: pairs need x2 and gx2");
  cudaStream_t s = as_stream(stream);
  const bool fast = c == kIfC && k <= 4 && a <= (1 << 16) && n1 * a < (1ll << 31) &&
                    ((reinterpret_cast<uintptr_t>(g) | reinterpret_cast<uintptr_t>(x1) |
                      reinterpret_cast<uintptr_t>(x2)) & 15) == 0;
  if (fast && n2 * a < (1ll << 31)) {
    const float inv_k = 1.f / (float)k;
    // rows into gx1, then columns into gx2 (gx1 for the per-sample covariances, or when
    // x2 is x1); two launches on one stream, so a shared gx is never written concurrently
    const unsigned grid_r = (unsigned)(n1 * a);
    const unsigned grid_c = (unsigned)((n2 > 0 ? n2 : n1) * a);
    float* gc = n2 > 0 ? gx2 : gx1;
    switch (k) {
      case 1:
        input_fs_pass_kernel<1, false><<<grid_r, 256, 0, s>>>(g, x1, x2, gx1, n1, n2, (int)a, inv_k);
        input_fs_pass_kernel<1, true><<<grid_c, 256, 0, s>>>(g, x1, x2, gc, n1, n2, (int)a, inv_k);
        break;
      case 2:
        input_fs_pass_kernel<2, false><<<grid_r, 256, 0, s>>>(g, x1, x2, gx1, n1, n2, (int)a, inv_k);
        input_fs_pass_kernel<2, true><<<grid_c, 256, 0, s>>>(g, x1, x2, gc, n1, n2, (int)a, inv_k);
        break;
      case 3:
        input_fs_pass_kernel<3, false><<<grid_r, 256, 0, s>>>(g, x1, x2, gx1, n1, n2, (int)a, inv_k);
        input_fs_pass_kernel<3, true><<<grid_c, 256, 0, s>>>(g, x1, x2, gc, n1, n2, (int)a, inv_k);
        break;
      default:
        input_fs_pass_kernel<4, false><<<grid_r, 256, 0, s>>>(g, x1, x2, gx1, n1, n2, (int)a, inv_k);
        input_fs_pass_kernel<4, true><<<grid_c, 256, 0, s>>>(g, x1, x2, gc, n1, n2, (int)a, inv_k);
        break;
    }
    note_launch();
    note_launch();
    return check_launch("ntg_input_fs_bwd2");
  }
  const size_t sm = sizeof(float) * c * k;
  NTG_REQUIRE(sm <= 48 * 1024, "ntg_input_fs_bwd2: C * K too large");
  const float inv_k = 1.f / (float)k;
  if (n2 == 0) {
    input_fs_t_kernel<<<(unsigned)(n1 * a), 128, sm, s>>>(g, x1, gx1, n1, n1, 0, a, c, k, 0, inv_k);
    input_fs_t_kernel<<<(unsigned)(n1 * a), 128, sm, s>>>(g, x1, gx1, n1, n1, 0, a, c, k, 1, inv_k);
  } else {
    input_fs_t_kernel<<<(unsigned)(n1 * a), 128, sm, s>>>(g, x2, gx1, n1, n2, n2, a, c, k, 0, inv_k);
    input_fs_t_kernel<<<(unsigned)(n2 * a), 128, sm, s>>>(g, x1, gx2, n2, n1, n2, a, c, k, 1, inv_k);
  }
  note_launch(2);
  return check_launch("ntg_input_fs_bwd2");
}

extern "C" int ntg_gemm_ex(void* stream, const float* a, const float* b, float* c, int64_t m,
                           int64_t n, int64_t k, int32_t trans_a, float alpha,
                           int32_t accumulate) {
  NTG_REQUIRE(a && b && c && m > 0 && n > 0 && k > 0, "ntg_gemm_ex: bad arguments");
  NTG_REQUIRE(ceil_div(m, 64) <= 65535, "ntg_gemm_ex: m too large");
  dim3 grid((unsigned)ceil_div(n, 64), (unsigned)ceil_div(m, 64));
  gemm_ex_kernel<<<grid, 256, 0, as_stream(stream)>>>(a, b, c, m, n, k, trans_a, alpha,
                                                      accumulate);
  note_launch();
  return check_launch("ntg_gemm_ex");
}

extern "C" int ntg_cov_diag_bwd(void* stream, const float* gcov, const float* x, float* gx,
                                int64_t n, int64_t d) {
  NTG_REQUIRE(gcov && x && gx && n > 0 && d > 0, "ntg_cov_diag_bwd: bad arguments");
  cov_diag_t_kernel<<<grid_for(n * d), kT, 0, as_stream(stream)>>>(gcov, x, gx, n, d,
                                                                   2.f / (float)d);
  note_launch();
  return check_launch("ntg_cov_diag_bwd");
}

// Adjoint of ntg_input_ds, ADDING into gx [nself, P, K]:
//   mode 0: gx[s, p, k] += scale sum_o g[s, o, p] xo[o, p, k]   (g is [nself, nother, P])
//   mode 1: gx[s, p, k] += scale sum_o g[o, s, p] xo[o, p, k]   (g is [nother, nself, P])
//   mode 2: gx[s, p, k] += scale g[s, p] xo[s, p, k]             (self covariances)
__global__ void input_ds_bwd_kernel(const float* __restrict__ g, const float* __restrict__ xo,
                                    float* __restrict__ gx, int64_t nself, int64_t nother,
                                    int64_t P, int64_t K, int mode, float scale) {
  const int64_t total = nself * P * K;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = idx % K, sp = idx / K, p = sp % P, sf = sp / P;
    float acc = 0.f;
    if (mode == 2) {
      acc = g[sf * P + p] * xo[idx];
    } else {
      for (int64_t o = 0; o < nother; ++o) {
        const float gv = mode == 0 ? g[(sf * nother + o) * P + p] : g[(o * nself + sf) * P + p];
        acc = fmaf(gv, xo[(o * P + p) * K + k], acc);
      }
    }
    gx[idx] += scale * acc;
  }
}

extern "C" int ntg_input_ds_bwd(void* stream, const float* g, const float* x1, const float* x2,
                                float* gx1, float* gx2, int64_t n1, int64_t n2, int64_t p,
                                int64_t k) {
  NTG_REQUIRE(g && x1 && gx1 && n1 > 0 && p > 0 && k > 0, "ntg_input_ds_bwd: bad arguments");
  NTG_REQUIRE(n2 == 0 || (x2 && gx2 && n2 > 0), "ntg_input_ds_bwd: pairs need x2, gx2, n2 > 0");
  cudaStream_t s = as_stream(stream);
  const float inv_k = 1.f / (float)k;
  if (n2 == 0) {
    input_ds_bwd_kernel<<<grid_for(n1 * p * k), kT, 0, s>>>(g, x1, gx1, n1, 1, p, k, 2,
                                                            2.f * inv_k);
    note_launch();
  } else {
    // two launches on one stream: gx2 may be gx1 (a symmetric call, x2 == x1)
    input_ds_bwd_kernel<<<grid_for(n1 * p * k), kT, 0, s>>>(g, x2, gx1, n1, n2, p, k, 0, inv_k);
    input_ds_bwd_kernel<<<grid_for(n2 * p * k), kT, 0, s>>>(g, x1, gx2, n2, n1, p, k, 1, inv_k);
    note_launch();
    note_launch();
  }
  return check_launch("ntg_input_ds_bwd");
}

namespace ntg {
int bwd_take_device_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_bwd_error, sizeof(int)) != cudaSuccess) return -1;
  const int zero = 0;
  if (v != 0 && cudaMemcpyToSymbol(g_bwd_error, &zero, sizeof(int)) != cudaSuccess) return -1;
  return v;
}
}  // namespace ntg

extern "C" int ntg_diag_add(void* stream, const float* src, float* dst, int64_t n, int64_t a,
                            int64_t c, int64_t s_n, int64_t s_a, int64_t s_c) {
  NTG_REQUIRE(src && dst && n > 0 && a > 0 && c > 0, "ntg_diag_add: bad arguments");
  diag_add_kernel<<<grid_for(n * a * c), kT, 0, as_stream(stream)>>>(src, dst, n, a, c, s_n, s_a,
                                                                     s_c);
  note_launch();
  return check_launch("ntg_diag_add");
}
