// Shared device helpers for the sm_103a kernels of the analytic NNGP/NTK path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "nt_gb300.h"

namespace ntg {

// ---------------------------------------------------------------------------
// Host-side error plumbing shared by every translation unit.
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_launch(const char* what);
void note_launch(uint64_t n = 1);
int32_t tune(int32_t knob);  // current value of an NTG_TUNE_* knob
// Read and clear the device error words of the adjoint kernels (ntg_bwd.cu)
// and of the tensor-core Gram (ntg_gram_tc.cu); -1 if the read failed.
int bwd_take_device_error();
int gram_take_device_error();
int gemm_take_device_error();  // ntg_gemm_tc.cu
int chol_take_device_error();  // ntg_chol_tc.cu

// Tensor-core (tcgen05) split-precision Gram; defined in ntg_gram_tc.cu.
int gram_tc(cudaStream_t stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
            int64_t d, float* out, void* workspace, size_t ws_bytes);
size_t gram_tc_workspace(int64_t n1, int64_t n2, int64_t d);

#define NTG_REQUIRE(cond, msg)                                   \
  do {                                                           \
    if (!(cond)) return ::ntg::fail(NTG_ERR_INVALID_ARG, (msg)); \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr float kPi = 3.14159265358979323846f;

// ---------------------------------------------------------------------------
// Bulk-copy rings: shared-memory addresses and bounded mbarrier waits. A wait
// that runs out returns false; the kernel then raises its device error word.
// ---------------------------------------------------------------------------
constexpr uint32_t kLineWaitLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
  for (uint32_t it = 0; it < kLineWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Activation rules.  All products that the reference evaluates as separate
// float32 operations use the non-contracting intrinsics so that a self pair
// (q == v1 == v2) gives v1*v2 - q*q == 0 exactly, as in the reference.
// ---------------------------------------------------------------------------

// v1*v2 - q*q.  compensated: exact two-product difference (error-free
// transformations of both products), accurate near correlation +-1.
__device__ __forceinline__ float prod_minus_sq(float v1, float v2, float q, int compensated) {
  float p = __fmul_rn(v1, v2);
  float qq = __fmul_rn(q, q);
  float d = __fsub_rn(p, qq);
  if (compensated) {
    float pe = __fmaf_rn(v1, v2, -p);
    float qe = __fmaf_rn(q, q, -qq);
    d = __fadd_rn(d, __fsub_rn(pe, qe));
  }
  return d;
}

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// atan(t) for t in [0, 1] as t * P(t^2), P of degree 7. The coefficients are a
// minimax fit made for this library (Lawson-weighted least squares on a dense
// grid of [0, 1]); max |error| 3.8e-8 in exact arithmetic, 1.4e-7 evaluated in
// float32.
__device__ __forceinline__ float atan_unit(float t) {
  const float z = t * t;
  float p = -0.00405457f;
  p = fmaf(p, z, 0.02186296f);
  p = fmaf(p, z, -0.05591233f);
  p = fmaf(p, z, 0.09642197f);
  p = fmaf(p, z, -0.13908629f);
  p = fmaf(p, z, 0.19946566f);
  p = fmaf(p, z, -0.3332986f);
  p = fmaf(p, z, 0.99999934f);
  return p * t;
}

// atan2(y, x) for x >= 0 (angle in [-pi/2, pi/2]); atan2(0, 0) = 0.
__device__ __forceinline__ float atan2_xpos(float y, float x) {
  const float ay = fabsf(y);
  const float mx = fmaxf(ay, x), mn = fminf(ay, x);
  float th = atan_unit(mn * rcp_approx(mx));
  th = (ay > x) ? (0.5f * kPi - th) : th;
  th = (mx == 0.f) ? 0.f : th;
  return copysignf(th, y);
}

// Packed float pairs on the sm_100-family f32x2 datapath: one instruction
// operates on two independent lanes, each rounded exactly as the scalar
// instruction would round it.
struct P2 {
  unsigned long long v;
};
__device__ __forceinline__ P2 p2(float a, float b) {
  P2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ P2 p2s(float a) { return p2(a, a); }
__device__ __forceinline__ void p2u(P2 x, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
}
__device__ __forceinline__ P2 p2ld(const float* ptr) {  // 8-byte aligned shared/global
  P2 r;
  r.v = *reinterpret_cast<const unsigned long long*>(ptr);
  return r;
}
__device__ __forceinline__ P2 add2(P2 a, P2 b) {
  P2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}
__device__ __forceinline__ P2 sub2(P2 a, P2 b) {
  P2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}
__device__ __forceinline__ P2 mul2(P2 a, P2 b) {
  P2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}
__device__ __forceinline__ P2 fma2(P2 a, P2 b, P2 c) {
  P2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return d;
}

// Per-layer activation constants, computed once per layer (uniform).
struct ActC {
  int kind;
  int comp;
  float factor, half;  // ABRelu: (a-b)^2 / (2 pi), (a^2 + b^2) / 2
  float f2, h_neg, h_zero;  // 2 factor, half - pi factor, half - pi/2 factor
  float a2, b2, c2;    // Erf: a^2, b^2, c^2; Sin: a^2 / 2, b^2, cos(2 c); Rbf: gamma in a2
  float stab;
};

__device__ __forceinline__ ActC act_consts(const ntg_act_t& act) {
  ActC c;
  c.kind = act.kind;
  c.comp = act.compensated;
  const float amb = act.a - act.b;
  c.factor = __fdiv_rn(__fmul_rn(amb, amb), 2.f * kPi);
  c.half = 0.5f * (__fmul_rn(act.a, act.a) + __fmul_rn(act.b, act.b));
  c.f2 = 2.f * c.factor;
  c.h_neg = fmaf(-kPi, c.factor, c.half);
  c.h_zero = fmaf(-0.5f * kPi, c.factor, c.half);
  c.a2 = __fmul_rn(act.a, act.a);
  c.b2 = __fmul_rn(act.b, act.b);
  c.c2 = __fmul_rn(act.c, act.c);
  c.stab = act.stabilize;
  if (act.kind == NTG_ACT_SIN) {
    c.a2 = 0.5f * c.a2;
    c.c2 = act.c;  // the caller passes cos(2 c)
  } else if (act.kind == NTG_ACT_RBF) {
    c.a2 = act.a;
  }
  return c;
}

// Sin / Rbf / Gelu rules. Kernels instantiate act_apply<false> to leave them out:
// compiled into the fused chain kernel, their library calls slow its ReLU path.
__device__ __forceinline__ void act_apply_rare(const ActC& c, float& q, float& t, float v1,
                                            float v2) {
  if (c.kind == NTG_ACT_SIN) {
    // elementwise.py:303-311: s1 = exp(b^2 (q - sum / 2)), s2 = exp(b^2 (-q - sum / 2)) cos 2c
    const float sum = v1 + v2;
    const float s1 = expf(c.b2 * fmaf(-0.5f, sum, q));
    const float s2 = expf(c.b2 * fmaf(-0.5f, sum, -q)) * c.c2;
    t = t * (c.a2 * c.b2 * (s1 + s2));
    q = c.a2 * (s1 - s2);
  } else if (c.kind == NTG_ACT_RBF) {
    // elementwise.py:380-384: q' = exp(gamma (2 q - sum)), ntk' = ntk 2 gamma q'
    const float qo = expf(c.a2 * fmaf(2.f, q, -(v1 + v2)));
    t = t * (2.f * c.a2 * qo);
    q = qo;
  } else if (c.kind == NTG_ACT_GELU) {
    // elementwise.py:230-250 with prod = v1 v2, prod + 1 = (v1 + 1)(v2 + 1)
    const float prod = v1 * v2;
    const float pp1 = (v1 + 1.f) * (v2 + 1.f);
    const float d2 = pp1 - q * q;
    const float dl = sqrtf(fmaxf(d2, 0.f));
    const float ang = atan2_xpos(q, dl);
    float qo = (q * q + prod * d2) / (pp1 * dl);
    qo = (qo + q * ang) / (2.f * kPi);
    qo = fmaf(0.25f, q, qo);
    float first = 1.f / d2 + (1.f - prod) / pp1 + 1.f;
    first *= q / dl / (2.f * kPi);
    t = t * (first + (0.25f + ang / (2.f * kPi)));
    q = qo;
  }
}

// ABRelu(a, b) rule, elementwise.py:447-455:
//   s = sqrt(max(prod - q^2, 0)); theta = atan2(s, q) (pi/2 if both 0)
//   dot = (a^2 + b^2)/2 - (a-b)^2/(2 pi) theta; q' = (a-b)^2/(2 pi) s + dot q; ntk' = ntk dot
// theta comes from the half-angle identities
//   theta = 2 atan(s / (n + q)) for q >= 0,  theta = pi - 2 atan(s / (n - q)) for q < 0,
// n = sqrt(v1) sqrt(v2) >= |q|, whose arguments lie in [0, 1] and carry no
// cancellation near correlation +-1. sv1, sv2 are sqrt(v1), sqrt(v2).
// Erf(a, b, c) rule, elementwise.py:67-112 (k *= b first, a*k + c last):
//   prod = (1 + 2 v1)(1 + 2 v2); s = sqrt(max(prod - 4q^2, 0));
//   q' = 2/pi atan2(2q, s); ntk' = ntk (4/pi) / s
template <bool RARE = true, bool ERF = true>
__device__ __forceinline__ void act_apply(const ActC& c, float& q, float& t, float v1, float v2,
                                          float sv1, float sv2) {
  if (c.kind == NTG_ACT_ABRELU) {
    float n = __fmul_rn(sv1, sv2);
    if (c.stab > 0.f) {
      q = __fdiv_rn(q, c.stab);
      v1 = __fdiv_rn(v1, c.stab);
      v2 = __fdiv_rn(v2, c.stab);
      n = __fdiv_rn(n, c.stab);
    }
    const float d = prod_minus_sq(v1, v2, q, c.comp);
    const float s = sqrt_approx(fmaxf(d, 0.f));
    const float den = n + fabsf(q);
    const float p = atan_unit(s * rcp_approx(den));
    float dot = (q < 0.f) ? fmaf(c.f2, p, c.h_neg) : fmaf(-c.f2, p, c.half);
    dot = (den == 0.f) ? c.h_zero : dot;
    float qo = fmaf(c.factor, s, __fmul_rn(dot, q));
    if (c.stab > 0.f) qo = __fmul_rn(qo, c.stab);
    q = qo;
    t = __fmul_rn(t, dot);
  } else if (ERF && c.kind == NTG_ACT_ERF) {
    const float qb = __fmul_rn(c.b2, q);
    const float d1 = fmaf(2.f * c.b2, v1, 1.f);
    const float d2 = fmaf(2.f * c.b2, v2, 1.f);
    const float q2 = 2.f * qb;
    const float d = prod_minus_sq(d1, d2, q2, c.comp);
    const float s = sqrt_approx(fmaxf(d, 0.f));
    const float qo = __fmul_rn(2.f / kPi, atan2_xpos(q2, s));
    const float dot = __fmul_rn(4.f / kPi, rcp_approx(s));
    q = fmaf(c.a2, qo, c.c2);
    t = __fmul_rn(c.a2, __fmul_rn(__fmul_rn(c.b2, t), dot));
  } else if (RARE && c.kind >= NTG_ACT_SIN) {
    act_apply_rare(c, q, t, v1, v2);
  }
}

// The ABRelu branch of act_apply (do_stabilize off) on a packed pair, with
// the same operation sequence per lane. COMP: -1 reads c.comp, 0 / 1 fix the
// plain / compensated var1 var2 - q^2 at compile time.
template <int COMP = -1>
__device__ __forceinline__ void abrelu2(const ActC& c, P2& q, P2& t, P2 v1, P2 v2, P2 sv1,
                                        P2 sv2) {
  const P2 n = mul2(sv1, sv2);
  const P2 pr = mul2(v1, v2), qq = mul2(q, q);
  P2 d = sub2(pr, qq);
  if (COMP == 1 || (COMP < 0 && c.comp)) {
    const P2 m1 = p2s(-1.f);
    const P2 pe = fma2(v1, v2, mul2(pr, m1)), qe = fma2(q, q, mul2(qq, m1));
    d = add2(d, sub2(pe, qe));
  }
  float d0, d1, q0, q1, n0, n1;
  p2u(d, d0, d1);
  p2u(q, q0, q1);
  p2u(n, n0, n1);
  const float s0 = sqrt_approx(fmaxf(d0, 0.f)), s1 = sqrt_approx(fmaxf(d1, 0.f));
  const float den0 = n0 + fabsf(q0), den1 = n1 + fabsf(q1);
  const P2 sp = p2(s0, s1);
  const P2 r = mul2(sp, p2(rcp_approx(den0), rcp_approx(den1)));
  const P2 z = mul2(r, r);
  P2 pp = fma2(p2s(-0.00405457f), z, p2s(0.02186296f));
  pp = fma2(pp, z, p2s(-0.05591233f));
  pp = fma2(pp, z, p2s(0.09642197f));
  pp = fma2(pp, z, p2s(-0.13908629f));
  pp = fma2(pp, z, p2s(0.19946566f));
  pp = fma2(pp, z, p2s(-0.3332986f));
  pp = fma2(pp, z, p2s(0.99999934f));
  pp = mul2(pp, r);
  const P2 dneg = fma2(p2s(c.f2), pp, p2s(c.h_neg));
  const P2 dpos = fma2(p2s(-c.f2), pp, p2s(c.half));
  float a0, a1, b0, b1;
  p2u(dneg, a0, a1);
  p2u(dpos, b0, b1);
  float dot0 = (q0 < 0.f) ? a0 : b0, dot1 = (q1 < 0.f) ? a1 : b1;
  dot0 = (den0 == 0.f) ? c.h_zero : dot0;
  dot1 = (den1 == 0.f) ? c.h_zero : dot1;
  const P2 dot = p2(dot0, dot1);
  q = fma2(p2s(c.factor), sp, mul2(dot, q));
  t = mul2(t, dot);
}

// sqrt(var) as every kernel of the library evaluates it (one approximate
// square root), so that the fused and the materialised paths round alike.
__device__ __forceinline__ float sqrt_var(float v) { return sqrt_approx(fmaxf(v, 0.f)); }

__device__ __forceinline__ void act_apply(const ActC& c, float& q, float& t, float v1, float v2) {
  act_apply<true>(c, q, t, v1, v2, sqrt_var(v1), sqrt_var(v2));
}

// Affine rule on an unscaled propagated sum u (nngp) and u_t (ntk) whose
// stencil normalisation `scale` (1 / filter size) is folded into the weights.
__device__ __forceinline__ void apply_affine(const ntg_affine_t& f, float u, float ut,
                                             bool has_ntk, float& q, float& t,
                                             float scale = 1.f) {
  q = fmaf(f.w2 * scale, u, f.b2);
  if (has_ntk) {
    float nn = f.nn_scaled ? q : u * scale;
    t = fmaf(f.ntk_w2 * scale, ut, fmaf(f.ntk_nn, nn, f.ntk_c));
  }
}

__device__ __forceinline__ float var_at(const ntg_var_t& v, int64_t n, int64_t a, int64_t c) {
  return __ldg(v.base + n * v.s_n + a * v.s_a + c * v.s_c);
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace ntg
