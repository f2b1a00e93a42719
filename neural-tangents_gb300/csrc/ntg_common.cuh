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

// Tensor-core (tcgen05) split-precision Gram; defined in ntg_gram_tc.cu.
int gram_tc(cudaStream_t stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
            int64_t d, float* out);

#define NTG_REQUIRE(cond, msg)                                   \
  do {                                                           \
    if (!(cond)) return ::ntg::fail(NTG_ERR_INVALID_ARG, (msg)); \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

constexpr float kPi = 3.14159265358979323846f;

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

// atan2(s, q) for s >= 0 (angle in [0, pi]); returns `fill` when s == q == 0
// (the fill_zero convention of elementwise.py:1293-1301).
__device__ __forceinline__ float atan2_ypos(float s, float q, float fill) {
  const float aq = fabsf(q);
  const float mx = fmaxf(aq, s), mn = fminf(aq, s);
  float th = atan_unit(mn * rcp_approx(mx));
  th = (s > aq) ? (0.5f * kPi - th) : th;
  th = (q < 0.f) ? (kPi - th) : th;
  return (mx == 0.f) ? fill : th;
}

// Per-layer activation constants, computed once per layer (uniform).
struct ActC {
  int kind;
  int comp;
  float factor, half;  // ABRelu: (a-b)^2 / (2 pi), (a^2 + b^2) / 2
  float a2, b2, c2;    // Erf: a^2, b^2, c^2
  float stab, inv_stab;
};

__device__ __forceinline__ ActC act_consts(const ntg_act_t& act) {
  ActC c;
  c.kind = act.kind;
  c.comp = act.compensated;
  const float amb = act.a - act.b;
  c.factor = __fdiv_rn(__fmul_rn(amb, amb), 2.f * kPi);
  c.half = 0.5f * (__fmul_rn(act.a, act.a) + __fmul_rn(act.b, act.b));
  c.a2 = __fmul_rn(act.a, act.a);
  c.b2 = __fmul_rn(act.b, act.b);
  c.c2 = __fmul_rn(act.c, act.c);
  c.stab = act.stabilize;
  c.inv_stab = act.stabilize > 0.f ? __fdiv_rn(1.f, act.stabilize) : 1.f;
  return c;
}

// ABRelu(a, b) rule, elementwise.py:447-455:
//   s = sqrt(max(prod - q^2, 0)); theta = atan2(s, q) (pi/2 if both 0)
//   dot = (a^2 + b^2)/2 - (a-b)^2/(2 pi) theta; q' = (a-b)^2/(2 pi) s + dot q; ntk' = ntk dot
// Erf(a, b, c) rule, elementwise.py:67-112 (k *= b first, a*k + c last):
//   prod = (1 + 2 v1)(1 + 2 v2); s = sqrt(max(prod - 4q^2, 0));
//   q' = 2/pi atan2(2q, s); ntk' = ntk (4/pi) / s
__device__ __forceinline__ void act_apply(const ActC& c, float& q, float& t, float v1, float v2) {
  if (c.kind == NTG_ACT_ABRELU) {
    if (c.stab > 0.f) {
      q = __fdiv_rn(q, c.stab);
      v1 = __fdiv_rn(v1, c.stab);
      v2 = __fdiv_rn(v2, c.stab);
    }
    const float d = prod_minus_sq(v1, v2, q, c.comp);
    const float s = sqrt_approx(fmaxf(d, 0.f));
    const float th = atan2_ypos(s, q, 0.5f * kPi);
    const float dot = fmaf(-c.factor, th, c.half);
    float qo = fmaf(c.factor, s, __fmul_rn(dot, q));
    if (c.stab > 0.f) qo = __fmul_rn(qo, c.stab);
    q = qo;
    t = __fmul_rn(t, dot);
  } else if (c.kind == NTG_ACT_ERF) {
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
  }
}

// Affine rule on an unscaled propagated value u (nngp) and u_t (ntk).
__device__ __forceinline__ void apply_affine(const ntg_affine_t& f, float u, float ut,
                                             bool has_ntk, float& q, float& t) {
  q = __fadd_rn(__fmul_rn(f.w2, u), f.b2);
  if (has_ntk) {
    float nn = f.nn_scaled ? q : u;
    t = __fadd_rn(__fadd_rn(__fmul_rn(f.ntk_w2, ut), __fmul_rn(f.ntk_nn, nn)), f.ntk_c);
  }
}

__device__ __forceinline__ float var_at(const ntg_var_t& v, int64_t n, int64_t a, int64_t c) {
  return __ldg(v.base + n * v.s_n + a * v.s_a + c * v.s_c);
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace ntg
