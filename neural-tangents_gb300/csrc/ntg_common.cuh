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

// ABRelu(a, b) rule, elementwise.py:447-455:
//   s = sqrt(max(prod - q^2, 0)); theta = atan2(s, q) (pi/2 if both 0)
//   dot = (a^2 + b^2)/2 - (a-b)^2/(2 pi) theta; q' = (a-b)^2/(2 pi) s + dot q
__device__ __forceinline__ void abrelu_rule(float q, float v1, float v2, float a, float b,
                                            int compensated, float& q_out, float& dot) {
  float d = prod_minus_sq(v1, v2, q, compensated);
  float s = sqrtf(fmaxf(d, 0.f));
  float th = (s == 0.f && q == 0.f) ? 0.5f * kPi : atan2f(s, q);
  float amb = a - b;
  float factor = __fdiv_rn(__fmul_rn(amb, amb), 2.f * kPi);
  float half = 0.5f * (__fmul_rn(a, a) + __fmul_rn(b, b));
  dot = __fsub_rn(half, __fmul_rn(factor, th));
  q_out = __fadd_rn(__fmul_rn(factor, s), __fmul_rn(dot, q));
}

// Erf(a, b, c) rule, elementwise.py:67-112, applied after k *= b and before
// a*k + c:  prod = (1 + 2 v1)(1 + 2 v2);  s = sqrt(max(prod - 4q^2, 0));
//   q' = 2/pi atan2(2q, s);  ntk' = ntk * (4/pi) / s
__device__ __forceinline__ void erf_rule(float q, float v1, float v2, int compensated,
                                         float& q_out, float& dot) {
  float d1 = __fadd_rn(1.f, __fmul_rn(2.f, v1));
  float d2 = __fadd_rn(1.f, __fmul_rn(2.f, v2));
  float q2 = 2.f * q;
  float d = prod_minus_sq(d1, d2, q2, compensated);
  float s = sqrtf(fmaxf(d, 0.f));
  q_out = __fmul_rn(2.f / kPi, atan2f(q2, s));
  dot = __fdiv_rn(4.f / kPi, s);
}

// Applies the activation to (q, t) with variances (v1, v2); t may be unused.
__device__ __forceinline__ void apply_act(const ntg_act_t& act, float& q, float& t, float v1,
                                          float v2) {
  if (act.kind == NTG_ACT_ABRELU) {
    float f = 1.f;
    if (act.stabilize > 0.f) {
      f = act.stabilize;
      q = __fdiv_rn(q, f);
      v1 = __fdiv_rn(v1, f);
      v2 = __fdiv_rn(v2, f);
    }
    float qo, dot;
    abrelu_rule(q, v1, v2, act.a, act.b, act.compensated, qo, dot);
    if (act.stabilize > 0.f) qo = __fmul_rn(qo, f);
    q = qo;
    t = __fmul_rn(t, dot);
  } else if (act.kind == NTG_ACT_ERF) {
    float b2 = __fmul_rn(act.b, act.b);
    float a2 = __fmul_rn(act.a, act.a);
    float c2 = __fmul_rn(act.c, act.c);
    float qo, dot;
    erf_rule(__fmul_rn(b2, q), __fmul_rn(b2, v1), __fmul_rn(b2, v2), act.compensated, qo, dot);
    q = __fadd_rn(__fmul_rn(a2, qo), c2);
    t = __fmul_rn(a2, __fmul_rn(__fmul_rn(b2, t), dot));
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
