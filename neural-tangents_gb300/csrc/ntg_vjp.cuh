// Activation-rule adjoints at one entry (and on packed pairs), shared by the
// VJP kernels and the fused activation-VJP + transposed-stencil kernel.
// Derivative conventions follow the reference's custom JVPs: _sqrt
// (elementwise.py:1278-1290) has derivative 0 where its argument is <= 1e-30,
// and _arctan2 (:1293-1310) divides by max(x^2 + y^2, 1e-30).
#pragma once

#include "ntg_common.cuh"

namespace ntg {
namespace {

// VJPs of the Sin / Rbf / Gelu rules at one entry (the forward rules are
// act_apply_rare's): reverse mode through the reference's expressions, with
// _sqrt's derivative 0 where its argument is <= 1e-30 (elementwise.py:1278-1290)
// and jnp.arctan2's plain derivative in the Gelu rule (elementwise.py:230-250).
__device__ __forceinline__ void act_vjp_rare(const ActC& c, float q, float t, float v1, float v2,
                                             float gq, float gt, float& oq, float& ot,
                                             float& ov1, float& ov2) {
  if (c.kind == NTG_ACT_SIN) {
    // q' = A (s1 - s2) = M, t' = t B A (s1 + s2) = t B P with dM/dq = B P, dP/dq = B M and
    // d/dv1 = d/dv2 = -B / 2 on both (A = a^2 / 2, B = b^2; elementwise.py:303-311)
    const float sum = v1 + v2;
    const float s1 = expf(c.b2 * fmaf(-0.5f, sum, q));
    const float s2 = expf(c.b2 * fmaf(-0.5f, sum, -q)) * c.c2;
    const float P = c.a2 * (s1 + s2), M = c.a2 * (s1 - s2);
    const float gP = c.b2 * t * gt;
    oq = c.b2 * fmaf(gq, P, gP * M);
    ot = c.b2 * P * gt;
    ov1 = ov2 = -0.5f * c.b2 * fmaf(gq, M, gP * P);
  } else if (c.kind == NTG_ACT_RBF) {
    // q' = exp(g (2 q - v1 - v2)), t' = t 2 g q' (g = gamma; elementwise.py:380-384)
    const float qo = expf(c.a2 * fmaf(2.f, q, -(v1 + v2)));
    const float g_qo = fmaf(2.f * c.a2 * t, gt, gq);
    oq = 2.f * c.a2 * qo * g_qo;
    ot = 2.f * c.a2 * qo * gt;
    ov1 = ov2 = -c.a2 * qo * g_qo;
  } else if (c.kind == NTG_ACT_GELU) {
    const float tol = 1e-30f;
    const float prod = v1 * v2;
    const float pp1 = (v1 + 1.f) * (v2 + 1.f);
    const float d2 = pp1 - q * q;
    const float dl = sqrtf(fmaxf(d2, 0.f));
    const float ang = atan2f(q, dl);
    const float num = q * q + prod * d2, dn = pp1 * dl;
    const float first0 = 1.f / d2 + (1.f - prod) / pp1 + 1.f;
    const float k2pi = 1.f / (2.f * kPi);
    const float first = first0 * q / dl * k2pi;
    const float second = 0.25f + ang * k2pi;
    ot = gt * (first + second);
    const float g_f = gt * t;  // cotangent of first and of second
    float g_q = gq * (ang * k2pi + 0.25f);
    const float g_ang = (g_f + gq * q) * k2pi;
    const float g_r = gq * k2pi;  // cotangent of num / dn
    // first = first0 q / dl / (2 pi)
    const float g_first0 = g_f * q / dl * k2pi;
    g_q += g_f * first0 / dl * k2pi;
    float g_dl = -g_f * first0 * q / (dl * dl) * k2pi;
    // first0 = 1 / d2 + (1 - prod) / pp1 + 1
    float g_d2 = -g_first0 / (d2 * d2);
    float g_prod = -g_first0 / pp1;
    float g_pp1 = -g_first0 * (1.f - prod) / (pp1 * pp1);
    // num / dn
    const float g_num = g_r / dn;
    const float g_dn = -g_r * num / (dn * dn);
    g_pp1 += g_dn * dl;
    g_dl += g_dn * pp1;
    g_q += 2.f * q * g_num;
    g_prod += g_num * d2;
    g_d2 += g_num * prod;
    // ang = arctan2(q, dl)
    const float den = q * q + dl * dl;
    g_q += g_ang * dl / den;
    g_dl -= g_ang * q / den;
    // dl = _sqrt(d2)
    g_d2 += (d2 > tol) ? g_dl * 0.5f / dl : 0.f;
    // d2 = pp1 - q^2
    g_pp1 += g_d2;
    g_q -= 2.f * q * g_d2;
    oq = g_q;
    ov1 = fmaf(g_pp1, v2 + 1.f, g_prod * v2);
    ov2 = fmaf(g_pp1, v1 + 1.f, g_prod * v1);
  } else {
    oq = gq;
    ot = gt;
    ov1 = ov2 = 0.f;
  }
}

__device__ __forceinline__ bool act_is_rare(int kind) {
  return kind == NTG_ACT_SIN || kind == NTG_ACT_RBF || kind == NTG_ACT_GELU;
}

// act_vjp with the library's one-instruction square roots and reciprocals and
// its arc tangent: the angle atan2(s, q) comes from the half-angle identities
// theta = 2 atan(s / (r + q)) (q >= 0), pi - 2 atan(s / (r - q)) (q < 0),
// r = |(q, s)|, and pi / 2 where s = q = 0 — the same derivative conventions
// as act_vjp (tolerance 1e-30 in the arctan2 and sqrt derivatives).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <bool RARE = false>
__device__ __forceinline__ void act_vjp_fast(const ntg_act_t& act, const ActC& c, float q,
                                             float t, float v1, float v2, float gq, float gt,
                                             float& oq, float& ot, float& ov1, float& ov2) {
  const float tol = 1e-30f;
  if (act.kind == NTG_ACT_ABRELU) {
    const float d = prod_minus_sq(v1, v2, q, c.comp);
    const float s = sqrt_approx(fmaxf(d, 0.f));
    const float den2 = fmaf(s, s, q * q);
    const float r = sqrt_approx(den2);
    const float hd = r + fabsf(q);
    const float p = atan_unit(s * rcp_approx(hd));
    float th = (q < 0.f) ? fmaf(-2.f, p, kPi) : 2.f * p;
    th = (hd == 0.f) ? 0.5f * kPi : th;
    const float dot = fmaf(-c.factor, th, c.half);
    const float g_dot = fmaf(q, gq, t * gt);
    float g_s = c.factor * gq;
    float g_q = dot * gq;
    ot = dot * gt;
    const float g_th = -c.factor * g_dot;
    const float inv = rcp_approx(fmaxf(den2, tol));
    g_s = fmaf(g_th * q, inv, g_s);
    g_q = fmaf(-g_th * s, inv, g_q);
    const float g_d = (d > tol) ? 0.5f * g_s * rsqrt_approx(d) : 0.f;
    g_q = fmaf(-2.f * q, g_d, g_q);
    ov1 = g_d * v2;
    ov2 = g_d * v1;
    oq = g_q;
  } else if (act.kind == NTG_ACT_ERF) {
    const float qb = c.b2 * q, tb = c.b2 * t;
    const float d1 = fmaf(2.f * c.b2, v1, 1.f), d2 = fmaf(2.f * c.b2, v2, 1.f);
    const float y = 2.f * qb;
    const float dd = prod_minus_sq(d1, d2, y, c.comp);
    const float s = sqrt_approx(fmaxf(dd, 0.f));
    const float gq2 = c.a2 * gq, gt2 = c.a2 * gt;
    const float rs = rcp_approx(s);
    const float dot = (4.f / kPi) * rs;
    const float g_tb = dot * gt2;
    const float g_dot = tb * gt2;
    float g_s = -(4.f / kPi) * rs * rs * g_dot;
    const float g_phi = (2.f / kPi) * gq2;
    const float den = fmaf(s, s, y * y);
    const float iden = den > 0.f ? rcp_approx(den) : 0.f;
    const float g_y = g_phi * s * iden;
    g_s = fmaf(-g_phi * y, iden, g_s);
    float g_qb = 2.f * g_y;
    const float g_dd = (dd > tol) ? 0.5f * g_s * rsqrt_approx(dd) : 0.f;
    g_qb = fmaf(-4.f * y, g_dd, g_qb);
    oq = c.b2 * g_qb;
    ot = c.b2 * g_tb;
    ov1 = c.b2 * 2.f * (g_dd * d2);
    ov2 = c.b2 * 2.f * (g_dd * d1);
  } else if (RARE && act_is_rare(act.kind)) {
    act_vjp_rare(c, q, t, v1, v2, gq, gt, oq, ot, ov1, ov2);
  } else {
    oq = gq;
    ot = gt;
    ov1 = ov2 = 0.f;
  }
}

// act_vjp_fast's ABRelu branch on a packed pair of entries (the f32x2 datapath
// for the products and sums, scalar square roots, reciprocals and selects).
__device__ __forceinline__ void abrelu_vjp2(const ActC& c, P2 q, P2 t, P2 v1, P2 v2, P2 gq,
                                            P2 gt, P2& oq, P2& ot, P2& ov1, P2& ov2) {
  const float tol = 1e-30f;
  const P2 pr = mul2(v1, v2), qq = mul2(q, q);
  P2 d = sub2(pr, qq);
  if (c.comp) {
    const P2 m1 = p2s(-1.f);
    const P2 pe = fma2(v1, v2, mul2(pr, m1)), qe = fma2(q, q, mul2(qq, m1));
    d = add2(d, sub2(pe, qe));
  }
  float d0, d1, q0, q1;
  p2u(d, d0, d1);
  p2u(q, q0, q1);
  const float s0 = sqrt_approx(fmaxf(d0, 0.f)), s1 = sqrt_approx(fmaxf(d1, 0.f));
  const P2 sp = p2(s0, s1);
  const P2 den2 = fma2(sp, sp, qq);
  float e0, e1;
  p2u(den2, e0, e1);
  const float hd0 = sqrt_approx(e0) + fabsf(q0), hd1 = sqrt_approx(e1) + fabsf(q1);
  const P2 r = mul2(sp, p2(rcp_approx(hd0), rcp_approx(hd1)));
  const P2 z = mul2(r, r);
  P2 pp = fma2(p2s(-0.00405457f), z, p2s(0.02186296f));
  pp = fma2(pp, z, p2s(-0.05591233f));
  pp = fma2(pp, z, p2s(0.09642197f));
  pp = fma2(pp, z, p2s(-0.13908629f));
  pp = fma2(pp, z, p2s(0.19946566f));
  pp = fma2(pp, z, p2s(-0.3332986f));
  pp = fma2(pp, z, p2s(0.99999934f));
  pp = mul2(pp, r);
  float p0, p1;
  p2u(pp, p0, p1);
  float th0 = (q0 < 0.f) ? fmaf(-2.f, p0, kPi) : 2.f * p0;
  float th1 = (q1 < 0.f) ? fmaf(-2.f, p1, kPi) : 2.f * p1;
  th0 = (hd0 == 0.f) ? 0.5f * kPi : th0;
  th1 = (hd1 == 0.f) ? 0.5f * kPi : th1;
  const P2 dot = fma2(p2s(-c.factor), p2(th0, th1), p2s(c.half));
  const P2 g_dot = fma2(q, gq, mul2(t, gt));
  P2 g_s = mul2(p2s(c.factor), gq);
  P2 g_q = mul2(dot, gq);
  ot = mul2(dot, gt);
  const P2 g_th = mul2(p2s(-c.factor), g_dot);
  const P2 inv = p2(rcp_approx(fmaxf(e0, tol)), rcp_approx(fmaxf(e1, tol)));
  g_s = fma2(mul2(g_th, q), inv, g_s);
  g_q = fma2(mul2(mul2(g_th, sp), p2s(-1.f)), inv, g_q);
  float gs0, gs1;
  p2u(g_s, gs0, gs1);
  const float gd0 = (d0 > tol) ? 0.5f * gs0 * rsqrt_approx(d0) : 0.f;
  const float gd1 = (d1 > tol) ? 0.5f * gs1 * rsqrt_approx(d1) : 0.f;
  const P2 g_d = p2(gd0, gd1);
  oq = fma2(mul2(p2s(-2.f), q), g_d, g_q);
  ov1 = mul2(g_d, v2);
  ov2 = mul2(g_d, v1);
}

}  // namespace
}  // namespace ntg
