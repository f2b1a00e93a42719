// Fused whole-network NNGP/NTK kernel for the Myrtle conv-net family on sm_103a.
//
// One CTA computes one (x1[i], x2[j]) pair end to end: first-layer Gram ->
// [3x3 SAME Conv + activation] x n0 -> AvgPool(2) -> [Conv + act] x n1 ->
// AvgPool(2) -> ... -> readout (mean of all spatial entries, or the mean of the
// spatial diagonal).  Nothing but the two readout scalars reaches HBM.
//
// Data layout.  The full-spatial kernel K[h, h', w, w'] of a pair is walked
// along its "lines": a line is the set of planes (h, h + delta) for a fixed
// delta; every Conv rule only couples planes of the same line
// (K'[h,h',..] = sum_d K[h+d, h'+d, ..]).  Inside a plane the (w, w') square is
// stored skewed: row r = (w' - w) mod S, column c = w, so the w-direction
// stencil neighbours (w +- 1, w' +- 1) are column neighbours of the same row
// (a row holds two diagonals of the square, split at c = S - r).  A thread owns
// EPT consecutive columns of one row in every plane of a line; the h-direction
// stencil is a 3-plane register ring, the w-direction one two warp shuffles.
// AvgPool(2) couples lines 2m-1, 2m, 2m+1 into pooled line m; pooled lines
// accumulate in shared memory and a completed pooled line is processed by the
// next segment right away, so the per-pair working set stays on chip.
#include "ntg_common.cuh"

namespace ntg {
namespace {

constexpr int NT = 512;

struct ChainCtx {
  const float* img1;  // [K][S0*S0] channel planes
  const float* img2;
  const float* img2s;  // img2 planes shifted one column left (segment-0 paired loads)
  int K;
  float* stage;        // [2 buffers][2 tensors][S0*S0]
  float inv_k;
  float acc_q, acc_t;  // per-thread readout partial sums
  int readout;
};

__device__ __forceinline__ float wshift_left(float v) {
  return __shfl_up_sync(0xffffffffu, v, 1);
}
__device__ __forceinline__ float wshift_right(float v) {
  return __shfl_down_sync(0xffffffffu, v, 1);
}

__device__ __forceinline__ void zero_slot(float* q, float* t, int n) {
  for (int i = threadIdx.x; i < n; i += NT) {
    q[i] = 0.f;
    t[i] = 0.f;
  }
}

// Processes line `delta` of a segment of size S with NC conv layers.
// FIRST: level-0 input is the first-layer Gram of the two images (its NTK is
// the scalar zero of an input kernel); otherwise it is pooled line
// `in_q/in_t` ([S][S*S], scaled by 1/16 for the AvgPool normalisation).
// LAST: the final level feeds the readout sums, otherwise it is average-pooled
// into the line slots of segment `seg + 1`.
// `vmaps` holds this segment's variance maps, layer k at vmaps + 4*k*S*S:
// var1, var2, sqrt(var1), sqrt(var2) as S x S maps; `out_slots` is the next segment's
// slot region ([parity][tensor][S/2][S/2 * S/2]).
// RO: which activation rules are compiled in — 0: ABRelu and Erf, 1: the ABRelu
// family only, 2: every rule (Sin / Rbf / Gelu as well).
template <int S, int NC, bool FIRST, bool LAST, int RO = 0>
__device__ __forceinline__ void process_line(ChainCtx& cx, const ntg_chain_t& pg, int lbase,
                                             const float* vmaps, float* out_slots, int delta,
                                             const float* in_q, const float* in_t) {
  constexpr int EPT = (S * S >= NT) ? (S * S / NT) : 1;
  constexpr int TPR = S / EPT;
  constexpr int ACTIVE = S * S / EPT;
  static_assert(TPR <= 32 && 32 % TPR == 0, "rows must tile warps");
  static_assert(ACTIVE % 32 == 0 && ACTIVE <= NT, "whole warps");
  const int tid = threadIdx.x;
  const bool on = tid < ACTIVE;
  const int r = on ? tid / TPR : 0;
  const int c0 = on ? (tid % TPR) * EPT : 0;
  const int lo = delta < 0 ? -delta : 0;
  const int hi = delta < 0 ? S : S - delta;

  // 1/0 weights of the left / right C-direction stencil neighbours (zero at
  // the row ends and at the split between the row's two diagonals)
  float ml[EPT], mr[EPT];
  int wp[EPT];
#pragma unroll
  for (int u = 0; u < EPT; ++u) {
    int c = c0 + u;
    ml[u] = (c >= 1 && c != S - r) ? 1.f : 0.f;
    mr[u] = (c <= S - 2 && c != S - 1 - r) ? 1.f : 0.f;
    wp[u] = (c + r) & (S - 1);
  }

  ActC acs[NC > 0 ? NC : 1];
#pragma unroll
  for (int k = 0; k < NC; ++k) acs[k] = act_consts(pg.act[lbase + k]);

  // Ring of the last two planes of every level (level 0 = input).
  float Aq[NC + 1][EPT], Bq[NC + 1][EPT], At[NC + 1][EPT], Bt[NC + 1][EPT];
#pragma unroll
  for (int k = 0; k <= NC; ++k)
#pragma unroll
    for (int u = 0; u < EPT; ++u) Aq[k][u] = Bq[k][u] = At[k][u] = Bt[k][u] = 0.f;

  int buf = 0;
  __syncthreads();
  for (int s = lo; s < hi + NC; ++s) {
    float nq[EPT], nt[EPT];
    // ---- level 0 at plane s ----
#pragma unroll
    for (int u = 0; u < EPT; ++u) nq[u] = nt[u] = 0.f;
    if (on && s < hi) {
      if (FIRST) {
        // first-layer Gram of the two images, channel by channel in the same
        // order as ntg_input_fs, so that both paths round alike
        const float* x1r = cx.img1 + s * S + c0;
        const float* x2r = cx.img2 + (s + delta) * S;
        float g[EPT];
#pragma unroll
        for (int u = 0; u < EPT; ++u) g[u] = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (k < cx.K) {
            const float* a = x1r + k * (S * S);
            const float* b = x2r + k * (S * S);
#pragma unroll
            for (int u = 0; u < EPT; ++u) g[u] = fmaf(a[u], b[wp[u]], g[u]);
          }
        }
#pragma unroll
        for (int u = 0; u < EPT; ++u) nq[u] = g[u] * cx.inv_k;
      } else {
        const float* pq = in_q + s * S * S + r * S + c0;
        const float* pt = in_t + s * S * S + r * S + c0;
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
          nq[u] = pq[u] * 0.0625f;
          nt[u] = pt[u] * 0.0625f;
        }
      }
    }
    // ---- conv layers: level k+1 at plane s-k-1 ----
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const int p = s - k - 1;
      const int l = lbase + k;
      const bool has_t = !(FIRST && k == 0);
      float hq[EPT], ht[EPT];
#pragma unroll
      for (int u = 0; u < EPT; ++u) {
        hq[u] = (Aq[k][u] + Bq[k][u]) + nq[u];
        ht[u] = has_t ? (At[k][u] + Bt[k][u]) + nt[u] : 0.f;
      }
      const float lq = wshift_left(hq[EPT - 1]), rq = wshift_right(hq[0]);
      const float lt = has_t ? wshift_left(ht[EPT - 1]) : 0.f;
      const float rt = has_t ? wshift_right(ht[0]) : 0.f;
      float oq[EPT], ot[EPT];
      const bool in_line = p >= lo && p < hi;  // uniform across the CTA
      if (in_line) {
        const ntg_affine_t& af = pg.aff[l];
        const ActC& ac = acs[k];
        const float* vm = vmaps + 4 * k * S * S;
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
          const float xl = (u > 0) ? hq[u - 1] : lq;
          const float xr = (u < EPT - 1) ? hq[u + 1] : rq;
          const float cq = fmaf(mr[u], xr, fmaf(ml[u], xl, hq[u]));
          float ct = 0.f;
          if (has_t) {
            const float yl = (u > 0) ? ht[u - 1] : lt;
            const float yr = (u < EPT - 1) ? ht[u + 1] : rt;
            ct = fmaf(mr[u], yr, fmaf(ml[u], yl, ht[u]));
          }
          float q, t = 0.f;
          apply_affine(af, cq, ct, true, q, t, 1.f / 9.f);
          if (ac.kind != NTG_ACT_NONE && on) {
            const int i1 = p * S + c0 + u, i2 = (p + delta) * S + wp[u];
            act_apply<RO == 2, RO != 1>(ac, q, t, vm[i1], vm[S * S + i2], vm[2 * S * S + i1],
                                        vm[3 * S * S + i2]);
          }
          oq[u] = q;
          ot[u] = t;
        }
      } else {
#pragma unroll
        for (int u = 0; u < EPT; ++u) oq[u] = ot[u] = 0.f;
      }
#pragma unroll
      for (int u = 0; u < EPT; ++u) {
        Aq[k][u] = Bq[k][u];
        Bq[k][u] = nq[u];
        At[k][u] = Bt[k][u];
        Bt[k][u] = nt[u];
        nq[u] = oq[u];
        nt[u] = ot[u];
      }
    }
    // ---- emit the last level at plane p = s - NC ----
    const int p = s - NC;
    if (p < lo || p >= hi) continue;
    if (LAST) {
      if (on) {
        if (cx.readout == 0) {
#pragma unroll
          for (int u = 0; u < EPT; ++u) {
            cx.acc_q += nq[u];
            cx.acc_t += nt[u];
          }
        } else if (delta == 0 && r == 0) {
#pragma unroll
          for (int u = 0; u < EPT; ++u) {
            cx.acc_q += nq[u];
            cx.acc_t += nt[u];
          }
        }
      }
    } else {
      float* sq = cx.stage + (2 * buf) * (S * S);
      float* st = sq + S * S;
      if (on) {
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
          sq[(c0 + u) * S + wp[u]] = nq[u];
          st[(c0 + u) * S + wp[u]] = nt[u];
        }
      }
      __syncthreads();
      constexpr int H = S / 2;
      if (tid < H * H) {
        const int rho = tid / H, kap = tid % H;
        const int j = kap, jp = (kap + rho) & (H - 1);
        const int o0 = (2 * j) * S + 2 * jp, o1 = o0 + S;
        float vq = (sq[o0] + sq[o0 + 1]) + (sq[o1] + sq[o1 + 1]);
        float vt = (st[o0] + st[o0 + 1]) + (st[o1] + st[o1 + 1]);
        const int I = p >> 1;
        const int m = ((p + delta) >> 1) - I;
        const int par = m & 1;
        float* dq = out_slots + (2 * par) * (H * H * H) + I * H * H + tid;
        float* dt = dq + H * H * H;
        *dq += vq;
        *dt += vt;
      }
      buf ^= 1;
    }
  }
  __syncthreads();
}

// Segment-0 line processor for 32x32 inputs: process_line<32, NC, true,
// LAST> with each thread's two elements held as one packed f32x2 pair.
// Thread t owns columns 2(t % 16), 2(t % 16) + 1 of skewed row t / 16. The
// per-lane operation sequence equals the scalar path's, so the result is bit
// for bit the same as process_line's and as the materialised layer kernels'.
template <int NC, bool LAST, int RO = 0, int COMP = -1, int KC = 0>
__device__ __forceinline__ void line_s32(ChainCtx& cx, const ntg_chain_t& pg, const float* vmaps,
                                         float* out_slots, int delta) {
  constexpr int S = 32;
  static_assert(NT == 512, "two columns per thread");
  const int tid = threadIdx.x;
  const int r = tid >> 4, c0 = (tid & 15) * 2;
  const int lo = delta < 0 ? -delta : 0;
  const int hi = delta < 0 ? S : S - delta;
  // 1/0 weights of the left / right neighbours of the thread's two columns
  const float ml0 = (c0 >= 1 && c0 != S - r) ? 1.f : 0.f, ml1 = (c0 + 1 != S - r) ? 1.f : 0.f;
  const float mr0 = (c0 != S - 1 - r) ? 1.f : 0.f;
  const float mr1 = (c0 + 1 <= S - 2 && c0 + 1 != S - 1 - r) ? 1.f : 0.f;
  const int wp0 = (c0 + r) & (S - 1), wp1 = (c0 + 1 + r) & (S - 1);
  // Sample-2 entries at the skewed columns (wp0, wp1 = wp0 + 1 mod 32) as one aligned
  // 8-byte load: from the plane itself for even rows (wp0 even), from its copy shifted
  // one column left (shifted[j] = plane[j + 1 mod 32]) at wp0 - 1 for odd rows.
  const int wpo = (r & 1) ? wp0 - 1 : wp0;
  const float* img2v = (r & 1) ? cx.img2s : cx.img2;
  const P2 zero = p2s(0.f);

  ActC acs[NC];
  P2 W2[NC], B2[NC], TW[NC], TN[NC], TC[NC];
  bool nns[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    acs[k] = act_consts(pg.act[k]);
    const ntg_affine_t& f = pg.aff[k];
    W2[k] = p2s(f.w2 * (1.f / 9.f));
    B2[k] = p2s(f.b2);
    TW[k] = p2s(f.ntk_w2 * (1.f / 9.f));
    TN[k] = p2s(f.ntk_nn);
    TC[k] = p2s(f.ntk_c);
    nns[k] = f.nn_scaled != 0;
  }
  const P2 INV9 = p2s(1.f / 9.f);
  const P2 INVK = p2s(cx.inv_k);

  P2 Aq[NC], Bq[NC], At[NC], Bt[NC];
#pragma unroll
  for (int k = 0; k < NC; ++k) Aq[k] = Bq[k] = At[k] = Bt[k] = zero;

  int buf = 0;
  __syncthreads();
  // unrolled by the period of the (A, B, new) plane ring, so that its rotation is a
  // renaming of registers rather than moves
#pragma unroll 3
  for (int s = lo; s < hi + NC; ++s) {
    P2 nq = zero, nt = zero;
    if (s < hi) {
      const float* x1r = cx.img1 + s * S + c0;
      const float* x2r = img2v + (s + delta) * S + wpo;
      P2 g = zero;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (KC > 0 ? k < KC : k < cx.K)  // KC > 0: channel count fixed at compile time
          g = fma2(p2ld(x1r + k * (S * S)), p2ld(x2r + k * (S * S)), g);
      }
      nq = mul2(g, INVK);
    }
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const int p = s - k - 1;
      const bool has_t = k > 0;
      const P2 hq = add2(add2(Aq[k], Bq[k]), nq);
      const P2 ht = has_t ? add2(add2(At[k], Bt[k]), nt) : zero;
      // the w-direction stencil per lane, in the order of the packed form
      // (h + ml * left) + mr * right, from the two shuffled neighbours
      float h0, h1, e0 = 0.f, e1 = 0.f;
      p2u(hq, h0, h1);
      const float lq = wshift_left(h1), rq = wshift_right(h0);
      const P2 cq = p2(fmaf(mr0, h1, fmaf(ml0, lq, h0)), fmaf(mr1, rq, fmaf(ml1, h0, h1)));
      P2 ct = zero;
      if (has_t) {
        p2u(ht, e0, e1);
        const float lt = wshift_left(e1), rt = wshift_right(e0);
        ct = p2(fmaf(mr0, e1, fmaf(ml0, lt, e0)), fmaf(mr1, rt, fmaf(ml1, e0, e1)));
      }
      P2 oq = zero, ot = zero;
      if (p >= lo && p < hi) {  // uniform across the CTA
        P2 q = fma2(W2[k], cq, B2[k]);
        const P2 nn = nns[k] ? q : mul2(cq, INV9);
        P2 t = fma2(TW[k], ct, fma2(TN[k], nn, TC[k]));
        const ActC& ac = acs[k];
        if (ac.kind != NTG_ACT_NONE) {
          // six maps per layer: v1, v2, sqrt v1, sqrt v2, and v2, sqrt v2 shifted
          const float* vm = vmaps + 6 * k * S * S;
          const int i1 = p * S + c0, i2 = (p + delta) * S;
          const P2 v1 = p2ld(vm + i1), sv1 = p2ld(vm + 2 * S * S + i1);
          const float* v2r = vm + S * S + i2;
          const float* s2r = vm + 3 * S * S + i2;
          if (RO == 1 || (ac.kind == NTG_ACT_ABRELU && ac.stab <= 0.f)) {
            // odd rows read the shifted copies: v2 at map 4, sqrt v2 at map 5
            const int shv = (r & 1) ? 3 * S * S : 0, shs = (r & 1) ? 2 * S * S : 0;
            abrelu2<COMP>(ac, q, t, v1, p2ld(v2r + shv + wpo), sv1, p2ld(s2r + shs + wpo));
          } else {
            float qa, qb, ta, tb, va, vb, sa, sb;
            p2u(q, qa, qb);
            p2u(t, ta, tb);
            p2u(v1, va, vb);
            p2u(sv1, sa, sb);
            act_apply<RO == 2>(ac, qa, ta, va, v2r[wp0], sa, s2r[wp0]);
            act_apply<RO == 2>(ac, qb, tb, vb, v2r[wp1], sb, s2r[wp1]);
            q = p2(qa, qb);
            t = p2(ta, tb);
          }
        }
        oq = q;
        ot = t;
      }
      Aq[k] = Bq[k];
      Bq[k] = nq;
      At[k] = Bt[k];
      Bt[k] = nt;
      nq = oq;
      nt = ot;
    }
    const int p = s - NC;
    if (p < lo || p >= hi) continue;
    float q0, q1, t0, t1;
    p2u(nq, q0, q1);
    p2u(nt, t0, t1);
    if (LAST) {
      if (cx.readout == 0 || (delta == 0 && r == 0)) {
        cx.acc_q += q0 + q1;
        cx.acc_t += t0 + t1;
      }
    } else {
      float* sq = cx.stage + (2 * buf) * (S * S);
      float* st = sq + S * S;
      sq[c0 * S + wp0] = q0;
      sq[(c0 + 1) * S + wp1] = q1;
      st[c0 * S + wp0] = t0;
      st[(c0 + 1) * S + wp1] = t1;
      __syncthreads();
      constexpr int H = S / 2;
      if (tid < H * H) {
        const int rho = tid / H, kap = tid % H;
        const int j = kap, jp = (kap + rho) & (H - 1);
        const int o0 = (2 * j) * S + 2 * jp, o1 = o0 + S;
        const float vq = (sq[o0] + sq[o0 + 1]) + (sq[o1] + sq[o1 + 1]);
        const float vt = (st[o0] + st[o0 + 1]) + (st[o1] + st[o1 + 1]);
        const int I = p >> 1;
        const int m = ((p + delta) >> 1) - I;
        float* dq = out_slots + (2 * (m & 1)) * (H * H * H) + I * H * H + tid;
        float* dt = dq + H * H * H;
        *dq += vq;
        *dt += vt;
      }
      buf ^= 1;
    }
  }
  __syncthreads();
}

// NCT >= 0: the segment's conv count is known at compile time (one instantiation).
template <int S, bool LAST, int NCT = -1, int RO = 0>
__device__ __forceinline__ void process_pooled_line(ChainCtx& cx, const ntg_chain_t& pg, int ncv,
                                                    int lbase, const float* vmaps,
                                                    const float* in_slots, float* out_slots,
                                                    int m) {
  const float* q = in_slots + (2 * (m & 1)) * (S * S * S);
  const float* t = q + S * S * S;
  if constexpr (NCT >= 0) {
    process_line<S, NCT, false, LAST, RO>(cx, pg, lbase, vmaps, out_slots, m, q, t);
    return;
  }
  switch (ncv) {
    case 0: process_line<S, 0, false, LAST, RO>(cx, pg, lbase, vmaps, out_slots, m, q, t); break;
    case 1: process_line<S, 1, false, LAST, RO>(cx, pg, lbase, vmaps, out_slots, m, q, t); break;
    case 2: process_line<S, 2, false, LAST, RO>(cx, pg, lbase, vmaps, out_slots, m, q, t); break;
    default: process_line<S, 3, false, LAST, RO>(cx, pg, lbase, vmaps, out_slots, m, q, t); break;
  }
}

// Segment sizes 32 -> 16 -> 8 (nseg <= 3); segment 0 has N0 conv layers.
// Pair p of the upper triangle (i <= j) of an n x n grid, row by row.
__device__ __forceinline__ void tri_pair(int64_t p, int64_t n, int64_t& i, int64_t& j) {
  auto start = [&](int64_t r) { return r * n - (r * (r - 1)) / 2; };  // first pair of row r
  const double b = 2.0 * (double)n + 1.0;
  int64_t r = (int64_t)floor((b - sqrt(fmax(b * b - 8.0 * (double)p, 0.0))) * 0.5);
  if (r < 0) r = 0;
  if (r > n - 1) r = n - 1;
  while (r > 0 && start(r) > p) --r;
  while (r + 1 < n && start(r + 1) <= p) ++r;
  i = r;
  j = r + (p - start(r));
}

// NSEG > 0: segment count and conv counts N1, N2 fixed at compile time (the common
// Myrtle shapes), so that only the code this network runs is in the kernel.
template <int N0, int NSEG, int N1, int N2, int RO, int COMP, int KC>
__device__ __forceinline__ void chain_pair(const ntg_chain_t& pg, const float* __restrict__ x1,
                                           const float* __restrict__ x2, int64_t gi, int64_t gj,
                                           const float* __restrict__ var1,
                                           const float* __restrict__ var2,
                                           float* __restrict__ out_q, float* __restrict__ out_t,
                                           int64_t o1, int64_t o2) {
  constexpr int S0 = 32, S1 = 16, S2 = 8;
  extern __shared__ __align__(16) float smem[];
  const int K = pg.channels;
  const int nseg = NSEG > 0 ? NSEG : pg.nseg;

  ChainCtx cx;
  float* img1 = smem;                 // [4][S0*S0]
  float* img2 = img1 + 4 * S0 * S0;
  float* img2s = img2 + 4 * S0 * S0;
  float* p = img2s + 4 * S0 * S0;
  // per-layer variance maps of both samples, segment by segment
  float* vseg[3] = {nullptr, nullptr, nullptr};
  {
    int l = 0;
    for (int sgi = 0; sgi < nseg; ++sgi) {
      const int S = S0 >> sgi;
      vseg[sgi] = p;
      for (int k = 0; k < pg.nconv[sgi]; ++k, ++l) {
        const float* g1 = var1 + gi * pg.var_stride + pg.var_off[l];
        const float* g2 = var2 + gj * pg.var_stride + pg.var_off[l];
        for (int e = threadIdx.x; e < S * S; e += NT) {
          const float a = __ldg(g1 + e), b = __ldg(g2 + e);
          p[e] = a;
          p[S * S + e] = b;
          p[2 * S * S + e] = sqrt_var(a);
          p[3 * S * S + e] = sqrt_var(b);
          if (sgi == 0) {  // shifted copies of the sample-2 maps: [row][j] = [row][j + 1]
            const int row = e / S, col = e % S;
            const float bs = __ldg(g2 + row * S + ((col + 1) & (S - 1)));
            p[4 * S * S + e] = bs;
            p[5 * S * S + e] = sqrt_var(bs);
          }
        }
        p += (sgi == 0 ? 6 : 4) * S * S;
      }
    }
  }
  float* slots1 = p;
  if (nseg > 1) p += 4 * S1 * S1 * S1;
  float* slots2 = p;
  if (nseg > 2) p += 4 * S2 * S2 * S2;
  cx.stage = p;
  p += 4 * S0 * S0;
  float* red = p;  // 2 * NT/32 floats

  // images as channel planes
  const float* im1 = x1 + gi * S0 * S0 * K;
  const float* im2 = x2 + gj * S0 * S0 * K;
  for (int e = threadIdx.x; e < S0 * S0; e += NT) {
    for (int k = 0; k < K; ++k) {
      img1[k * S0 * S0 + e] = __ldg(im1 + e * K + k);
      img2[k * S0 * S0 + e] = __ldg(im2 + e * K + k);
      const int es = (e & ~(S0 - 1)) | ((e + 1) & (S0 - 1));  // same row, next column
      img2s[k * S0 * S0 + e] = __ldg(im2 + es * K + k);
    }
  }
  cx.img1 = img1;
  cx.img2 = img2;
  cx.img2s = img2s;
  cx.K = K;
  cx.inv_k = 1.f / (float)K;
  cx.acc_q = cx.acc_t = 0.f;
  cx.readout = pg.readout;
  __syncthreads();

  const int lb1 = N0;
  const int nc1 = NSEG > 0 ? (NSEG > 1 ? N1 : 0) : (nseg > 1 ? pg.nconv[1] : 0);
  const int nc2 = NSEG > 0 ? (NSEG > 2 ? N2 : 0) : (nseg > 2 ? pg.nconv[2] : 0);
  const int lb2 = lb1 + nc1;
  for (int d0 = -(S0 - 1); d0 <= S0 - 1; ++d0) {
    if (nseg > 1 && (d0 & 1)) {
      const int m = (d0 + 1) / 2;
      if (m <= S1 - 1) {
        float* z = slots1 + (2 * (m & 1)) * (S1 * S1 * S1);
        zero_slot(z, z + S1 * S1 * S1, S1 * S1 * S1);
      }
    }
    if (nseg == 1)
      line_s32<N0, true, RO, COMP, KC>(cx, pg, vseg[0], nullptr, d0);
    else
      line_s32<N0, false, RO, COMP, KC>(cx, pg, vseg[0], slots1, d0);
    if (nseg > 1 && (d0 & 1)) {
      const int m1 = (d0 - 1) / 2;
      if (m1 >= -(S1 - 1)) {
        if (nseg > 2 && (m1 & 1)) {
          const int m = (m1 + 1) / 2;
          if (m <= S2 - 1) {
            float* z = slots2 + (2 * (m & 1)) * (S2 * S2 * S2);
            zero_slot(z, z + S2 * S2 * S2, S2 * S2 * S2);
          }
        }
        if (nseg == 2)
          process_pooled_line<S1, true, NSEG == 2 ? N1 : -1, RO>(cx, pg, nc1, lb1, vseg[1], slots1,
                                                            nullptr, m1);
        else
          process_pooled_line<S1, false, NSEG == 3 ? N1 : -1, RO>(cx, pg, nc1, lb1, vseg[1], slots1,
                                                             slots2, m1);
        if (nseg > 2 && (m1 & 1)) {
          const int m2 = (m1 - 1) / 2;
          if (m2 >= -(S2 - 1))
            process_pooled_line<S2, true, NSEG == 3 ? N2 : -1, RO>(cx, pg, nc2, lb2, vseg[2], slots2,
                                                              nullptr, m2);
        }
      }
    }
  }

  // block reduction of the readout sums
  float aq = cx.acc_q, at = cx.acc_t;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    aq += __shfl_xor_sync(0xffffffffu, aq, o);
    at += __shfl_xor_sync(0xffffffffu, at, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[warp] = aq;
    red[NT / 32 + warp] = at;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float sq = 0.f, st = 0.f;
    for (int w = 0; w < NT / 32; ++w) {
      sq += red[w];
      st += red[NT / 32 + w];
    }
    const int Sl = S0 >> (nseg - 1);
    const float cnt = pg.readout == 0 ? (float)Sl * Sl * Sl * Sl : (float)Sl * Sl;
    out_q[o1] = sq / cnt;
    if (out_t) out_t[o1] = st / cnt;
    if (o2 >= 0) {
      out_q[o2] = sq / cnt;
      if (out_t) out_t[o2] = st / cnt;
    }
  }
}

// One CTA per pair. sym == 0: the pairs (r0 + i, c0 + j) of x1 x x2, result at
// out[i * ld + j] (out points at the tile). sym == 1: the pairs i <= j of the
// square tile of x1 with itself (r0 == c0, n1 == n2); sym == 2: all pairs of a
// tile of x1 with itself whose row and column ranges are disjoint. For sym != 0
// out points at element (0, 0) of the whole kernel and each result is written at
// (gi, gj) and (gj, gi).
template <int N0, int NSEG = 0, int N1 = 0, int N2 = 0, int RO = 0, int COMP = -1,
          int KC = 0>
__global__ void __launch_bounds__(NT, 1)
    chain_fwd_kernel(const __grid_constant__ ntg_chain_t pg, const float* __restrict__ x1,
                     const float* __restrict__ x2, int64_t r0, int64_t n1, int64_t c0,
                     int64_t n2, const float* __restrict__ var1, const float* __restrict__ var2,
                     float* __restrict__ out_q, float* __restrict__ out_t, int64_t ld_out,
                     int sym) {
  const int64_t pair = blockIdx.x;
  int64_t i, j;
  if (sym == 1) {
    tri_pair(pair, n1, i, j);
  } else {
    i = pair / n2;
    j = pair - i * n2;
  }
  const int64_t gi = r0 + i, gj = c0 + j;
  const int64_t o1 = sym ? gi * ld_out + gj : i * ld_out + j;
  const int64_t o2 = (sym && gi != gj) ? gj * ld_out + gi : -1;
  chain_pair<N0, NSEG, N1, N2, RO, COMP, KC>(pg, x1, x2, gi, gj, var1, var2, out_q, out_t,
                                              o1, o2);
}

size_t chain_smem_bytes(const ntg_chain_t& pg) {
  size_t f = 3 * 4 * 32 * 32;  // images (4 channel planes each), image 2 shifted
  for (int sgi = 0; sgi < pg.nseg; ++sgi) {
    size_t S = 32 >> sgi;
    f += (sgi == 0 ? 6 : 4) * S * S * pg.nconv[sgi];
    if (sgi > 0) f += 4 * S * S * S;
  }
  f += 4 * 32 * 32;  // staging
  f += 2 * NT / 32;
  return f * sizeof(float);
}

}  // namespace
}  // namespace ntg

using namespace ntg;

namespace {

template <int N0, int NSEG, int N1, int N2, int RO = 0, int COMP = -1, int KC = 0>
cudaError_t launch_chain_k(unsigned grid, size_t sm, cudaStream_t s, const ntg_chain_t& pg,
                           const float* x1, const float* x2, int64_t r0, int64_t n1, int64_t c0,
                           int64_t n2, const float* var1, const float* var2, float* out_q,
                           float* out_t, int64_t ld_out, int sym) {
  cudaError_t e = cudaFuncSetAttribute(chain_fwd_kernel<N0, NSEG, N1, N2, RO, COMP, KC>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess)
    chain_fwd_kernel<N0, NSEG, N1, N2, RO, COMP, KC><<<grid, NT, sm, s>>>(
        pg, x1, x2, r0, n1, c0, n2, var1, var2, out_q, out_t, ld_out, sym);
  return e;
}

// The Myrtle shapes: segment-specialised kernels, ReLU-family-only variants where they apply.
template <int N0, int N1, int N2>
cudaError_t launch_myrtle(bool relu_only, unsigned grid, size_t sm, cudaStream_t s,
                          const ntg_chain_t& pg, const float* x1, const float* x2, int64_t r0,
                          int64_t n1, int64_t c0, int64_t n2, const float* var1,
                          const float* var2, float* out_q, float* out_t, int64_t ld_out,
                          int sym) {
  if (relu_only) {
    bool comp = false;  // all layers share the precision of one call
    for (int l = 0; l < NTG_CHAIN_MAX_LAYERS; ++l) comp = comp || pg.act[l].compensated != 0;
    // three input channels (images) get their own instantiation
    if (comp)
      return pg.channels == 3
                 ? launch_chain_k<N0, 3, N1, N2, 1, 1, 3>(grid, sm, s, pg, x1, x2, r0, n1,
                                                             c0, n2, var1, var2, out_q, out_t,
                                                             ld_out, sym)
                 : launch_chain_k<N0, 3, N1, N2, 1, 1>(grid, sm, s, pg, x1, x2, r0, n1, c0,
                                                          n2, var1, var2, out_q, out_t, ld_out,
                                                          sym);
    return pg.channels == 3
               ? launch_chain_k<N0, 3, N1, N2, 1, 0, 3>(grid, sm, s, pg, x1, x2, r0, n1, c0,
                                                           n2, var1, var2, out_q, out_t, ld_out,
                                                           sym)
               : launch_chain_k<N0, 3, N1, N2, 1, 0>(grid, sm, s, pg, x1, x2, r0, n1, c0, n2,
                                                        var1, var2, out_q, out_t, ld_out, sym);
  }
  return launch_chain_k<N0, 3, N1, N2, 0>(grid, sm, s, pg, x1, x2, r0, n1, c0, n2, var1,
                                              var2, out_q, out_t, ld_out, sym);
}

int launch_chain(const char* who, void* stream, const ntg_chain_t* prog, const float* x1,
                 const float* x2, int64_t r0, int64_t n1_, int64_t c0, int64_t n2_,
                 const float* var1, const float* var2, float* out_q, float* out_t, int64_t ld_out,
                 int sym) {
  const int64_t n1 = n1_, n2 = n2_;
  const std::string w(who);
  NTG_REQUIRE(prog && x1 && x2 && var1 && var2 && out_q, w + ": null pointer");
  const ntg_chain_t& pg = *prog;
  NTG_REQUIRE(pg.s0 == 32, w + ": the fused chain needs 32x32 inputs");
  NTG_REQUIRE(pg.nseg >= 1 && pg.nseg <= 3, w + ": 1 to 3 segments");
  NTG_REQUIRE(pg.channels >= 1 && pg.channels <= 4, w + ": 1 to 4 input channels");
  NTG_REQUIRE(pg.nconv[0] >= 1 && pg.nconv[0] <= 3, w + ": 1 to 3 convs in segment 0");
  int nl = 0;
  for (int sg = 0; sg < pg.nseg; ++sg) {
    NTG_REQUIRE(pg.nconv[sg] >= 0 && pg.nconv[sg] <= 3, w + ": 0 to 3 convs per segment");
    nl += pg.nconv[sg];
  }
  NTG_REQUIRE(nl <= NTG_CHAIN_MAX_LAYERS, w + ": too many layers");
  bool rare = false;  // Sin / Rbf / Gelu: the instances with every rule compiled in
  for (int l = 0; l < nl; ++l) {
    NTG_REQUIRE(pg.act[l].kind >= NTG_ACT_NONE && pg.act[l].kind <= NTG_ACT_GELU,
                w + ": unknown activation kind");
    rare = rare || pg.act[l].kind >= NTG_ACT_SIN;
  }
  NTG_REQUIRE(pg.readout == 0 || pg.readout == 1, w + ": readout must be 0 or 1");
  NTG_REQUIRE(n1 > 0 && n2 > 0 && r0 >= 0 && c0 >= 0, w + ": bad tile");
  NTG_REQUIRE(sym ? ld_out >= (r0 + n1 > c0 + n2 ? r0 + n1 : c0 + n2) : ld_out >= n2,
              w + ": ld_out smaller than the kernel");
  NTG_REQUIRE(n1 <= (1ll << 24) && n2 <= (1ll << 24), w + ": tile too large");
  const int64_t total = sym == 1 ? n1 * (n1 + 1) / 2 : n1 * n2;
  NTG_REQUIRE(total < (1ll << 31), w + ": too many pairs for one launch");
  const unsigned grid = (unsigned)total;  // one CTA per pair
  size_t sm = chain_smem_bytes(pg);
  NTG_REQUIRE(sm <= 232448, w + ": network needs more shared memory than a CTA has");
  cudaStream_t s = as_stream(stream);
  const int n0 = pg.nconv[0];
  const int c1 = pg.nseg > 1 ? pg.nconv[1] : -1, c2 = pg.nseg > 2 ? pg.nconv[2] : -1;
  cudaError_t e;
  // the Myrtle-5 / -7 / -10 shapes get kernels specialised to their segments
  bool relu_only = true;
  for (int l = 0; l < nl; ++l)
    relu_only = relu_only && (pg.act[l].kind == NTG_ACT_NONE || pg.act[l].kind == NTG_ACT_ABRELU);
  if (rare)
    e = n0 == 1 ? launch_chain_k<1, 0, 0, 0, 2>(grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1,
                                                var2, out_q, out_t, ld_out, sym)
        : n0 == 2 ? launch_chain_k<2, 0, 0, 0, 2>(grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1,
                                                  var2, out_q, out_t, ld_out, sym)
                  : launch_chain_k<3, 0, 0, 0, 2>(grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1,
                                                  var2, out_q, out_t, ld_out, sym);
  else if (pg.nseg == 3 && n0 == 2 && c1 == 1 && c2 == 1)
    e = launch_myrtle<2, 1, 1>(relu_only, grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1, var2,
                               out_q, out_t, ld_out, sym);
  else if (pg.nseg == 3 && n0 == 2 && c1 == 2 && c2 == 2)
    e = launch_myrtle<2, 2, 2>(relu_only, grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1, var2,
                               out_q, out_t, ld_out, sym);
  else if (pg.nseg == 3 && n0 == 3 && c1 == 3 && c2 == 3)
    e = launch_myrtle<3, 3, 3>(relu_only, grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1, var2,
                               out_q, out_t, ld_out, sym);
  else if (n0 == 1)
    e = launch_chain_k<1, 0, 0, 0>(grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1, var2, out_q,
                                   out_t, ld_out, sym);
  else if (n0 == 2)
    e = launch_chain_k<2, 0, 0, 0>(grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1, var2, out_q,
                                   out_t, ld_out, sym);
  else
    e = launch_chain_k<3, 0, 0, 0>(grid, sm, s, pg, x1, x2, r0, n1_, c0, n2_, var1, var2, out_q,
                                   out_t, ld_out, sym);
  if (e != cudaSuccess) return fail(NTG_ERR_CUDA, w + ": " + cudaGetErrorString(e));
  note_launch();
  return check_launch(who);
}

}  // namespace

extern "C" int ntg_chain_fwd(void* stream, const ntg_chain_t* prog, const float* x1,
                             const float* x2, int64_t r0, int64_t n1, int64_t c0, int64_t n2,
                             const float* var1, const float* var2, float* out_q, float* out_t,
                             int64_t ld_out) {
  return launch_chain("ntg_chain_fwd", stream, prog, x1, x2, r0, n1, c0, n2, var1, var2, out_q,
                      out_t, ld_out, 0);
}

extern "C" int ntg_chain_fwd_sym(void* stream, const ntg_chain_t* prog, const float* x,
                                 int64_t r0, int64_t n1, int64_t c0, int64_t n2, const float* var,
                                 float* out_q, float* out_t, int64_t ld_out) {
  int sym;
  if (r0 == c0 && n1 == n2) {
    sym = 1;
  } else if (r0 + n1 <= c0 || c0 + n2 <= r0) {
    sym = 2;
  } else {
    return fail(NTG_ERR_INVALID_ARG,
                "ntg_chain_fwd_sym: the row and column ranges must be equal or disjoint");
  }
  return launch_chain("ntg_chain_fwd_sym", stream, prog, x, x, r0, n1, c0, n2, var, var, out_q,
                      out_t, ld_out, sym);
}
