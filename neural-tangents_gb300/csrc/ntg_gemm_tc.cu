// FP32-accurate GEMM on the sm_103a tensor cores: C = alpha A B^T + beta C with
// A [M, K] and B [N, K] row-major float32 (both K-major), the products split as
// x = hi + lo with hi = tf32(x), lo = tf32(x - hi) and accumulated in FP32 in
// tensor memory as hi_a hi_b + hi_a lo_b + lo_a hi_b (tcgen05.mma kind::tf32;
// about 22 significant bits per operand, the lo lo term being below that).
//
// One CTA per 128 x 128 tile of C. TMA brings 128 x 32 float32 tiles of A and B
// (one 128-byte swizzled row per matrix row) into a 3-stage shared-memory ring;
// four converter warps split each tile in place (hi) and into a second buffer
// (lo) and hand the stage to the MMA thread, which issues 12 MMAs per stage and
// frees it with tcgen05.commit; the converter warps then drain the accumulator
// with tcgen05.ld into the idle ring, from which all warps write C row by row
// (coalesced) with alpha, beta applied. With `lower` set only the tiles on or
// below the diagonal are computed and only entries with col <= row written (the
// symmetric rank-k update of a Cholesky factorisation). Every wait is bounded:
// one that runs out raises the device error word, lets the copies and MMAs in
// flight land (bounded), frees the tensor memory and returns.
#include <mutex>
#include <string>

#include "ntg_tc.cuh"

namespace ntg {
namespace tc {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int make_map_2d(CUtensorMap* m, CUtensorMapDataType dtype, int elem_bytes, const void* base,
                int64_t rows, int64_t cols, int64_t ld, int box_rows, int box_cols,
                const char* who) {
  auto fn = encode_fn();
  if (!fn) return fail(NTG_ERR_CUDA, std::string(who) + ": cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * elem_bytes)};
  cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, dtype, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(NTG_ERR_CUDA, std::string(who) + ": cuTensorMapEncodeTiled failed");
  return NTG_OK;
}

}  // namespace tc

namespace {

constexpr int GM = 128, GN = 128, GK = 32;     // GK float32 = one 128-byte swizzled row
constexpr int GSTAGES = 3;
constexpr int GTILE = GM * GK * 4;             // 16 KB per operand tile
constexpr int GSTAGE = 4 * GTILE;              // A (hi in place), A lo, B (hi in place), B lo
constexpr int GSMEM = GSTAGES * GSTAGE + 1024 + 256;
constexpr int GTHREADS = 192;                  // warp 0 TMA, warp 1 MMA, warps 2-5 split + epilogue
constexpr uint32_t GTMEM_COLS = 128;
constexpr uint64_t GWAIT = 1ull << 21;
constexpr uint32_t GIDESC = tc::idesc(2, GM, GN);  // kind::tf32

__device__ int g_gemm_error = 0;

struct GemmArgs {
  float* c;
  int64_t ldc, m, n, k;
  float alpha, beta;
  int32_t lower;
  int32_t tiles_n;
};

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(GIDESC), "r"(acc));
}

__device__ __forceinline__ float tf32_rn(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// hi = tf32(x) in place, lo = tf32(x - hi) into lo_buf at the same offset, for the
// 16-byte chunks tid, tid + 128, ... of one operand tile (same swizzled layout).
__device__ __forceinline__ void split_tile(uint8_t* tile, uint8_t* lo_buf, int tid) {
#pragma unroll
  for (int i = 0; i < GTILE / 16 / 128; ++i) {
    const int off = (tid + 128 * i) * 16;
    float4 v = *reinterpret_cast<float4*>(tile + off);
    float4 h, l;
    h.x = tf32_rn(v.x); l.x = tf32_rn(v.x - h.x);
    h.y = tf32_rn(v.y); l.y = tf32_rn(v.y - h.y);
    h.z = tf32_rn(v.z); l.z = tf32_rn(v.z - h.z);
    h.w = tf32_rn(v.w); l.w = tf32_rn(v.w - h.w);
    *reinterpret_cast<float4*>(tile + off) = h;
    *reinterpret_cast<float4*>(lo_buf + off) = l;
  }
}

__global__ void __launch_bounds__(GTHREADS, 1)
    gemm_tf32x3_kernel(const __grid_constant__ CUtensorMap ta,
                       const __grid_constant__ CUtensorMap tb, GemmArgs p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GSTAGES * GSTAGE);
  // bars[0, S): TMA landed; [S, 2S): split done; [2S, 3S): stage free; [3S]: accumulator ready
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3 * GSTAGES + 1);
  __shared__ int s_fail;

  int64_t tm, tn;
  if (p.lower) {
    const int64_t idx = blockIdx.x;
    int64_t i = (int64_t)((sqrt(8.0 * (double)idx + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > idx) --i;
    while ((i + 1) * (i + 2) / 2 <= idx) ++i;
    tm = i;
    tn = idx - i * (i + 1) / 2;
  } else {
    tm = blockIdx.x / p.tiles_n;
    tn = blockIdx.x - tm * p.tiles_n;
  }
  const int64_t m0 = tm * GM, n0 = tn * GN;
  const int nk = (int)((p.k + GK - 1) / GK);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GSTAGES; ++s) {
      tc::mbar_init(tc::smem_u32(&bars[s]), 1);
      tc::mbar_init(tc::smem_u32(&bars[GSTAGES + s]), 4);
      tc::mbar_init(tc::smem_u32(&bars[2 * GSTAGES + s]), 1);
    }
    tc::mbar_init(tc::smem_u32(&bars[3 * GSTAGES]), 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::smem_u32(tmem_slot)),
                 "r"(GTMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;
  int issued = 0;
  bool ready = true;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      bool ok = true;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % GSTAGES;
        if (kc >= GSTAGES)
          ok = tc::mbar_wait(tc::smem_u32(&bars[2 * GSTAGES + s]), ((kc / GSTAGES) - 1) & 1, GWAIT);
        if (!ok) break;
        const uint32_t full = tc::smem_u32(&bars[s]);
        uint8_t* st = smem + s * GSTAGE;
        tc::mbar_expect_tx(full, 2 * GTILE);
        tc::tma_load_2d(tc::smem_u32(st), &ta, full, kc * GK, (int32_t)m0);
        tc::tma_load_2d(tc::smem_u32(st + 2 * GTILE), &tb, full, kc * GK, (int32_t)n0);
        issued = kc + 1;
      }
      if (!ok) {
        atomicExch(&g_gemm_error, NTG_ERR_WAIT_TIMEOUT);
        s_fail = 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      bool ok = true;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % GSTAGES;
        ok = tc::mbar_wait(tc::smem_u32(&bars[GSTAGES + s]), (kc / GSTAGES) & 1, GWAIT);
        if (!ok) break;
        tc::fence_after();
        const uint32_t st = tc::smem_u32(smem + s * GSTAGE);
        const uint32_t a_hi = st, a_lo = st + GTILE, b_hi = st + 2 * GTILE,
                       b_lo = st + 3 * GTILE;
#pragma unroll
        for (int kk = 0; kk < GK / 8; ++kk) {
          const uint32_t off = kk * 32;  // 8 float32 along K
          mma_tf32(tmem, tc::smem_desc_sw128(a_hi + off), tc::smem_desc_sw128(b_hi + off),
                   (kc | kk) ? 1u : 0u);
          mma_tf32(tmem, tc::smem_desc_sw128(a_hi + off), tc::smem_desc_sw128(b_lo + off), 1u);
          mma_tf32(tmem, tc::smem_desc_sw128(a_lo + off), tc::smem_desc_sw128(b_hi + off), 1u);
        }
        tc::commit(tc::smem_u32(&bars[2 * GSTAGES + s]));  // frees the stage
      }
      tc::commit(tc::smem_u32(&bars[3 * GSTAGES]));  // accumulator complete (or all issued)
      if (!ok) {
        atomicExch(&g_gemm_error, NTG_ERR_WAIT_TIMEOUT);
        s_fail = 1;
      }
    }
  } else {
    // split warps (2..5): each stage's A and B tiles, then the epilogue
    const int tid = threadIdx.x - 64;
    bool ok = true;
    for (int kc = 0; kc < nk; ++kc) {
      const int s = kc % GSTAGES;
      ok = tc::mbar_wait(tc::smem_u32(&bars[s]), (kc / GSTAGES) & 1, GWAIT);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      uint8_t* st = smem + s * GSTAGE;
      split_tile(st, st + GTILE, tid);
      split_tile(st + 2 * GTILE, st + 3 * GTILE, tid);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tc::smem_u32(&bars[GSTAGES + s]));
    }
    if (!ok && lane == 0) {
      atomicExch(&g_gemm_error, NTG_ERR_WAIT_TIMEOUT);
      s_fail = 1;
    }
    ready = tc::mbar_wait(tc::smem_u32(&bars[3 * GSTAGES]), 0, GWAIT);
    ready = __all_sync(0xffffffffu, ready);
    if (!ready && lane == 0) {
      atomicExch(&g_gemm_error, NTG_ERR_WAIT_TIMEOUT);
      s_fail = 1;
    }
  }

  // Epilogue through shared memory: the split warps move the accumulator from TMEM into
  // the (now idle) stage buffers, then all six warps write C row by row, coalesced.
  tc::fence_before();
  __syncthreads();
  const bool acc_ok = !s_fail;
  float* stile = reinterpret_cast<float*>(smem);  // [128][129] floats, 66 KB of the ring
  constexpr int SP = GN + 1;
  if (acc_ok && warp >= 2) {
    tc::fence_after();
    const int q = warp & 3;
#pragma unroll 1
    for (int c0 = 0; c0 < GN; c0 += 32) {
      uint32_t v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
      float* dst = stile + (q * 32 + lane) * SP + c0;
#pragma unroll
      for (int j = 0; j < 32; ++j) dst[j] = __uint_as_float(v[j]);
    }
  }
  __syncthreads();
  if (acc_ok) {
    // groups of 4 columns; four groups per thread in flight (the read of C for beta != 0
    // is latency-bound otherwise); whole groups move as float4 when C allows it
    const bool vec = ((p.ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(p.c) & 15) == 0);
    constexpr int G = GM * GN / 4, GPR = GN / 4;
    for (int g0 = threadIdx.x; g0 < G; g0 += 4 * GTHREADS) {
      float4 cv[4];
      bool whole[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int g = g0 + u * GTHREADS;
        const int r = g / GPR, c4 = (g % GPR) * 4;
        const int64_t row = m0 + r, col = n0 + c4;
        whole[u] = g < G && vec && row < p.m && col + 3 < p.n && (!p.lower || col + 3 <= row);
        cv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (whole[u] && p.beta != 0.f)
          cv[u] = *reinterpret_cast<const float4*>(p.c + row * p.ldc + col);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int g = g0 + u * GTHREADS;
        if (g >= G) continue;
        const int r = g / GPR, c4 = (g % GPR) * 4;
        const int64_t row = m0 + r, col = n0 + c4;
        const float* sv = stile + r * SP + c4;
        if (whole[u]) {
          float4 o;
          o.x = fmaf(p.beta, cv[u].x, p.alpha * sv[0]);
          o.y = fmaf(p.beta, cv[u].y, p.alpha * sv[1]);
          o.z = fmaf(p.beta, cv[u].z, p.alpha * sv[2]);
          o.w = fmaf(p.beta, cv[u].w, p.alpha * sv[3]);
          *reinterpret_cast<float4*>(p.c + row * p.ldc + col) = o;
        } else if (row < p.m) {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int64_t cl = col + e;
            if (cl < p.n && (!p.lower || cl <= row)) {
              float* cp = p.c + row * p.ldc + cl;
              float val = p.alpha * sv[e];
              if (p.beta != 0.f) val = fmaf(p.beta, *cp, val);
              *cp = val;
            }
          }
        }
      }
    }
  }
  tc::fence_before();
  __syncthreads();
  if (s_fail) {
    // a wait ran out: let the TMA loads still in flight land (the last use of each
    // stage) and the issued MMAs finish (their final commit), both bounded, before
    // the shared and tensor memory are released
    if (warp == 0 && lane == 0)
      for (int kc = issued > GSTAGES ? issued - GSTAGES : 0; kc < issued; ++kc)
        tc::mbar_wait(tc::smem_u32(&bars[kc % GSTAGES]), (kc / GSTAGES) & 1, GWAIT);
    if (warp == 1 && lane == 0) tc::mbar_wait(tc::smem_u32(&bars[3 * GSTAGES]), 0, GWAIT);
    __syncthreads();
  }
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(GTMEM_COLS));
}

}  // namespace

int gemm_take_device_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_gemm_error, sizeof(int)) != cudaSuccess) return -1;
  const int zero = 0;
  if (v != 0 && cudaMemcpyToSymbol(g_gemm_error, &zero, sizeof(int)) != cudaSuccess) return -1;
  return v;
}

int gemm_tf32x3(cudaStream_t s, const float* a, int64_t lda, const float* b, int64_t ldb,
                float* c, int64_t ldc, int64_t m, int64_t n, int64_t k, float alpha, float beta,
                int lower) {
  NTG_REQUIRE(a && b && c, "ntg_gemm_tc: null pointer");
  NTG_REQUIRE(m > 0 && n > 0 && k > 0, "ntg_gemm_tc: sizes must be positive");
  NTG_REQUIRE(lda >= k && ldb >= k && ldc >= n, "ntg_gemm_tc: leading dimensions too small");
  NTG_REQUIRE(lda % 4 == 0 && ldb % 4 == 0,
              "ntg_gemm_tc: lda and ldb must be multiples of 4 (16-byte rows for TMA)");
  NTG_REQUIRE((reinterpret_cast<uintptr_t>(a) & 15) == 0 && (reinterpret_cast<uintptr_t>(b) & 15) == 0,
              "ntg_gemm_tc: A and B must be 16-byte aligned");
  NTG_REQUIRE(!lower || m == n, "ntg_gemm_tc: the lower-triangle update needs m == n");
  NTG_REQUIRE(m <= (1ll << 31) - GM && n <= (1ll << 31) - GN && k <= (1ll << 31) - GK,
              "ntg_gemm_tc: sizes too large");
  const int64_t tm = ceil_div(m, GM), tn = ceil_div(n, GN);
  const int64_t tiles = lower ? tm * (tm + 1) / 2 : tm * tn;
  NTG_REQUIRE(tiles <= (1ll << 31) - 1, "ntg_gemm_tc: too many tiles");
  CUtensorMap ma, mb;
  int rc = tc::make_map_2d(&ma, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a, m, k, lda, GM, GK,
                           "ntg_gemm_tc");
  if (rc) return rc;
  rc = tc::make_map_2d(&mb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b, n, k, ldb, GN, GK,
                       "ntg_gemm_tc");
  if (rc) return rc;
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(gemm_tf32x3_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, GSMEM);
  });
  if (attr_err != cudaSuccess)
    return fail(NTG_ERR_CUDA, std::string("ntg_gemm_tc: ") + cudaGetErrorString(attr_err));
  GemmArgs p{c, ldc, m, n, k, alpha, beta, lower, (int32_t)tn};
  gemm_tf32x3_kernel<<<(unsigned)tiles, GTHREADS, GSMEM, s>>>(ma, mb, p);
  note_launch();
  return check_launch("ntg_gemm_tc");
}

}  // namespace ntg

extern "C" int ntg_gemm_tc(void* stream, const float* a, int64_t lda, const float* b,
                           int64_t ldb, float* c, int64_t ldc, int64_t m, int64_t n, int64_t k,
                           float alpha, float beta, int32_t lower) {
  return ntg::gemm_tf32x3(ntg::as_stream(stream), a, lda, b, ldb, c, ldc, m, n, k, alpha, beta,
                          lower);
}
