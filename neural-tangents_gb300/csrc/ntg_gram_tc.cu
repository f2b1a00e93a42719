// Split-precision Gram x1 x2^T / D on the sm_103a tensor cores (tcgen05).
//
// Each float32 input is split into bf16 hi = bf16(x) and lo = bf16(x - hi);
// x1 x2^T ~ hi1 hi2^T + hi1 lo2^T + lo1 hi2^T, the three products accumulated
// in FP32 in tensor memory (the lo lo^T term is below float32 resolution of
// the sum). For x1 == x2 only the tiles on or below the diagonal are computed and
// the output is mirrored, so that it is exactly symmetric. Tiles: 128 x 128 outputs per CTA, K chunks of 64 bf16 (one 128-byte
// swizzled row) moved by TMA into a 3-stage shared-memory ring; one thread
// issues tcgen05.mma (M=128, N=128, K=16) and tcgen05.commit frees each stage;
// four warps drain the accumulator with tcgen05.ld. Every mbarrier wait is
// bounded: a wait that runs out sets the error words (the workspace word and
// the library's device word read by ntg_device_status), waits (bounded) for the
// copies and MMAs already issued, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <mutex>
#include <string>

#include "ntg_tc.cuh"

namespace ntg {
namespace {

constexpr int BM = 128, BN = 256, BK = 64;
constexpr int STAGES = 2;
constexpr int A_BYTES = BM * BK * 2;              // an A operand tile: 16 KB
constexpr int B_BYTES = BN * BK * 2;              // a B operand tile: 32 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // A_hi, A_lo, B_hi, B_lo: 96 KB
constexpr uint32_t TMEM_COLS = BN;
constexpr uint64_t WAIT_LIMIT = 1ull << 20;   // about a second of polling

__device__ int g_gram_error = 0;

// hi = bf16(x), lo = bf16(x - hi) for x [n, d] into [npad, dpad] (zero padding), eight
// consecutive entries of a row per thread: two 16-byte loads (when rows are 16-byte
// aligned) and one 16-byte store into each of hi and lo.
__global__ void split_bf16_kernel(const float* __restrict__ x, int64_t n, int64_t d,
                                  int64_t npad, int64_t dpad, __nv_bfloat16* __restrict__ hi,
                                  __nv_bfloat16* __restrict__ lo) {
  const int64_t groups = dpad / 8, total = npad * groups;
  const bool vec = (d & 3) == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / groups, c = (idx - r * groups) * 8;
    float v[8];
    if (r < n && vec && c + 8 <= d) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(x + r * d + c));
      const float4 b = __ldg(reinterpret_cast<const float4*>(x + r * d + c + 4));
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
      v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = (r < n && c + u < d) ? __ldg(x + r * d + c + u) : 0.f;
    }
    __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      h[u] = __float2bfloat16_rn(v[u]);
      l[u] = __float2bfloat16_rn(v[u] - __bfloat162float(h[u]));
    }
    *reinterpret_cast<uint4*>(hi + r * dpad + c) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(lo + r * dpad + c) = *reinterpret_cast<const uint4*>(l);
  }
}

using tc::commit;
using tc::mbar_expect_tx;
using tc::mbar_init;
using tc::smem_u32;
using tc::tma_load_2d;

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  return tc::mbar_wait(bar, parity, WAIT_LIMIT);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) { return tc::smem_desc_sw128(addr); }

// Instruction descriptor, kind::f16: D F32, A/B BF16, both K-major, M=128, N=128.
constexpr uint32_t IDESC = tc::idesc(1, BM, BN);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) { commit(bar); }

constexpr int kThreads = 192;            // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr uint32_t TMEM_ALLOC = 2 * TMEM_COLS;  // two accumulators
constexpr int STG_FLOATS = 4 * 32 * 33;  // each epilogue warp's 32 x 32 staging block
constexpr int P_SMEM_BYTES = STAGES * STAGE_BYTES + STG_FLOATS * 4 + 1024 + 256;

// Output tile t of the schedule (128-row x 256-column tiles): with sym (x1 == x2) t
// enumerates, row tile by row tile, the column tiles j <= i / 2 that reach the diagonal
// or below it (row tile i has i / 2 + 1 of them: S(2a) = a (a + 1) and S(2a + 1) =
// (a + 1)^2 tiles precede row tiles 2a and 2a + 1), else the nbn-wide grid row by row.
__device__ __forceinline__ void tile_of(int64_t t, int sym, int64_t nbn, int64_t& ti,
                                        int64_t& tj) {
  if (sym) {
    int64_t a = (int64_t)((sqrt(4.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (a * (a + 1) > t) --a;
    while ((a + 1) * (a + 2) <= t) ++a;
    if (t >= (a + 1) * (a + 1)) {
      ti = 2 * a + 1;
      tj = t - (a + 1) * (a + 1);
    } else {
      ti = 2 * a;
      tj = t - a * (a + 1);
    }
  } else {
    ti = t / nbn;
    tj = t - ti * nbn;
  }
}

// Persistent: CTA c computes the tiles c, c + gridDim.x, ... of the schedule. The TMA
// producer and the MMA issuer run through the tiles' K chunks in one continuous ring; the
// MMAs of a tile go to one of two TMEM accumulators while the four epilogue warps drain
// the other (tcgen05.ld -> shared-memory staging -> row-coalesced stores), so that a tile's
// epilogue overlaps the next tile's MMAs. With sym each off-diagonal tile is also written
// transposed: the entries on or below the diagonal are stored directly and those strictly
// below it also at their mirrored position, so that the output is exactly symmetric.
__global__ void __launch_bounds__(kThreads, 1)
    gram_tc_kernel(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                   const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo,
                   float* __restrict__ out, int64_t n1, int64_t n2, int64_t dpad, float inv_d,
                   int sym, int64_t ntiles, int64_t nbn, int* err) {
  extern __shared__ uint8_t smem_raw[];
  // 1024-byte alignment for the swizzled tiles
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  float* stg_all = reinterpret_cast<float*>(smem + STAGES * STAGE_BYTES);
  uint64_t* bars = reinterpret_cast<uint64_t*>(stg_all + STG_FLOATS);
  // bars[0..S) full, [S..2S) empty, 2S + b: accumulator b full, 2S + 2 + b: accumulator b
  // drained, 2S + 4: all MMAs retired
  uint64_t* tfull = bars + 2 * STAGES;
  uint64_t* tempty = bars + 2 * STAGES + 2;
  uint64_t* drain = bars + 2 * STAGES + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 5);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (int)(dpad / BK);

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[STAGES + s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), 4);  // one arrival per epilogue warp
    }
    mbar_init(smem_u32(drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_ALLOC));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tmem_slot;
  int64_t issued = 0;  // K chunks whose TMA loads the producer issued

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      bool ok = true;
      int64_t g = 0;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        int64_t ti, tj;
        tile_of(t, sym, nbn, ti, tj);
        for (int kc = 0; kc < nk; ++kc, ++g) {
          const int s = (int)(g % STAGES);
          if (g >= STAGES && !(ok = mbar_wait(smem_u32(&bars[STAGES + s]),
                                              (uint32_t)(((g / STAGES) - 1) & 1))))
            break;
          const uint32_t full = smem_u32(&bars[s]);
          uint8_t* st = smem + s * STAGE_BYTES;
          mbar_expect_tx(full, STAGE_BYTES);
          const int32_t x = kc * BK;
          tma_load_2d(smem_u32(st), &ta_hi, full, x, (int32_t)(ti * BM));
          tma_load_2d(smem_u32(st + A_BYTES), &ta_lo, full, x, (int32_t)(ti * BM));
          tma_load_2d(smem_u32(st + 2 * A_BYTES), &tb_hi, full, x, (int32_t)(tj * BN));
          tma_load_2d(smem_u32(st + 2 * A_BYTES + B_BYTES), &tb_lo, full, x, (int32_t)(tj * BN));
          issued = g + 1;
        }
      }
      if (!ok) {
        atomicExch(err, 1);
        atomicExch(&g_gram_error, NTG_ERR_WAIT_TIMEOUT);
        s_fail = 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      bool ok = true;
      int64_t g = 0;
      int it = 0;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
        const int b = it & 1;
        // the accumulator's previous tile has been drained (its first use passes at once)
        if (!(ok = mbar_wait(smem_u32(&tempty[b]), (uint32_t)(((it >> 1) & 1) ^ 1)))) break;
        tc::fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * TMEM_COLS);
        for (int kc = 0; kc < nk; ++kc, ++g) {
          const int s = (int)(g % STAGES);
          if (!(ok = mbar_wait(smem_u32(&bars[s]), (uint32_t)((g / STAGES) & 1)))) break;
          tc::fence_after();
          const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
          const uint32_t a_hi = st, a_lo = st + A_BYTES, b_hi = st + 2 * A_BYTES,
                         b_lo = st + 2 * A_BYTES + B_BYTES;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 along K
            mma_bf16(acc, smem_desc(a_hi + off), smem_desc(b_hi + off), (kc | kk) ? 1u : 0u);
            mma_bf16(acc, smem_desc(a_hi + off), smem_desc(b_lo + off), 1u);
            mma_bf16(acc, smem_desc(a_lo + off), smem_desc(b_hi + off), 1u);
          }
          mma_commit(smem_u32(&bars[STAGES + s]));  // frees the stage once these MMAs finish
        }
        if (!ok) break;
        mma_commit(smem_u32(&tfull[b]));  // the tile's accumulator is complete
      }
      mma_commit(smem_u32(drain));  // every MMA issued, retired before TMEM is freed
      if (!ok) {
        atomicExch(err, 2);
        atomicExch(&g_gram_error, NTG_ERR_WAIT_TIMEOUT);
        s_fail = 1;
      }
    }
  } else {  // epilogue: warp w drains TMEM lanes 32 (w % 4) .. + 31 (rows of the tile)
    const int rq = warp & 3;
    float* stg = stg_all + (warp - 2) * 32 * 33;
    int it = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
      const int b = it & 1;
      if (!mbar_wait(smem_u32(&tfull[b]), (uint32_t)((it >> 1) & 1))) {
        if (lane == 0) {
          atomicExch(err, 3);
          atomicExch(&g_gram_error, NTG_ERR_WAIT_TIMEOUT);
          s_fail = 1;
        }
        break;
      }
      tc::fence_after();
      int64_t ti, tj;
      tile_of(t, sym, nbn, ti, tj);
      const int64_t m0 = ti * BM, n0 = tj * BN;
      const int64_t rbase = m0 + rq * 32;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(rq * 32) << 16) + (uint32_t)(b * TMEM_COLS + c0), v);
        // lane = row rbase + lane of the tile, v[j] = column n0 + c0 + j
#pragma unroll
        for (int j = 0; j < 32; ++j) stg[lane * 33 + j] = __uint_as_float(v[j]) * inv_d;
        __syncwarp();
        const int64_t col = n0 + c0 + lane;
        if (col < n2) {
#pragma unroll 4
          for (int rr = 0; rr < 32; ++rr)
            if (rbase + rr < n1 && (!sym || col <= rbase + rr))
              out[(rbase + rr) * n2 + col] = stg[rr * 33 + lane];
        }
        if (sym && rbase + lane < n1) {  // out[n0 + c0 + j][rbase + lane] = tile[lane][j]
#pragma unroll 4
          for (int j = 0; j < 32; ++j)
            if (n0 + c0 + j < rbase + lane)  // strictly below the diagonal (and < n1)
              out[(n0 + c0 + j) * n2 + rbase + lane] = stg[lane * 33 + j];
        }
        __syncwarp();
      }
      tc::fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(smem_u32(&tempty[b]));
    }
  }
  __syncthreads();
  if (warp == 1 && lane == 0) mbar_wait(smem_u32(drain), 0);  // bounded
  if (s_fail && warp == 0 && lane == 0) {
    // a wait ran out: let the TMA loads still in flight land (the last use of each stage;
    // bounded) before the shared memory is released
    for (int64_t g = issued > STAGES ? issued - STAGES : 0; g < issued; ++g)
      mbar_wait(smem_u32(&bars[g % STAGES]), (uint32_t)((g / STAGES) & 1));
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_ALLOC));
  }
}

int make_map(CUtensorMap* m, const void* base, int64_t rows, int64_t dpad, int box_rows) {
  return tc::make_map_2d(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, rows, dpad, dpad,
                         box_rows, BK, "ntg_gram");
}

}  // namespace

int gram_take_device_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_gram_error, sizeof(int)) != cudaSuccess) return -1;
  const int zero = 0;
  if (v != 0 && cudaMemcpyToSymbol(g_gram_error, &zero, sizeof(int)) != cudaSuccess) return -1;
  return v;
}

size_t gram_tc_workspace(int64_t n1, int64_t n2, int64_t d) {
  const int64_t dpad = ceil_div(d, BK) * BK;
  const int64_t p1 = ceil_div(n1, BM) * BM, p2 = ceil_div(n2, BN) * BN;
  return (size_t)(2 * (p1 + p2) * dpad) * sizeof(__nv_bfloat16) + 256 + 256;
}

int gram_tc(cudaStream_t s, const float* x1, const float* x2, int64_t n1, int64_t n2, int64_t d,
            float* out, void* workspace, size_t ws_bytes) {
  NTG_REQUIRE(workspace && ws_bytes >= gram_tc_workspace(n1, n2, d),
              "ntg_gram: precision 1 needs ntg_gram_workspace_bytes(n1, n2, d) of workspace");
  NTG_REQUIRE(ceil_div(n1, BM) <= 65535, "ntg_gram: n1 too large");
  const int64_t dpad = ceil_div(d, BK) * BK;
  const int64_t p1 = ceil_div(n1, BM) * BM, p2 = ceil_div(n2, BN) * BN;
  uint8_t* ws = static_cast<uint8_t*>(workspace);
  int* err = reinterpret_cast<int*>(ws);
  __nv_bfloat16* a_hi = reinterpret_cast<__nv_bfloat16*>(ws + 256);
  __nv_bfloat16* a_lo = a_hi + p1 * dpad;
  __nv_bfloat16* b_hi = a_lo + p1 * dpad;
  __nv_bfloat16* b_lo = b_hi + p2 * dpad;
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return check_launch("ntg_gram memset");
  // x1 == x2: one split, the lower triangle of tiles, mirrored (the result exactly symmetric)
  const bool sym = x1 == x2 && n1 == n2;
  auto grid = [](int64_t n) { return (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 32); };
  split_bf16_kernel<<<grid(p1 * dpad / 8), 256, 0, s>>>(x1, n1, d, p1, dpad, a_hi, a_lo);
  note_launch();
  if (!sym) {
    split_bf16_kernel<<<grid(p2 * dpad / 8), 256, 0, s>>>(x2, n2, d, p2, dpad, b_hi, b_lo);
    note_launch();
  } else {
    b_hi = a_hi;
    b_lo = a_lo;
  }
  CUtensorMap m[4];
  int rc;
  // B tiles are 256 rows: for sym the A buffers (rows padded to 128) serve as B, the rows
  // beyond them read as zero
  const int64_t brows = sym ? p1 : p2;
  if ((rc = make_map(&m[0], a_hi, p1, dpad, BM)) || (rc = make_map(&m[1], a_lo, p1, dpad, BM)) ||
      (rc = make_map(&m[2], b_hi, brows, dpad, BN)) || (rc = make_map(&m[3], b_lo, brows, dpad, BN)))
    return rc;
  static std::once_flag attr_once;
  static cudaError_t attr_err = cudaSuccess;
  static int num_sms = 0;
  std::call_once(attr_once, [] {
    attr_err = cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    P_SMEM_BYTES);
    int dev = 0;
    if (attr_err == cudaSuccess) attr_err = cudaGetDevice(&dev);
    if (attr_err == cudaSuccess)
      attr_err = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  });
  if (attr_err != cudaSuccess)
    return fail(NTG_ERR_CUDA, std::string("ntg_gram: ") + cudaGetErrorString(attr_err));
  const int64_t nb1 = p1 / BM, nbn = p2 / BN;
  // sym: S(nb1) tiles, S(2a) = a (a + 1), S(2a + 1) = (a + 1)^2
  const int64_t ha = nb1 / 2;
  const int64_t ntiles = sym ? ((nb1 & 1) ? (ha + 1) * (ha + 1) : ha * (ha + 1)) : nb1 * nbn;
  const unsigned ctas = (unsigned)std::min<int64_t>(ntiles, num_sms > 0 ? num_sms : 148);
  gram_tc_kernel<<<ctas, kThreads, P_SMEM_BYTES, s>>>(m[0], m[1], m[2], m[3], out, n1, n2, dpad,
                                                      1.f / (float)d, sym ? 1 : 0, ntiles, nbn,
                                                      err);
  note_launch();
  return check_launch("ntg_gram (tcgen05)");
}

}  // namespace ntg
