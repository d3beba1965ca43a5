// tcgen05 GEMM for 16-bit operands (F16 or BF16) with FP32 accumulation in tensor memory.
//
// D (M x N) = A' B with A stored K x M and B stored K x N, both column-major, i.e. both operands
// K-contiguous ("TN").  This is the shape of every large contraction on the path:
//   * A'U and the Gram products V'V, V'(AV)        (A, V column-major, K = rows),
//   * A V through a one-time transposed copy of the fixed operator A.
// Structure (one 128 x BN output tile per CTA, optional split over K):
//   warp 0      TMA producer: 128-byte-swizzled tiles of A and B into a STAGES-deep ring;
//   warp 1      allocates TMEM and issues tcgen05.mma (M=128, N=BN, K=16) from one elected lane,
//               committing each stage back to the producer through an mbarrier;
//   warps 2..5  epilogue: tcgen05.ld of the FP32 accumulator, conversion, coalesced stores
//               (or FP32 partials when K is split; a fixed-order reduction then sums them).
// Every mbarrier wait is bounded by a ~2 s timer; on timeout the kernel records an error word,
// drains and returns, so a fault in the pipeline cannot hang the GPU.
#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "ofrr_internal.cuh"
#include "tcgen05.cuh"

namespace ofrr {
namespace tc {

constexpr int STAGES = 4;
constexpr int THREADS = 192;

template <int BN>
struct Smem {
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int TOTAL = STAGES * STAGE + 1024 /*align*/ + 256 /*barriers*/;
};

template <int BN, class TOUT>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
              int kblocks_total, int kblocks_per_split, uint32_t idesc, TOUT* __restrict__ D, int64_t ldd,
              float* __restrict__ partial, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base;
  uint8_t* sB = base + STAGES * Smem<BN>::A_BYTES;
  uint64_t* bars = (uint64_t*)(base + STAGES * Smem<BN>::STAGE);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* accum = bars + 2 * STAGES;
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int kb0 = blockIdx.z * kblocks_per_split;
  const int kb1 = min(kb0 + kblocks_per_split, kblocks_total);
  const int nkb = max(kb1 - kb0, 0);
  constexpr uint32_t TMEM_COLS = (BN < 32) ? 32 : BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        if (i >= STAGES && !mbar_wait(&empty[s], ((i / STAGES) + 1) & 1, err, 11)) break;
        mbar_expect_tx(&full[s], Smem<BN>::STAGE);
        const int kx = (kb0 + i) * BK;
        tma_load_2d(&tmA, &full[s], sA + s * Smem<BN>::A_BYTES, kx, m0);
        tma_load_2d(&tmB, &full[s], sB + s * Smem<BN>::B_BYTES, kx, n0);
        issued = i + 1;
      }
      // drain: every issued stage must have landed before the CTA may exit
      for (int i = max(0, issued - STAGES); i < issued; ++i) mbar_wait(&full[i % STAGES], (i / STAGES) & 1, err, 12);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        if (!mbar_wait(&full[s], (i / STAGES) & 1, err, 13)) break;
        fence_after();
        const uint32_t a0 = smem_u32(sA + s * Smem<BN>::A_BYTES);
        const uint32_t b0 = smem_u32(sB + s * Smem<BN>::B_BYTES);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          umma_f16(tmem, desc_sw128(a0 + 32 * k), desc_sw128(b0 + 32 * k), idesc, (i > 0 || k > 0) ? 1u : 0u);
        }
        umma_commit(&empty[s]);
      }
      umma_commit(accum);
    }
    __syncwarp();
  } else {
    // epilogue warps 2..5 -> TMEM lane quarter (warp % 4)
    const int q = warp & 3;
    const bool ok = mbar_wait(accum, 0, err, 14);
    fence_after();
    const int row = m0 + 32 * q + lane;
    const bool split = (partial != nullptr);
#pragma unroll 1
    for (int c = 0; c < BN; c += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c, v);
      if (!ok || nkb == 0) {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0.f;
      }
      if (row < M) {
        if (split) {
          float* P = partial + (size_t)blockIdx.z * (size_t)M * N;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c + j;
            if (n < N) P[row + (size_t)n * M] = v[j];
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c + j;
            if (n < N) D[row + (size_t)n * ldd] = cvt_out<TOUT>(v[j]);
          }
        }
      }
    }
    fence_before();
  }
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// Fixed-order sum of the K-split partials (deterministic).  WIDE (many splits): loads issued eight at
// a time; otherwise the plain loop, whose low register count keeps more loads resident.
template <class TOUT, bool WIDE>
__global__ void k_splitk_reduce(int M, int N, int splits, const float* __restrict__ partial, TOUT* __restrict__ D,
                                int64_t ldd) {
  const int64_t total = (int64_t)M * N;
  OFRR_FOR_2D(m, n, M, N) {
    const int64_t e = m + n * (int64_t)M;
    float s = 0.f;
    int z = 0;
    if (WIDE) {
      for (; z + 8 <= splits; z += 8) {
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = partial[(size_t)(z + u) * total + e];
#pragma unroll
        for (int u = 0; u < 8; ++u) s += v[u];
      }
    }
    for (; z < splits; ++z) s += partial[(size_t)z * total + e];
    D[m + n * ldd] = cvt_out<TOUT>(s);
  }
}

// ---- host side ------------------------------------------------------------------------
template <int BN, class TOUT>
static int launch(ofrr_ctx* ctx, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, ofrr_dtype t16,
                  TOUT* D, int64_t ldd, int splits) {
  const int kbt = (K + BK - 1) / BK;
  const int kbps = (kbt + splits - 1) / splits;
  splits = (kbt + kbps - 1) / kbps;
  const int gm = (M + BM - 1) / BM, gn = (N + BN - 1) / BN;
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  float* partial = nullptr;
  if (splits > 1) {
    partial = ws_get<float>(ctx, (size_t)splits * M * N, &st);
    if (!partial) return st;
  }
  const size_t smem = Smem<BN>::TOTAL;
  static std::atomic<bool> attr_set{false};
  if (!attr_set) {
    OFRR_TRY(allow_smem(k_gemm_tn<BN, TOUT>));
    attr_set = true;
  }
  dim3 grid(gm, gn, splits);
  k_gemm_tn<BN, TOUT><<<grid, THREADS, smem, ctx->stream>>>(ma, mb, M, N, kbt, kbps, make_idesc(t16, BN), D, ldd,
                                                            partial, ctx->dev_flags + kFlagTcWait);
  OFRR_LAUNCHED(ctx, "k_gemm_tn");
  if (splits > 1) {
    if (splits >= 12)
      k_splitk_reduce<TOUT, true><<<grid_2d(M, N, 256), 256, 0, ctx->stream>>>(M, N, splits, partial, D, ldd);
    else
      k_splitk_reduce<TOUT, false><<<grid_2d(M, N, 256), 256, 0, ctx->stream>>>(M, N, splits, partial, D, ldd);
    OFRR_LAUNCHED(ctx, "k_splitk_reduce");
  }
  return OFRR_SUCCESS;
}

}  // namespace tc

// Route a 16-bit TN product to the tcgen05 kernel when its layout allows TMA (16-byte aligned
// base and leading dimensions); *handled = false leaves the call to the caller's fallback.
int gemm_tc_try(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype t16, int64_t M, int64_t N, int64_t K,
                const void* A, int64_t lda, const void* B, int64_t ldb, ofrr_dtype tout, void* C, int64_t ldc,
                bool* handled) {
  *handled = false;
  if (!(transA == 1 && transB == 0)) return OFRR_SUCCESS;
  if (K < 16 || M < 1 || N < 1 || M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) return OFRR_SUCCESS;
  if (((uintptr_t)A & 15) || ((uintptr_t)B & 15) || ((lda * 2) & 15) || ((ldb * 2) & 15)) return OFRR_SUCCESS;
  if (getenv("OFRR_DISABLE_TC")) return OFRR_SUCCESS;
  const int BN = (N <= 32) ? 32 : (N <= 64 ? 64 : 128);
  CUtensorMap ma, mb;
  if (!tc::make_map(&ma, t16, A, K, M, lda, tc::BM)) return OFRR_SUCCESS;
  if (!tc::make_map(&mb, t16, B, K, N, ldb, BN)) return OFRR_SUCCESS;
  // enough CTAs to cover the SMs: split K when the output grid is small
  const int tiles = (int)(((M + tc::BM - 1) / tc::BM) * ((N + BN - 1) / BN));
  const int kbt = (int)((K + tc::BK - 1) / tc::BK);
  int splits = 1;
  while (tiles * splits < 148 && splits * 2 <= kbt && splits < 64) splits *= 2;
  if (const char* e = getenv("OFRR_TC_SPLITS")) splits = std::max(1, std::min(atoi(e), kbt));  // tuning override
  int st = OFRR_SUCCESS;
  OFRR_DISPATCH_STORAGE(tout, TO, {
    if (BN == 32) st = tc::launch<32, TO>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (TO*)C, ldc, splits);
    else if (BN == 64) st = tc::launch<64, TO>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (TO*)C, ldc, splits);
    else st = tc::launch<128, TO>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (TO*)C, ldc, splits);
  });
  if (st != OFRR_SUCCESS) return st;
  *handled = true;
  return OFRR_SUCCESS;
}

}  // namespace ofrr
