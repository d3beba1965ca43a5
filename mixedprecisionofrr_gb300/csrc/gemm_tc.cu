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
#include <cuda_fp8.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <type_traits>

#include "ofrr_internal.cuh"
#include "tcgen05.cuh"

#include <mutex>

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

// F8: E4M3 operands (kind::f8f6f4, 128-element K blocks of the same 128 bytes), the FP32 result scaled by
// sa[row] sb[col] (powers of two, so the scaling is exact and commutes with the split-K sum)
template <int BN, class TOUT, bool F8 = false>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
              int kblocks_total, int kblocks_per_split, uint32_t idesc, TOUT* __restrict__ D, int64_t ldd,
              float* __restrict__ partial, int* __restrict__ err, const float* __restrict__ sa = nullptr,
              const float* __restrict__ sb = nullptr) {
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
        const int kx = (kb0 + i) * (F8 ? 2 * BK : BK);
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
          if (F8)
            umma_f8(tmem, desc_sw128(a0 + 32 * k), desc_sw128(b0 + 32 * k), idesc, (i > 0 || k > 0) ? 1u : 0u);
          else
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
      if (F8 && row < M) {
        const float ra = sa[row];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c + j;
          v[j] *= ra * ((n < N) ? sb[n] : 0.f);
        }
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

// The split-K reduction fused with scalecols (16-bit storage TO, FP32 compute) for a product the power
// iteration scales at once (subspace_iter_svd.m:63-69): each CTA sums the FP32 partials of its rows in
// the order k_splitk_reduce uses and rounds them to TO (the values that kernel would store), then
// scales them as k_scalecols_small does (pivot: lowest row of maximum modulus, across the cluster of
// CL CTAs that shares a column).  The result is the reduction followed by scalecols, bit for bit.
template <class TO, bool FAST, int U, int CL>
__global__ void __launch_bounds__(SCS_T) k_splitk_scalecols(int M, int N, int splits, const float* __restrict__ partial,
                                                            TO* __restrict__ D, int64_t ldd) {
  using TC = float;
  if (CL > 1) cluster_arrive_relaxed();
  __shared__ ArgMaxK red[SCS_T / 32];
  __shared__ TC s_t, s_y;
  __shared__ long long s_k;
  __shared__ bool s_pf;
  __shared__ unsigned long long s_ckey[CL], s_crow[CL], s_cval[CL];  // filled by the cluster
  const int n = blockIdx.x / CL;
  const int64_t r0 = (int64_t)(blockIdx.x % CL) * SCS_T * U;
  const int64_t total = (int64_t)M * N;
  const float* pc = partial + (int64_t)n * M;
  float acc[U];
#pragma unroll
  for (int u = 0; u < U; ++u) acc[u] = 0.f;
#pragma unroll 4
  for (int z = 0; z < splits; ++z) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
      if (i < M) acc[u] += pc[(size_t)z * total + i];
    }
  }
  TO v[U];
  ArgMaxK a{-1, 0x7fffffffffffffffLL};
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
    v[u] = (i < M) ? cvt_out<TO>(acc[u]) : TO(0);
    if (i < M) {
      const long long key = amax_key(v[u]);
      if (key > a.key) a = ArgMaxK{key, i};  // per-thread rows ascend: strict > keeps the lowest
    }
  }
  const ArgMaxK r = block_argmaxk(a, red);
  if (r.key >= 0 && threadIdx.x == (int)((r.i - r0) % SCS_T)) {  // the owner of this CTA's candidate
    const int ku = (int)((r.i - r0) / SCS_T);
    TO pv = TO(0);
#pragma unroll
    for (int u = 0; u < U; ++u) pv = (u == ku) ? v[u] : pv;
    const TC t0 = to_c<TC, TO>(pv);
    s_t = t0;
    if (CL == 1) {
      s_k = r.i;
      s_y = (t0 != TC(0)) ? pivot_recip(t0) : TC(0);  // once per column
      s_pf = pivot_fast(t0);
    }
  }
  if (CL > 1) {
    __syncthreads();
    cluster_wait();  // every CTA of the cluster has started: its shared memory may be written
    const unsigned me = cluster_rank();
    if (threadIdx.x < CL) {
      st_cluster_u64(cluster_map(&s_ckey[me], threadIdx.x), (unsigned long long)r.key);
      st_cluster_u64(cluster_map(&s_crow[me], threadIdx.x), (unsigned long long)r.i);
      st_cluster_u64(cluster_map(&s_cval[me], threadIdx.x), (unsigned long long)__float_as_uint(r.key >= 0 ? s_t : 0.f));
    }
    cluster_arrive();
    cluster_wait();  // the last access to another CTA's shared memory is before this barrier
    if (threadIdx.x == 0) {
      ArgMaxK g{-1, 0x7fffffffffffffffLL};
      TC gv = TC(0);
#pragma unroll
      for (int q = 0; q < CL; ++q) {  // in row order: max key, lowest row on ties
        const ArgMaxK c{(long long)s_ckey[q], (long long)s_crow[q]};
        const ArgMaxK pk = argmaxk_pick(g, c);
        if (pk.key != g.key || pk.i != g.i) gv = __uint_as_float((unsigned)s_cval[q]);
        g = pk;
      }
      s_t = gv;
      s_k = g.i;
      s_y = (gv != TC(0)) ? pivot_recip(gv) : TC(0);
      s_pf = pivot_fast(gv);
    }
  }
  __syncthreads();
  const TC t = s_t, y = s_y;
  const int64_t k = s_k;
  const bool pf = s_pf;
  TO* col = D + (int64_t)n * ldd;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
    if (i < M) col[i] = (t != TC(0)) ? from_c<TO, TC>(scale_by<TC, FAST>(to_c<TC, TO>(v[u]), t, y, pf, i == k)) : v[u];
  }
}

// ---- host side ------------------------------------------------------------------------
// scale >= 0: the product is followed by scalecols (FAST when scale == 1) of the 16-bit result, fused
// with the split-K reduction when K is split
template <int BN, class TOUT>
static int launch(ofrr_ctx* ctx, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, ofrr_dtype t16,
                  TOUT* D, int64_t ldd, int splits, int scale = -1) {
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
  constexpr bool k16 = std::is_same<TOUT, __half>::value || std::is_same<TOUT, __nv_bfloat16>::value;
  if (scale >= 0 && !k16) return OFRR_ERR_INTERNAL;
  if constexpr (k16) {
    if (scale >= 0 && splits > 1) {
      OFRR_TRY(scs_dispatch(M, [&](auto u, auto cl) {
        constexpr int RU = decltype(u)::value, CL = decltype(cl)::value;
        if (scale == 1)
          return launch_cols(ctx, CL, N, k_splitk_scalecols<TOUT, true, RU, CL>, M, N, splits, (const float*)partial,
                             D, ldd);
        return launch_cols(ctx, CL, N, k_splitk_scalecols<TOUT, false, RU, CL>, M, N, splits, (const float*)partial,
                           D, ldd);
      }));
      OFRR_LAUNCHED(ctx, "k_splitk_scalecols");
      return OFRR_SUCCESS;
    }
    if (scale >= 0) return scalecols_impl(ctx, t16, OFRR_F32, M, N, D, ldd, nullptr, scale == 1);
  }
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

namespace tc {
// enough CTAs to cover the SMs: split K when the output grid is small
// Tile plans found by the autotuner (ofrr_autotune_gemm16), process-wide, keyed by the exact shape and type;
// shapes without a tuned plan take the heuristic below.
struct TunedPlan {
  int64_t M, N, K;
  int t16, BN, splits;
};
static std::mutex g_plan_mu;
static std::vector<TunedPlan> g_plans;

static bool find_plan(int64_t M, int64_t N, int64_t K, int t16, int* BN, int* splits) {
  std::lock_guard<std::mutex> lock(g_plan_mu);
  for (const TunedPlan& p : g_plans)
    if (p.M == M && p.N == N && p.K == K && p.t16 == t16) {
      *BN = p.BN;
      *splits = p.splits;
      return true;
    }
  return false;
}

static void store_plan(int64_t M, int64_t N, int64_t K, int t16, int BN, int splits) {
  std::lock_guard<std::mutex> lock(g_plan_mu);
  for (TunedPlan& p : g_plans)
    if (p.M == M && p.N == N && p.K == K && p.t16 == t16) {
      p.BN = BN;
      p.splits = splits;
      return;
    }
  g_plans.push_back(TunedPlan{M, N, K, t16, BN, splits});
}

static int plan_splits(int64_t M, int64_t N, int64_t K, int BN) {
  const int tiles = (int)(((M + BM - 1) / BM) * ((N + BN - 1) / BN));
  const int kbt = (int)((K + BK - 1) / BK);
  int splits = 1;
  while (tiles * splits < 148 && splits * 2 <= kbt && splits < 64) splits *= 2;
  if (const char* e = getenv("OFRR_TC_SPLITS")) splits = std::max(1, std::min(atoi(e), kbt));  // tuning override
  return splits;
}

// E4M3 product C (M x N, FP32) = diag(sa) (A8' B8) diag(sb): A8 (K x M) and B8 (K x N) E4M3 bytes,
// K-contiguous with leading dimensions lda8, ldb8 (multiples of 16 bytes)
template <int BN>
static int launch_f8(ofrr_ctx* ctx, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, float* D,
                     int64_t ldd, int splits, const float* sa, const float* sb) {
  const int kbt = (K + 2 * BK - 1) / (2 * BK);
  splits = std::max(1, std::min(splits, kbt));
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
  static std::atomic<bool> attr_set{false};
  if (!attr_set) {
    OFRR_TRY(allow_smem(k_gemm_tn<BN, float, true>));
    attr_set = true;
  }
  dim3 grid(gm, gn, splits);
  k_gemm_tn<BN, float, true><<<grid, THREADS, Smem<BN>::TOTAL, ctx->stream>>>(
      ma, mb, M, N, kbt, kbps, make_idesc(OFRR_F16, BN), D, ldd, partial, ctx->dev_flags + kFlagTcWait, sa, sb);
  OFRR_LAUNCHED(ctx, "k_gemm_tn_e4m3");
  if (splits > 1) {
    k_splitk_reduce<float, false><<<grid_2d(M, N, 256), 256, 0, ctx->stream>>>(M, N, splits, partial, D, ldd);
    OFRR_LAUNCHED(ctx, "k_splitk_reduce");
  }
  return OFRR_SUCCESS;
}

// the tile width and K split of a product: the tuned plan when there is one, else the heuristic
static void choose_plan(int64_t M, int64_t N, int64_t K, int t16, int* BN, int* splits) {
  if (find_plan(M, N, K, t16, BN, splits)) return;
  *BN = (N <= 32) ? 32 : (N <= 64 ? 64 : 128);
  *splits = plan_splits(M, N, K, *BN);
}
}  // namespace tc

// A 16-bit K x cols operand as TMA takes it (16-byte aligned base and leading dimension): a misaligned
// one (an odd row count) is copied once, as one pitched copy, into an aligned workspace buffer.  The
// tensor-core path then serves every shape, so results never depend on a library fallback.
static int tc_operand(ofrr_ctx* ctx, const void* X, int64_t ld, int64_t K, int64_t cols, const void** out,
                      int64_t* ldo) {
  if (!((uintptr_t)X & 15) && !((ld * 2) & 15)) {
    *out = X;
    *ldo = ld;
    return OFRR_SUCCESS;
  }
  const int64_t ldp = (K + 7) & ~int64_t(7);
  int st = OFRR_SUCCESS;
  void* w = ws_alloc(ctx, (size_t)ldp * cols * 2, &st);
  if (!w) return st;
  OFRR_CUDA(cudaMemcpy2DAsync(w, (size_t)ldp * 2, X, (size_t)ld * 2, (size_t)K * 2, (size_t)cols,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  *out = w;
  *ldo = ldp;
  return OFRR_SUCCESS;
}

// Route a 16-bit TN product to the tcgen05 kernel (operands staged to TMA-aligned layouts when needed);
// *handled = false leaves the call to the caller's fallback.
int gemm_tc_try(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype t16, int64_t M, int64_t N, int64_t K,
                const void* A, int64_t lda, const void* B, int64_t ldb, ofrr_dtype tout, void* C, int64_t ldc,
                bool* handled) {
  *handled = false;
  if (!(transA == 1 && transB == 0)) return OFRR_SUCCESS;
  if (K < 16 || M < 1 || N < 1 || M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) return OFRR_SUCCESS;
  if (getenv("OFRR_DISABLE_TC")) return OFRR_SUCCESS;
  OFRR_TRY(tc_operand(ctx, A, lda, K, M, &A, &lda));
  OFRR_TRY(tc_operand(ctx, B, ldb, K, N, &B, &ldb));
  int BN = 64, splits = 1;
  tc::choose_plan(M, N, K, t16, &BN, &splits);
  CUtensorMap ma, mb;
  if (!tc::make_map(&ma, t16, A, K, M, lda, tc::BM)) return OFRR_SUCCESS;
  if (!tc::make_map(&mb, t16, B, K, N, ldb, BN)) return OFRR_SUCCESS;
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

// C (t16, M x N) = A' B (16-bit TN product, FP32 accumulation), then scalecols of C in FP32 (fast: the
// reciprocal-multiply form): the power step of the 16-bit phase.  With K split, the partial sums are
// combined inside the scaling kernel; the result equals gemm_tc_try followed by scalecols_impl bit for
// bit.  *handled = false (nothing launched) leaves both steps to the caller.
int gemm_tc_scalecols(ofrr_ctx* ctx, ofrr_dtype t16, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                      const void* B, int64_t ldb, void* C, int64_t ldc, bool fast, bool* handled) {
  *handled = false;
  if (t16 != OFRR_F16 && t16 != OFRR_BF16) return OFRR_SUCCESS;
  if (K < 16 || M < 1 || N < 1 || M > 8192 || N > 65535 || K > (1 << 30)) return OFRR_SUCCESS;
  if (getenv("OFRR_DISABLE_TC")) return OFRR_SUCCESS;
  OFRR_TRY(tc_operand(ctx, A, lda, K, M, &A, &lda));
  OFRR_TRY(tc_operand(ctx, B, ldb, K, N, &B, &ldb));
  int BN = 64, splits = 1;
  tc::choose_plan(M, N, K, t16, &BN, &splits);
  CUtensorMap ma, mb;
  if (!tc::make_map(&ma, t16, A, K, M, lda, tc::BM)) return OFRR_SUCCESS;
  if (!tc::make_map(&mb, t16, B, K, N, ldb, BN)) return OFRR_SUCCESS;
  const int sc = fast ? 1 : 0;
  int st;
  if (t16 == OFRR_F16) {
    if (BN == 32) st = tc::launch<32, __half>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (__half*)C, ldc, splits, sc);
    else if (BN == 64) st = tc::launch<64, __half>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (__half*)C, ldc, splits, sc);
    else st = tc::launch<128, __half>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (__half*)C, ldc, splits, sc);
  } else {
    using B16 = __nv_bfloat16;
    if (BN == 32) st = tc::launch<32, B16>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (B16*)C, ldc, splits, sc);
    else if (BN == 64) st = tc::launch<64, B16>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (B16*)C, ldc, splits, sc);
    else st = tc::launch<128, B16>(ctx, ma, mb, (int)M, (int)N, (int)K, t16, (B16*)C, ldc, splits, sc);
  }
  if (st != OFRR_SUCCESS) return st;
  *handled = true;
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

// Self-test of the 16-bit power step: C = A' B (A: K x M, B: K x N, both t16; C t16), then scalecols of C
// in FP32, with the split-K reduction fused into the scaling kernel.  Returns OFRR_ERR_INVALID_ARGUMENT
// for a shape or layout the fused path does not take.
extern "C" int ofrr_debug_gemm16_scalecols(ofrr_ctx* ctx, int t16, int64_t M, int64_t N, int64_t K, const void* A,
                                           int64_t lda, const void* B, int64_t ldb, void* C, int64_t ldc, int fast) {
  if (!ctx || !A || !B || !C || ldc < M) return OFRR_ERR_INVALID_ARGUMENT;
  bool handled = false;
  OFRR_TRY(gemm_tc_scalecols(ctx, (ofrr_dtype)t16, M, N, K, A, lda, B, ldb, C, ldc, fast != 0, &handled));
  return handled ? OFRR_SUCCESS : OFRR_ERR_INVALID_ARGUMENT;
}

// Tile autotuner of the 16-bit tcgen05 product (no reference counterpart): for C (M x N, FP32) = A' B with
// A (K x M) and B (K x N) of type t16, every tile width BN in {32, 64, 128} and K split in {1, 2, 4, ...,
// 64} (at most the number of 64-wide K blocks) is timed over reps launches (CUDA events, synchronous) on
// seeded operands of that shape; the fastest plan is kept for the shape and used by every later product of
// exactly that shape and type (the 16-bit power steps, Gram products and Ritz updates).
extern "C" int ofrr_autotune_gemm16(ofrr_ctx* ctx, int t16, int64_t M, int64_t N, int64_t K, int reps, int* best_bn,
                                    int* best_splits, double* best_us) {
  if (!ctx || (t16 != OFRR_F16 && t16 != OFRR_BF16) || M < 1 || N < 1 || K < 16 || reps < 1)
    return OFRR_ERR_INVALID_ARGUMENT;
  if (M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t Kp = (K + 7) / 8 * 8;
  void* A = ws_alloc(ctx, (size_t)Kp * M * 2, &st);
  void* B = ws_alloc(ctx, (size_t)Kp * N * 2, &st);
  float* C = ws_get<float>(ctx, (size_t)M * N, &st);
  if (!A || !B || !C) return st;
  OFRR_TRY(ofrr_randn(ctx, 1, K, M, (ofrr_dtype)t16, A, Kp));
  OFRR_TRY(ofrr_randn(ctx, 2, K, N, (ofrr_dtype)t16, B, Kp));
  cudaEvent_t e0, e1;
  OFRR_CUDA(cudaEventCreate(&e0));
  OFRR_CUDA(cudaEventCreate(&e1));
  const int kbt = (int)((K + tc::BK - 1) / tc::BK);
  double best = INFINITY;
  int bbn = 64, bsp = 1;
  const int bns[3] = {32, 64, 128};
  for (int bi = 0; bi < 3 && st == OFRR_SUCCESS; ++bi) {
    const int BN = bns[bi];
    CUtensorMap ma, mb;
    if (!tc::make_map(&ma, (ofrr_dtype)t16, A, K, M, Kp, tc::BM) || !tc::make_map(&mb, (ofrr_dtype)t16, B, K, N, Kp, BN)) {
      st = OFRR_ERR_INTERNAL;
      break;
    }
    for (int sp = 1; sp <= 64 && sp <= kbt && st == OFRR_SUCCESS; sp *= 2) {
      auto run = [&]() {
        if (BN == 32) return tc::launch<32, float>(ctx, ma, mb, (int)M, (int)N, (int)K, (ofrr_dtype)t16, C, M, sp);
        if (BN == 64) return tc::launch<64, float>(ctx, ma, mb, (int)M, (int)N, (int)K, (ofrr_dtype)t16, C, M, sp);
        return tc::launch<128, float>(ctx, ma, mb, (int)M, (int)N, (int)K, (ofrr_dtype)t16, C, M, sp);
      };
      st = run();  // warm-up
      if (st != OFRR_SUCCESS) break;
      st = map_cuda_error(cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < reps && st == OFRR_SUCCESS; ++r) st = run();
      if (st == OFRR_SUCCESS) st = map_cuda_error(cudaEventRecord(e1, ctx->stream));
      if (st == OFRR_SUCCESS) st = sync_and_check(ctx);
      float ms = 0.f;
      if (st == OFRR_SUCCESS) st = map_cuda_error(cudaEventElapsedTime(&ms, e0, e1));
      const double us = 1e3 * ms / reps;
      if (st == OFRR_SUCCESS && us < best) {
        best = us;
        bbn = BN;
        bsp = sp;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  OFRR_TRY(st);
  tc::store_plan(M, N, K, t16, bbn, bsp);
  if (best_bn) *best_bn = bbn;
  if (best_splits) *best_splits = bsp;
  if (best_us) *best_us = best;
  return OFRR_SUCCESS;
}

// The plan a 16-bit product of this shape would use now; *tuned = 1 when it came from the autotuner.
extern "C" int ofrr_gemm16_plan(int t16, int64_t M, int64_t N, int64_t K, int* bn, int* splits, int* tuned) {
  if (!bn || !splits) return OFRR_ERR_INVALID_ARGUMENT;
  const bool t = tc::find_plan(M, N, K, t16, bn, splits);
  if (!t) tc::choose_plan(M, N, K, t16, bn, splits);
  if (tuned) *tuned = t ? 1 : 0;
  return OFRR_SUCCESS;
}

namespace ofrr {
namespace {
// Per-column E4M3 copy of X (K x M, type TI, column-major): scale_j = 2^e with 2^e >= max_k |X(k, j)| / 448,
// X8(k, j) = e4m3(X(k, j) / scale_j) (saturating); one CTA per column, ld8 bytes between columns
template <class TI>
__global__ void __launch_bounds__(256) k_quant_e4m3(int64_t K, int64_t M, const TI* __restrict__ X, int64_t ldx,
                                                    __nv_fp8_e4m3* __restrict__ X8, int64_t ld8,
                                                    float* __restrict__ scale) {
  __shared__ float red[8];
  const int64_t j = blockIdx.x;
  const TI* x = X + j * ldx;
  float mx = 0.f;
  for (int64_t k = threadIdx.x; k < K; k += blockDim.x) mx = fmaxf(mx, fabsf(to_c<float, TI>(x[k])));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  float m = 0.f;
  for (int w = 0; w < 8; ++w) m = fmaxf(m, red[w]);
  // power-of-two scale: the largest entry lands in [224, 448]
  const float sc = (m > 0.f) ? exp2f(ceilf(log2f(m / 448.f))) : 1.f;
  const float inv = 1.f / sc;
  if (threadIdx.x == 0) scale[j] = sc;
  __nv_fp8_e4m3* y = X8 + j * ld8;
  for (int64_t k = threadIdx.x; k < ld8; k += blockDim.x)
    y[k] = (k < K) ? __nv_fp8_e4m3(to_c<float, TI>(x[k]) * inv) : __nv_fp8_e4m3(0.f);
}
}  // namespace

int quant_e4m3(ofrr_ctx* ctx, ofrr_dtype tin, int64_t K, int64_t M, const void* X, int64_t ldx, void* X8,
               int64_t ld8, float* scale) {
  if (M <= 0) return OFRR_SUCCESS;
  if (M > 0x7fffffffLL) return OFRR_ERR_BLAS_INVALID_SIZE;
  OFRR_DISPATCH_STORAGE(tin, TI, {
    k_quant_e4m3<TI><<<(unsigned)M, 256, 0, ctx->stream>>>(K, M, (const TI*)X, ldx, (__nv_fp8_e4m3*)X8, ld8, scale);
    OFRR_LAUNCHED(ctx, "k_quant_e4m3");
  });
  return OFRR_SUCCESS;
}

// C (M x N, FP32) = diag(sa) A8' B8 diag(sb) on the tcgen05 tensor cores (kind::f8f6f4)
int gemm_e4m3_tn(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const void* A8, int64_t lda8, const float* sa,
                 const void* B8, int64_t ldb8, const float* sb, float* C, int64_t ldc) {
  if (M < 1 || N < 1 || K < 32 || M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (((uintptr_t)A8 & 15) || ((uintptr_t)B8 & 15) || (lda8 & 15) || (ldb8 & 15)) return OFRR_ERR_INVALID_ARGUMENT;
  const int BN = (N <= 32) ? 32 : (N <= 64 ? 64 : 128);
  CUtensorMap ma, mb;
  if (!tc::make_map_u8(&ma, A8, K, M, lda8, tc::BM) || !tc::make_map_u8(&mb, B8, K, N, ldb8, BN))
    return OFRR_ERR_INTERNAL;
  const int tiles = (int)(((M + tc::BM - 1) / tc::BM) * ((N + BN - 1) / BN));
  const int kbt = (int)((K + 127) / 128);
  int splits = 1;
  while (tiles * splits < 148 && splits * 2 <= kbt && splits < 64) splits *= 2;
  if (BN == 32) return tc::launch_f8<32>(ctx, ma, mb, (int)M, (int)N, (int)K, C, ldc, splits, sa, sb);
  if (BN == 64) return tc::launch_f8<64>(ctx, ma, mb, (int)M, (int)N, (int)K, C, ldc, splits, sa, sb);
  return tc::launch_f8<128>(ctx, ma, mb, (int)M, (int)N, (int)K, C, ldc, splits, sa, sb);
}

}  // namespace ofrr

// C (M x N, FP32) = A' B with FP32 A (K x M) and B (K x N): both quantized per column to E4M3 with
// power-of-two scales, multiplied on the tensor cores (FP32 accumulation), scaled back (no reference
// counterpart; the FP8 variant of the 16-bit power steps).
extern "C" int ofrr_gemm_e4m3(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const float* A, int64_t lda,
                              const float* B, int64_t ldb, float* C, int64_t ldc) {
  if (!ctx || !A || !B || !C || M < 1 || N < 1 || K < 32 || lda < K || ldb < K || ldc < M)
    return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t ld8 = (K + 127) / 128 * 128;
  void* A8 = ws_alloc(ctx, (size_t)ld8 * M, &st);
  void* B8 = ws_alloc(ctx, (size_t)ld8 * N, &st);
  float* sa = ws_get<float>(ctx, (size_t)M, &st);
  float* sb = ws_get<float>(ctx, (size_t)N, &st);
  if (!A8 || !B8 || !sa || !sb) return st;
  OFRR_TRY(quant_e4m3(ctx, OFRR_F32, K, M, A, lda, A8, ld8, sa));
  OFRR_TRY(quant_e4m3(ctx, OFRR_F32, K, N, B, ldb, B8, ld8, sb));
  return gemm_e4m3_tn(ctx, M, N, ld8, A8, ld8, sa, B8, ld8, sb, C, ldc);
}
