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
#include <cstdlib>

#include "ofrr_internal.cuh"

namespace ofrr {
namespace tc {

constexpr int BM = 128;
constexpr int BK = 64;  // one 128-byte swizzle row of 16-bit elements
constexpr int STAGES = 4;
constexpr int THREADS = 192;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait (about 2 s); records code in *err and returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer() - t0 > 2000000000ull) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map, uint64_t* bar, void* dst, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// UMMA shared-memory descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address (16-byte units)
  d |= (uint64_t)1 << 16;                    // leading byte offset (ignored for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset between 8-row groups
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

template <class TOUT> __device__ __forceinline__ TOUT cvt_out(float x);
template <> __device__ __forceinline__ float cvt_out<float>(float x) { return x; }
template <> __device__ __forceinline__ double cvt_out<double>(float x) { return (double)x; }
template <> __device__ __forceinline__ __half cvt_out<__half>(float x) { return __float2half_rn(x); }
template <> __device__ __forceinline__ __nv_bfloat16 cvt_out<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }

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

template <class TOUT>
__global__ void k_splitk_reduce(int M, int N, int splits, const float* __restrict__ partial, TOUT* __restrict__ D,
                                int64_t ldd) {
  const int64_t total = (int64_t)M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += partial[(size_t)z * total + e];  // fixed order: deterministic
    const int64_t m = e % M, n = e / M;
    D[m + n * ldd] = cvt_out<TOUT>(s);
  }
}

// ---- host side ------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// 2D map over a K-contiguous operand: dims {K, rows}, row stride ld elements, box {64, box_rows}
static bool make_map(CUtensorMap* map, ofrr_dtype t, const void* ptr, int64_t K, int64_t rows, int64_t ld,
                     int box_rows) {
  EncodeTiledFn enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, t == OFRR_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                   const_cast<void*>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

static uint32_t make_idesc(ofrr_dtype t, int BN) {
  const uint32_t fmt = (t == OFRR_BF16) ? 1u : 0u;
  uint32_t d = 0;
  d |= 1u << 4;                     // D format: F32
  d |= fmt << 7;                    // A format
  d |= fmt << 10;                   // B format
  d |= 0u << 15;                    // A K-major
  d |= 0u << 16;                    // B K-major
  d |= (uint32_t)(BN >> 3) << 17;   // N >> 3
  d |= (uint32_t)(BM >> 4) << 24;   // M >> 4
  return d;
}

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
  static bool attr_set = false;
  if (!attr_set) {
    OFRR_CUDA(cudaFuncSetAttribute(k_gemm_tn<BN, TOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  dim3 grid(gm, gn, splits);
  k_gemm_tn<BN, TOUT><<<grid, THREADS, smem, ctx->stream>>>(ma, mb, M, N, kbt, kbps, make_idesc(t16, BN), D, ldd,
                                                            partial, ctx->dev_flags + 2);
  OFRR_LAUNCHED(ctx, "k_gemm_tn");
  if (splits > 1) {
    k_splitk_reduce<TOUT><<<grid_for((int64_t)M * N, 256, 1024), 256, 0, ctx->stream>>>(M, N, splits, partial, D, ldd);
    OFRR_LAUNCHED(ctx, "k_splitk_reduce");
  }
  return OFRR_SUCCESS;
}

}  // namespace tc

// FP32 partial products of a 16-bit TN GEMM: partial[z] (M x N, ld M) holds the sum over the z-th
// contiguous range of kblocks_per_split * 64 entries of K.  Used by the exact-slice FP64 emulation,
// which chooses the ranges so that every partial sum is exact.  Requires TMA-compatible layouts.
int tc_gemm_partials(ofrr_ctx* ctx, ofrr_dtype t16, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                     const void* B, int64_t ldb, int kblocks_per_split, float* partial, int* splits_out) {
  if (K < 16 || M < 1 || N < 1) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (((uintptr_t)A & 15) || ((uintptr_t)B & 15) || ((lda * 2) & 15) || ((ldb * 2) & 15))
    return OFRR_ERR_BLAS_INVALID_SIZE;
  const int BN = (N <= 32) ? 32 : (N <= 64 ? 64 : 128);
  CUtensorMap ma, mb;
  if (!tc::make_map(&ma, t16, A, K, M, lda, tc::BM) || !tc::make_map(&mb, t16, B, K, N, ldb, BN))
    return OFRR_ERR_INTERNAL;
  const int kbt = (int)((K + tc::BK - 1) / tc::BK);
  const int kbps = std::max(1, std::min(kblocks_per_split, kbt));
  const int splits = (kbt + kbps - 1) / kbps;
  const int gm = (int)((M + tc::BM - 1) / tc::BM), gn = (int)((N + BN - 1) / BN);
  dim3 grid(gm, gn, splits);
  const uint32_t idesc = tc::make_idesc(t16, BN);
  float* none = nullptr;
  if (BN == 32) {
    const size_t smem = tc::Smem<32>::TOTAL;
    OFRR_CUDA(cudaFuncSetAttribute(tc::k_gemm_tn<32, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tc::k_gemm_tn<32, float><<<grid, tc::THREADS, smem, ctx->stream>>>(ma, mb, (int)M, (int)N, kbt, kbps, idesc, none,
                                                                       M, partial, ctx->dev_flags + 2);
  } else if (BN == 64) {
    const size_t smem = tc::Smem<64>::TOTAL;
    OFRR_CUDA(cudaFuncSetAttribute(tc::k_gemm_tn<64, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tc::k_gemm_tn<64, float><<<grid, tc::THREADS, smem, ctx->stream>>>(ma, mb, (int)M, (int)N, kbt, kbps, idesc, none,
                                                                       M, partial, ctx->dev_flags + 2);
  } else {
    const size_t smem = tc::Smem<128>::TOTAL;
    OFRR_CUDA(cudaFuncSetAttribute(tc::k_gemm_tn<128, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tc::k_gemm_tn<128, float><<<grid, tc::THREADS, smem, ctx->stream>>>(ma, mb, (int)M, (int)N, kbt, kbps, idesc,
                                                                        none, M, partial, ctx->dev_flags + 2);
  }
  OFRR_LAUNCHED(ctx, "k_gemm_tn");
  *splits_out = splits;
  return OFRR_SUCCESS;
}

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
