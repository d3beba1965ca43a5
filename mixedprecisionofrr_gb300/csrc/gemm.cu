// Dense contractions with MATLAB gemm.m semantics (MATLAB/+src/+mvops/gemm.m:27-59):
// operands converted to the compute type, accumulated there, stored in the output type.
//
// Routing:
//   * 16-bit operands (both F16 or both BF16) with F32 compute -> the hand-written tcgen05
//     kernel (gemm_tc.cu) when the shape fits its tiling, else cuBLAS GemmEx;
//   * F32 x F32 / F64 x F64 -> cuBLAS S/DGEMM (plain library GEMMs, pedantic math mode);
//   * mixed operand types -> the narrower operand is widened to the compute type first.
#include "ofrr_internal.cuh"

namespace ofrr {

int gemm_tc_try(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype t16, int64_t M, int64_t N, int64_t K,
                const void* A, int64_t lda, const void* B, int64_t ldb, ofrr_dtype tout, void* C, int64_t ldc,
                bool* handled);

static cudaDataType_t cuda_type(ofrr_dtype t) {
  switch (t) {
    case OFRR_F64: return CUDA_R_64F;
    case OFRR_F32: return CUDA_R_32F;
    case OFRR_F16: return CUDA_R_16F;
    case OFRR_BF16: return CUDA_R_16BF;
  }
  return CUDA_R_32F;
}

constexpr int64_t kSlicedMaxK = int64_t(1) << 20;

// C += T (FP64, M x N)
__global__ void k_add_f64(int64_t m, int64_t n, const double* __restrict__ T, int64_t ldt, double* __restrict__ C,
                          int64_t ldc) {
  OFRR_FOR_2D(i, j, m, n) C[i + j * ldc] += T[i + j * ldt];
}

// ---- FP64 Gram products on the CUDA cores ------------------------------------------------------------
// C (M x N) = A' B for FP64 A (K x M), B (K x N), M, N <= 128: the Gram and cross-Gram matrices of a
// Rayleigh-Ritz step.  The exact-slice emulation's element error (2^-35 of |A|'|B|) is amplified by the
// condition number of a non-orthogonal basis (10^3 .. 10^4 for power-iterated Hessenberg bases); the small
// products (K M N <= 2^22 FMAs: small requests) run in FP64, larger ones stay emulated until a solve meets
// that floor (the solvers then switch to FP64 products).
// One CTA per K chunk: 32-row slabs of both operands staged in shared memory, a 64 x 64 output tile per
// pass (4 x 4 per thread of a 16 x 16 grid), the chunk's partial written out; k_gram_sum adds the
// partials in chunk order (results do not depend on the schedule).
constexpr int kGramSlab = 32;

__global__ void __launch_bounds__(256) k_gram_f64(int64_t K, int M, int N, const double* __restrict__ A, int64_t lda,
                                                  const double* __restrict__ B, int64_t ldb, int64_t kc,
                                                  double* __restrict__ partial) {
  __shared__ double sA[kGramSlab][65], sB[kGramSlab][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t k0 = (int64_t)blockIdx.x * kc, k1 = min(K, k0 + kc);
  double* P = partial + (size_t)blockIdx.x * M * N;
  for (int m0 = 0; m0 < M; m0 += 64)
    for (int n0 = 0; n0 < N; n0 += 64) {
      double acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
      for (int64_t kb = k0; kb < k1; kb += kGramSlab) {
        for (int e = threadIdx.x; e < kGramSlab * 64; e += 256) {
          const int r = e % kGramSlab, c = e / kGramSlab;
          const int64_t k = kb + r;
          sA[r][c] = (k < k1 && m0 + c < M) ? A[k + (int64_t)(m0 + c) * lda] : 0.0;
          sB[r][c] = (k < k1 && n0 + c < N) ? B[k + (int64_t)(n0 + c) * ldb] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kGramSlab; ++kk) {
          double a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            a[i] = sA[kk][ty + 16 * i];
            b[i] = sB[kk][tx + 16 * i];
          }
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
          if (m < M && n < N) P[m + (size_t)n * M] = acc[i][j];
        }
    }
}

__global__ void k_gram_sum(int M, int N, int chunks, const double* __restrict__ partial, double* __restrict__ C,
                           int64_t ldc) {
  const int mn = M * N;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < mn; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += partial[(size_t)c * mn + e];
    C[(e % M) + (int64_t)(e / M) * ldc] = s;
  }
}

int gram_f64(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
             int64_t ldb, double* C, int64_t ldc) {
  if (M > 128 || N > 128 || M < 1 || N < 1) return OFRR_ERR_BLAS_INVALID_SIZE;
  int st = OFRR_SUCCESS;
  const int64_t slabs = (K + kGramSlab - 1) / kGramSlab;
  const int chunks = (int)std::max<int64_t>(1, std::min<int64_t>(slabs, 152 * 2));
  const int64_t kc = ((slabs + chunks - 1) / chunks) * kGramSlab;
  const int used = (int)((K + kc - 1) / kc);
  double* partial = ws_get<double>(ctx, (size_t)used * M * N, &st);
  if (!partial) return st;
  k_gram_f64<<<used, 256, 0, ctx->stream>>>(K, (int)M, (int)N, A, lda, B, ldb, kc, partial);
  OFRR_LAUNCHED(ctx, "k_gram_f64");
  k_gram_sum<<<(int)std::min<int64_t>((M * N + 255) / 256, 152 * 4), 256, 0, ctx->stream>>>((int)M, (int)N, used,
                                                                                            partial, C, ldc);
  OFRR_LAUNCHED(ctx, "k_gram_sum");
  return OFRR_SUCCESS;
}

// C (M x N) = A (M x K) B (K x N) in FP64 for K, N <= 128: the Ritz-vector back-transform X = Q Z of a
// Rayleigh-Ritz step.  Q is a non-orthogonal basis and Z's columns cancel across it (|Q||z| is 10^3 ..
// 10^4 times |Qz|), so the emulation's error is relative to a much larger number than the result; small
// products (and every back-transform once a solve meets the emulation floor) run in FP64.  B in shared
// memory, a thread per row and 16 columns, A read with coalesced loads.
__global__ void __launch_bounds__(128) k_tsmm_f64(int64_t M, int N, int K, const double* __restrict__ A, int64_t lda,
                                                  const double* __restrict__ B, int64_t ldb, double* __restrict__ C,
                                                  int64_t ldc) {
  extern __shared__ double sBm[];  // K x 16 slice of B (row-major)
  const int c0 = blockIdx.y * 16, nc = min(16, N - c0);
  for (int e = threadIdx.x; e < K * 16; e += blockDim.x) {
    const int k = e / 16, c = e % 16;
    sBm[e] = (c < nc) ? B[k + (int64_t)(c0 + c) * ldb] : 0.0;
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (int64_t)gridDim.x * blockDim.x) {
    double acc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) acc[c] = 0.0;
    for (int k = 0; k < K; ++k) {
      const double a = A[i + (int64_t)k * lda];
      const double* b = sBm + k * 16;
#pragma unroll
      for (int c = 0; c < 16; ++c) acc[c] = fma(a, b[c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (c < nc) C[i + (int64_t)(c0 + c) * ldc] = acc[c];
  }
}

int tsmm_f64(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
             int64_t ldb, double* C, int64_t ldc) {
  if (K > 256 || K < 1) return OFRR_ERR_BLAS_INVALID_SIZE;
  const dim3 grid((unsigned)std::min<int64_t>((M + 127) / 128, 152 * 8), (unsigned)((N + 15) / 16));
  const size_t smem = (size_t)K * 16 * sizeof(double);
  if (smem > 48 * 1024) OFRR_TRY(allow_smem(k_tsmm_f64));
  k_tsmm_f64<<<grid, 128, smem, ctx->stream>>>(M, (int)N, (int)K, A, lda, B, ldb, C, ldc);
  OFRR_LAUNCHED(ctx, "k_tsmm_f64");
  return OFRR_SUCCESS;
}

int gemm_impl(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype ta, ofrr_dtype tb, ofrr_dtype tc, ofrr_dtype tout,
              int64_t M, int64_t N, int64_t K, double alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
              double beta, void* C, int64_t ldc) {
  if (M <= 0 || N <= 0) return OFRR_SUCCESS;
  if (tc != OFRR_F64 && tc != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t Ar = transA ? K : M, Ac = transA ? M : K;
  const int64_t Br = transB ? N : K, Bc = transB ? K : N;
  if (K <= 0) {
    // C = beta C (alpha * empty product)
    if (beta == 0.0) {
      for (int64_t j = 0; j < N; ++j)
        OFRR_TRY(fill_zero(ctx, (char*)C + (size_t)j * ldc * dtype_size(tout), (size_t)M * dtype_size(tout)));
      return OFRR_SUCCESS;
    }
    if (beta == 1.0) return OFRR_SUCCESS;
  }
  // FP64 TN products in the refinement phase of the mixed solver: exact BF16 slices on the tensor cores
  if (ctx->emulate_f64 && tc == OFRR_F64 && ta == OFRR_F64 && tb == OFRR_F64 && tout == OFRR_F64 && transB == 0 &&
      alpha == 1.0 && beta == 0.0 && transA == 1 && M <= 128 && N <= 128 && K * M * N <= (int64_t(1) << 22))
    return gram_f64(ctx, M, N, K, (const double*)A, lda, (const double*)B, ldb, (double*)C, ldc);
  if (ctx->emulate_f64 && tc == OFRR_F64 && ta == OFRR_F64 && tb == OFRR_F64 && tout == OFRR_F64 && transA == 0 &&
      transB == 0 && alpha == 1.0 && beta == 0.0 && K <= 128 && N <= 128 && M * N * K <= (int64_t(1) << 22))
    return tsmm_f64(ctx, M, N, K, (const double*)A, lda, (const double*)B, ldb, (double*)C, ldc);
  if (ctx->emulate_f64 && tc == OFRR_F64 && ta == OFRR_F64 && tb == OFRR_F64 && tout == OFRR_F64 && transB == 0 &&
      alpha == 1.0 && beta == 0.0 && K >= 16 && (transA == 1 || (M >= 1024 && K <= 1024))) {
    if (K > kSlicedMaxK) {
      // the exact integer combination holds for K <= 2^20: longer contractions (Gram products of
      // millions of rows) are summed over K chunks in FP64, each chunk product emulated
      double* T = ws_get<double>(ctx, (size_t)M * N, &st);
      if (!T) return st;
      for (int64_t k0 = 0; k0 < K; k0 += kSlicedMaxK) {
        const int64_t kc = std::min<int64_t>(kSlicedMaxK, K - k0);
        const double* Ak = (const double*)A + k0;  // transA == 1: A is K x M, its rows k0 ..
        const double* Bk = (const double*)B + k0;
        OFRR_TRY(gemm_impl(ctx, 1, 0, ta, tb, tc, tout, M, N, kc, 1.0, Ak, lda, Bk, ldb, 0.0, k0 ? T : C,
                           k0 ? M : ldc));
        if (k0) {
          k_add_f64<<<grid_2d(M, N, 256), 256, 0, ctx->stream>>>(M, N, T, M, (double*)C, ldc);
          OFRR_LAUNCHED(ctx, "k_add_f64");
        }
      }
      return OFRR_SUCCESS;
    }
    SlicedOperand As;
    if (transA == 1) {
      OFRR_TRY(sliced_prepare(ctx, K, M, (const double*)A, lda, &As));
    } else {
      // tall-skinny A (M x K, e.g. the Ritz update basis x coefficients): slice the transposed copy
      double* At = ws_get<double>(ctx, (size_t)M * K, &st);
      if (!At) return st;
      OFRR_TRY(cast_transpose_impl(ctx, OFRR_F64, OFRR_F64, M, K, A, lda, At, K));
      OFRR_TRY(sliced_prepare(ctx, K, M, At, K, &As));
    }
    return sliced_gemm_tn(ctx, As, N, (const double*)B, ldb, (double*)C, ldc);
  }
  // 16-bit tensor-core path
  if (tc == OFRR_F32 && ta == tb && (ta == OFRR_F16 || ta == OFRR_BF16) && alpha == 1.0 && beta == 0.0) {
    bool handled = false;
    OFRR_TRY(gemm_tc_try(ctx, transA, transB, ta, M, N, K, A, lda, B, ldb, tout, C, ldc, &handled));
    if (handled) return OFRR_SUCCESS;
    cublasComputeType_t ct = CUBLAS_COMPUTE_32F;  // FP32 accumulation (the pedantic variant rejects bf16)
    void* Cout = C;
    int64_t ldco = ldc;
    ofrr_dtype tco = tout;
    if (tout == OFRR_F64) {  // GemmEx cannot write F64 from 16-bit inputs: go through F32
      Cout = ws_get<float>(ctx, (size_t)M * N, &st);
      if (!Cout) return st;
      ldco = M;
      tco = OFRR_F32;
    }
    const float fa = 1.0f, fb = 0.0f;
    const cublasStatus_t cs =
        cublasGemmEx(ctx->cublas, transA ? CUBLAS_OP_T : CUBLAS_OP_N, transB ? CUBLAS_OP_T : CUBLAS_OP_N, (int)M,
                     (int)N, (int)K, &fa, A, cuda_type(ta), (int)lda, B, cuda_type(tb), (int)ldb, &fb, Cout,
                     cuda_type(tco), (int)ldco, ct, CUBLAS_GEMM_DEFAULT);
    if (cs == CUBLAS_STATUS_SUCCESS) {
      ctx->library_calls++;
      if (Cout != C) OFRR_TRY(cast_impl(ctx, OFRR_F32, tout, M, N, Cout, ldco, C, ldc));
      return OFRR_SUCCESS;
    }
    if (cs != CUBLAS_STATUS_NOT_SUPPORTED) OFRR_CUBLAS(cs);
    // unsupported layout for the 16-bit library kernels: widen to FP32 below (same values)
  }
  // widen operands to the compute type
  const void* Ac_ptr = A;
  int64_t ldac = lda;
  if (ta != tc) {
    void* w = ws_alloc(ctx, (size_t)Ar * Ac * dtype_size(tc), &st);
    if (!w) return st;
    OFRR_TRY(cast_impl(ctx, ta, tc, Ar, Ac, A, lda, w, Ar));
    Ac_ptr = w;
    ldac = Ar;
  }
  const void* Bc_ptr = B;
  int64_t ldbc = ldb;
  if (tb != tc) {
    void* w = ws_alloc(ctx, (size_t)Br * Bc * dtype_size(tc), &st);
    if (!w) return st;
    OFRR_TRY(cast_impl(ctx, tb, tc, Br, Bc, B, ldb, w, Br));
    Bc_ptr = w;
    ldbc = Br;
  }
  void* Cc = C;
  int64_t ldcc = ldc;
  if (tout != tc) {
    Cc = ws_alloc(ctx, (size_t)M * N * dtype_size(tc), &st);
    if (!Cc) return st;
    ldcc = M;
    if (beta != 0.0) OFRR_TRY(cast_impl(ctx, tout, tc, M, N, C, ldc, Cc, ldcc));
  }
  const cublasOperation_t oa = transA ? CUBLAS_OP_T : CUBLAS_OP_N, ob = transB ? CUBLAS_OP_T : CUBLAS_OP_N;
  if (tc == OFRR_F64) {
    OFRR_CUBLAS(cublasDgemm(ctx->cublas, oa, ob, (int)M, (int)N, (int)K, &alpha, (const double*)Ac_ptr, (int)ldac,
                            (const double*)Bc_ptr, (int)ldbc, &beta, (double*)Cc, (int)ldcc));
  } else {
    const float fa = (float)alpha, fb = (float)beta;
    OFRR_CUBLAS(cublasSgemm(ctx->cublas, oa, ob, (int)M, (int)N, (int)K, &fa, (const float*)Ac_ptr, (int)ldac,
                            (const float*)Bc_ptr, (int)ldbc, &fb, (float*)Cc, (int)ldcc));
  }
  ctx->library_calls++;
  if (Cc != C) OFRR_TRY(cast_impl(ctx, tc, tout, M, N, Cc, ldcc, C, ldc));
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_gemm(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype ta, ofrr_dtype tb, ofrr_dtype tcompute,
                         ofrr_dtype tout, int64_t M, int64_t N, int64_t K, double alpha, const void* A, int64_t lda,
                         const void* B, int64_t ldb, double beta, void* C, int64_t ldc) {
  if (!ctx || M < 0 || N < 0 || K < 0) return OFRR_ERR_INVALID_ARGUMENT;
  if (!dtype_valid(ta) || !dtype_valid(tb) || !dtype_valid(tout)) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (tcompute != OFRR_F64 && tcompute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  // gemm.m:84-89: FP64 output needs FP64 compute; F32 output needs >= F32 compute
  if (tout == OFRR_F64 && tcompute != OFRR_F64) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  const int64_t Ar = transA ? K : M, Br = transB ? N : K;
  if (M > 0 && N > 0 && K > 0) {
    if (!A || !B || lda < (Ar > 1 ? Ar : 1) || ldb < (Br > 1 ? Br : 1)) return OFRR_ERR_INVALID_ARGUMENT;
  }
  if (M > 0 && N > 0 && (!C || ldc < M)) return OFRR_ERR_INVALID_ARGUMENT;
  return gemm_impl(ctx, transA, transB, ta, tb, tcompute, tout, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
