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
