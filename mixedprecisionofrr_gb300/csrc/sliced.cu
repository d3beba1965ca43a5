// Exact-slice FP64 emulation of dense products on the tcgen05 tensor cores (Ozaki-style splitting).
//
// The refinement phase of the mixed solver needs A V and A' U in FP64 accuracy; GB300 runs FP64
// at 1/64 of its FP32 rate, while BF16 tensor cores run at ~1 PFLOP/s.  Each FP64 operand column is
// scaled by a power of two (x = 2^e y, |y| < 1) and split into S signed digits of BETA bits,
// y = sum_s d_s 2^{-BETA (s+1)}, every d_s an integer with |d_s| <= 2^BETA, stored exactly in BF16.
// The product of two columns is then sum_{s,t} 2^{e_a + e_b - BETA (s+t+2)} (d_s . d'_t).  Terms with
// s + t = L share one scale, so the digits are stacked along K ([d_0; d_1; ...] against
// [d'_L; d'_{L-1}; ...]) and every level L <= LMAX is ONE tensor-core GEMM of depth (L+1) K.
// Integer products summed in FP32 are exact while the partial sum stays below 2^24: the GEMM is
// split along K into ranges short enough for that on the two leading levels (where an FP32 rounding
// would show), and the exact FP32 partials are combined and scaled in FP64.  Dropped terms
// (s + t > LMAX) and the digit truncation are below 2^-(BETA (LMAX+1)) relative.
#include "ofrr_internal.cuh"

#include <algorithm>
#include <vector>

namespace ofrr {

int tc_gemm_partials(ofrr_ctx* ctx, ofrr_dtype t16, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                     const void* B, int64_t ldb, int kblocks_per_split, float* partial, int* splits_out);

namespace slice {
constexpr int BETA = 7;  // digit width: |leading digit| <= 128, later digits <= 64
constexpr int S = 5;     // digits per operand (35 bits)
constexpr int LMAX = 4;  // levels kept: pairs with s + t <= 4 (15 of 25), error ~ 2^-35

// Digits of every column of X (K x N, column-major).  Stacked layout: column n occupies
// stack[(n * S + s) * Kp + k] for digit s; rows k >= K are zero.  expo[n] = exponent e_n.
__global__ void k_slice_cols(int64_t K, int64_t Kp, int64_t N, const double* __restrict__ X, int64_t ldx,
                             __nv_bfloat16* __restrict__ stack, int* __restrict__ expo) {
  __shared__ double red[32];
  __shared__ int s_e;
  for (int64_t n = blockIdx.x; n < N; n += gridDim.x) {
    const double* x = X + n * ldx;
    double mx = 0.0;
    for (int64_t k = threadIdx.x; k < K; k += blockDim.x) mx = fmax(mx, fabs(x[k]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
      int e = 0;
      if (m > 0.0) frexp(m, &e);  // m = f 2^e, f in [0.5, 1): |x| 2^-e < 1
      s_e = e;
      expo[n] = e;
    }
    __syncthreads();
    const int e = s_e;
    // fixed point: Y = round(x 2^(BETA S - e)), |Y| <= 2^35; digits by integer arithmetic (GB300's
    // FP64 pipe is 1/64 rate, so only one FP64 multiply and one conversion per element)
    __nv_bfloat16* col = stack + (size_t)n * S * Kp;
    for (int64_t k = threadIdx.x; k < Kp; k += blockDim.x) {
      long long r = (k < K) ? __double2ll_rn(ldexp(x[k], BETA * S - e)) : 0ll;
#pragma unroll
      for (int s = S - 1; s > 0; --s) {  // centred base-2^BETA digits, least significant first
        const long long d = ((r + (1 << (BETA - 1))) & ((1 << BETA) - 1)) - (1 << (BETA - 1));
        r = (r - d) >> BETA;  // exact: r - d is a multiple of 2^BETA
        col[(size_t)s * Kp + k] = __float2bfloat16_rn((float)d);  // |d| <= 64
      }
      col[k] = __float2bfloat16_rn((float)r);  // leading digit, |r| <= 128: exact in bf16
    }
    __syncthreads();
  }
}

// Level stacks of the second operand: for level L, column n holds [d_L; d_{L-1}; ...; d_0]
// (length (L+1) Kp), built from the digit stack of k_slice_cols.  Level L starts at offset
// off(L) = N Kp L (L+1) / 2.
__global__ void k_level_stacks(int64_t Kp, int64_t N, const __nv_bfloat16* __restrict__ digits,
                               __nv_bfloat16* __restrict__ levels) {
  const int64_t per = (int64_t)N * Kp;
  const int64_t total = per * (LMAX + 1) * (LMAX + 2) / 2;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    // locate level L and the position p inside column n
    int L = 0;
    int64_t base = 0;
    while (L < LMAX && e >= base + per * (L + 1)) {
      base += per * (L + 1);
      ++L;
    }
    const int64_t r = e - base;
    const int64_t len = (int64_t)(L + 1) * Kp;
    const int64_t n = r / len, q = r % len;
    const int p = (int)(q / Kp);
    const int64_t k = q % Kp;
    const int s = L - p;
    levels[e] = digits[((size_t)n * S + s) * Kp + k];
  }
}

// C (+)= 2^{ea_m + eb_n - shift} * sum_z P_z   (FP64)
__global__ void k_combine(int64_t M, int64_t N, int splits, const float* __restrict__ P, double* __restrict__ C,
                          int64_t ldc, const int* __restrict__ ea, const int* __restrict__ eb, int shift, int first) {
  const int64_t total = M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    // partials are integer-valued (digit products) below 2^31 in magnitude: sum them exactly as integers
    long long s = 0;
    for (int z = 0; z < splits; ++z) s += (long long)__float2ll_rn(P[(size_t)z * total + e]);
    const int64_t m = e % M, n = e / M;
    const double v = ldexp((double)s, ea[m] + eb[n] - shift);
    double* c = C + m + n * ldc;
    *c = first ? v : (*c + v);
  }
}

}  // namespace slice

static_assert(slice::S == kSliceDigits, "digit count");

// Digit stack of X (K x M, column-major FP64) into caller buffers (M * S * roundup(K, 64) bf16, M ints)
int sliced_prepare_into(ofrr_ctx* ctx, int64_t K, int64_t M, const double* X, int64_t ldx, __nv_bfloat16* stack,
                        int* expo, SlicedOperand* out) {
  out->K = K;
  out->Kp = (K + 63) / 64 * 64;
  out->M = M;
  out->stack = stack;
  out->expo = expo;
  const int grid = (int)std::min<int64_t>(M, 65535);
  slice::k_slice_cols<<<grid, 256, 0, ctx->stream>>>(K, out->Kp, M, X, ldx, out->stack, out->expo);
  OFRR_LAUNCHED(ctx, "k_slice_cols");
  return OFRR_SUCCESS;
}

// Build the digit stack of X (K x M, column-major FP64) in the workspace.
int sliced_prepare(ofrr_ctx* ctx, int64_t K, int64_t M, const double* X, int64_t ldx, SlicedOperand* out) {
  int st = OFRR_SUCCESS;
  const int64_t Kp = (K + 63) / 64 * 64;
  __nv_bfloat16* stack = ws_get<__nv_bfloat16>(ctx, (size_t)M * slice::S * Kp, &st);
  if (!stack) return st;
  int* expo = ws_get<int>(ctx, (size_t)M, &st);
  if (!expo) return st;
  return sliced_prepare_into(ctx, K, M, X, ldx, stack, expo, out);
}

// C (M x N, FP64) = A_op' B with A_op the prepared stack (K x M) and B (K x N, FP64, column-major)
int sliced_gemm_tn(ofrr_ctx* ctx, const SlicedOperand& A, int64_t N, const double* B, int64_t ldb, double* C,
                   int64_t ldc) {
  using namespace slice;
  const int64_t K = A.K, Kp = A.Kp, M = A.M;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  SlicedOperand Bs;
  OFRR_TRY(sliced_prepare(ctx, K, N, B, ldb, &Bs));
  __nv_bfloat16* levels = ws_get<__nv_bfloat16>(ctx, (size_t)N * Kp * (LMAX + 1) * (LMAX + 2) / 2, &st);
  if (!levels) return st;
  slice::k_level_stacks<<<grid_for(N * Kp * 15, 256, 4096), 256, 0, ctx->stream>>>(Kp, N, Bs.stack, levels);
  OFRR_LAUNCHED(ctx, "k_level_stacks");
  // partial buffer: largest split count over the levels
  const int64_t kb = Kp / 64;
  const int tiles = (int)(((M + 127) / 128) * ((N + 63) / 64));
  std::vector<int> kbps(LMAX + 1);
  int max_splits = 1;
  for (int L = 0; L <= LMAX; ++L) {
    const int64_t kbl = kb * (L + 1);
    // exact ranges on the two leading levels: |d_s d_t| <= 2^14 (L = 0), 2^13 (L = 1); 2^24 bound
    int64_t lim = (L == 0) ? (1 << 10) / 64 : (L == 1 ? (1 << 11) / 64 : kbl);
    int64_t per = std::min<int64_t>(lim, kbl);
    // at least ~one wave of CTAs
    while (tiles * ((kbl + per - 1) / per) < 148 && per > 2) per = (per + 1) / 2;
    kbps[L] = (int)per;
    max_splits = std::max<int>(max_splits, (int)((kbl + per - 1) / per));
  }
  float* P = ws_get<float>(ctx, (size_t)max_splits * M * N, &st);
  if (!P) return st;
  for (int L = 0; L <= LMAX; ++L) {
    const __nv_bfloat16* Bl = levels + (size_t)N * Kp * L * (L + 1) / 2;
    int splits = 0;
    OFRR_TRY(tc_gemm_partials(ctx, OFRR_BF16, M, N, (L + 1) * Kp, A.stack, S * Kp, Bl, (L + 1) * Kp, kbps[L], P,
                              &splits));
    slice::k_combine<<<grid_for(M * N, 256, 2048), 256, 0, ctx->stream>>>(M, N, splits, P, C, ldc, A.expo, Bs.expo,
                                                                         BETA * (L + 2), L == 0 ? 1 : 0);
    OFRR_LAUNCHED(ctx, "k_combine");
  }
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

// C ABI wrapper used by the tests: C = A' B in emulated FP64 (A: K x M, B: K x N, all FP64, column-major)
extern "C" int ofrr_gemm_f64_emulated(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                                      const double* B, int64_t ldb, double* C, int64_t ldc) {
  if (!ctx || M < 0 || N < 0 || K < 0) return OFRR_ERR_INVALID_ARGUMENT;
  if (M == 0 || N == 0) return OFRR_SUCCESS;
  if (!A || !B || !C || lda < K || ldb < K || ldc < M || K < 1) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  SlicedOperand As;
  OFRR_TRY(sliced_prepare(ctx, K, M, A, lda, &As));
  return sliced_gemm_tn(ctx, As, N, B, ldb, C, ldc);
}
