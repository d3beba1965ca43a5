// Column-pivoted LU basis, MATLAB/+src/+qr/lu.m:47-94, on the GPU.  Right-looking with the rows of
// the working copy W swapped in place, as the MATLAB code does, so the pivot of column j is the first
// maximum of |W(j:m, j)| in the current row order; a column whose maximum is below select_tol is
// dropped (its row j is consumed all the same, U(j, j:n) keeps the row).  Per column one single-CTA
// kernel (pivot search, swaps, select flag, U row, L column) and one trailing-update kernel over all
// SMs; the select decision stays on the device (no host synchronisation per column).  Every operation
// is element-wise or an exact argmax with MATLAB's tie rule, so the result equals the oracle's
// restatement bit for bit.  The basis leaves in the solvers' contract: Q(r, j) = L(position of row r,
// j) (the un-permuted L of lu.m's two-output form), dropped columns zero, select flags, R = U.
#include <vector>

#include "ofrr_internal.cuh"

namespace ofrr {
namespace {

constexpr int LU_T = 1024;

// step j: pivot, swaps, U(j, j:n), L(j:m, j); sel[j] = 0 for a dropped column
template <class TO, class TC>
__global__ void __launch_bounds__(LU_T) k_lu_pivot(int64_t m, int64_t n, int64_t j, TO* __restrict__ W,
                                                   TO* __restrict__ Lm, int* __restrict__ perm, double* __restrict__ U,
                                                   int* __restrict__ sel, double stol) {
  __shared__ ArgMaxK red[LU_T / 32];
  __shared__ int s_p;
  __shared__ bool s_keep;
  TO* wj = W + j * m;  // column j of W
  ArgMaxK a{-1, 0x7fffffffffffffffLL};
  for (int64_t r = j + threadIdx.x; r < m; r += LU_T) {  // rows ascend per thread: strict > keeps the first
    const long long key = amax_key(wj[r]);
    if (key > a.key) a = ArgMaxK{key, r};
  }
  const ArgMaxK b = block_argmaxk(a, red);
  if (threadIdx.x == 0) {
    const int64_t p = (b.key < 0) ? j : b.i;
    const double mx = fabs((double)to_c<double, TO>(wj[p]));
    s_keep = !(mx < stol);  // a NaN maximum keeps the column, as max() in lu.m does
    s_p = (int)p;
    sel[j] = s_keep ? 1 : 0;
  }
  __syncthreads();
  const int64_t p = s_p;
  if (s_keep && p != j) {  // swap rows j and p of W (all columns) and of L (columns < j), and perm
    for (int64_t c = threadIdx.x; c < n; c += LU_T) {
      const TO t = W[j + c * m];
      W[j + c * m] = W[p + c * m];
      W[p + c * m] = t;
      if (c < j) {
        const TO u = Lm[j + c * m];
        Lm[j + c * m] = Lm[p + c * m];
        Lm[p + c * m] = u;
      }
    }
    if (threadIdx.x == 0) {
      const int t = perm[j];
      perm[j] = perm[p];
      perm[p] = t;
    }
  }
  __syncthreads();
  for (int64_t c = j + threadIdx.x; c < n; c += LU_T) U[j + c * n] = (double)to_c<double, TO>(W[j + c * m]);
  if (!s_keep) return;
  const TC piv = to_c<TC, TO>(wj[j]);
  for (int64_t r = j + threadIdx.x; r < m; r += LU_T) Lm[r + j * m] = from_c<TO, TC>(div_rn(to_c<TC, TO>(wj[r]), piv));
}

// W(i, c) = po(pc(W(i, c)) - pc(L(i, j)) pc(W(j, c))) for i > j, c > j (kept columns only)
template <class TO, class TC>
__global__ void k_lu_update(int64_t m, int64_t n, int64_t j, TO* __restrict__ W, const TO* __restrict__ Lm,
                            const int* __restrict__ sel) {
  if (!sel[j]) return;
  const int64_t rows = m - j - 1;
  OFRR_FOR_2D(ii, cc, rows, n - j - 1) {
    const int64_t i = j + 1 + ii, c = j + 1 + cc;
    const TC p = mul_rn(to_c<TC, TO>(Lm[i + j * m]), to_c<TC, TO>(W[j + c * m]));
    W[i + c * m] = from_c<TO, TC>(sub_rn(to_c<TC, TO>(W[i + c * m]), p));
  }
}

// Q(perm[k], c) = L(k, c) for kept columns, 0 for dropped ones
template <class TO>
__global__ void k_lu_unpermute(int64_t m, int64_t n, const TO* __restrict__ Lm, const int* __restrict__ perm,
                               const int* __restrict__ sel, TO* __restrict__ Q, int64_t ldq) {
  OFRR_FOR_2D(k, c, m, n) Q[perm[k] + c * ldq] = sel[c] ? Lm[k + c * m] : TO(0);
}

__global__ void k_iota(int64_t m, int* __restrict__ perm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    perm[i] = (int)i;
}

}  // namespace

int lu_basis_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n, const void* A,
                  int64_t lda, void* Q, int64_t ldq, double select_tol, double* R_dev, int* select_dev) {
  if (n <= 0 || m <= 0) return OFRR_SUCCESS;
  if (m < n) return OFRR_ERR_BLAS_INVALID_SIZE;  // lu.m:50 asserts a tall-thin A
  if (m > 0x7fffffffLL) return OFRR_ERR_BLAS_INVALID_SIZE;
  double stol = select_tol < 0 ? dtype_eps(tout) : select_tol;
  stol = (tout == OFRR_F32) ? (double)(float)stol
       : (tout == OFRR_F16) ? (double)__half2float(__double2half(stol))
       : (tout == OFRR_BF16) ? (double)__bfloat162float(__double2bfloat16(stol)) : stol;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const size_t es = dtype_size(tout);
  void* W = ws_alloc(ctx, (size_t)m * n * es, &st);
  void* Lm = ws_alloc(ctx, (size_t)m * n * es, &st);
  int* perm = ws_get<int>(ctx, (size_t)m, &st);
  if (!W || !Lm || !perm) return st;
  OFRR_TRY(cast_impl(ctx, tin, tout, m, n, A, lda, W, m));  // A_work = precision_output(A)
  OFRR_CUDA(cudaMemsetAsync(Lm, 0, (size_t)m * n * es, ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(R_dev, 0, sizeof(double) * n * n, ctx->stream));
  k_iota<<<(unsigned)std::min<int64_t>((m + 255) / 256, 1024), 256, 0, ctx->stream>>>(m, perm);
  OFRR_LAUNCHED(ctx, "k_iota");
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    for (int64_t j = 0; j < n; ++j) {
      k_lu_pivot<TO, TC><<<1, LU_T, 0, ctx->stream>>>(m, n, j, (TO*)W, (TO*)Lm, perm, R_dev, select_dev, stol);
      OFRR_LAUNCHED(ctx, "k_lu_pivot");
      if (j + 1 < n) {
        k_lu_update<TO, TC><<<grid_2d(m - j - 1, n - j - 1, 256), 256, 0, ctx->stream>>>(m, n, j, (TO*)W,
                                                                                        (const TO*)Lm, select_dev);
        OFRR_LAUNCHED(ctx, "k_lu_update");
      }
    }
    k_lu_unpermute<TO><<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, (const TO*)Lm, perm, select_dev, (TO*)Q, ldq);
    OFRR_LAUNCHED(ctx, "k_lu_unpermute");
  }));
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_lu_basis(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute, int64_t m, int64_t n,
                             const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol, double* U_host,
                             int* skip_host) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(tin) || !dtype_valid(tout)) return OFRR_ERR_INVALID_ARGUMENT;
  if (tcompute != OFRR_F64 && tcompute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (m < n) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (n == 0) return OFRR_SUCCESS;
  if (!A || !Q || lda < m || ldq < m) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double* R = ws_get<double>(ctx, (size_t)n * n, &st);
  int* sel = ws_get<int>(ctx, (size_t)n, &st);
  if (!R || !sel) return st;
  OFRR_TRY(lu_basis_impl(ctx, tin, tout, tcompute, m, n, A, lda, Q, ldq, select_tol, R, sel));
  std::vector<int> hsel((size_t)n);
  OFRR_CUDA(cudaMemcpyAsync(hsel.data(), sel, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (U_host) OFRR_CUDA(cudaMemcpyAsync(U_host, R, sizeof(double) * n * n, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  if (skip_host)
    for (int64_t j = 0; j < n; ++j) skip_host[j] = hsel[(size_t)j] ? 0 : 1;
  return OFRR_SUCCESS;
}
