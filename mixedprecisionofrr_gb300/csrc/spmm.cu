// CSR operator applications: Y = op(A) X for a block of right-hand sides.
//
// Behaviour: MATLAB/+src/+csr/csrmv.m:27-78 -- the value copy of the compute precision is used
// (sparse2csr.m:48-49), products are accumulated in that precision and the result is stored in
// the output type.  Layout: thread per row, right-hand sides in register chunks of RC columns;
// for stencil matrices consecutive rows touch consecutive columns, so a warp's gathers of X are
// coalesced, and the row's nonzeros are read once per chunk.  'T' is a scatter with atomics.
#include "ofrr_internal.cuh"

namespace ofrr {

template <class TC> struct CsrVals;
template <> struct CsrVals<double> {
  static const double* get(const ofrr_csr* A) { return A->a_double; }
  using T = double;
};
template <> struct CsrVals<float> {
  static const float* get(const ofrr_csr* A) { return A->a_single; }
  using T = float;
};

template <class TX, class TC, class TY, int RC>
__global__ void __launch_bounds__(256) k_csrmm_n(int64_t nrows, const int32_t* __restrict__ indptr,
                                                 const int32_t* __restrict__ indices, const TC* __restrict__ vals,
                                                 int64_t nrhs, const TX* __restrict__ X, int64_t ldx,
                                                 TY* __restrict__ Y, int64_t ldy) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < nrows; row += stride) {
    const int32_t p0 = __ldg(indptr + row), p1 = __ldg(indptr + row + 1);
    for (int64_t c0 = 0; c0 < nrhs; c0 += RC) {
      TC acc[RC];
#pragma unroll
      for (int r = 0; r < RC; ++r) acc[r] = TC(0);
      for (int32_t p = p0; p < p1; ++p) {
        const int64_t col = __ldg(indices + p);
        const TC a = __ldg(vals + p);
#pragma unroll
        for (int r = 0; r < RC; ++r) {
          if (c0 + r < nrhs) acc[r] = fma(a, to_c<TC, TX>(X[col + (c0 + r) * ldx]), acc[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < RC; ++r)
        if (c0 + r < nrhs) Y[row + (c0 + r) * ldy] = from_c<TY, TC>(acc[r]);
    }
  }
}

template <class TX, class TC>
__global__ void k_csrmm_t(int64_t nrows, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                          const TC* __restrict__ vals, int64_t nrhs, const TX* __restrict__ X, int64_t ldx,
                          TC* __restrict__ Yacc, int64_t ldy) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < nrows; row += stride) {
    const int32_t p0 = indptr[row], p1 = indptr[row + 1];
    for (int64_t c = 0; c < nrhs; ++c) {
      const TC x = to_c<TC, TX>(X[row + c * ldx]);
      for (int32_t p = p0; p < p1; ++p) atomicAdd(&Yacc[indices[p] + c * ldy], vals[p] * x);
    }
  }
}

int csrmm_impl(ofrr_ctx* ctx, const ofrr_csr* A, int trans, ofrr_dtype tx, ofrr_dtype tc, ofrr_dtype ty,
               int64_t nrhs, const void* X, int64_t ldx, void* Y, int64_t ldy) {
  if (nrhs <= 0) return OFRR_SUCCESS;
  const int64_t nout = trans ? A->ncols : A->nrows;
  if (nout <= 0) return OFRR_SUCCESS;
  const int block = 256;
  if (!trans) {
    const int grid = grid_for(A->nrows, block, 1 << 20);
    OFRR_DISPATCH_COMPUTE(tc, TC, {
      const TC* vals = CsrVals<TC>::get(A);
      if (!vals) return OFRR_ERR_INVALID_ARGUMENT;
      OFRR_DISPATCH_STORAGE(tx, TX, OFRR_DISPATCH_STORAGE(ty, TY, {
        if (nrhs == 1) {
          k_csrmm_n<TX, TC, TY, 1><<<grid, block, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs,
                                                                      (const TX*)X, ldx, (TY*)Y, ldy);
        } else if (nrhs <= 4) {
          k_csrmm_n<TX, TC, TY, 4><<<grid, block, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs,
                                                                      (const TX*)X, ldx, (TY*)Y, ldy);
        } else {
          k_csrmm_n<TX, TC, TY, 8><<<grid, block, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs,
                                                                      (const TX*)X, ldx, (TY*)Y, ldy);
        }
        OFRR_LAUNCHED(ctx, "k_csrmm_n");
      }));
    });
    return OFRR_SUCCESS;
  }
  // transposed: accumulate in the compute type, then store
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  void* acc = ws_alloc(ctx, (size_t)nout * nrhs * dtype_size(tc), &st);
  if (!acc) return st;
  OFRR_TRY(fill_zero(ctx, acc, (size_t)nout * nrhs * dtype_size(tc)));
  const int grid = grid_for(A->nrows, block, 1 << 20);
  OFRR_DISPATCH_COMPUTE(tc, TC, {
    const TC* vals = CsrVals<TC>::get(A);
    if (!vals) return OFRR_ERR_INVALID_ARGUMENT;
    OFRR_DISPATCH_STORAGE(tx, TX, {
      k_csrmm_t<TX, TC><<<grid, block, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs, (const TX*)X,
                                                          ldx, (TC*)acc, nout);
      OFRR_LAUNCHED(ctx, "k_csrmm_t");
    });
  });
  return cast_impl(ctx, tc, ty, nout, nrhs, acc, nout, Y, ldy);
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_csrmm(ofrr_ctx* ctx, const ofrr_csr* A, int trans, ofrr_dtype tx, ofrr_dtype tcompute,
                          ofrr_dtype ty, int64_t nrhs, const void* X, int64_t ldx, void* Y, int64_t ldy) {
  if (!ctx || !A || nrhs < 0 || A->nrows < 0 || A->ncols < 0) return OFRR_ERR_INVALID_ARGUMENT;
  if (!dtype_valid(tx) || !dtype_valid(ty)) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (tcompute != OFRR_F64 && tcompute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  const int64_t nin = trans ? A->nrows : A->ncols, nout = trans ? A->ncols : A->nrows;
  if (nrhs > 0 && nout > 0 && (!X || !Y || !A->indptr || (A->nnz > 0 && !A->indices) || ldx < nin || ldy < nout))
    return OFRR_ERR_INVALID_ARGUMENT;
  return csrmm_impl(ctx, A, trans, tx, tcompute, ty, nrhs, X, ldx, Y, ldy);
}
