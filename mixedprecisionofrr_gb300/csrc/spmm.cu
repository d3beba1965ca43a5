// CSR operator applications: Y = op(A) X for a block of right-hand sides.
//
// Behaviour: MATLAB/+src/+csr/csrmv.m:27-78 -- the value copy of the compute precision is used
// (sparse2csr.m:48-49), products are accumulated in that precision and the result is stored in
// the output type.
//
// Layout ('N'): a CTA owns 256 consecutive rows, one per thread.  The CTA's nonzeros (a contiguous
// range of the value and index arrays) are first copied into shared memory with coalesced loads, so
// the CSR arrays are read from HBM once for all right-hand sides; each thread then walks its row in
// shared memory for every chunk of RC columns.  For stencil operators consecutive rows touch
// consecutive columns, so a warp's gathers of X are coalesced.  CTAs whose nonzeros exceed the staging
// capacity read them from global memory instead (same arithmetic, same order).
// 'T' applies the 'N' kernel to the transpose, built once per call (or once per solve, Op::prepare_csr_t)
// with a deterministic counting sort, so results never depend on the schedule (no floating-point
// atomics).
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

constexpr int kSpmmRows = 256;
constexpr int kSpmmCap = 2048;  // staged nonzeros per CTA (8 per row on average)

template <class TX, class TC, class TY, int RC>
__global__ void __launch_bounds__(kSpmmRows) k_csrmm_n(int64_t nrows, const int32_t* __restrict__ indptr,
                                                       const int32_t* __restrict__ indices,
                                                       const TC* __restrict__ vals, int64_t nrhs,
                                                       const TX* __restrict__ X, int64_t ldx, TY* __restrict__ Y,
                                                       int64_t ldy, int nchunks) {
  __shared__ TC s_val[kSpmmCap];
  __shared__ int32_t s_idx[kSpmmCap];
  // CTA b: row block b / nchunks, right-hand sides [RC (b % nchunks), ...) -- the CTAs of one row block are
  // adjacent, so the block's nonzeros are read from HBM once and from L2 by the others
  const int64_t r0 = (int64_t)(blockIdx.x / nchunks) * kSpmmRows;
  const int64_t cbeg = (nchunks > 1) ? (int64_t)(blockIdx.x % nchunks) * RC : 0;
  const int64_t cend = (nchunks > 1) ? min(nrhs, cbeg + RC) : nrhs;
  if (r0 >= nrows) return;
  const int64_t rend = min(nrows, r0 + kSpmmRows);
  const int32_t pbase = __ldg(indptr + r0), pend = __ldg(indptr + rend);
  const bool staged = (pend - pbase) <= kSpmmCap;
  if (staged) {
    for (int32_t e = threadIdx.x; e < pend - pbase; e += kSpmmRows) {
      s_val[e] = __ldg(vals + pbase + e);
      s_idx[e] = __ldg(indices + pbase + e);
    }
  }
  __syncthreads();
  const int64_t row = r0 + threadIdx.x;
  if (row >= rend) return;
  const int32_t p0 = __ldg(indptr + row), p1 = __ldg(indptr + row + 1);
  for (int64_t c0 = cbeg; c0 < cend; c0 += RC) {
    TC acc[RC];
#pragma unroll
    for (int r = 0; r < RC; ++r) acc[r] = TC(0);
    for (int32_t p = p0; p < p1; ++p) {
      const int64_t col = staged ? s_idx[p - pbase] : __ldg(indices + p);
      const TC a = staged ? s_val[p - pbase] : __ldg(vals + p);
#pragma unroll
      for (int r = 0; r < RC; ++r) {
        if (c0 + r < cend) acc[r] = fma(a, to_c<TC, TX>(X[col + (c0 + r) * ldx]), acc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < RC; ++r)
      if (c0 + r < cend) Y[row + (c0 + r) * ldy] = from_c<TY, TC>(acc[r]);
  }
}

// ---- deterministic CSR transpose -------------------------------------------------------------
__global__ void k_csrt_count(int64_t nnz, const int32_t* __restrict__ indices, int32_t* __restrict__ cnt) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[indices[p]], 1);  // integer counts: the result does not depend on the order
}

// exclusive scan of n counts into out (n + 1 entries) by one CTA of 1024 threads, chunk by chunk
__global__ void __launch_bounds__(1024) k_csrt_scan(int64_t n, const int32_t* __restrict__ cnt,
                                                    int32_t* __restrict__ out) {
  __shared__ int32_t s[1024];
  __shared__ int32_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const int32_t v = (i < n) ? cnt[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan
      const int32_t t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) out[i] = s_carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 0) s_carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = s_carry;
}

// each nonzero (row i, column j) goes to column j's segment; rows taken in order by one thread per row
// chunk would serialise, so the slot comes from an atomic cursor and each segment is sorted afterwards
__global__ void k_csrt_fill(int64_t nrows, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                            const int32_t* __restrict__ colptr, int32_t* __restrict__ cursor,
                            int32_t* __restrict__ rowidx, int32_t* __restrict__ src) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    for (int32_t p = indptr[r]; p < indptr[r + 1]; ++p) {
      const int32_t j = indices[p];
      const int32_t slot = colptr[j] + atomicAdd(&cursor[j], 1);
      rowidx[slot] = (int32_t)r;
      src[slot] = p;
    }
  }
}

// sort each column segment by row (insertion sort: segments of sparse operators are short), carrying
// the source position; then gather the values of every precision present
__global__ void k_csrt_sort(int64_t ncols, const int32_t* __restrict__ colptr, int32_t* __restrict__ rowidx,
                            int32_t* __restrict__ src) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < ncols; j += (int64_t)gridDim.x * blockDim.x) {
    const int32_t b = colptr[j], e = colptr[j + 1];
    for (int32_t p = b + 1; p < e; ++p) {
      const int32_t r = rowidx[p], sp = src[p];
      int32_t q = p - 1;
      while (q >= b && rowidx[q] > r) {
        rowidx[q + 1] = rowidx[q];
        src[q + 1] = src[q];
        --q;
      }
      rowidx[q + 1] = r;
      src[q + 1] = sp;
    }
  }
}

template <class TV>
__global__ void k_csrt_gather(int64_t nnz, const int32_t* __restrict__ src, const TV* __restrict__ v,
                              TV* __restrict__ vt) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x)
    vt[p] = v[src[p]];
}

int csr_transpose_impl(ofrr_ctx* ctx, const ofrr_csr* A, ofrr_csr* At) {
  int st = OFRR_SUCCESS;
  const int64_t m = A->nrows, n = A->ncols, nnz = A->nnz;
  *At = ofrr_csr{};
  At->nrows = n;
  At->ncols = m;
  At->nnz = nnz;
  int32_t* colptr = ws_get<int32_t>(ctx, (size_t)n + 1, &st);
  int32_t* cursor = ws_get<int32_t>(ctx, (size_t)n + 1, &st);
  int32_t* rowidx = ws_get<int32_t>(ctx, (size_t)std::max<int64_t>(nnz, 1), &st);
  int32_t* src = ws_get<int32_t>(ctx, (size_t)std::max<int64_t>(nnz, 1), &st);
  if (!colptr || !cursor || !rowidx || !src) return st;
  OFRR_TRY(fill_zero(ctx, cursor, sizeof(int32_t) * ((size_t)n + 1)));
  const int g = grid_for(std::max<int64_t>(nnz, 1), 256, 152 * 16);
  if (nnz > 0) {
    k_csrt_count<<<g, 256, 0, ctx->stream>>>(nnz, A->indices, cursor);
    OFRR_LAUNCHED(ctx, "k_csrt_count");
  }
  k_csrt_scan<<<1, 1024, 0, ctx->stream>>>(n, cursor, colptr);
  OFRR_LAUNCHED(ctx, "k_csrt_scan");
  OFRR_TRY(fill_zero(ctx, cursor, sizeof(int32_t) * ((size_t)n + 1)));
  if (nnz > 0) {
    k_csrt_fill<<<grid_for(m, 256, 152 * 16), 256, 0, ctx->stream>>>(m, A->indptr, A->indices, colptr,
                                                                             cursor, rowidx, src);
    OFRR_LAUNCHED(ctx, "k_csrt_fill");
    k_csrt_sort<<<grid_for(n, 256, 152 * 16), 256, 0, ctx->stream>>>(n, colptr, rowidx, src);
    OFRR_LAUNCHED(ctx, "k_csrt_sort");
  }
  At->indptr = colptr;
  At->indices = rowidx;
  if (A->a_double) {
    double* v = ws_get<double>(ctx, (size_t)std::max<int64_t>(nnz, 1), &st);
    if (!v) return st;
    if (nnz > 0) {
      k_csrt_gather<double><<<g, 256, 0, ctx->stream>>>(nnz, src, A->a_double, v);
      OFRR_LAUNCHED(ctx, "k_csrt_gather");
    }
    At->a_double = v;
  }
  if (A->a_single) {
    float* v = ws_get<float>(ctx, (size_t)std::max<int64_t>(nnz, 1), &st);
    if (!v) return st;
    if (nnz > 0) {
      k_csrt_gather<float><<<g, 256, 0, ctx->stream>>>(nnz, src, A->a_single, v);
      OFRR_LAUNCHED(ctx, "k_csrt_gather");
    }
    At->a_single = v;
  }
  if (A->a_half) {
    __half* v = ws_get<__half>(ctx, (size_t)std::max<int64_t>(nnz, 1), &st);
    if (!v) return st;
    if (nnz > 0) {
      k_csrt_gather<__half><<<g, 256, 0, ctx->stream>>>(nnz, src, (const __half*)A->a_half, v);
      OFRR_LAUNCHED(ctx, "k_csrt_gather");
    }
    At->a_half = v;
  }
  return OFRR_SUCCESS;
}

static int csrmm_n(ofrr_ctx* ctx, const ofrr_csr* A, ofrr_dtype tx, ofrr_dtype tc, ofrr_dtype ty, int64_t nrhs,
                   const void* X, int64_t ldx, void* Y, int64_t ldy) {
  const int64_t blocks = (A->nrows + kSpmmRows - 1) / kSpmmRows;
  // many right-hand sides: one CTA per (row block, 8-column chunk), for more loads in flight per SM
  const int nchunks = (nrhs > 8) ? (int)((nrhs + 7) / 8) : 1;
  if (blocks * nchunks > 0x7fffffffLL) return OFRR_ERR_BLAS_INVALID_SIZE;
  const unsigned grid = (unsigned)(blocks * nchunks);
  OFRR_DISPATCH_COMPUTE(tc, TC, {
    const TC* vals = CsrVals<TC>::get(A);
    if (!vals) return OFRR_ERR_INVALID_ARGUMENT;
    OFRR_DISPATCH_STORAGE(tx, TX, OFRR_DISPATCH_STORAGE(ty, TY, {
      if (nrhs == 1) {
        k_csrmm_n<TX, TC, TY, 1><<<grid, kSpmmRows, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs,
                                                                      (const TX*)X, ldx, (TY*)Y, ldy, nchunks);
      } else if (nrhs <= 4) {
        k_csrmm_n<TX, TC, TY, 4><<<grid, kSpmmRows, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs,
                                                                      (const TX*)X, ldx, (TY*)Y, ldy, nchunks);
      } else {
        k_csrmm_n<TX, TC, TY, 8><<<grid, kSpmmRows, 0, ctx->stream>>>(A->nrows, A->indptr, A->indices, vals, nrhs,
                                                                      (const TX*)X, ldx, (TY*)Y, ldy, nchunks);
      }
      OFRR_LAUNCHED(ctx, "k_csrmm_n");
    }));
  });
  return OFRR_SUCCESS;
}

int csrmm_impl(ofrr_ctx* ctx, const ofrr_csr* A, int trans, ofrr_dtype tx, ofrr_dtype tc, ofrr_dtype ty,
               int64_t nrhs, const void* X, int64_t ldx, void* Y, int64_t ldy) {
  if (nrhs <= 0) return OFRR_SUCCESS;
  const int64_t nout = trans ? A->ncols : A->nrows;
  if (nout <= 0) return OFRR_SUCCESS;
  if (!trans) return csrmm_n(ctx, A, tx, tc, ty, nrhs, X, ldx, Y, ldy);
  // transposed: the 'N' product of the transpose (same arithmetic per output entry in a fixed order)
  WsScope scope(ctx);
  ofrr_csr At;
  OFRR_TRY(csr_transpose_impl(ctx, A, &At));
  return csrmm_n(ctx, &At, tx, tc, ty, nrhs, X, ldx, Y, ldy);
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
