// Cast + transpose of a column-major matrix through 32 x 33 shared-memory tiles (coalesced on
// both sides).  Used once per solve to keep a K-contiguous copy of the fixed operator A, so that
// A V runs on the tcgen05 TN kernel like every other contraction.
#include "ofrr_internal.cuh"

#include <algorithm>
#include <type_traits>

namespace ofrr {

template <class TI, class TO>
__global__ void k_cast_transpose(int64_t m, int64_t n, const TI* __restrict__ in, int64_t ldin, TO* __restrict__ out,
                                 int64_t ldout) {
  // staged in FP32 unless a side is FP64 (every 16/32-bit value is a float; one rounding either way)
  using TT = typename std::conditional<std::is_same<TI, double>::value || std::is_same<TO, double>::value, double,
                                       float>::type;
  __shared__ TT tile[32][33];
  for (int64_t bj = blockIdx.y; bj * 32 < n; bj += gridDim.y) {
    for (int64_t bi = blockIdx.x; bi * 32 < m; bi += gridDim.x) {
      const int64_t i0 = bi * 32, j0 = bj * 32;
      for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, j = j0 + r;
        tile[r][threadIdx.x] = (i < m && j < n) ? to_c<TT, TI>(in[i + j * ldin]) : TT(0);
      }
      __syncthreads();
      for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t j = j0 + threadIdx.x, i = i0 + r;  // out(j, i) = in(i, j)
        if (i < m && j < n) out[j + i * ldout] = from_c<TO, TT>(tile[threadIdx.x][r]);
      }
      __syncthreads();
    }
  }
}

// out (n x m, column-major, ldout >= n) = tout(in') for in (m x n, column-major)
int cast_transpose_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, int64_t m, int64_t n, const void* in,
                        int64_t ldin, void* out, int64_t ldout) {
  if (m <= 0 || n <= 0) return OFRR_SUCCESS;
  dim3 block(32, 8);
  dim3 grid((unsigned)std::min<int64_t>((m + 31) / 32, 1024), (unsigned)std::min<int64_t>((n + 31) / 32, 1024));
  OFRR_DISPATCH_STORAGE(tin, TI, OFRR_DISPATCH_STORAGE(tout, TO, {
    k_cast_transpose<TI, TO><<<grid, block, 0, ctx->stream>>>(m, n, (const TI*)in, ldin, (TO*)out, ldout);
    OFRR_LAUNCHED(ctx, "k_cast_transpose");
  }));
  return OFRR_SUCCESS;
}

}  // namespace ofrr
