// Test-problem generators on the GPU: point sets (MATLAB/+src/+kernel/generate_pts.m, and the uniform
// box of CPP/testproblems/gaussian_kernel.hpp:36-40) and Gaussian kernel matrices, in the C++ form
// generate_gaussian_kernel (gaussian_kernel.hpp:14-77: diagonal f^2 (1 + s^2), off-diagonal
// f^2 exp(-|x_i - x_j|^2 / (2 l^2)), 0 where the exponent is below -700) and the MATLAB form
// gaussian.m:21-27 (D2 = -2 X Y' + |x|^2 + |y|^2, K = f^2 exp(-D2 / (2 l^2)) + s^2 eye).
// Points: the reference draws with its own generators (std / MATLAB rand), which cannot be reproduced;
// here uniform draws come from the library's counter-based generator: u(e) = (splitmix64(key + e) >>
// 11) 2^-53 with key = splitmix64(seed), e = row + n * (draw index), so the oracle gives the same
// values.  Every kernel value is computed in FP64 with the reference's operation order (no fused
// multiply-add), then rounded once to the output type; the matrix is written once (HBM-bound for
// small d, FP64-pipe-bound in exp otherwise).
#include <cmath>

#include "ofrr_internal.cuh"

namespace ofrr {
namespace {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double unif(uint64_t key, uint64_t e) {
  return (double)(mix64(key + e) >> 11) * 0x1p-53;
}

// type 0 / 20 / 30: box u * scale (scale = n^(1/d)); 21: disk; 22: circle; 23: grid; 31: ball;
// 32: sphere (generate_pts.m).  radius: the type's radius constant computed on the host.
__global__ void k_points(uint64_t key, int64_t n, int d, int type, double scale, double* __restrict__ X,
                         int64_t ldx) {
  const double two_pi = 6.283185307179586;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t e = (uint64_t)i, nn = (uint64_t)n;
    if (type == 0 || type == 20 || type == 30) {
      for (int k = 0; k < d; ++k) X[i + k * ldx] = __dmul_rn(scale, unif(key, e + nn * (uint64_t)k));
    } else if (type == 21 || type == 22) {
      const double theta = __dmul_rn(two_pi, unif(key, e));
      const double r = (type == 21) ? __dmul_rn(scale, sqrt(unif(key, e + nn))) : scale;
      X[i] = __dmul_rn(r, sin(theta));
      X[i + ldx] = __dmul_rn(r, cos(theta));
    } else if (type == 23) {
      const int64_t nx = (int64_t)llround(sqrt((double)n));
      X[i] = (double)(i % nx + 1);
      X[i + ldx] = (double)(i / nx + 1);
    } else {  // 31, 32: sph2cart(azimuth, asin(2u - 1), r)
      const double el = asin(__dsub_rn(__dmul_rn(2.0, unif(key, e)), 1.0));
      const double az = __dmul_rn(two_pi, unif(key, e + nn));
      const double r = (type == 31) ? __dmul_rn(scale, cbrt(unif(key, e + 2 * nn))) : scale;
      const double rc = __dmul_rn(r, cos(el));
      X[i] = __dmul_rn(rc, cos(az));
      X[i + ldx] = __dmul_rn(rc, sin(az));
      X[i + 2 * ldx] = __dmul_rn(r, sin(el));
    }
  }
}

// generate_gaussian_kernel's value at (i, j), i != j (symmetric in i, j bit for bit: the squared
// differences do not depend on the order of the two points)
__device__ __forceinline__ double gauss_cpp(const double* __restrict__ X, int64_t ldx, int d, int64_t i, int64_t j,
                                            double l2x2, double f2) {
  double dist = 0.0;
  for (int k = 0; k < d; ++k) {
    const double diff = __dsub_rn(X[i + k * ldx], X[j + k * ldx]);
    dist = __dadd_rn(dist, __dmul_rn(diff, diff));
  }
  const double arg = __ddiv_rn(-dist, l2x2);
  return (arg < -700.0) ? 0.0 : __dmul_rn(exp(arg), f2);
}

// The symmetric form by 32 x 32 tile pairs (bi <= bj): each value computed once (the FP64 divide and
// exp bound this kernel), staged in shared memory and written to both K(bi, bj) and K(bj, bi) with
// coalesced column stores.
template <class TO>
__global__ void __launch_bounds__(256) k_gauss_sym(int64_t n, int d, const double* __restrict__ X, int64_t ldx,
                                                   double l2x2, double f2, double s, TO* __restrict__ K,
                                                   int64_t ldk) {
  const int64_t bi = blockIdx.x, bj = blockIdx.y;
  if (bj < bi) return;
  const double diag = __dmul_rn(__dadd_rn(1.0, __dmul_rn(s, s)), f2);  // gaussian_kernel.hpp:45, then * f^2
  __shared__ double t[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t i = bi * 32 + tx;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int jj = ty + 8 * r;
    const int64_t j = bj * 32 + jj;
    double v = 0.0;
    if (i < n && j < n) v = (i == j) ? diag : gauss_cpp(X, ldx, d, i, j, l2x2, f2);
    t[jj][tx] = v;
    if (i < n && j < n) K[i + j * ldk] = from_c<TO, double>(v);
  }
  if (bi == bj) return;
  __syncthreads();
  const int64_t i2 = bj * 32 + tx;  // rows of the mirrored tile
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int ii = ty + 8 * r;
    const int64_t j2 = bi * 32 + ii;
    if (i2 < n && j2 < n) K[i2 + j2 * ldk] = from_c<TO, double>(t[tx][ii]);
  }
}

template <class TO>
__global__ void k_gauss(int form, int64_t m, int64_t n, int d, const double* __restrict__ X, int64_t ldx,
                        const double* __restrict__ Y, int64_t ldy, double l2x2, double f2, double s,
                        TO* __restrict__ K, int64_t ldk) {
  OFRR_FOR_2D(i, j, m, n) {
    double v;
    if (form == 0) {  // generate_gaussian_kernel: K = f^2 * (i == j ? 1 + s^2 : exp(-dist^2 / 2l^2))
      if (i == j) {
        v = __dmul_rn(__dadd_rn(1.0, __dmul_rn(s, s)), f2);
      } else {
        double dist = 0.0;
        for (int k = 0; k < d; ++k) {
          const double diff = __dsub_rn(X[i + k * ldx], Y[j + k * ldy]);
          dist = __dadd_rn(dist, __dmul_rn(diff, diff));
        }
        const double arg = __ddiv_rn(-dist, l2x2);
        v = (arg < -700.0) ? 0.0 : __dmul_rn(exp(arg), f2);
      }
    } else {  // gaussian.m: f^2 exp(-((-2 xy + xx) + yy) / (2 l^2)) + s^2 [i == j]
      double xy = 0.0, xx = 0.0, yy = 0.0;
      for (int k = 0; k < d; ++k) {
        const double a = X[i + k * ldx], b = Y[j + k * ldy];
        xy = __dadd_rn(xy, __dmul_rn(a, b));
        xx = __dadd_rn(xx, __dmul_rn(a, a));
        yy = __dadd_rn(yy, __dmul_rn(b, b));
      }
      const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(-2.0, xy), xx), yy);
      v = __dmul_rn(f2, exp(__ddiv_rn(-d2, l2x2)));
      if (i == j) v = __dadd_rn(v, __dmul_rn(s, s));
    }
    K[i + j * ldk] = from_c<TO, double>(v);
  }
}

}  // namespace
}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_rand_points(ofrr_ctx* ctx, uint64_t seed, int64_t n, int d, int type, double* X, int64_t ldx) {
  if (n <= 0 || d <= 0) return OFRR_ERR_INVALID_ARGUMENT;  // gaussian_kernel.hpp:27-29
  int need = 0;
  double scale = 0.0;
  const double pi = 3.141592653589793, dn = (double)n;
  switch (type) {
    case 0: need = d; scale = std::pow(dn, 1.0 / d); break;
    case 20: need = 2; scale = std::pow(dn, 1.0 / 2); break;
    case 30: need = 3; scale = std::pow(dn, 1.0 / 3); break;
    case 21: need = 2; scale = std::pow(dn / pi, 1.0 / 2); break;
    case 22: need = 2; scale = dn / 2 / pi; break;
    case 23: {
      need = 2;
      const long long nx = std::llround(std::sqrt(dn));
      if (nx * nx != n) return OFRR_ERR_INVALID_ARGUMENT;  // generate_pts.m: sqrt(n) must be an integer
      break;
    }
    case 31: need = 3; scale = std::pow(3 * dn / 4 / pi, 1.0 / 3); break;
    case 32: need = 3; scale = std::pow(dn / 4 / pi, 1.0 / 2); break;
    default: return OFRR_ERR_INVALID_ARGUMENT;
  }
  if (d != need || !ctx || !X || ldx < n) return OFRR_ERR_INVALID_ARGUMENT;
  const uint64_t key = mix64(seed);
  k_points<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8), 256, 0, ctx->stream>>>(key, n, d, type, scale, X,
                                                                                           ldx);
  OFRR_LAUNCHED(ctx, "k_points");
  return OFRR_SUCCESS;
}

extern "C" int ofrr_gaussian_kernel(ofrr_ctx* ctx, int form, int64_t m, int64_t n, int d, const double* X, int64_t ldx,
                                    const double* Y, int64_t ldy, double l, double f, double s, ofrr_dtype tout,
                                    void* K, int64_t ldk) {
  if (!(l > 0.0) || !(s >= 0.0) || m <= 0 || n <= 0 || d <= 0) return OFRR_ERR_INVALID_ARGUMENT;
  if (form != 0 && form != 1) return OFRR_ERR_INVALID_ARGUMENT;
  if (form == 0 && (X != Y || m != n || ldx != ldy)) return OFRR_ERR_INVALID_ARGUMENT;  // K(X, X) only
  if (!ctx || !X || !Y || !K || ldx < m || ldy < n || ldk < m || !dtype_valid(tout)) return OFRR_ERR_INVALID_ARGUMENT;
  const double l2x2 = 2.0 * l * l, f2 = f * f;
  const int64_t tiles = (n + 31) / 32;
  OFRR_DISPATCH_STORAGE(tout, TO, {
    if (form == 0 && tiles <= 65535) {
      k_gauss_sym<TO><<<dim3((unsigned)tiles, (unsigned)tiles), 256, 0, ctx->stream>>>(n, d, X, ldx, l2x2, f2, s,
                                                                                       (TO*)K, ldk);
      OFRR_LAUNCHED(ctx, "k_gauss_sym");
    } else {
      k_gauss<TO><<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(form, m, n, d, X, ldx, Y, ldy, l2x2, f2, s, (TO*)K,
                                                               ldk);
      OFRR_LAUNCHED(ctx, "k_gauss");
    }
  });
  return OFRR_SUCCESS;
}

// ---- dense matrices with a prescribed spectrum (the batched and serving workloads) ------------------
// A = H_1 .. H_r [diag(s); 0] G_1 .. G_r (SVD form, m x n, m >= n) or A = H_1 .. H_r diag(s) H_r .. H_1
// (symmetric form, m = n), with Householder reflectors H = I - 2 u u' / (u'u) whose vectors u are
// Gaussian draws of the library's generator: the singular values (eigenvalues) are exactly s, the
// singular vectors dense.  Each reflector is one matrix-vector product and one rank-1 update in FP64.
namespace ofrr {
namespace {
__global__ void k_diag_fill(int64_t m, int64_t n, const double* __restrict__ s, double* __restrict__ A, int64_t lda) {
  OFRR_FOR_2D(i, j, m, n) A[i + j * lda] = (i == j) ? s[j] : 0.0;
}
// y (m) = A x (trans 0) or y (n) = A' x (trans 1), one thread per output entry (FP64)
__global__ void k_gemv_f64(int trans, int64_t m, int64_t n, const double* __restrict__ A, int64_t lda,
                           const double* __restrict__ x, double* __restrict__ y) {
  const int64_t nout = trans ? n : m;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < nout; o += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    if (trans) {
      for (int64_t i = 0; i < m; ++i) acc = fma(A[i + o * lda], x[i], acc);
    } else {
      for (int64_t j = 0; j < n; ++j) acc = fma(A[o + j * lda], x[j], acc);
    }
    y[o] = acc;
  }
}
// A -= alpha x y'
__global__ void k_rank1_f64(int64_t m, int64_t n, double alpha, const double* __restrict__ x,
                            const double* __restrict__ y, double* __restrict__ A, int64_t lda) {
  OFRR_FOR_2D(i, j, m, n) A[i + j * lda] -= alpha * x[i] * y[j];
}
}  // namespace
}  // namespace ofrr

extern "C" int ofrr_test_matrix_spectrum(ofrr_ctx* ctx, int symmetric, uint64_t seed, int64_t m, int64_t n,
                                         int reflectors, const double* s, double* A, int64_t lda) {
  using namespace ofrr;
  if (!ctx || !s || !A || m < 1 || n < 1 || lda < m || reflectors < 0 || reflectors > 16)
    return OFRR_ERR_INVALID_ARGUMENT;
  if ((symmetric && m != n) || (!symmetric && m < n)) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *sd = ws_get<double>(ctx, (size_t)n, &st), *u = ws_get<double>(ctx, (size_t)m, &st),
         *w = ws_get<double>(ctx, (size_t)std::max(m, n), &st);
  if (!sd || !u || !w) return st;
  OFRR_CUDA(cudaMemcpyAsync(sd, s, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  k_diag_fill<<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, sd, A, lda);
  OFRR_LAUNCHED(ctx, "k_diag_fill");
  const int gv = grid_for(std::max(m, n), 128, 152 * 8);
  for (int r = 0; r < reflectors; ++r) {
    for (int side = 0; side < 2; ++side) {  // side 0: from the left (length m), 1: from the right (length n)
      const int64_t len = side ? n : m;
      OFRR_TRY(ofrr_randn(ctx, seed * 64 + 2 * r + side + 1, len, 1, OFRR_F64, u, len));
      std::vector<double> hu(len);
      OFRR_CUDA(cudaMemcpyAsync(hu.data(), u, sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
      double uu = 0.0;
      for (double v : hu) uu += v * v;
      if (side == 0) {  // A = (I - 2 u u'/uu) A: w = A' u, A -= (2/uu) u w'
        k_gemv_f64<<<gv, 128, 0, ctx->stream>>>(1, m, n, A, lda, u, w);
        OFRR_LAUNCHED(ctx, "k_gemv_f64");
        k_rank1_f64<<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, 2.0 / uu, u, w, A, lda);
      } else {  // A = A (I - 2 u u'/uu): w = A u, A -= (2/uu) w u'
        k_gemv_f64<<<gv, 128, 0, ctx->stream>>>(0, m, n, A, lda, u, w);
        OFRR_LAUNCHED(ctx, "k_gemv_f64");
        k_rank1_f64<<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, 2.0 / uu, w, u, A, lda);
      }
      OFRR_LAUNCHED(ctx, "k_rank1_f64");
      if (symmetric && side == 0) {  // the same reflector on the right keeps A symmetric
        k_gemv_f64<<<gv, 128, 0, ctx->stream>>>(0, m, n, A, lda, u, w);
        OFRR_LAUNCHED(ctx, "k_gemv_f64");
        k_rank1_f64<<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, 2.0 / uu, w, u, A, lda);
        OFRR_LAUNCHED(ctx, "k_rank1_f64");
        break;
      }
    }
  }
  return OFRR_SUCCESS;
}
