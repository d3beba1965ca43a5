// Orthogonal comparison bases for subspace iteration: modified (MATLAB/+src/+qr/mgs.m:49-101) and
// classical (MATLAB/+src/+qr/cgs.m:49-110) Gram-Schmidt with the reference's adaptive
// re-orthogonalisation.  mgs.m is the default `function_orth` of subspace_iter_eig.m:114-115; the
// orthogonalization-free runs pass hessenberg instead.  For column i of A (m x n, tall):
//   normv = norm2(a_i); normv < select_tol -> column dropped
//   projection pass over the selected earlier columns j (in order):
//     MGS: r_j = dot(v, q_j), v = po(pc(v) - pc(r_j) pc(q_j)) one j at a time
//     CGS: all r_j = dot(v, q_j) first, then the same updates in j order
//   t = norm2(v); while t >= orth_tol and t < reorth_tol normv: normv = t, another pass with
//   R(j,i) = po(pc(R(j,i)) + pc(r_j)), t = norm2(v)
//   t < select_tol -> dropped; else q_i = po(pc(v) / pc(t)), R(i,i) = t.
// Dots and norms are grid reductions in the compute type (per-CTA partial sums, the last CTA adds
// them in a fixed order: deterministic); the updates are row-parallel and apply the j terms in order
// with one rounding to the output type per term, as the MATLAB code does.  The while-loop decisions
// need t on the host: one synchronisation per column and pass (the comparison path, not the hot one).
// Q keeps the input's column positions (dropped columns zero) with select flags, like the Hessenberg
// basis, so the solvers compact both the same way.
#include <cmath>
#include <vector>

#include "ofrr_internal.cuh"

namespace ofrr {
namespace {

constexpr int GS_T = 256;
constexpr int GS_G = 152;  // CTAs per reduction

// host-side conversions of the storage types
inline double host_double(double x) { return x; }
inline double host_double(float x) { return (double)x; }
inline double host_double(__half x) { return (double)__half2float(x); }
inline double host_double(__nv_bfloat16 x) { return (double)__bfloat162float(x); }
// x rounded to the storage type t (a tolerance compared in the output precision)
inline double round_to(ofrr_dtype t, double x) {
  switch (t) {
    case OFRR_F32: return (double)(float)x;
    case OFRR_F16: return (double)__half2float(__double2half(x));
    case OFRR_BF16: return (double)__bfloat162float(__double2bfloat16(x));
    default: return x;
  }
}

// out[c] = po(sum_i pc(v_i) pc(Q[i, cols[c]])) for c = blockIdx.y; Q == nullptr: out[0] = po(sqrt(sum pc(v_i)^2))
template <class TO, class TC>
__global__ void __launch_bounds__(GS_T) k_gs_reduce(int64_t m, const TO* __restrict__ v, const TO* __restrict__ Q,
                                                    int64_t ldq, const int* __restrict__ cols, TC* __restrict__ partial,
                                                    unsigned int* __restrict__ counters, TO* __restrict__ out) {
  __shared__ TC red[GS_T / 32];
  __shared__ bool last;
  const int c = blockIdx.y;
  const TO* q = Q ? Q + (int64_t)cols[c] * ldq : nullptr;
  TC s = TC(0);
  for (int64_t i = blockIdx.x * (int64_t)GS_T + threadIdx.x; i < m; i += (int64_t)gridDim.x * GS_T) {
    const TC a = to_c<TC, TO>(v[i]);
    s += a * (q ? to_c<TC, TO>(q[i]) : a);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    TC b = TC(0);
    for (int w = 0; w < GS_T / 32; ++w) b += red[w];
    partial[(size_t)c * gridDim.x + blockIdx.x] = b;
    __threadfence();
    last = (atomicAdd(counters + c, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const volatile TC* vp = partial + (size_t)c * gridDim.x;
  TC tot = TC(0);
  for (unsigned int b = 0; b < gridDim.x; ++b) tot += vp[b];
  counters[c] = 0;  // self-resetting for the next reduction
  out[c] = q ? from_c<TO, TC>(tot) : from_c<TO, TC>(sqrt(tot));
}

// v_i <- po(pc(v_i) - pc(r_c) pc(Q[i, cols[c]])) for c = 0..ncols-1 in order (one rounding to po per
// term, no fused multiply-add: the MATLAB arithmetic); one thread also records R(cols[c], i) = r_c
// (acc: po(pc(R) + pc(r_c))) in the FP64 copy of R (column Rcol)
template <class TO, class TC>
__global__ void __launch_bounds__(GS_T) k_gs_update(int64_t m, TO* __restrict__ v, const TO* __restrict__ Q,
                                                    int64_t ldq, const int* __restrict__ cols, int ncols,
                                                    const TO* __restrict__ r, double* __restrict__ Rcol, int acc) {
  for (int64_t i = blockIdx.x * (int64_t)GS_T + threadIdx.x; i < m; i += (int64_t)gridDim.x * GS_T) {
    TC x = to_c<TC, TO>(v[i]);
    for (int c = 0; c < ncols; ++c) {
      const TC p = mul_rn(to_c<TC, TO>(r[c]), to_c<TC, TO>(Q[i + (int64_t)cols[c] * ldq]));
      x = to_c<TC, TO>(from_c<TO, TC>(sub_rn(x, p)));
    }
    v[i] = from_c<TO, TC>(x);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int c = 0; c < ncols; ++c) {
      const int j = cols[c];
      const TC rc = to_c<TC, TO>(r[c]);
      Rcol[j] = acc ? (double)to_c<TC, TO>(from_c<TO, TC>(add_rn(to_c<TC, double>(Rcol[j]), rc))) : (double)rc;
    }
  }
}

// q = po(pc(v) / pc(t)), R(i,i) = t
template <class TO, class TC>
__global__ void __launch_bounds__(GS_T) k_gs_scale(int64_t m, const TO* __restrict__ v, const TO* __restrict__ t,
                                                   TO* __restrict__ q, double* __restrict__ Rii) {
  const TC tc = to_c<TC, TO>(*t);
  for (int64_t i = blockIdx.x * (int64_t)GS_T + threadIdx.x; i < m; i += (int64_t)gridDim.x * GS_T)
    q[i] = from_c<TO, TC>(div_rn(to_c<TC, TO>(v[i]), tc));
  if (blockIdx.x == 0 && threadIdx.x == 0) *Rii = (double)to_c<TC, TO>(*t);
}

template <class TO, class TC>
int gs_run(ofrr_ctx* ctx, bool classical, int64_t m, int64_t n, const TO* A, int64_t lda, TO* Q, int64_t ldq,
           double stol, double otol, double rtol, double* R, int* select_dev) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  TO* v = ws_get<TO>(ctx, (size_t)m, &st);
  TO* rr = ws_get<TO>(ctx, (size_t)n + 2, &st);  // r_0..r_{n-1}, then norm scratch
  TC* partial = ws_get<TC>(ctx, (size_t)GS_G * n, &st);
  unsigned int* counters = ws_get<unsigned int>(ctx, (size_t)n, &st);
  int* cols = ws_get<int>(ctx, (size_t)n, &st);
  TO* norms = ws_get<TO>(ctx, (size_t)n, &st);
  if (!v || !rr || !partial || !counters || !cols || !norms) return st;
  OFRR_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned int) * n, ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(R, 0, sizeof(double) * n * n, ctx->stream));
  for (int64_t j = 0; j < n; ++j)
    OFRR_CUDA(cudaMemsetAsync(Q + j * ldq, 0, sizeof(TO) * m, ctx->stream));
  const unsigned gu = (unsigned)std::min<int64_t>((m + GS_T - 1) / GS_T, 4 * 152);
  auto norm_of = [&](const TO* x, TO* out) -> int {
    k_gs_reduce<TO, TC><<<dim3(GS_G, 1), GS_T, 0, ctx->stream>>>(m, x, nullptr, 0, nullptr, partial, counters, out);
    OFRR_LAUNCHED(ctx, "k_gs_reduce");
    return OFRR_SUCCESS;
  };
  // the norms of the original columns (column i is untouched until its turn)
  for (int64_t i = 0; i < n; ++i) OFRR_TRY(norm_of(A + i * lda, norms + i));
  std::vector<TO> hn((size_t)n);
  OFRR_CUDA(cudaMemcpyAsync(hn.data(), norms, sizeof(TO) * n, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  std::vector<int> sel((size_t)n, 0), hcols;
  // one projection pass of v against the selected columns hcols (R column i; acc: accumulate)
  auto pass = [&](int64_t i, int acc) -> int {
    const int nc = (int)hcols.size();
    if (nc == 0) return OFRR_SUCCESS;
    double* Rcol = R + i * n;
    if (classical) {
      k_gs_reduce<TO, TC><<<dim3(GS_G, nc), GS_T, 0, ctx->stream>>>(m, v, Q, ldq, cols, partial, counters, rr);
      OFRR_LAUNCHED(ctx, "k_gs_reduce");
      k_gs_update<TO, TC><<<gu, GS_T, 0, ctx->stream>>>(m, v, Q, ldq, cols, nc, rr, Rcol, acc);
      OFRR_LAUNCHED(ctx, "k_gs_update");
    } else {
      for (int c = 0; c < nc; ++c) {
        k_gs_reduce<TO, TC><<<dim3(GS_G, 1), GS_T, 0, ctx->stream>>>(m, v, Q, ldq, cols + c, partial, counters, rr);
        OFRR_LAUNCHED(ctx, "k_gs_reduce");
        k_gs_update<TO, TC><<<gu, GS_T, 0, ctx->stream>>>(m, v, Q, ldq, cols + c, 1, rr, Rcol, acc);
        OFRR_LAUNCHED(ctx, "k_gs_update");
      }
    }
    return OFRR_SUCCESS;
  };
  for (int64_t i = 0; i < n; ++i) {
    double normv = host_double(hn[(size_t)i]);
    if (normv < stol) continue;
    OFRR_CUDA(cudaMemcpyAsync(v, A + i * lda, sizeof(TO) * m, cudaMemcpyDeviceToDevice, ctx->stream));
    OFRR_TRY(pass(i, 0));
    TO ht;
    OFRR_TRY(norm_of(v, rr + n));
    OFRR_CUDA(cudaMemcpyAsync(&ht, rr + n, sizeof(TO), cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
    double t = host_double(ht);
    // (at most 64 passes: the reference loops until the norm stops dropping, which takes 1-2)
    for (int guard = 0; rtol >= 0 && t >= otol && t < rtol * normv && guard < 64; ++guard) {
      normv = t;
      OFRR_TRY(pass(i, 1));
      OFRR_TRY(norm_of(v, rr + n));
      OFRR_CUDA(cudaMemcpyAsync(&ht, rr + n, sizeof(TO), cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
      t = host_double(ht);
    }
    if (t < stol) continue;
    k_gs_scale<TO, TC><<<gu, GS_T, 0, ctx->stream>>>(m, v, rr + n, Q + i * ldq, R + i * n + i);
    OFRR_LAUNCHED(ctx, "k_gs_scale");
    sel[(size_t)i] = 1;
    hcols.push_back((int)i);
    OFRR_CUDA(cudaMemcpyAsync(cols + hcols.size() - 1, &hcols.back(), sizeof(int), cudaMemcpyHostToDevice,
                              ctx->stream));
    OFRR_TRY(sync_and_check(ctx));  // the pageable source of the index copy stays valid until here
  }
  OFRR_CUDA(cudaMemcpyAsync(select_dev, sel.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
  return sync_and_check(ctx);
}

}  // namespace

int gs_basis_impl(ofrr_ctx* ctx, bool classical, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m,
                  int64_t n, const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol, double* R_dev,
                  int* select_dev, double orth_tol, double reorth_tol) {
  if (n <= 0 || m <= 0) return OFRR_SUCCESS;
  if (m < n) return OFRR_ERR_BLAS_INVALID_SIZE;  // mgs.m:50 / cgs.m:50 assert a tall-thin A
  const double e = dtype_eps(tout);
  const double stol = select_tol < 0 ? e : select_tol;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const void* Ain = A;
  int64_t ldin = lda;
  const char* qb = (const char*)Q;
  const char* ab = (const char*)A;
  const bool alias = ab < qb + (size_t)ldq * n * dtype_size(tout) && qb < ab + (size_t)lda * n * dtype_size(tin);
  if (tin != tout || alias) {  // A = precision_output(A), in a copy when it overlaps Q
    void* w = ws_alloc(ctx, (size_t)m * n * dtype_size(tout), &st);
    if (!w) return st;
    OFRR_TRY(cast_impl(ctx, tin, tout, m, n, A, lda, w, m));
    Ain = w;
    ldin = m;
  }
  // the tolerances are compared in the output precision, as mgs.m:141-152 casts them
  const double s_t = round_to(tout, stol), o_t = round_to(tout, std::isnan(orth_tol) ? e : orth_tol),
               r_t = round_to(tout, std::isnan(reorth_tol) ? 1.0 / std::sqrt(2.0) : reorth_tol);
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    OFRR_TRY((gs_run<TO, TC>(ctx, classical, m, n, (const TO*)Ain, ldin, (TO*)Q, ldq, s_t, o_t, r_t, R_dev,
                             select_dev)));
  }));
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_gs_basis(ofrr_ctx* ctx, int classical, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute,
                             int64_t m, int64_t n, const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol,
                             double orth_tol, double reorth_tol, double* R_host, int* skip_host) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(tin) || !dtype_valid(tout)) return OFRR_ERR_INVALID_ARGUMENT;
  if (tcompute != OFRR_F64 && tcompute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (m < n) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (n == 0) return OFRR_SUCCESS;
  if (!A || !Q || lda < m || ldq < m) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double* R = ws_get<double>(ctx, (size_t)n * n, &st);
  if (!R) return st;
  int* sel = ws_get<int>(ctx, (size_t)n, &st);
  if (!sel) return st;
  OFRR_TRY(gs_basis_impl(ctx, classical != 0, tin, tout, tcompute, m, n, A, lda, Q, ldq, select_tol, R, sel,
                         orth_tol, reorth_tol));
  std::vector<int> hsel((size_t)n);
  OFRR_CUDA(cudaMemcpyAsync(hsel.data(), sel, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (R_host) OFRR_CUDA(cudaMemcpyAsync(R_host, R, sizeof(double) * n * n, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  if (skip_host)
    for (int64_t j = 0; j < n; ++j) skip_host[j] = hsel[(size_t)j] ? 0 : 1;
  return OFRR_SUCCESS;
}
