// Krylov steps of the thick-restart Hessenberg process (the production modes of the Krylov
// eigensolver), one fused kernel per new basis column, and the Rayleigh-Ritz helpers of a restart.
//
// Behaviour followed: the Krylov step of MATLAB/+src/+krylov/arnoldi_hess_eig.m:73-87 -- the new
// column is A times the previous one, eliminated against every earlier column in MGS order with the
// coefficients read at the earlier pivot rows, then pivoted on its largest entry and scaled by it.
// The restart keeps a block of Ritz vectors (solvers.cu); the steps below do not depend on it.
//
// Design (one launch per step i, columns 0 .. i-2 final in V, column i-1 unscaled in a staging
// vector Sprev of the arithmetic type TE, its pivot reciprocal in pvinv[i-1]):
//  * the elimination coefficients are known before the launch: with L(j, k) = q_k(perm_j) (unit lower
//    triangular because every column is zero at the earlier pivot rows) the MGS coefficients of the
//    new vector w are c = L^-1 w(perm).  L^-1 is kept explicitly and grown by one row per step, and the
//    last CTA of step i-1 evaluates w_i at the i pivot rows (i short CSR rows) and forms c, so the
//    bulk of step i is one pass over the rows with no dependence between CTAs;
//  * every thread owns R = 16 / sizeof(T) consecutive rows: it writes its rows of column i-1
//    (T(Sprev * pvinv), the stored basis values), computes its rows of A q_{i-1} from the CSR arrays
//    (the gathered neighbours scaled and rounded the same way), subtracts sum_j c_j q_j with one
//    16-byte load per earlier column, zeroes the earlier pivot rows, writes the unscaled result to the
//    staging vector Scur and keeps its integer argmax key (lowest row on ties);
//  * the last CTA to finish (atomic ticket) picks the pivot, appends row i to L and L^-1, and
//    evaluates the coefficients of step i+1.  A pivot below select_tol records a breakdown in
//    stop[0] and turns the remaining launches of the cycle into no-ops.
// HBM traffic of step i: CSR (nnz (4 + s_a) + 4 n) + staging read and write (2 n s_e) + the column
// write (n s) + i - 1 earlier columns (n s each) + the pivot marks (n), s = sizeof(T).
#include "ofrr_internal.cuh"

namespace ofrr {

constexpr int kKryThreads = 128;

template <class T>
struct KryVec {
  static constexpr int R = 16 / (int)sizeof(T);
};

template <class T, class TE>
__device__ __forceinline__ void kry_load16(const T* p, TE* out) {
  const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
  const T* t = reinterpret_cast<const T*>(&u);
#pragma unroll
  for (int k = 0; k < KryVec<T>::R; ++k) out[k] = to_c<TE, T>(t[k]);
}

// stored basis value of a staging entry: T(s * pinv), the same expression wherever it is needed
template <class T, class TE>
__device__ __forceinline__ T kry_q(TE s, TE pinv) {
  return from_c<T, TE>(mul_rn(s, pinv));
}

template <class TE>
__device__ __forceinline__ TE kry_warp_sum(TE v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

// Last CTA of a step (or of the start kernel): for the new column i (its unscaled values in S, its
// pivot row k = perm[i] and reciprocal pinv already chosen) append row i of L and L^-1, then the
// coefficients c = L^-1 w(perm) of step i + 1, w = A q_i evaluated at the pivot rows 0 .. i.
template <class T, class TE>
__device__ void kry_extend(int64_t k, int i, int nb, const T* V, int64_t ldv, const int32_t* indptr,
                           const int32_t* indices, const TE* vals, const TE* S, TE pinv, const int* perm, TE* Lrows,
                           TE* Linv, TE* coef, TE* s_L, TE* s_w) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int j = tid; j < i; j += nthr) {
    const TE l = to_c<TE, T>(__ldcg(V + k + (int64_t)j * ldv));
    s_L[j] = l;
    Lrows[(int64_t)i * nb + j] = l;
  }
  if (tid == 0) Lrows[(int64_t)i * nb + i] = TE(1);
  __syncthreads();
  for (int j = tid; j < i; j += nthr) {
    TE s = TE(0);
    for (int m = j; m < i; ++m) s = fma(s_L[m], Linv[(int64_t)m * nb + j], s);
    Linv[(int64_t)i * nb + j] = -s;
  }
  if (tid == 0) Linv[(int64_t)i * nb + i] = TE(1);
  if (i + 1 >= nb) return;
  __syncthreads();
  // w_{i+1} at the pivot rows: one warp per row, lanes over its nonzeros
  const int lane = tid & 31, wid = tid >> 5, nw = nthr >> 5;
  for (int j = wid; j <= i; j += nw) {
    const int64_t r = (j == i) ? k : (int64_t)perm[j];
    const int32_t p0 = indptr[r], p1 = indptr[r + 1];
    TE acc = TE(0);
    for (int32_t p = p0 + lane; p < p1; p += 32) {
      const int32_t col = indices[p];
      acc = fma(vals[p], to_c<TE, T>(kry_q<T, TE>(__ldcg(S + col), pinv)), acc);
    }
    acc = kry_warp_sum(acc);
    if (lane == 0) s_w[j] = acc;
  }
  __syncthreads();
  for (int j = tid; j <= i; j += nthr) {
    TE c = TE(0);
    for (int m = 0; m <= j; ++m) c = fma(Linv[(int64_t)j * nb + m], s_w[m], c);
    coef[j] = c;
  }
}

template <class T, class TE>
__global__ void __launch_bounds__(kKryThreads) k_kry_step(int64_t n, int nb, int i, T* __restrict__ V, int64_t ldv,
                                                          const int32_t* __restrict__ indptr,
                                                          const int32_t* __restrict__ indices,
                                                          const TE* __restrict__ vals, const TE* __restrict__ Sprev,
                                                          TE* __restrict__ Scur, unsigned char* __restrict__ mark,
                                                          TE* __restrict__ pvinv, TE* __restrict__ coef,
                                                          TE* __restrict__ Lrows, TE* __restrict__ Linv,
                                                          int* __restrict__ perm, ArgMaxK* __restrict__ partial,
                                                          unsigned int* __restrict__ counter, int* __restrict__ stop,
                                                          double stol) {
  constexpr int R = KryVec<T>::R;
  __shared__ TE s_c[kKryMaxNb];
  __shared__ TE s_L[kKryMaxNb];
  __shared__ TE s_w[kKryMaxNb];
  __shared__ ArgMaxK red[kKryThreads / 32];
  __shared__ bool s_last;
  if (*((volatile int*)stop) >= 0) return;  // breakdown earlier in this cycle (set by an earlier launch)
  const int tid = threadIdx.x;
  for (int j = tid; j < i; j += blockDim.x) s_c[j] = coef[j];
  const TE pinv = pvinv[i - 1];
  __syncthreads();
  const int64_t r0 = ((int64_t)blockIdx.x * blockDim.x + tid) * R;
  ArgMaxK best{-1, 0x7fffffffffffffffLL};
  if (r0 < n) {
    const int nr = (int)min((int64_t)R, n - r0);
    TE x[R], w[R];
    {  // column i-1 on this thread's rows: the stored basis values
      T xs[R];
#pragma unroll
      for (int rr = 0; rr < R; ++rr) {
        xs[rr] = kry_q<T, TE>(rr < nr ? Sprev[r0 + rr] : TE(0), pinv);
        x[rr] = to_c<TE, T>(xs[rr]);
      }
      *reinterpret_cast<uint4*>(V + (int64_t)(i - 1) * ldv + r0) = *reinterpret_cast<const uint4*>(xs);
    }
    // A q_{i-1} on this thread's rows (its nonzeros are contiguous)
    int32_t p = __ldg(indptr + r0);
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      TE acc = TE(0);
      if (rr < nr) {
        const int32_t pe = __ldg(indptr + r0 + rr + 1);
        for (; p < pe; ++p) {
          const int32_t col = __ldg(indices + p);
          acc = fma(__ldg(vals + p), to_c<TE, T>(kry_q<T, TE>(__ldg(Sprev + col), pinv)), acc);
        }
      }
      w[rr] = acc;
    }
    // eliminations: w -= sum_j c_j q_j (columns 0 .. i-2 from V, column i-1 from registers)
    const T* Vr = V + r0;
#pragma unroll 4
    for (int j = 0; j < i - 1; ++j) {
      TE q[R];
      kry_load16<T, TE>(Vr + (int64_t)j * ldv, q);
      const TE c = s_c[j];
#pragma unroll
      for (int rr = 0; rr < R; ++rr) w[rr] = fma(-c, q[rr], w[rr]);
    }
    {
      const TE c = s_c[i - 1];
#pragma unroll
      for (int rr = 0; rr < R; ++rr) w[rr] = fma(-c, x[rr], w[rr]);
    }
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
      if (rr < nr) {
        const TE v = mark[r0 + rr] ? TE(0) : w[rr];  // earlier pivot rows stay exactly zero
        Scur[r0 + rr] = v;
        const long long key = amax_key(v);
        if (key > best.key) best = ArgMaxK{key, r0 + rr};
      }
    }
  }
  const ArgMaxK b = block_argmaxk(best, red);
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    partial[blockIdx.x] = b;
    __threadfence();
    s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // ---- last CTA: pivot of column i ----
  ArgMaxK a{-1, 0x7fffffffffffffffLL};
  for (int t = tid; t < (int)gridDim.x; t += blockDim.x) {
    ArgMaxK q;
    q.key = __ldcg(&partial[t].key);
    q.i = __ldcg(&partial[t].i);
    a = argmaxk_pick(a, q);
  }
  const ArgMaxK f = block_argmaxk(a, red);
  const int64_t k = (f.key < 0) ? 0 : f.i;
  const TE pv = __ldcg(Scur + k);
  if (fabs((double)pv) < stol || pv == TE(0)) {  // breakdown: the cycle ends with columns 0 .. i-1
    if (tid == 0) {
      *stop = i;
      *counter = 0u;
    }
    return;
  }
  const TE pinv_i = div_rn(TE(1), pv);
  if (tid == 0) {
    perm[i] = (int)k;
    pvinv[i] = pinv_i;
    mark[k] = 1;
  }
  kry_extend<T, TE>(k, i, nb, V, ldv, indptr, indices, vals, Scur, pinv_i, perm, Lrows, Linv, coef, s_L, s_w);
  if (tid == 0) *counter = 0u;
}

// Start of the Krylov steps after the basis block 0 .. q-1 (final in V, pivot rows perm[0 .. q-1]):
// column q-1 copied into the staging vector (reciprocal 1), the earlier pivot rows marked, L and L^-1
// of the block, and the coefficients of step q.
template <class T, class TE>
__global__ void __launch_bounds__(kKryThreads) k_kry_begin(int64_t n, int nb, int q, const T* __restrict__ V,
                                                           int64_t ldv, const int32_t* __restrict__ indptr,
                                                           const int32_t* __restrict__ indices,
                                                           const TE* __restrict__ vals, TE* __restrict__ Sprev,
                                                           unsigned char* __restrict__ mark, TE* __restrict__ pvinv,
                                                           TE* __restrict__ coef, TE* __restrict__ Lrows,
                                                           TE* __restrict__ Linv, const int* __restrict__ perm,
                                                           unsigned int* __restrict__ counter) {
  __shared__ TE s_L[kKryMaxNb];
  __shared__ TE s_w[kKryMaxNb];
  __shared__ bool s_last;
  const int tid = threadIdx.x;
  const T* col = V + (int64_t)(q - 1) * ldv;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + tid; r < n; r += (int64_t)gridDim.x * blockDim.x)
    Sprev[r] = to_c<TE, T>(col[r]);
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int j = tid; j < q; j += blockDim.x) mark[perm[j]] = 1;
  if (tid == 0) pvinv[q - 1] = TE(1);
  // rows 0 .. q-2 of L and L^-1 one after another, then row q-1 with the coefficients of step q
  for (int i = 0; i < q - 1; ++i) {
    for (int j = tid; j < i; j += blockDim.x) {
      const TE l = to_c<TE, T>(V[perm[i] + (int64_t)j * ldv]);
      s_L[j] = l;
      Lrows[(int64_t)i * nb + j] = l;
    }
    if (tid == 0) Lrows[(int64_t)i * nb + i] = TE(1);
    __syncthreads();
    for (int j = tid; j < i; j += blockDim.x) {
      TE s = TE(0);
      for (int m = j; m < i; ++m) s = fma(s_L[m], Linv[(int64_t)m * nb + j], s);
      Linv[(int64_t)i * nb + j] = -s;
    }
    if (tid == 0) Linv[(int64_t)i * nb + i] = TE(1);
    __syncthreads();
  }
  kry_extend<T, TE>(perm[q - 1], q - 1, nb, V, ldv, indptr, indices, vals, Sprev, TE(1), perm, Lrows, Linv, coef, s_L,
                    s_w);
  if (tid == 0) *counter = 0u;
}

// the last column of a cycle: V(:, i) = T(S * pvinv[i]) unless the cycle broke down
template <class T, class TE>
__global__ void k_kry_end(int64_t n, int i, T* __restrict__ V, int64_t ldv, const TE* __restrict__ S,
                          const TE* __restrict__ pvinv, const int* __restrict__ stop) {
  if (*stop >= 0) return;
  const TE pinv = pvinv[i];
  T* col = V + (int64_t)i * ldv;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    col[r] = kry_q<T, TE>(S[r], pinv);
}

// ---- host side of the steps ----------------------------------------------------------------------
namespace {
template <class TE>
const TE* kry_vals(const ofrr_csr* A);
template <>
const float* kry_vals<float>(const ofrr_csr* A) {
  return A->a_single;
}
template <>
const double* kry_vals<double>(const ofrr_csr* A) {
  return A->a_double;
}

template <class T, class TE>
int kry_launch(ofrr_ctx* ctx, KryState& s, int what, int i) {
  const TE* vals = kry_vals<TE>(s.A);
  if (!vals) return OFRR_ERR_INVALID_ARGUMENT;
  T* V = (T*)s.V;
  TE* S0 = (TE*)s.S[0];
  TE* S1 = (TE*)s.S[1];
  if (what == 0) {  // begin with q = i columns
    TE* Sp = ((i - 1) & 1) ? S1 : S0;
    const int grid = grid_for(s.n, kKryThreads, 152 * 8);
    k_kry_begin<T, TE><<<grid, kKryThreads, 0, ctx->stream>>>(s.n, s.nb, i, V, s.ldv, s.A->indptr, s.A->indices,
                                                              vals, Sp, s.mark, (TE*)s.pvinv, (TE*)s.coef,
                                                              (TE*)s.Lrows, (TE*)s.Linv, s.perm, s.counter);
    OFRR_LAUNCHED(ctx, "k_kry_begin");
  } else if (what == 1) {  // step i
    TE* Sp = ((i - 1) & 1) ? S1 : S0;
    TE* Sc = (i & 1) ? S1 : S0;
    k_kry_step<T, TE><<<s.grid, kKryThreads, 0, ctx->stream>>>(
        s.n, s.nb, i, V, s.ldv, s.A->indptr, s.A->indices, vals, Sp, Sc, s.mark, (TE*)s.pvinv, (TE*)s.coef,
        (TE*)s.Lrows, (TE*)s.Linv, s.perm, (ArgMaxK*)s.partial, s.counter, s.stop, s.stol);
    OFRR_LAUNCHED(ctx, "k_kry_step");
  } else {  // end: scale column i
    const TE* Sc = (i & 1) ? S1 : S0;
    k_kry_end<T, TE><<<grid_for(s.n, 256, 152 * 8), 256, 0, ctx->stream>>>(s.n, i, V, s.ldv, Sc, (const TE*)s.pvinv,
                                                                          s.stop);
    OFRR_LAUNCHED(ctx, "k_kry_end");
  }
  return OFRR_SUCCESS;
}

int kry_dispatch(ofrr_ctx* ctx, KryState& s, int what, int i) {
  switch (s.t) {
    case OFRR_F16: return kry_launch<__half, float>(ctx, s, what, i);
    case OFRR_BF16: return kry_launch<__nv_bfloat16, float>(ctx, s, what, i);
    case OFRR_F32: return kry_launch<float, float>(ctx, s, what, i);
    case OFRR_F64: return kry_launch<double, double>(ctx, s, what, i);
  }
  return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
}
}  // namespace

ofrr_dtype kry_arith_type(ofrr_dtype t) { return t == OFRR_F64 ? OFRR_F64 : OFRR_F32; }

int64_t kry_ld(int64_t n) { return (n + 7) / 8 * 8; }

int kry_state_init(ofrr_ctx* ctx, KryState* s, const ofrr_csr* A, ofrr_dtype t, int nb, double stol) {
  if (nb < 2 || nb > kKryMaxNb) return OFRR_ERR_BLAS_INVALID_SIZE;
  const ofrr_dtype te = kry_arith_type(t);
  if ((te == OFRR_F32 && !A->a_single) || (te == OFRR_F64 && !A->a_double)) return OFRR_ERR_INVALID_ARGUMENT;
  int st = OFRR_SUCCESS;
  s->A = A;
  s->t = t;
  s->te = te;
  s->n = A->nrows;
  s->ldv = kry_ld(s->n);
  s->nb = nb;
  s->stol = stol;
  const size_t es = dtype_size(te);
  const int64_t rows_per_cta = (int64_t)kKryThreads * (16 / (int64_t)dtype_size(t));
  s->grid = (int)std::max<int64_t>(1, (s->n + rows_per_cta - 1) / rows_per_cta);
  if (!(s->V = ws_alloc(ctx, (size_t)s->ldv * nb * dtype_size(t), &st))) return st;
  for (int b = 0; b < 2; ++b)
    if (!(s->S[b] = ws_alloc(ctx, (size_t)s->ldv * es, &st))) return st;
  if (!(s->mark = (unsigned char*)ws_alloc(ctx, (size_t)s->ldv, &st))) return st;
  if (!(s->perm = ws_get<int>(ctx, (size_t)nb, &st))) return st;
  if (!(s->pvinv = ws_alloc(ctx, (size_t)nb * es, &st))) return st;
  if (!(s->coef = ws_alloc(ctx, (size_t)nb * es, &st))) return st;
  if (!(s->Lrows = ws_alloc(ctx, (size_t)nb * nb * es, &st))) return st;
  if (!(s->Linv = ws_alloc(ctx, (size_t)nb * nb * es, &st))) return st;
  if (!(s->partial = ws_alloc(ctx, (size_t)s->grid * sizeof(ArgMaxK), &st))) return st;
  if (!(s->counter = ws_get<unsigned int>(ctx, 1, &st))) return st;
  if (!(s->stop = ws_get<int>(ctx, 1, &st))) return st;
  OFRR_TRY(fill_zero(ctx, s->V, (size_t)s->ldv * nb * dtype_size(t)));
  OFRR_TRY(fill_zero(ctx, s->counter, sizeof(unsigned int)));
  return OFRR_SUCCESS;
}

int kry_cycle_steps(ofrr_ctx* ctx, KryState& s, int q) {
  if (q < 1 || q >= s.nb) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_CUDA(cudaMemsetAsync(s.stop, 0xFF, sizeof(int), ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(s.mark, 0, (size_t)s.ldv, ctx->stream));
  OFRR_TRY(fill_zero(ctx, s.Lrows, (size_t)s.nb * s.nb * dtype_size(s.te)));
  OFRR_TRY(fill_zero(ctx, s.Linv, (size_t)s.nb * s.nb * dtype_size(s.te)));
  OFRR_TRY(kry_dispatch(ctx, s, 0, q));
  for (int i = q; i < s.nb; ++i) OFRR_TRY(kry_dispatch(ctx, s, 1, i));
  return kry_dispatch(ctx, s, 2, s.nb - 1);
}

// ---- Rayleigh-Ritz helpers of the thick-restart cycle ----------------------------------------
// W (n x k, type TO) = V (n x nc, type T) Cf (nc x k, FP64 read as FP32): FP32 arithmetic, one thread per
// row and up to 32 output columns, the coefficient block in shared memory
template <class T, class TO>
__global__ void __launch_bounds__(128) k_kry_vmul(int64_t n, int nc, const T* __restrict__ V, int64_t ldv,
                                                  const double* __restrict__ Cf, int k, TO* __restrict__ W,
                                                  int64_t ldw) {
  __shared__ float Zs[kKryMaxNb + 15][33];
  const int j0 = blockIdx.y * 32;
  const int nj = min(32, k - j0);
  for (int e = threadIdx.x; e < (kKryMaxNb + 15) * 32; e += blockDim.x) {  // rows past nc are zero
    const int r = e >> 5, jj = e & 31;
    Zs[r][jj] = (jj < nj && r < nc) ? __double2float_rn(Cf[r + (int64_t)(j0 + jj) * nc]) : 0.f;
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float acc[32];
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) acc[jj] = 0.f;
    for (int r0 = 0; r0 < nc; r0 += 16) {
      float u[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) u[t] = (r0 + t < nc) ? to_c<float, T>(V[i + (int64_t)(r0 + t) * ldv]) : 0.f;
#pragma unroll
      for (int t = 0; t < 16; ++t) {
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) acc[jj] = fmaf(u[t], Zs[r0 + t][jj], acc[jj]);
      }
    }
#pragma unroll
    for (int jj = 0; jj < 32; ++jj)
      if (jj < nj) W[i + (int64_t)(j0 + jj) * ldw] = from_c<TO, float>(acc[jj]);
  }
}

template <class TW, class TA>
__global__ void k_kry_addcol(int64_t n, TW* __restrict__ w, const TA* __restrict__ a) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    w[i] = from_c<TW, double>(to_c<double, TW>(w[i]) + to_c<double, TA>(a[i]));
}

// x = M^-1 g for the SPD Gram matrix M (nc x nc, FP64): Cholesky in shared memory, one CTA
__global__ void __launch_bounds__(256) k_kry_spd_solve(int nc, const double* __restrict__ M,
                                                       const double* __restrict__ g, double* __restrict__ x) {
  extern __shared__ double sl[];  // nc x nc (column-major), then nc
  __shared__ double s_d;
  double* y = sl + (size_t)nc * nc;
  const int tid = threadIdx.x;
  for (int e = tid; e < nc * nc; e += blockDim.x) sl[e] = M[e];
  for (int e = tid; e < nc; e += blockDim.x) y[e] = g[e];
  __syncthreads();
  for (int j = 0; j < nc; ++j) {  // right-looking: column j, then the trailing update
    if (tid == 0) s_d = sqrt(fmax(sl[j + (size_t)j * nc], 0.0));
    __syncthreads();
    const double d = s_d;
    for (int i = j + 1 + tid; i < nc; i += blockDim.x)
      sl[i + (size_t)j * nc] = (d > 0.0) ? sl[i + (size_t)j * nc] / d : 0.0;
    if (tid == 0) sl[j + (size_t)j * nc] = d;
    __syncthreads();
    const int w = nc - j - 1;
    for (int e = tid; e < w * w; e += blockDim.x) {
      const int c = j + 1 + e / w, r = j + 1 + e % w;
      if (r >= c) sl[r + (size_t)c * nc] -= sl[r + (size_t)j * nc] * sl[c + (size_t)j * nc];
    }
    __syncthreads();
  }
  if (tid == 0) {  // L y = g, then L' x = y
    for (int i = 0; i < nc; ++i) {
      double t = y[i];
      for (int k = 0; k < i; ++k) t -= sl[i + (size_t)k * nc] * y[k];
      y[i] = (sl[i + (size_t)i * nc] > 0.0) ? t / sl[i + (size_t)i * nc] : 0.0;
    }
    for (int i = nc - 1; i >= 0; --i) {
      double t = y[i];
      for (int k = i + 1; k < nc; ++k) t -= sl[k + (size_t)i * nc] * y[k];
      y[i] = (sl[i + (size_t)i * nc] > 0.0) ? t / sl[i + (size_t)i * nc] : 0.0;
    }
    for (int i = 0; i < nc; ++i) x[i] = y[i];
  }
}

// Cf (nc x (k1 + k2 + 1)) = [U1(:, 0 .. k1-1), U2(:, 0 .. k2-1), -x]
__global__ void k_kry_coefmat(int nc, int k1, const double* __restrict__ U1, int k2, const double* __restrict__ U2,
                              const double* __restrict__ x, double* __restrict__ Cf) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nc * (k1 + k2 + 1); e += gridDim.x * blockDim.x) {
    const int r = e % nc, c = e / nc;
    Cf[e] = (c < k1) ? U1[r + (int64_t)c * nc] : (c < k1 + k2) ? U2[r + (int64_t)(c - k1) * nc] : -x[r];
  }
}

// s = sum_j W(:, j) / nrm_j (FP64)
template <class TW>
__global__ void k_kry_sumcols(int64_t n, int k, const TW* __restrict__ W, int64_t ldw, const double* __restrict__ nrm,
                              double* __restrict__ s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < k; ++j) acc += (nrm[j] > 0.0) ? to_c<double, TW>(W[i + (int64_t)j * ldw]) / nrm[j] : 0.0;
    s[i] = acc;
  }
}

int kry_backtransform(ofrr_ctx* ctx, ofrr_dtype t, int64_t n, int nc, const void* V, int64_t ldv, const double* Cf,
                      int k, ofrr_dtype tw, void* W, int64_t ldw, bool exact) {
  if (k <= 0) return OFRR_SUCCESS;
  if (exact && t == OFRR_F64 && tw == OFRR_F64)
    return tsmm_f64(ctx, n, k, nc, (const double*)V, ldv, Cf, nc, (double*)W, ldw);
  if (t == OFRR_F64 || tw == OFRR_F64)
    return gemm_impl(ctx, 0, 0, t, OFRR_F64, OFRR_F64, tw, n, k, nc, 1.0, V, ldv, Cf, nc, 0.0, W, ldw);
  if (tw != OFRR_F32 || nc > kKryMaxNb) return OFRR_ERR_INVALID_ARGUMENT;
  const dim3 grid((unsigned)std::min<int64_t>((n + 127) / 128, 152 * 8), (unsigned)((k + 31) / 32));
  switch (t) {
    case OFRR_F16:
      k_kry_vmul<__half, float><<<grid, 128, 0, ctx->stream>>>(n, nc, (const __half*)V, ldv, Cf, k, (float*)W, ldw);
      break;
    case OFRR_BF16:
      k_kry_vmul<__nv_bfloat16, float><<<grid, 128, 0, ctx->stream>>>(n, nc, (const __nv_bfloat16*)V, ldv, Cf, k,
                                                                      (float*)W, ldw);
      break;
    case OFRR_F32:
      k_kry_vmul<float, float><<<grid, 128, 0, ctx->stream>>>(n, nc, (const float*)V, ldv, Cf, k, (float*)W, ldw);
      break;
    default: return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  }
  OFRR_LAUNCHED(ctx, "k_kry_vmul");
  return OFRR_SUCCESS;
}

int kry_add_col(ofrr_ctx* ctx, ofrr_dtype tw, int64_t n, void* w, ofrr_dtype ta, const void* a) {
  const int grid = grid_for(n, 256, 152 * 8);
  if (tw == OFRR_F32 && ta == OFRR_F32) {
    k_kry_addcol<float, float><<<grid, 256, 0, ctx->stream>>>(n, (float*)w, (const float*)a);
  } else if (tw == OFRR_F64 && ta == OFRR_F64) {
    k_kry_addcol<double, double><<<grid, 256, 0, ctx->stream>>>(n, (double*)w, (const double*)a);
  } else {
    return OFRR_ERR_INVALID_ARGUMENT;
  }
  OFRR_LAUNCHED(ctx, "k_kry_addcol");
  return OFRR_SUCCESS;
}

int kry_spd_solve(ofrr_ctx* ctx, int nc, const double* M, const double* g, double* x) {
  if (nc <= 0 || nc > kKryMaxNb) return OFRR_ERR_INVALID_ARGUMENT;
  const size_t smem = ((size_t)nc * nc + nc) * sizeof(double);
  OFRR_TRY(allow_smem(k_kry_spd_solve));
  k_kry_spd_solve<<<1, 256, smem, ctx->stream>>>(nc, M, g, x);
  OFRR_LAUNCHED(ctx, "k_kry_spd_solve");
  return OFRR_SUCCESS;
}

int kry_coef_matrix(ofrr_ctx* ctx, int nc, int k1, const double* U1, int k2, const double* U2, const double* x,
                    double* Cf) {
  k_kry_coefmat<<<grid_for((int64_t)nc * (k1 + k2 + 1), 256, 64), 256, 0, ctx->stream>>>(nc, k1, U1, k2, U2, x, Cf);
  OFRR_LAUNCHED(ctx, "k_kry_coefmat");
  return OFRR_SUCCESS;
}

// ---- cross-Gram V' (A V) of the 16-bit phase on the tensor cores --------------------------------------
// A V is FP32 and V 16-bit, and a tcgen05 product takes one operand type: each column of A V is scaled by a
// power of two (its maximum into [2^13, 2^14)), split into hi = T(y) and lo = T(y - hi), and
// G = 2^e (V' hi + V' lo) with FP32 accumulation.  The split keeps about 22 bits of A V (FP16) -- the
// library FP32 path that it replaces (operands widened to FP32, SGEMM with K in the millions and a 65 x 65
// result) ran on a handful of SMs.
__global__ void k_kry_colmax_f32(int64_t n, int nc, const float* __restrict__ X, int64_t ldx,
                                 unsigned int* __restrict__ mx) {
  const int c = blockIdx.y;
  float m = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(X[i + (int64_t)c * ldx]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(mx + c, __float_as_uint(m));  // order-free for m >= 0
}

template <class T>
__global__ void k_kry_split_hilo(int64_t n, int nc, const float* __restrict__ X, int64_t ldx,
                                 const unsigned int* __restrict__ mx, T* __restrict__ hi, T* __restrict__ lo,
                                 int64_t ldh) {
  const int c = blockIdx.y;
  const float m = __uint_as_float(mx[c]);
  int e = 0;
  if (m > 0.f) frexpf(m, &e);                // m = f 2^e, f in [0.5, 1)
  const float sc = (m > 0.f) ? ldexpf(1.f, 14 - e) : 0.f;  // maximum into [2^13, 2^14)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float y = X[i + (int64_t)c * ldx] * sc;
    const T h = from_c<T, float>(y);
    hi[i + (int64_t)c * ldh] = h;
    lo[i + (int64_t)c * ldh] = from_c<T, float>(y - to_c<float, T>(h));
  }
}

__global__ void k_kry_gram_combine(int nc, const double* __restrict__ G1, const double* __restrict__ G2,
                                   const unsigned int* __restrict__ mx, double* __restrict__ G) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nc * nc; e += gridDim.x * blockDim.x) {
    const int c = e / nc;
    const float m = __uint_as_float(mx[c]);
    int ex = 0;
    if (m > 0.f) frexpf(m, &ex);
    G[e] = (m > 0.f) ? ldexp(G1[e] + G2[e], ex - 14) : 0.0;
  }
}

int kry_gram16(ofrr_ctx* ctx, ofrr_dtype t, int64_t n, int nc, const void* V, int64_t ldv, const float* AV,
               int64_t ldav, double* G) {
  if (t != OFRR_F16 && t != OFRR_BF16) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t ldh = kry_ld(n);
  void* hi = ws_alloc(ctx, (size_t)ldh * nc * 2, &st);
  void* lo = ws_alloc(ctx, (size_t)ldh * nc * 2, &st);
  unsigned int* mx = ws_get<unsigned int>(ctx, (size_t)nc, &st);
  double* G1 = ws_get<double>(ctx, (size_t)nc * nc, &st);
  double* G2 = ws_get<double>(ctx, (size_t)nc * nc, &st);
  if (!hi || !lo || !mx || !G1 || !G2) return st;
  OFRR_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned int) * nc, ctx->stream));
  const dim3 grid((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)nc);
  k_kry_colmax_f32<<<grid, 256, 0, ctx->stream>>>(n, nc, AV, ldav, mx);
  OFRR_LAUNCHED(ctx, "k_kry_colmax_f32");
  if (t == OFRR_F16)
    k_kry_split_hilo<__half><<<grid, 256, 0, ctx->stream>>>(n, nc, AV, ldav, mx, (__half*)hi, (__half*)lo, ldh);
  else
    k_kry_split_hilo<__nv_bfloat16><<<grid, 256, 0, ctx->stream>>>(n, nc, AV, ldav, mx, (__nv_bfloat16*)hi,
                                                                  (__nv_bfloat16*)lo, ldh);
  OFRR_LAUNCHED(ctx, "k_kry_split_hilo");
  OFRR_TRY(gemm_impl(ctx, 1, 0, t, t, OFRR_F32, OFRR_F64, nc, nc, n, 1.0, V, ldv, hi, ldh, 0.0, G1, nc));
  OFRR_TRY(gemm_impl(ctx, 1, 0, t, t, OFRR_F32, OFRR_F64, nc, nc, n, 1.0, V, ldv, lo, ldh, 0.0, G2, nc));
  k_kry_gram_combine<<<(nc * nc + 255) / 256, 256, 0, ctx->stream>>>(nc, G1, G2, mx, G);
  OFRR_LAUNCHED(ctx, "k_kry_gram_combine");
  return OFRR_SUCCESS;
}

int kry_sum_unit_cols(ofrr_ctx* ctx, ofrr_dtype tw, int64_t n, int k, const void* W, int64_t ldw, const double* nrm,
                      double* s) {
  const int grid = grid_for(n, 256, 152 * 8);
  if (tw == OFRR_F32)
    k_kry_sumcols<float><<<grid, 256, 0, ctx->stream>>>(n, k, (const float*)W, ldw, nrm, s);
  else if (tw == OFRR_F64)
    k_kry_sumcols<double><<<grid, 256, 0, ctx->stream>>>(n, k, (const double*)W, ldw, nrm, s);
  else
    return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_LAUNCHED(ctx, "k_kry_sumcols");
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

// Profiling form of one Krylov step (no reference counterpart): a basis of i + 1 columns of type t on
// the CSR operator A (Gaussian columns scaled to a unit maximum, distinct pivot rows, identity L^-1),
// then reps launches of step i timed with CUDA events on the context's stream (synchronous).  Returns the
// mean time per launch and the step's algorithmic HBM bytes: CSR values and indices once, row pointers
// once, the staging vector read and written once, column i-1 written once, the i-1 earlier columns read
// once and the pivot marks.
extern "C" int ofrr_profile_krylov_step(ofrr_ctx* ctx, const ofrr_csr* A, ofrr_dtype t, int i, int reps,
                                        double* us_per_launch, double* bytes_per_launch) {
  if (!ctx || !A || !us_per_launch || !bytes_per_launch || reps < 2 || i < 1 || i + 1 > kKryMaxNb)
    return OFRR_ERR_INVALID_ARGUMENT;
  if (A->nrows != A->ncols || A->nrows < 2 * kKryMaxNb || !dtype_valid(t)) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  KryState s;
  OFRR_TRY(kry_state_init(ctx, &s, A, t, i + 1, 0.0));
  const ofrr_dtype te = s.te;
  const size_t es = dtype_size(te);
  OFRR_TRY(ofrr_randn(ctx, 11, s.n, i, t, s.V, s.ldv));
  OFRR_TRY(ofrr_randn(ctx, 12, s.n, 1, te, s.S[0], s.ldv));
  OFRR_TRY(ofrr_randn(ctx, 13, s.n, 1, te, s.S[1], s.ldv));
  OFRR_TRY(scalecols_impl(ctx, t, te, s.n, i, s.V, s.ldv, nullptr));
  std::vector<int> hp(i + 1);
  for (int j = 0; j <= i; ++j) hp[j] = (int)((int64_t)j * (s.n / (i + 1)));
  OFRR_CUDA(cudaMemcpyAsync(s.perm, hp.data(), sizeof(int) * (i + 1), cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(s.mark, 0, (size_t)s.ldv, ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(s.stop, 0xFF, sizeof(int), ctx->stream));
  std::vector<double> h((size_t)(i + 1) * (i + 1) + 2 * (i + 1), 0.0);
  for (int j = 0; j <= i; ++j) {
    h[(size_t)j * (i + 1) + j] = 1.0;                 // L^-1 = I
    h[(size_t)(i + 1) * (i + 1) + j] = 1.0;           // reciprocal pivots 1
    h[(size_t)(i + 1) * (i + 1) + (i + 1) + j] = 0.01;  // coefficients
  }
  {
    WsScope tmp(ctx);
    int st = OFRR_SUCCESS;
    double* hd = ws_get<double>(ctx, h.size(), &st);
    if (!hd) return st;
    OFRR_CUDA(cudaMemcpyAsync(hd, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream));
    const size_t o1 = (size_t)(i + 1) * (i + 1), o2 = o1 + (i + 1);
    OFRR_TRY(cast_impl(ctx, OFRR_F64, te, i + 1, i + 1, hd, i + 1, s.Linv, i + 1));
    OFRR_TRY(cast_impl(ctx, OFRR_F64, te, i + 1, 1, hd + o1, i + 1, s.pvinv, i + 1));
    OFRR_TRY(cast_impl(ctx, OFRR_F64, te, i + 1, 1, hd + o2, i + 1, s.coef, i + 1));
    OFRR_TRY(sync_and_check(ctx));
  }
  cudaEvent_t e0, e1;
  OFRR_CUDA(cudaEventCreate(&e0));
  OFRR_CUDA(cudaEventCreate(&e1));
  int st = kry_dispatch(ctx, s, 1, i);  // warm-up
  if (st == OFRR_SUCCESS) st = map_cuda_error(cudaEventRecord(e0, ctx->stream));
  for (int r = 0; r < reps && st == OFRR_SUCCESS; ++r) st = kry_dispatch(ctx, s, 1, i);
  if (st == OFRR_SUCCESS) st = map_cuda_error(cudaEventRecord(e1, ctx->stream));
  if (st == OFRR_SUCCESS) st = sync_and_check(ctx);
  float ms = 0.f;
  if (st == OFRR_SUCCESS) st = map_cuda_error(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  OFRR_TRY(st);
  *us_per_launch = 1e3 * ms / reps;
  const double n = (double)s.n, nnz = (double)A->nnz, sz = (double)dtype_size(t);
  *bytes_per_launch = nnz * (4.0 + es) + 4.0 * (n + 1) + n * (2.0 * es + sz * i + 1.0);
  return OFRR_SUCCESS;
}
