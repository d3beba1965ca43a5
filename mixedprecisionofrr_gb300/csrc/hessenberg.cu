// Hessenberg-process oblique basis (pivoted elimination, unit-max columns).
//
// Behaviour: MATLAB/+src/+qr/hessenberg.m:45-85 (left-looking, MGS order).  Replaces the three
// GPU variants of the reference (CPP/linalg/factorization/hessenberg.cu:197-801), which issue a
// blocking device->host copy per column, cudaMalloc inside iamax and <<<1,1>>> launches.
//
// Design: one launch per column i.  Every CTA first recovers the elimination coefficients
// r_j = v_j(perm_j) for j < i by a forward substitution over the i pivot rows only (the matrix
// Q(perm,:) is unit lower triangular); that substitution performs, for each pivot row, exactly the
// rounding sequence MATLAB performs on that row.  Each thread then applies the i eliminations to its
// own rows in the same order (one rounding to the output type per elimination, as
// v = po(pc(v) - pc(R(j,i)) * pc(Q(:,j)))), so every element of Q is bit-identical to the MATLAB
// restatement.  The per-CTA argmax partials are combined by the last CTA to finish (atomic
// ticket), which also records the pivot, R(:,i), the selection flag and the pivot row of Q.  The
// division of column i by its pivot is fused into launch i+1 (each thread scales its own rows
// before using them), and a final launch scales the last column.  No host synchronisation
// happens inside the loop, so the whole build can be captured in a CUDA graph.
#include "ofrr_internal.cuh"

namespace ofrr {

template <class TO, class TC>
__global__ void __launch_bounds__(256) k_hess_col(int64_t m, int n, int i, TO* __restrict__ Q, int64_t ldq,
                                                   int* __restrict__ select, int* __restrict__ perm,
                                                   TO* __restrict__ pivrows, TO* __restrict__ pvals,
                                                   double* __restrict__ R, ArgMax* __restrict__ partial,
                                                   unsigned int* __restrict__ counter, double select_tol,
                                                   int scale_prev, int* __restrict__ stop, int stage_L,
                                                   TO* __restrict__ snap = nullptr) {
  extern __shared__ unsigned char smem_raw[];
  TC* s_r = reinterpret_cast<TC*>(smem_raw);                       // n entries
  TO* s_x = reinterpret_cast<TO*>(s_r + n);                        // n entries
  int* s_sel = reinterpret_cast<int*>(((uintptr_t)(s_x + n) + 15) & ~(uintptr_t)15);  // n entries
  __shared__ ArgMax red[32];
  __shared__ bool s_last;
  __shared__ TC s_pprev;

  const int tid = threadIdx.x;
  // Krylov mode: a breakdown earlier in this cycle turns the rest of the cycle into no-ops
  if (stop != nullptr && *((volatile int*)stop) >= 0) return;
  // column i at the earlier pivot rows: from the snapshot the previous launch's last CTA took (every
  // column is given up front), else from Q itself -- which is only safe while all CTAs of the launch
  // read it before any of them rewrites its rows of column i, i.e. for grids that are resident at once
  for (int j = tid; j < i; j += blockDim.x) {
    int sj = select[j];
    s_sel[j] = sj;
    s_x[j] = sj ? (snap ? snap[j] : Q[(int64_t)perm[j] + (int64_t)i * ldq]) : TO(0);
  }
  if (tid == 0) s_pprev = (i > 0) ? to_c<TC, TO>(pvals[i - 1]) : TC(0);
  // stage the strictly lower i x i block of pivot rows in shared memory when it fits, so that the
  // sequential substitution below never waits on global memory
  TO* s_L = stage_L ? reinterpret_cast<TO*>(((uintptr_t)(s_sel + n) + 15) & ~(uintptr_t)15) : nullptr;
  if (stage_L) {
    for (int e = tid; e < i * i; e += blockDim.x) {
      const int jj = e / i, l = e % i;
      if (l < jj) s_L[e] = pivrows[(int64_t)jj * n + l];
    }
  }
  __syncthreads();

  // forward substitution over the pivot rows (warp 0): r_j = value at perm_j after j eliminations
  if (tid < 32) {
    for (int j = 0; j < i; ++j) {
      __syncwarp();
      if (!s_sel[j]) {
        if (tid == 0) s_r[j] = TC(0);
        continue;
      }
      const TC rc = to_c<TC, TO>(s_x[j]);
      for (int jj = j + 1 + tid; jj < i; jj += 32) {
        if (s_sel[jj]) {
          const TC l = to_c<TC, TO>(stage_L ? s_L[jj * i + j] : pivrows[(int64_t)jj * n + j]);
          s_x[jj] = from_c<TO, TC>(sub_rn(to_c<TC, TO>(s_x[jj]), mul_rn(rc, l)));
        }
      }
      if (tid == 0) s_r[j] = rc;
    }
  }
  __syncthreads();

  // eliminations on this thread's rows (MGS order), fused scaling of column i-1
  const int prev_sel = (i > 0) ? s_sel[i - 1] : 0;
  ArgMax a{-1.0, 0x7fffffffffffffffLL};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + tid; row < m; row += stride) {
    TO qprev = TO(0);
    if (i > 0) {
      qprev = Q[row + (int64_t)(i - 1) * ldq];
      if (scale_prev) {
        qprev = prev_sel ? from_c<TO, TC>(div_rn(to_c<TC, TO>(qprev), s_pprev)) : TO(0);
        Q[row + (int64_t)(i - 1) * ldq] = qprev;
      }
    }
    TC v = to_c<TC, TO>(Q[row + (int64_t)i * ldq]);
    TO vo = Q[row + (int64_t)i * ldq];
    // eliminations in MGS order; the previous columns are loaded 8 at a time ahead of the
    // dependent chain so that the loads overlap
    for (int j0 = 0; j0 < i; j0 += 8) {
      TO qb[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u;
        qb[u] = (j < i - 1) ? Q[row + (int64_t)j * ldq] : ((j == i - 1) ? qprev : TO(0));
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u;
        if (j < i && s_sel[j]) {
          vo = from_c<TO, TC>(sub_rn(v, mul_rn(s_r[j], to_c<TC, TO>(qb[u]))));
          v = to_c<TC, TO>(vo);
        }
      }
    }
    Q[row + (int64_t)i * ldq] = vo;
    const double av = absd(vo);
    if (av > a.v) a = ArgMax{av, row};
  }
  ArgMax r = block_argmax(a, red);
  if (tid == 0) {
    partial[blockIdx.x] = r;
    __threadfence();
    unsigned int ticket = atomicAdd(counter, 1u);
    s_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // last CTA: global pivot, R(:,i), selection and pivot row
  ArgMax b{-1.0, 0x7fffffffffffffffLL};
  const volatile ArgMax* vp = partial;
  for (int t = tid; t < (int)gridDim.x; t += blockDim.x) {
    ArgMax p;
    p.v = vp[t].v;
    p.i = vp[t].i;
    b = argmax_pick(b, p);
  }
  ArgMax f = block_argmax(b, red);
  const int64_t k = (f.v < 0.0) ? 0 : f.i;
  const TO pv = __ldcg(reinterpret_cast<const TO*>(Q + k + (int64_t)i * ldq));
  const double tol_o = to_c<double, TO>(from_c<TO, double>(select_tol));
  // kept unless |pivot| < select_tol: a column that is NaN throughout (no row wins the search, row 0
  // is taken) stays selected, as in hessenberg.m where abs(NaN) < select_tol is false
  const bool keep = !(absd(pv) < tol_o);
  for (int j = tid; j < i; j += blockDim.x) R[j + (int64_t)i * n] = s_sel[j] ? to_c<double, TC>(s_r[j]) : 0.0;
  if (keep) {
    for (int l = tid; l < i; l += blockDim.x) {
      pivrows[(int64_t)i * n + l] = __ldcg(reinterpret_cast<const TO*>(Q + k + (int64_t)l * ldq));
    }
  }
  if (snap && i + 1 < n) {  // column i + 1 (untouched so far) at the pivot rows 0 .. i
    for (int j = tid; j <= i; j += blockDim.x) {
      const int64_t row = (j == i) ? k : (int64_t)perm[j];
      snap[j] = (j == i || s_sel[j]) ? __ldcg(reinterpret_cast<const TO*>(Q + row + (int64_t)(i + 1) * ldq)) : TO(0);
    }
  }
  if (tid == 0) {
    R[i + (int64_t)i * n] = to_c<double, TO>(pv);
    if (stop != nullptr && !keep) *stop = i;
    select[i] = keep ? 1 : 0;
    perm[i] = keep ? (int)k : -1;
    pvals[i] = keep ? pv : TO(0);
    *counter = 0u;
  }
}

// scale (or zero) the last column by its pivot
template <class TO, class TC>
__global__ void k_hess_scale(int64_t m, int i, TO* __restrict__ Q, int64_t ldq, const int* __restrict__ select,
                             const TO* __restrict__ pvals, const int* __restrict__ stop) {
  if (stop != nullptr && *stop >= 0) return;
  const int keep = select[i];
  const TC p = to_c<TC, TO>(pvals[i]);
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < m; row += (int64_t)gridDim.x * blockDim.x) {
    TO q = Q[row + (int64_t)i * ldq];
    Q[row + (int64_t)i * ldq] = keep ? from_c<TO, TC>(div_rn(to_c<TC, TO>(q), p)) : TO(0);
  }
}

template <class TO, class TC>
static int hess_run(ofrr_ctx* ctx, int64_t m, int n, TO* Q, int64_t ldq, double select_tol, double* R, int* select,
                    int* perm) {
  int st = OFRR_SUCCESS;
  TO* pivrows = ws_get<TO>(ctx, (size_t)n * n, &st);
  if (!pivrows) return st;
  TO* pvals = ws_get<TO>(ctx, (size_t)n, &st);
  if (!pvals) return st;
  const int block = 128;  // one row per thread: 64 CTAs for 8192 rows
  // tall bases (millions of rows, the Krylov restart block): enough threads that each walks only a few
  // rows -- a thread's rows are a chain of dependent loads of the earlier columns.  The launches read
  // the next column's pivot-row values from a snapshot, so the grid need not be resident at once.
  int grid = grid_for(m, block, 152 * 16);
  ArgMax* partial = ws_get<ArgMax>(ctx, grid, &st);
  TO* snap = ws_get<TO>(ctx, (size_t)n, &st);
  if (!partial || !snap) return st;
  OFRR_TRY(fill_zero(ctx, R, sizeof(double) * (size_t)n * n));
  OFRR_TRY(fill_zero(ctx, pivrows, sizeof(TO) * (size_t)n * n));
  const int stage = ((size_t)n * n * sizeof(TO) <= 96 * 1024) ? 1 : 0;
  size_t smem = (size_t)n * (sizeof(TC) + sizeof(TO)) + 16 + (size_t)n * sizeof(int);
  if (stage) smem += 16 + (size_t)n * n * sizeof(TO);
  if (smem > 48 * 1024) {
    OFRR_TRY(allow_smem(k_hess_col<TO, TC>));
  }
  for (int i = 0; i < n; ++i) {
    k_hess_col<TO, TC><<<grid, block, smem, ctx->stream>>>(m, n, i, Q, ldq, select, perm, pivrows, pvals, R, partial,
                                                            ctx->dev_counters, select_tol, 1, nullptr, stage, snap);
    OFRR_LAUNCHED(ctx, "k_hess_col");
  }
  k_hess_scale<TO, TC><<<grid, block, 0, ctx->stream>>>(m, n - 1, Q, ldq, select, pvals, nullptr);
  OFRR_LAUNCHED(ctx, "k_hess_scale");
  return OFRR_SUCCESS;
}

int hess_run_blocked(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n, void* Q, int64_t ldq,
                     double select_tol, double* R, int* select, int* perm, bool fast, bool* done);

int hessenberg_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n,
                    const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol, double* R_dev,
                    int* select_dev, int* perm_dev, bool fast) {
  if (n <= 0 || m <= 0) return OFRR_SUCCESS;
  if (n > 4096) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (select_tol < 0) select_tol = dtype_eps(tout);
  // Q <- tout(A); an in-place call must keep the element type and the leading dimension
  if (A == Q && (tin != tout || lda != ldq)) return OFRR_ERR_INVALID_ARGUMENT;
  if (A != Q) OFRR_TRY(cast_impl(ctx, tin, tout, m, n, A, lda, Q, ldq));
  WsScope scope(ctx);
  // blocked cluster schedule (hessenberg_blocked.cu) when the block fits on chip, else per column
  bool done = false;
  OFRR_TRY(hess_run_blocked(ctx, tout, tc, m, n, Q, ldq, select_tol, R_dev, select_dev, perm_dev, fast, &done));
  if (done) return OFRR_SUCCESS;
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    OFRR_TRY((hess_run<TO, TC>(ctx, m, (int)n, (TO*)Q, ldq, select_tol, R_dev, select_dev, perm_dev)));
  }));
  return OFRR_SUCCESS;
}

// ---- Krylov (Hessenberg-process Arnoldi) steps: one new column at a time -------------------
template <class TO, class TC>
static int kry_col(ofrr_ctx* ctx, int64_t m, int nb, int i, TO* V, int64_t ldv, double stol, int* sel, int* perm,
                   TO* pivrows, TO* pvals, double* R, int* stop) {
  const int block = 256;
  const int grid = grid_for(m, block, 152 * 4);  // resident at once: column i is read from V itself
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  ArgMax* partial = ws_get<ArgMax>(ctx, grid, &st);
  if (!partial) return st;
  const int stage = ((size_t)nb * nb * sizeof(TO) <= 96 * 1024) ? 1 : 0;
  size_t smem = (size_t)nb * (sizeof(TC) + sizeof(TO)) + 16 + (size_t)nb * sizeof(int);
  if (stage) smem += 16 + (size_t)nb * nb * sizeof(TO);
  if (smem > 48 * 1024) {
    OFRR_TRY(allow_smem(k_hess_col<TO, TC>));
  }
  k_hess_col<TO, TC><<<grid, block, smem, ctx->stream>>>(m, nb, i, V, ldv, sel, perm, pivrows, pvals, R, partial,
                                                          ctx->dev_counters, stol, 0, stop, stage);
  OFRR_LAUNCHED(ctx, "k_hess_col");
  return OFRR_SUCCESS;
}

int hess_krylov_first(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int nb, void* V, int64_t ldv,
                      double stol, int* sel, int* perm, void* pivrows, void* pvals, double* R, int* stop) {
  OFRR_CUDA(cudaMemsetAsync(stop, 0xFF, 2 * sizeof(int), ctx->stream));
  OFRR_TRY(fill_zero(ctx, R, sizeof(double) * (size_t)nb * nb));
  OFRR_TRY(fill_zero(ctx, pivrows, dtype_size(tout) * (size_t)nb * nb));
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    OFRR_TRY((kry_col<TO, TC>(ctx, m, nb, 0, (TO*)V, ldv, stol, sel, perm, (TO*)pivrows, (TO*)pvals, R, stop)));
    k_hess_scale<TO, TC><<<grid_for(m, 256, 152 * 4), 256, 0, ctx->stream>>>(m, 0, (TO*)V, ldv, sel, (const TO*)pvals,
                                                                            stop);
    OFRR_LAUNCHED(ctx, "k_hess_scale");
  }));
  return OFRR_SUCCESS;
}

int hess_krylov_step(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int nb, int i, void* V, int64_t ldv,
                     double stol, int* sel, int* perm, void* pivrows, void* pvals, double* R, int* stop) {
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    OFRR_TRY((kry_col<TO, TC>(ctx, m, nb, i, (TO*)V, ldv, stol, sel, perm, (TO*)pivrows, (TO*)pvals, R, stop)));
  }));
  return OFRR_SUCCESS;
}

int hess_scale_col(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int i, void* V, int64_t ldv,
                   const int* sel, const void* pvals, const int* stop) {
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    k_hess_scale<TO, TC><<<grid_for(m, 256, 152 * 4), 256, 0, ctx->stream>>>(m, i, (TO*)V, ldv, sel,
                                                                            (const TO*)pvals, stop);
    OFRR_LAUNCHED(ctx, "k_hess_scale");
  }));
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_hessenberg(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute, int64_t m,
                               int64_t n, const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol,
                               double* R_host, int* skip_host, int* perm_host) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(tin) || !dtype_valid(tout)) return OFRR_ERR_INVALID_ARGUMENT;
  if (tcompute != OFRR_F64 && tcompute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (m < n) return OFRR_ERR_BLAS_INVALID_SIZE;  // hessenberg.m:52 asserts a tall-thin A
  if (n == 0) return OFRR_SUCCESS;
  if (!A || !Q || lda < m || ldq < m) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double* R = ws_get<double>(ctx, (size_t)n * n, &st);
  if (!R) return st;
  int* sel = ws_get<int>(ctx, (size_t)n, &st);
  if (!sel) return st;
  int* perm = ws_get<int>(ctx, (size_t)n, &st);
  if (!perm) return st;
  OFRR_TRY(hessenberg_impl(ctx, tin, tout, tcompute, m, n, A, lda, Q, ldq, select_tol, R, sel, perm));
  std::vector<int> hsel(n), hperm(n);
  OFRR_CUDA(cudaMemcpyAsync(hsel.data(), sel, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(hperm.data(), perm, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (R_host) OFRR_CUDA(cudaMemcpyAsync(R_host, R, sizeof(double) * n * n, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  for (int64_t j = 0; j < n; ++j) {
    if (skip_host) skip_host[j] = hsel[j] ? 0 : 1;
    if (perm_host) perm_host[j] = hperm[j];
  }
  return OFRR_SUCCESS;
}

// ======================================================================================
// Hessenberg basis without any allocation
// ======================================================================================
// Some callers of this library cannot allocate GPU memory: an application whose memory pool has
// already reserved all of HBM (a cudaMalloc would fail), or a latency-bound request handler that
// must not pay the implicit device-wide synchronisation of cudaMalloc/cudaFree on other streams.
// ofrr_hessenberg needs a context (its creation allocates) and a cached workspace; this entry point
// needs neither.  Its scratch -- the pivot rows and pivot values of the process, the per-CTA argmax
// partials and the last-CTA ticket counter -- lives in one file-scope __device__ array of
// kNoAllocScratchBytes (1 MiB), which every GPU that loads the library holds until the process exits.
// The caller passes the input, the outputs and a stream.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;
constexpr int kNoAllocGrid = 304;  // 2 CTAs per SM: the argmax partials need this many slots
__device__ __align__(256) unsigned char g_hess_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device.  Looked up on every call (cheap once the
// module is loaded), so a device reset or a new primary context never leaves a stale address behind.
int noalloc_scratch(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_hess_noalloc_scratch);
  if (e != cudaSuccess) {
    note_cuda_error(e, "cudaGetSymbolAddress(g_hess_noalloc_scratch)", __FILE__, __LINE__);
    return map_cuda_error(e);
  }
  *out = (unsigned char*)p;
  return OFRR_SUCCESS;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// bytes of scratch for an n-column basis of element size es
size_t noalloc_bytes(int64_t n, size_t es) {
  return align256(sizeof(unsigned int)) + align256(sizeof(ArgMax) * kNoAllocGrid) + align256((size_t)n * es) +
         align256((size_t)n * n * es);
}

template <class TO, class TC>
int hess_run_noalloc(ofrr_ctx* sctx, unsigned char* scratch, int64_t m, int n, TO* Q, int64_t ldq, double select_tol,
                     double* R, int* select, int* perm) {
  unsigned int* counter = (unsigned int*)scratch;
  ArgMax* partial = (ArgMax*)(scratch + align256(sizeof(unsigned int)));
  TO* pvals = (TO*)((unsigned char*)partial + align256(sizeof(ArgMax) * kNoAllocGrid));
  TO* pivrows = (TO*)((unsigned char*)pvals + align256((size_t)n * sizeof(TO)));
  const int block = 256;
  const int grid = grid_for(m, block, kNoAllocGrid);
  // everything that must start at zero: the ticket counter, R and the pivot rows
  OFRR_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), sctx->stream));
  OFRR_TRY(fill_zero(sctx, R, sizeof(double) * (size_t)n * n));
  OFRR_TRY(fill_zero(sctx, pivrows, sizeof(TO) * (size_t)n * n));
  const size_t smem = (size_t)n * (sizeof(TC) + sizeof(TO)) + 16 + (size_t)n * sizeof(int);
  if (smem > 48 * 1024) return OFRR_ERR_BLAS_INVALID_SIZE;
  for (int i = 0; i < n; ++i) {
    k_hess_col<TO, TC><<<grid, block, smem, sctx->stream>>>(m, n, i, Q, ldq, select, perm, pivrows, pvals, R, partial,
                                                             counter, select_tol, 1, nullptr, 0);
    OFRR_LAUNCHED(sctx, "k_hess_col");
  }
  k_hess_scale<TO, TC><<<grid, block, 0, sctx->stream>>>(m, n - 1, Q, ldq, select, pvals, nullptr);
  OFRR_LAUNCHED(sctx, "k_hess_scale");
  return OFRR_SUCCESS;
}

}  // namespace

extern "C" size_t ofrr_hessenberg_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int ofrr_hessenberg_noalloc(void* stream, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute, int64_t m,
                                       int64_t n, const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol,
                                       double* R, int* select, int* perm) {
  if (m < 0 || n < 0 || !dtype_valid(tin) || !dtype_valid(tout)) return OFRR_ERR_INVALID_ARGUMENT;
  if (tcompute != OFRR_F64 && tcompute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (m < n) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (n == 0) return OFRR_SUCCESS;
  if (!A || !Q || !R || !select || !perm || lda < m || ldq < m) return OFRR_ERR_INVALID_ARGUMENT;
  const size_t es = dtype_size(tout);
  if (n > 1024 || noalloc_bytes(n, es) > kNoAllocScratchBytes) {
    fprintf(stderr,
            "[ofrr] ofrr_hessenberg_noalloc: %lld columns of %zu-byte elements need %zu bytes of scratch, "
            "more than the fixed %zu-byte array\n",
            (long long)n, es, noalloc_bytes(n, es), kNoAllocScratchBytes);
    return OFRR_ERR_BLAS_INVALID_SIZE;
  }
  unsigned char* scratch = nullptr;
  OFRR_TRY(noalloc_scratch(&scratch));
  // a stack context that only carries the stream (no handle, no workspace, no allocation)
  ofrr_ctx sctx;
  sctx.stream = (cudaStream_t)stream;
  if (select_tol < 0) select_tol = dtype_eps(tout);
  if (A == Q && (tin != tout || lda != ldq)) return OFRR_ERR_INVALID_ARGUMENT;
  if (A != Q) OFRR_TRY(cast_impl(&sctx, tin, tout, m, n, A, lda, Q, ldq));
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tcompute, TC, {
    OFRR_TRY((hess_run_noalloc<TO, TC>(&sctx, scratch, m, (int)n, (TO*)Q, ldq, select_tol, R, select, perm)));
  }));
  return OFRR_SUCCESS;
}
