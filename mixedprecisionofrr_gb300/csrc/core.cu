// Context, workspace, status handling and the level-1/2 kernels of libofrr_gb300.so:
// project RNG, casts, column argmax / scalecols, iamax, NaN/Inf scan, column norms.
#include <mutex>
#include <set>
#include <type_traits>

#include "ofrr_internal.cuh"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

namespace ofrr {

int aux_begin(ofrr_ctx* ctx, ofrr_ctx** aux) {
  if (!ctx->aux) {
    OFRR_TRY(ofrr_ctx_create(&ctx->aux, ctx->device, nullptr));
    trace_destroy(ctx->aux);  // phases are traced on the main context only
    OFRR_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    OFRR_CUDA(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  }
  ctx->aux->emulate_f64 = ctx->emulate_f64;
  OFRR_CUDA(cudaEventRecord(ctx->ev_fork, ctx->stream));
  OFRR_CUDA(cudaStreamWaitEvent(ctx->aux->stream, ctx->ev_fork, 0));
  *aux = ctx->aux;
  return OFRR_SUCCESS;
}

int aux_end(ofrr_ctx* ctx) {
  if (!ctx->aux) return OFRR_SUCCESS;
  OFRR_CUDA(cudaEventRecord(ctx->ev_join, ctx->aux->stream));
  OFRR_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
  return OFRR_SUCCESS;
}

int allow_dynamic_smem(const void* func) {
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> done;
  int dev = 0;
  OFRR_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (done.count({dev, func})) return OFRR_SUCCESS;
  int optin = 0;
  OFRR_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  OFRR_CUDA(cudaFuncGetAttributes(&fa, func));
  const int cap = optin - (int)fa.sharedSizeBytes;
  OFRR_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
  done.insert({dev, func});
  return OFRR_SUCCESS;
}

int map_cuda_error(cudaError_t e) {
  switch (e) {
    case cudaSuccess: return OFRR_SUCCESS;
    case cudaErrorMemoryAllocation: return OFRR_ERR_CUDA_MEMORY;
    case cudaErrorLaunchFailure:
    case cudaErrorInvalidConfiguration:
    case cudaErrorLaunchOutOfResources: return OFRR_ERR_CUDA_LAUNCH;
    default: return OFRR_ERR_CUDA_GENERAL;
  }
}

void note_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  fprintf(stderr, "[ofrr] CUDA error %s (%d) in %s at %s:%d\n", cudaGetErrorString(e), (int)e, what, file,
          line);
  (void)cudaGetLastError();  // reported here: do not charge it to this thread's next launch
}

void* ws_alloc(ofrr_ctx* ctx, size_t bytes, int* status) {
  const size_t align = 256;
  bytes = (bytes + align - 1) / align * align;
  if (bytes == 0) bytes = align;
  while (true) {
    if (ctx->cur_chunk < ctx->chunks.size()) {
      Chunk& c = ctx->chunks[ctx->cur_chunk];
      if (ctx->cur_off + bytes <= c.size) {
        void* p = c.ptr + ctx->cur_off;
        ctx->cur_off += bytes;
        return p;
      }
      // move to the next chunk (later chunks are only used after earlier ones fill up)
      if (ctx->cur_chunk + 1 < ctx->chunks.size()) {
        ctx->cur_chunk++;
        ctx->cur_off = 0;
        continue;
      }
    }
    size_t prev = ctx->chunks.empty() ? 0 : ctx->chunks.back().size;
    size_t sz = bytes > 2 * prev ? bytes : 2 * prev;
    if (sz < (size_t(64) << 20)) sz = size_t(64) << 20;
    Chunk c;
    cudaError_t e = cudaMalloc(&c.ptr, sz);
    if (e != cudaSuccess) {
      note_cuda_error(e, "workspace cudaMalloc", __FILE__, __LINE__);
      *status = OFRR_ERR_OUT_OF_MEMORY;
      return nullptr;
    }
    c.size = sz;
    ctx->chunks.push_back(c);
    ctx->cur_chunk = ctx->chunks.size() - 1;
    ctx->cur_off = 0;
  }
}

int after_launch(ofrr_ctx* ctx, const char* name) {
  ctx->launches++;
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    cudaGetLastError();
    note_cuda_error(e, name, __FILE__, __LINE__);
    return OFRR_ERR_CUDA_LAUNCH;
  }
  return OFRR_SUCCESS;
}

int sync_and_check(ofrr_ctx* ctx) {
  // words 2..4 of this context and of its auxiliary context (ordered behind ctx's stream by aux_end)
  OFRR_CUDA(cudaMemcpyAsync(ctx->host_flags, ctx->dev_flags + kFlagTcWait, 3 * sizeof(int), cudaMemcpyDeviceToHost,
                            ctx->stream));
  if (ctx->aux)
    OFRR_CUDA(cudaMemcpyAsync(ctx->host_flags + 3, ctx->aux->dev_flags + kFlagTcWait, 3 * sizeof(int),
                              cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_CUDA(cudaStreamSynchronize(ctx->stream));
  const int* h = ctx->host_flags;
  const bool timed_out = h[0] || h[2] || (ctx->aux && (h[3] || h[5]));
  if (timed_out) {
    OFRR_CUDA(cudaMemsetAsync(ctx->dev_flags + kFlagTcWait, 0, 3 * sizeof(int), ctx->stream));
    if (ctx->aux) OFRR_CUDA(cudaMemsetAsync(ctx->aux->dev_flags + kFlagTcWait, 0, 3 * sizeof(int), ctx->stream));
    OFRR_CUDA(cudaStreamSynchronize(ctx->stream));
    return OFRR_ERR_DEVICE_TIMEOUT;
  }
  return OFRR_SUCCESS;
}

int fill_zero(ofrr_ctx* ctx, void* p, size_t bytes) {
  if (bytes == 0) return OFRR_SUCCESS;
  OFRR_CUDA(cudaMemsetAsync(p, 0, bytes, ctx->stream));
  return OFRR_SUCCESS;
}

// --------------------------------------------------------------------------------------
// RNG: splitmix64 counter hash + Box-Muller (identical definition to the CPU oracle)
// --------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <class T>
__global__ void k_randn(uint64_t key, int64_t n, int64_t k, T* out, int64_t ld) {
  const int64_t total = n * k;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    uint64_t h1 = splitmix64(key + 2ull * (uint64_t)e);
    uint64_t h2 = splitmix64(key + 2ull * (uint64_t)e + 1ull);
    double u1 = ((double)(h1 >> 11) + 0.5) * 1.1102230246251565e-16;
    double u2 = (double)(h2 >> 11) * 1.1102230246251565e-16;
    double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    int64_t i = e % n, j = e / n;
    out[i + j * ld] = from_c<T, double>(z);
  }
}

// --------------------------------------------------------------------------------------
// casts
// --------------------------------------------------------------------------------------
template <class TI, class TO>
__global__ void k_cast(int64_t m, int64_t n, const TI* in, int64_t ldin, TO* out, int64_t ldout) {
  OFRR_FOR_2D(i, j, m, n) {
    // through FP32 when neither side is FP64 (exact: every 16/32-bit value is a float; RN once)
    if constexpr (std::is_same<TI, double>::value || std::is_same<TO, double>::value)
      out[i + j * ldout] = from_c<TO, double>(to_c<double, TI>(in[i + j * ldin]));
    else
      out[i + j * ldout] = from_c<TO, float>(to_c<float, TI>(in[i + j * ldin]));
  }
}

// --------------------------------------------------------------------------------------
// column argmax + scaling (scalecols.m:27-32)
// Argmax on integer keys of |x| (no FP64 compares); lowest row among equal maxima.  Columns up to
// 4 SC_CHUNK rows: one CTA (256 or 1024 threads) per column, values held in registers between the
// search and the scaling.
// Longer columns: a grid of (chunks x columns) CTAs finds per-chunk maxima (with their values),
// then the same grid reduces a column's chunk maxima and scales its chunk.
// --------------------------------------------------------------------------------------
constexpr int SC_T = 256;
constexpr int SC_U = 8;
constexpr int64_t SC_CHUNK = (int64_t)SC_T * SC_U;


template <class TO, class TC, bool FAST, int T>
__global__ void __launch_bounds__(T) k_scalecols_small(int64_t m, TO* U, int64_t ldu, int* piv, int do_scale) {
  __shared__ ArgMaxK red[T / 32];
  __shared__ TO s_t;
  __shared__ TC s_y;
  __shared__ bool s_pf;
  TO* col = U + (int64_t)blockIdx.x * ldu;
  TO v[SC_U];
  ArgMaxK a{-1, 0x7fffffffffffffffLL};
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = threadIdx.x + (int64_t)u * T;
    v[u] = (i < m) ? col[i] : TO(0);
  }
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = threadIdx.x + (int64_t)u * T;
    if (i < m) {
      const long long key = amax_key(v[u]);
      if (key > a.key) a = ArgMaxK{key, i};  // per-thread rows ascend: strict > keeps the lowest
    }
  }
  const ArgMaxK r = block_argmaxk(a, red);
  const int64_t k = (r.key < 0) ? 0 : r.i;
  if (threadIdx.x == 0) {
    if (piv) piv[blockIdx.x] = (int)k;
    s_t = (m > 0) ? col[k] : TO(0);
    const TC t0 = to_c<TC, TO>(s_t);
    // the reciprocal once per column: an FP64 reciprocal is a sequence of 1/64-rate instructions
    s_y = (t0 != TC(0)) ? pivot_recip(t0) : TC(0);
    s_pf = pivot_fast(t0);
  }
  __syncthreads();
  const TC t = to_c<TC, TO>(s_t);
  if (!do_scale || t == TC(0)) return;
  const TC y = s_y;
  const bool pf = s_pf;
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = threadIdx.x + (int64_t)u * T;
    if (i < m) col[i] = from_c<TO, TC>(scale_by<TC, FAST>(to_c<TC, TO>(v[u]), t, y, pf, i == k));
  }
}

template <class TO>
__global__ void __launch_bounds__(SC_T) k_colamax(int64_t m, const TO* U, int64_t ldu, ArgMaxK* part, double* pval) {
  __shared__ ArgMaxK red[SC_T / 32];
  const TO* col = U + (int64_t)blockIdx.y * ldu;
  const int64_t r0 = (int64_t)blockIdx.x * SC_CHUNK;
  TO v[SC_U];
  ArgMaxK a{-1, 0x7fffffffffffffffLL};
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SC_T;
    v[u] = (i < m) ? col[i] : TO(0);
  }
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SC_T;
    if (i < m) {
      const long long key = amax_key(v[u]);
      if (key > a.key) a = ArgMaxK{key, i};
    }
  }
  const ArgMaxK r = block_argmaxk(a, red);
  const size_t slot = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
  if (threadIdx.x == 0) part[slot] = r;
  // the maximum's value, read by the thread that holds it (before any CTA scales the column)
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SC_T;
    if (r.key >= 0 && i == r.i) pval[slot] = to_c<double, TO>(v[u]);
  }
}

template <class TO, class TC, bool FAST>
__global__ void __launch_bounds__(SC_T) k_colscale(int64_t m, TO* U, int64_t ldu, const ArgMaxK* part,
                                                   const double* pval, int* piv, int do_scale) {
  __shared__ double s_t;
  __shared__ long long s_k;
  __shared__ TC s_y;
  __shared__ bool s_pf;
  const int nchunks = gridDim.x;
  TO* col = U + (int64_t)blockIdx.y * ldu;
  if (threadIdx.x < 32) {
    ArgMaxK b{-1, 0x7fffffffffffffffLL};
    for (int c = threadIdx.x; c < nchunks; c += 32) b = argmaxk_pick(b, part[(size_t)blockIdx.y * nchunks + c]);
    b = warp_argmaxk(b);
    if (threadIdx.x == 0) {
      const int64_t k = (b.key < 0) ? 0 : b.i;
      s_k = k;
      s_t = (b.key < 0) ? 0.0 : pval[(size_t)blockIdx.y * nchunks + k / SC_CHUNK];
      if (piv && blockIdx.x == 0) piv[blockIdx.y] = (int)k;
      const TC t0 = to_c<TC, double>(s_t);
      s_y = (t0 != TC(0)) ? pivot_recip(t0) : TC(0);
      s_pf = pivot_fast(t0);
    }
  }
  __syncthreads();
  const TC t = to_c<TC, double>(s_t);
  if (!do_scale || t == TC(0)) return;
  const int64_t k = s_k;
  const TC y = s_y;
  const bool pf = s_pf;
  const int64_t r0 = (int64_t)blockIdx.x * SC_CHUNK;
  TO v[SC_U];
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SC_T;
    v[u] = (i < m) ? col[i] : TO(0);
  }
#pragma unroll
  for (int u = 0; u < SC_U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SC_T;
    if (i < m) col[i] = from_c<TO, TC>(scale_by<TC, FAST>(to_c<TC, TO>(v[u]), t, y, pf, i == k));
  }
}

// single-vector argmax with a grid of CTAs and a last-block-done reduction
template <class T>
__global__ void k_iamax(int64_t n, const T* x, ArgMax* partial, unsigned int* counter, int* out_idx1,
                        double* out_val) {
  __shared__ ArgMax red[32];
  __shared__ bool last;
  ArgMax a{-1.0, 0x7fffffffffffffffLL};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = absd(x[i]);
    if (v > a.v) a = ArgMax{v, i};
  }
  ArgMax r = block_argmax(a, red);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = r;
    __threadfence();
    unsigned int done = atomicAdd(counter, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  ArgMax b{-1.0, 0x7fffffffffffffffLL};
  const volatile ArgMax* vp = partial;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
    ArgMax p;
    p.v = vp[i].v;
    p.i = vp[i].i;
    b = argmax_pick(b, p);
  }
  ArgMax f = block_argmax(b, red);
  if (threadIdx.x == 0) {
    int64_t k = (f.v < 0.0) ? 0 : f.i;
    *out_idx1 = (n > 0) ? (int)(k + 1) : 0;
    *out_val = (n > 0) ? to_c<double, T>(x[k]) : 0.0;
    *counter = 0u;  // self-reset for the next call
  }
}

template <class T>
__global__ void k_special(int64_t m, int64_t n, const T* A, int64_t lda, int* flags) {
  int nan = 0, inf = 0;
  OFRR_FOR_2D(i, j, m, n) {
    double v = to_c<double, T>(A[i + j * lda]);
    if (isnan(v)) nan = 1;
    else if (isinf(v)) inf = 1;
  }
  if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1);
  if (__any_sync(0xffffffffu, inf) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 2);
}

// column 2-norms in FP64 (one CTA per column, fixed reduction order -> deterministic)
template <class T>
__global__ void k_colnorm(int64_t m, int64_t n, const T* X, int64_t ldx, double* out) {
  __shared__ double red[32];
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      double v = to_c<double, T>(X[i + j * ldx]);
      s = fma(v, v, s);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
      for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
      if (threadIdx.x == 0) out[j] = sqrt(t);
    }
    __syncthreads();
  }
}

// sqrt(sum_i f(i, j)^2) per column j over a grid of (row chunks x columns) CTAs: each CTA reduces its
// chunk in a fixed order (rows loaded CS_R at a time), the last CTA of a column (a self-resetting
// counter) adds the chunk sums in chunk order -- deterministic, and the FP64 work of a column spread
// over many SMs (one CTA per column was bound by one SM's 1/64-rate FP64 pipe).
constexpr int CS_T = 256, CS_R = 4;
template <class F>
__global__ void __launch_bounds__(CS_T) k_colsumsq(int64_t m, F f, double* __restrict__ part,
                                                  unsigned int* __restrict__ counters, double* __restrict__ out) {
  __shared__ double red[CS_T / 32];
  __shared__ bool last;
  const int64_t j = blockIdx.y;
  const int64_t r0 = (int64_t)blockIdx.x * CS_T * CS_R;
  double v[CS_R];
#pragma unroll
  for (int u = 0; u < CS_R; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * CS_T;
    v[u] = (i < m) ? f(i, j) : 0.0;
  }
  double s = 0.0;
#pragma unroll
  for (int u = 0; u < CS_R; ++u) s = fma(v[u], v[u], s);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < CS_T / 32; ++w) t += red[w];
    part[j * gridDim.x + blockIdx.x] = t;
    __threadfence();
    last = (atomicAdd(&counters[j], 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  const volatile double* pp = part + j * gridDim.x;
  double t = 0.0;
  for (unsigned c = 0; c < gridDim.x; ++c) t += pp[c];
  counters[j] = 0u;
  out[j] = sqrt(t);
}

template <class T>
struct ColValue {
  const T* X;
  int64_t ldx;
  __device__ double operator()(int64_t i, int64_t j) const { return to_c<double, T>(X[i + j * ldx]); }
};
struct ColResidualX {  // A x_j - lam_j x_j (separate leading dimensions)
  const double* AX;
  int64_t ldax;
  const double* X;
  int64_t ldx;
  const double* lam;
  __device__ double operator()(int64_t i, int64_t j) const { return AX[i + j * ldax] - lam[j] * X[i + j * ldx]; }
};
struct ColResidual {  // A v_j - s_j u_j
  const double* AV;
  const double* U;
  const double* s;
  int64_t ld;
  __device__ double operator()(int64_t i, int64_t j) const { return AV[i + j * ld] - s[j] * U[i + j * ld]; }
};

template <class F>
static int colsumsq_launch(ofrr_ctx* ctx, int64_t m, int64_t n, F f, double* out) {
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  const int64_t chunks = (m + CS_T * CS_R - 1) / (CS_T * CS_R);
  double* part = ws_get<double>(ctx, (size_t)chunks * n, &st);
  if (!part) return st;
  k_colsumsq<F><<<dim3((unsigned)chunks, (unsigned)n), CS_T, 0, ctx->stream>>>(m, f, part, ctx->dev_counters, out);
  OFRR_LAUNCHED(ctx, "k_colsumsq");
  return OFRR_SUCCESS;
}

// ||A v_j - s_j u_j||_2 per column (FP64; AV and U m x n with leading dimension m)
int residual_columns2(ofrr_ctx* ctx, int64_t m, int64_t n, const double* AV, const double* U, const double* s,
                      double* out) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 1024 || m <= 0 || (m + CS_T * CS_R - 1) / (CS_T * CS_R) > 65535) return OFRR_ERR_BLAS_INVALID_SIZE;
  return colsumsq_launch(ctx, m, n, ColResidual{AV, U, s, m}, out);
}

// ||AX(:,j) - lam_j X(:,j)||_2 per column, FP64
__global__ void k_rescol(int64_t m, int64_t n, const double* AX, int64_t ldax, const double* X, int64_t ldx,
                         const double* lam, double* out) {
  __shared__ double red[32];
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const double l = lam[j];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      double r = AX[i + j * ldax] - l * X[i + j * ldx];
      s = fma(r, r, s);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      double t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
      for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
      if (threadIdx.x == 0) out[j] = sqrt(t);
    }
    __syncthreads();
  }
}

int cast_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, int64_t m, int64_t n, const void* in, int64_t ldin,
              void* out, int64_t ldout) {
  if (m <= 0 || n <= 0) return OFRR_SUCCESS;
  OFRR_DISPATCH_STORAGE(tin, TI, OFRR_DISPATCH_STORAGE(tout, TO, {
    k_cast<TI, TO><<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, (const TI*)in, ldin, (TO*)out, ldout);
    OFRR_LAUNCHED(ctx, "k_cast");
  }));
  return OFRR_SUCCESS;
}

template <class TO, class TC, bool FAST>
static int scalecols_t(ofrr_ctx* ctx, int64_t m, int64_t n, TO* U, int64_t ldu, int* piv, int do_scale = 1) {
  if (m <= SC_CHUNK) {
    k_scalecols_small<TO, TC, FAST, SC_T><<<(unsigned)n, SC_T, 0, ctx->stream>>>(m, U, ldu, piv, do_scale);
    OFRR_LAUNCHED(ctx, "k_scalecols_small");
    return OFRR_SUCCESS;
  }
  if (m <= 4 * SC_CHUNK) {  // up to 8192 rows: still one CTA per column, 1024 threads
    k_scalecols_small<TO, TC, FAST, 4 * SC_T><<<(unsigned)n, 4 * SC_T, 0, ctx->stream>>>(m, U, ldu, piv, do_scale);
    OFRR_LAUNCHED(ctx, "k_scalecols_small");
    return OFRR_SUCCESS;
  }
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  const int64_t nchunks = (m + SC_CHUNK - 1) / SC_CHUNK;
  if (nchunks > 65535) return OFRR_ERR_BLAS_INVALID_SIZE;
  ArgMaxK* part = ws_get<ArgMaxK>(ctx, (size_t)nchunks * n, &st);
  if (!part) return st;
  double* pval = ws_get<double>(ctx, (size_t)nchunks * n, &st);
  if (!pval) return st;
  const dim3 grid((unsigned)nchunks, (unsigned)n);
  k_colamax<TO><<<grid, SC_T, 0, ctx->stream>>>(m, U, ldu, part, pval);
  OFRR_LAUNCHED(ctx, "k_colamax");
  k_colscale<TO, TC, FAST><<<grid, SC_T, 0, ctx->stream>>>(m, U, ldu, part, pval, piv, do_scale);
  OFRR_LAUNCHED(ctx, "k_colscale");
  return OFRR_SUCCESS;
}

int scalecols_impl(ofrr_ctx* ctx, ofrr_dtype po, ofrr_dtype pc, int64_t m, int64_t n, void* U, int64_t ldu,
                   int* piv, bool fast) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 65535) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (fast && pc == OFRR_F64) {
    OFRR_DISPATCH_STORAGE(po, TO, { OFRR_TRY((scalecols_t<TO, double, true>(ctx, m, n, (TO*)U, ldu, piv))); });
    return OFRR_SUCCESS;
  }
  OFRR_DISPATCH_STORAGE(po, TO, OFRR_DISPATCH_COMPUTE(pc, TC, {
    OFRR_TRY((scalecols_t<TO, TC, false>(ctx, m, n, (TO*)U, ldu, piv)));
  }));
  return OFRR_SUCCESS;
}

int column_norms(ofrr_ctx* ctx, ofrr_dtype t, int64_t m, int64_t n, const void* X, int64_t ldx, double* out) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n <= 1024 && m >= 2048 && (m + CS_T * CS_R - 1) / (CS_T * CS_R) <= 65535) {  // tall columns: many CTAs each
    OFRR_DISPATCH_STORAGE(t, T, { OFRR_TRY(colsumsq_launch(ctx, m, n, ColValue<T>{(const T*)X, ldx}, out)); });
    return OFRR_SUCCESS;
  }
  int grid = (int)(n < 65535 ? n : 65535);
  OFRR_DISPATCH_STORAGE(t, T, {
    k_colnorm<T><<<grid, 256, 0, ctx->stream>>>(m, n, (const T*)X, ldx, out);
    OFRR_LAUNCHED(ctx, "k_colnorm");
  });
  return OFRR_SUCCESS;
}

int residual_columns(ofrr_ctx* ctx, int64_t m, int64_t n, const double* AX, int64_t ldax, const double* X,
                     int64_t ldx, const double* lam, double* out) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n <= 1024 && m >= 2048 && (m + CS_T * CS_R - 1) / (CS_T * CS_R) <= 65535)
    return colsumsq_launch(ctx, m, n, ColResidualX{AX, ldax, X, ldx, lam}, out);
  int grid = (int)(n < 65535 ? n : 65535);
  k_rescol<<<grid, 256, 0, ctx->stream>>>(m, n, AX, ldax, X, ldx, lam, out);
  OFRR_LAUNCHED(ctx, "k_rescol");
  return OFRR_SUCCESS;
}

// One CTA waits on an mbarrier that nothing arrives on; the bounded wait gives up after timeout_ns,
// records the timeout in the status word of the tcgen05 pipelines and returns.
__global__ void k_bounded_wait_probe(unsigned long long timeout_ns, int* err) {
  __shared__ __align__(8) unsigned long long bar;
  const unsigned baddr = (unsigned)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(baddr) : "memory");
  __syncthreads();
  if (threadIdx.x != 0) return;
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  while (true) {
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(baddr)
                 : "memory");
    if (ok) return;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > timeout_ns) {
      atomicCAS(err, 0, 99);
      return;
    }
  }
}

}  // namespace ofrr

using namespace ofrr;

// ======================================================================================
// C ABI: context and level-1/2 entry points
// ======================================================================================
extern "C" {

const char* ofrr_version(void) { return "ofrr-gb300 0.1 (sm_103a)"; }

const char* ofrr_status_string(int s) {
  switch (s) {
    case OFRR_SUCCESS: return "Success";
    case OFRR_ERR_INVALID_ARGUMENT: return "Invalid argument";
    case OFRR_ERR_INVALID_OPERATION: return "Invalid operation";
    case OFRR_ERR_OUT_OF_MEMORY: return "Out of memory";
    case OFRR_ERR_NOT_IMPLEMENTED: return "Not implemented";
    case OFRR_ERR_INTERNAL: return "Internal error";
    case OFRR_ERR_NAN: return "NaN value detected";
    case OFRR_ERR_INF: return "Inf value detected";
    case OFRR_ERR_BLAS_INVALID_LOCATION: return "BLAS: invalid location";
    case OFRR_ERR_BLAS_UNSUPPORTED_TYPE: return "BLAS: unsupported type";
    case OFRR_ERR_BLAS_CUBLAS: return "BLAS: cuBLAS failure";
    case OFRR_ERR_BLAS_INVALID_SIZE: return "BLAS: invalid size";
    case OFRR_ERR_FACTORIZATION_FAILED: return "Factorization failed";
    case OFRR_ERR_SINGULAR_MATRIX: return "Singular matrix";
    case OFRR_ERR_SOLVER_DIVERGENCE: return "Solver divergence";
    case OFRR_ERR_SOLVER_MAX_ITERATIONS: return "Solver reached max iterations";
    case OFRR_ERR_FILE_NOT_FOUND: return "File not found";
    case OFRR_ERR_INVALID_FORMAT: return "Invalid format";
    case OFRR_ERR_CUDA_GENERAL: return "CUDA error";
    case OFRR_ERR_CUDA_MEMORY: return "CUDA memory error";
    case OFRR_ERR_CUDA_LAUNCH: return "CUDA launch error";
    case OFRR_ERR_CUDA_SYNC: return "CUDA synchronization error";
    case OFRR_ERR_DEVICE_TIMEOUT: return "Device-side wait timed out";
  }
  return "Unknown status";
}

int ofrr_ctx_create(ofrr_ctx** out, int device, void* stream) {
  if (!out) return OFRR_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  ofrr_ctx* ctx = new (std::nothrow) ofrr_ctx();
  if (!ctx) return OFRR_ERR_OUT_OF_MEMORY;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete ctx;
    return map_cuda_error(e);
  }
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      return map_cuda_error(e);
    }
    ctx->owns_stream = true;
  }
  if (cublasCreate(&ctx->cublas) != CUBLAS_STATUS_SUCCESS) {
    if (ctx->owns_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return OFRR_ERR_BLAS_CUBLAS;
  }
  cublasSetStream(ctx->cublas, ctx->stream);
  cublasSetMathMode(ctx->cublas, CUBLAS_PEDANTIC_MATH);  // no TF32 / reduced-precision shortcuts
  e = cudaMalloc(&ctx->dev_flags, 64 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&ctx->dev_counters, 1024 * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(ctx->dev_flags, 0, 64 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(ctx->dev_counters, 0, 1024 * sizeof(unsigned int));
  if (e == cudaSuccess) {
    ctx->pinned_size = 1 << 20;
    e = cudaMallocHost(&ctx->pinned, ctx->pinned_size);
  }
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->host_flags, 8 * sizeof(int));
  if (e == cudaSuccess) memset(ctx->host_flags, 0, 8 * sizeof(int));
  if (e == cudaSuccess) {
    const char* tp = getenv("OFRR_TRACE_FILE");
    if (tp && *tp) ofrr_ctx_set_trace(ctx, tp);
  }
  if (e != cudaSuccess) {
    ofrr_ctx_destroy(ctx);
    return map_cuda_error(e);
  }
  *out = ctx;
  return OFRR_SUCCESS;
}

int ofrr_ctx_destroy(ofrr_ctx* ctx) {
  if (!ctx) return OFRR_SUCCESS;
  cudaSetDevice(ctx->device);
  if (ctx->aux) ofrr_ctx_destroy(ctx->aux);
  trace_destroy(ctx);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& c : ctx->chunks) cudaFree(c.ptr);
  if (ctx->dev_flags) cudaFree(ctx->dev_flags);
  if (ctx->dev_counters) cudaFree(ctx->dev_counters);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->host_flags) cudaFreeHost(ctx->host_flags);
  if (ctx->cublas) cublasDestroy(ctx->cublas);
  if (ctx->owns_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return OFRR_SUCCESS;
}

int ofrr_ctx_set_stream(ofrr_ctx* ctx, void* stream) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  if (ctx->owns_stream && ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  ctx->owns_stream = false;
  ctx->stream = (cudaStream_t)stream;
  cublasSetStream(ctx->cublas, ctx->stream);
  return OFRR_SUCCESS;
}

void* ofrr_ctx_get_stream(ofrr_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int ofrr_debug_bounded_wait(ofrr_ctx* ctx, int64_t timeout_ns) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  const long long t = timeout_ns < 1000 ? 1000 : (timeout_ns > 1000000000LL ? 1000000000LL : timeout_ns);
  ofrr::k_bounded_wait_probe<<<1, 32, 0, ctx->stream>>>((unsigned long long)t, ctx->dev_flags + kFlagTcWait);
  OFRR_LAUNCHED(ctx, "k_bounded_wait_probe");
  return OFRR_SUCCESS;
}

int ofrr_ctx_synchronize(ofrr_ctx* ctx) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  return sync_and_check(ctx);
}

uint64_t ofrr_ctx_launch_count(ofrr_ctx* ctx) {
  return ctx ? ctx->launches + (ctx->aux ? ctx->aux->launches : 0) : 0;
}
void ofrr_ctx_reset_launch_count(ofrr_ctx* ctx) {
  if (ctx) ctx->launches = 0;
  if (ctx && ctx->aux) ctx->aux->launches = 0;
}
int ofrr_ctx_trim(ofrr_ctx* ctx) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  if (ctx->cur_chunk != 0 || ctx->cur_off != 0) return OFRR_ERR_INVALID_ARGUMENT;  // allocations live
  OFRR_CUDA(cudaStreamSynchronize(ctx->stream));
  for (Chunk& c : ctx->chunks) cudaFree(c.ptr);
  ctx->chunks.clear();
  return OFRR_SUCCESS;
}

size_t ofrr_ctx_workspace_bytes(ofrr_ctx* ctx) {
  size_t s = 0;
  if (ctx)
    for (auto& c : ctx->chunks) s += c.size;
  return s;
}

int ofrr_randn(ofrr_ctx* ctx, uint64_t seed, int64_t n, int64_t k, ofrr_dtype dt, void* out, int64_t ld) {
  if (!ctx || n < 0 || k < 0 || (n > 0 && k > 0 && (!out || ld < n))) return OFRR_ERR_INVALID_ARGUMENT;
  if (n == 0 || k == 0) return OFRR_SUCCESS;
  uint64_t key = splitmix64(seed);
  OFRR_DISPATCH_STORAGE(dt, T, {
    k_randn<T><<<grid_for(n * k, 256), 256, 0, ctx->stream>>>(key, n, k, (T*)out, ld);
    OFRR_LAUNCHED(ctx, "k_randn");
  });
  return OFRR_SUCCESS;
}

void ofrr_randn_host(uint64_t seed, int64_t n, int64_t k, double* out) {
  if (!out) return;
  uint64_t key = splitmix64(seed);
  for (int64_t e = 0; e < n * k; ++e) {
    uint64_t h1 = splitmix64(key + 2ull * (uint64_t)e);
    uint64_t h2 = splitmix64(key + 2ull * (uint64_t)e + 1ull);
    double u1 = ((double)(h1 >> 11) + 0.5) * 1.1102230246251565e-16;
    double u2 = (double)(h2 >> 11) * 1.1102230246251565e-16;
    out[e] = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
}

int ofrr_cast(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, int64_t m, int64_t n, const void* in, int64_t ldin,
              void* out, int64_t ldout) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(tin) || !dtype_valid(tout)) return OFRR_ERR_INVALID_ARGUMENT;
  if (m > 0 && n > 0 && (!in || !out || ldin < m || ldout < m)) return OFRR_ERR_INVALID_ARGUMENT;
  return cast_impl(ctx, tin, tout, m, n, in, ldin, out, ldout);
}

int ofrr_scalecols(ofrr_ctx* ctx, ofrr_dtype po, ofrr_dtype pc, int64_t m, int64_t n, void* U, int64_t ldu,
                   int* piv) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(po)) return OFRR_ERR_INVALID_ARGUMENT;
  if (pc != OFRR_F64 && pc != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (m > 0 && n > 0 && (!U || ldu < m)) return OFRR_ERR_INVALID_ARGUMENT;
  if (m == 0) return OFRR_SUCCESS;
  return scalecols_impl(ctx, po, pc, m, n, U, ldu, piv);
}

int ofrr_matrix_iamax(ofrr_ctx* ctx, ofrr_dtype dt, int64_t m, int64_t n, const void* A, int64_t lda, int* idx) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(dt)) return OFRR_ERR_INVALID_ARGUMENT;
  if (m > 0 && n > 0 && (!A || !idx || lda < m)) return OFRR_ERR_INVALID_ARGUMENT;
  if (m == 0 || n == 0) return OFRR_SUCCESS;
  if (n > 65535) return OFRR_ERR_BLAS_INVALID_SIZE;
  OFRR_DISPATCH_STORAGE(dt, T, { OFRR_TRY((scalecols_t<T, double, false>(ctx, m, n, (T*)A, lda, idx, 0))); });
  return OFRR_SUCCESS;
}

int ofrr_iamax(ofrr_ctx* ctx, ofrr_dtype dt, int64_t n, const void* x, int* idx1, double* val) {
  if (!ctx || n < 0 || !dtype_valid(dt) || !idx1 || !val) return OFRR_ERR_INVALID_ARGUMENT;
  if (n == 0) {
    *idx1 = 0;
    *val = 0.0;
    return OFRR_SUCCESS;
  }
  if (!x) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int grid = grid_for(n, 1024, 304);
  ArgMax* partial = ws_get<ArgMax>(ctx, grid, &st);
  if (!partial) return st;
  int* dres = ws_get<int>(ctx, 4, &st);
  if (!dres) return st;
  double* dval = reinterpret_cast<double*>(dres + 2);
  OFRR_DISPATCH_STORAGE(dt, T, {
    k_iamax<T><<<grid, 1024, 0, ctx->stream>>>(n, (const T*)x, partial, ctx->dev_counters, dres, dval);
    OFRR_LAUNCHED(ctx, "k_iamax");
  });
  int* hp = (int*)ctx->pinned;
  OFRR_CUDA(cudaMemcpyAsync(hp, dres, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  *idx1 = hp[0];
  std::memcpy(val, hp + 2, sizeof(double));
  return OFRR_SUCCESS;
}

int ofrr_check_special_values(ofrr_ctx* ctx, ofrr_dtype dt, int64_t m, int64_t n, const void* A, int64_t lda) {
  if (!ctx || m < 0 || n < 0 || !dtype_valid(dt)) return OFRR_ERR_INVALID_ARGUMENT;
  if (m == 0 || n == 0) return OFRR_SUCCESS;
  if (!A || lda < m) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_CUDA(cudaMemsetAsync(ctx->dev_flags, 0, sizeof(int), ctx->stream));
  OFRR_DISPATCH_STORAGE(dt, T, {
    k_special<T><<<grid_2d(m, n, 256), 256, 0, ctx->stream>>>(m, n, (const T*)A, lda, ctx->dev_flags);
    OFRR_LAUNCHED(ctx, "k_special");
  });
  int* hp = (int*)ctx->pinned;
  OFRR_CUDA(cudaMemcpyAsync(hp, ctx->dev_flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  if (hp[0] & 1) return OFRR_ERR_NAN;
  if (hp[0] & 2) return OFRR_ERR_INF;
  return OFRR_SUCCESS;
}

}  // extern "C"
