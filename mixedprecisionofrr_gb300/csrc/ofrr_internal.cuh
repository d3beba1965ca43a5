// Internal declarations shared by the translation units of libofrr_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <type_traits>
#include <utility>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cublas_v2.h>
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <cstdio>
#include <vector>
#include <algorithm>

#include "../../include/ofrr.h"

// --------------------------------------------------------------------------------------
// status helpers
// --------------------------------------------------------------------------------------
#define OFRR_TRY(expr)                        \
  do {                                        \
    int _st = (expr);                         \
    if (_st != OFRR_SUCCESS) return _st;      \
  } while (0)

#define OFRR_CUDA(expr)                                                   \
  do {                                                                    \
    cudaError_t _e = (expr);                                              \
    if (_e != cudaSuccess) {                                              \
      ofrr::note_cuda_error(_e, #expr, __FILE__, __LINE__);               \
      return ofrr::map_cuda_error(_e);                                    \
    }                                                                     \
  } while (0)

#define OFRR_CUBLAS(expr)                                                 \
  do {                                                                    \
    cublasStatus_t _s = (expr);                                           \
    if (_s != CUBLAS_STATUS_SUCCESS) {                                    \
      fprintf(stderr, "[ofrr] cuBLAS error %d at %s:%d\n", (int)_s, __FILE__, __LINE__); \
      return OFRR_ERR_BLAS_CUBLAS;                                        \
    }                                                                     \
  } while (0)

namespace ofrr {

int map_cuda_error(cudaError_t e);
void note_cuda_error(cudaError_t e, const char* what, const char* file, int line);

// --------------------------------------------------------------------------------------
// context: stream, cuBLAS handle, chunked device workspace (never moves once handed out)
// --------------------------------------------------------------------------------------
struct Chunk {
  char* ptr = nullptr;
  size_t size = 0;
};

struct WsMark {
  size_t chunk;
  size_t offset;
};

struct Tracer;

}  // namespace ofrr

struct ofrr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  cublasHandle_t cublas = nullptr;
  std::vector<ofrr::Chunk> chunks;
  size_t cur_chunk = 0;
  size_t cur_off = 0;
  unsigned long long launches = 0;        // kernels of this library
  unsigned long long library_calls = 0;   // cuBLAS calls (library kernels, counted apart)
  int* dev_flags = nullptr;        // device status words written by kernels (bounded waits etc.)
  int* host_flags = nullptr;       // pinned copy of the wait-timeout words, read after each stream sync
  unsigned int* dev_counters = nullptr;  // grid "last block" counters (self-resetting)
  void* pinned = nullptr;          // small pinned host staging buffer
  bool emulate_f64 = false;        // FP64 TN products through exact BF16 slices on the tensor cores
  bool power_f8 = false;           // 16-bit power steps through E4M3 copies (the FP8 variant)
  size_t pinned_size = 0;
  ofrr_ctx* aux = nullptr;         // second stream + workspace for independent work run beside this one
  ofrr::Tracer* tracer = nullptr;  // per-solve phase events and the JSON-lines sink (trace.cu), or null
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace ofrr {

// workspace ---------------------------------------------------------------------------
void* ws_alloc(ofrr_ctx* ctx, size_t bytes, int* status);
inline WsMark ws_mark(ofrr_ctx* ctx) { return WsMark{ctx->cur_chunk, ctx->cur_off}; }
inline void ws_release(ofrr_ctx* ctx, WsMark m) {
  ctx->cur_chunk = m.chunk;
  ctx->cur_off = m.offset;
}
template <class T>
inline T* ws_get(ofrr_ctx* ctx, size_t count, int* status) {
  return static_cast<T*>(ws_alloc(ctx, count * sizeof(T), status));
}
// RAII scope: everything allocated inside is released at scope exit
struct WsScope {
  ofrr_ctx* ctx;
  WsMark m;
  explicit WsScope(ofrr_ctx* c) : ctx(c), m(ws_mark(c)) {}
  ~WsScope() { ws_release(ctx, m); }
};

// launch accounting -------------------------------------------------------------------
int after_launch(ofrr_ctx* ctx, const char* name);
#define OFRR_LAUNCHED(ctx, name) OFRR_TRY(ofrr::after_launch((ctx), (name)))

// Device status words (ctx->dev_flags): 0 special values found by the input check, 1 small-solver
// breakdown, 2 a tcgen05 pipeline wait that ran out (TMA / MMA / epilogue barriers), 3 non-convergence
// of the nonsymmetric small solver, 4 a cluster wait of the blocked Hessenberg build that ran out.
constexpr int kFlagTcWait = 2;
constexpr int kFlagHessWait = 4;

// Synchronise ctx's stream; OFRR_ERR_DEVICE_TIMEOUT when a bounded device wait gave up since the
// last check (the words are cleared again).
int sync_and_check(ofrr_ctx* ctx);

// Concurrency inside one solve: aux_begin() returns the context's auxiliary context (created on
// first use: same device, its own stream, cuBLAS handle and workspace) after ordering its stream
// behind everything queued on ctx's stream; work queued on it runs beside ctx's own; aux_end()
// orders ctx's stream behind it again.
int aux_begin(ofrr_ctx* ctx, ofrr_ctx** aux);

// Phase tracing (trace.cu): a TraceScope opens an NVTX range and, with a sink set on the context,
// brackets the phase with CUDA events on ctx's stream; trace_end_solve appends the solve's record.
struct TraceScope {
  ofrr_ctx* ctx;
  int idx = -1;
  TraceScope(ofrr_ctx* c, const char* name);
  ~TraceScope();
  void next(const char* name);  // ends this phase and opens the next one
  TraceScope(const TraceScope&) = delete;
  TraceScope& operator=(const TraceScope&) = delete;
};
void trace_begin_solve(ofrr_ctx* ctx);
void trace_end_solve(ofrr_ctx* ctx, const char* solver, int64_t m, int64_t n, const ofrr_options* opt, int status,
                     const ofrr_info* info, unsigned long long launches);
void trace_destroy(ofrr_ctx* ctx);
int aux_end(ofrr_ctx* ctx);

// kernel attributes ---------------------------------------------------------------------
// Raises a kernel's dynamic shared memory cap to the device's opt-in maximum, once per (device,
// kernel).  Kernels size their shared memory per launch; a fixed cap keeps concurrent host threads
// (the solve engine) from lowering each other's limit between an attribute call and a launch.
int allow_dynamic_smem(const void* func);
template <class F>
inline int allow_smem(F* f) {
  return allow_dynamic_smem(reinterpret_cast<const void*>(f));
}

// element sizes -----------------------------------------------------------------------
inline size_t dtype_size(ofrr_dtype t) {
  switch (t) {
    case OFRR_F64: return 8;
    case OFRR_F32: return 4;
    case OFRR_F16: return 2;
    case OFRR_BF16: return 2;
  }
  return 0;
}
inline bool dtype_valid(int t) { return t >= 0 && t <= 3; }
inline double dtype_eps(ofrr_dtype t) {
  switch (t) {
    case OFRR_F64: return 2.220446049250313e-16;
    case OFRR_F32: return 1.1920928955078125e-07;
    case OFRR_F16: return 9.765625e-04;  // 2^-10, MATLAB/+src/+utils/eps.m:24
    case OFRR_BF16: return 7.8125e-03;   // 2^-7
  }
  return 0;
}

// conversions with explicit round-to-nearest-even (no contraction, no fast-math) ------
template <class TC, class T> __device__ __forceinline__ TC to_c(T x);
template <> __device__ __forceinline__ double to_c<double, double>(double x) { return x; }
template <> __device__ __forceinline__ double to_c<double, float>(float x) { return (double)x; }
template <> __device__ __forceinline__ double to_c<double, __half>(__half x) { return (double)__half2float(x); }
template <> __device__ __forceinline__ double to_c<double, __nv_bfloat16>(__nv_bfloat16 x) { return (double)__bfloat162float(x); }
template <> __device__ __forceinline__ float to_c<float, double>(double x) { return __double2float_rn(x); }
template <> __device__ __forceinline__ float to_c<float, float>(float x) { return x; }
template <> __device__ __forceinline__ float to_c<float, __half>(__half x) { return __half2float(x); }
template <> __device__ __forceinline__ float to_c<float, __nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }

template <class T, class TC> __device__ __forceinline__ T from_c(TC x);
template <> __device__ __forceinline__ double from_c<double, double>(double x) { return x; }
template <> __device__ __forceinline__ float from_c<float, double>(double x) { return __double2float_rn(x); }
template <> __device__ __forceinline__ __half from_c<__half, double>(double x) { return __double2half(x); }
template <> __device__ __forceinline__ __nv_bfloat16 from_c<__nv_bfloat16, double>(double x) { return __double2bfloat16(x); }
template <> __device__ __forceinline__ double from_c<double, float>(float x) { return (double)x; }
template <> __device__ __forceinline__ float from_c<float, float>(float x) { return x; }
template <> __device__ __forceinline__ __half from_c<__half, float>(float x) { return __float2half_rn(x); }
template <> __device__ __forceinline__ __nv_bfloat16 from_c<__nv_bfloat16, float>(float x) { return __float2bfloat16_rn(x); }

// |x| as a double for comparisons (exact for every storage type)
template <class T> __device__ __forceinline__ double absd(T x) { return fabs(to_c<double, T>(x)); }

// IEEE single-rounding arithmetic helpers
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

// x / p, correctly rounded, for many x and one p (a pivot, a column maximum), given y = RN(1/p).  In FP64 (a 1/64-rate pipe on GB300) the
// correctly rounded quotient comes from one multiply and four FMAs: q0 = RN(x y), one correction
// q1 = RN(q0 + RN(x - p q0) y) makes q1 faithful, and by Markstein's theorem (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34, 1990) the
// second correction RN(q1 + (x - p q1) y), with x - p q1 exact, is RN(x / p).  Operands outside
// [2^-900, 2^900] (where an intermediate could underflow or overflow) use the division itself.
__device__ __forceinline__ double pivot_recip(double p) { return __drcp_rn(p); }
__device__ __forceinline__ float pivot_recip(float p) { return __frcp_rn(p); }
__device__ __forceinline__ bool pivot_fast(double p) {
  const double a = fabs(p);
  return a >= 0x1p-450 && a <= 0x1p+450;
}
__device__ __forceinline__ bool pivot_fast(float) { return false; }
__device__ __forceinline__ double pivot_div(double x, double p, double y, bool fast) {
  const double ax = fabs(x);
  if (fast && ax >= 0x1p-900 && ax <= 0x1p+900) {
    const double q0 = __dmul_rn(x, y);
    const double r0 = __fma_rn(-p, q0, x);
    const double q1 = __fma_rn(r0, y, q0);
    const double r1 = __fma_rn(-p, q1, x);
    return __fma_rn(r1, y, q1);
  }
  return __ddiv_rn(x, p);
}
__device__ __forceinline__ float pivot_div(float x, float p, float, bool) { return __fdiv_rn(x, p); }

// q / t for scalecols: FAST (FP64 production phase) multiplies by the reciprocal (within an ulp of
// q / t, the pivot itself exactly 1), otherwise the correctly rounded quotient
template <class TC, bool FAST>
__device__ __forceinline__ TC scale_by(TC q, TC t, TC y, bool pf, bool is_pivot) {
  if (FAST && pf) return is_pivot ? TC(1) : mul_rn(q, y);
  return pivot_div(q, t, y, pf);
}


// argmax reduction on (|value|, index): larger value wins, lower index on ties, NaN ignored
struct ArgMax {
  double v;  // -1 means "empty"
  long long i;
};
__device__ __forceinline__ ArgMax argmax_pick(ArgMax a, ArgMax b) {
  if (b.v > a.v || (b.v == a.v && b.i < a.i && b.v >= 0.0)) return b;
  return a;
}
__device__ __forceinline__ ArgMax warp_argmax(ArgMax a) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ArgMax b;
    b.v = __shfl_down_sync(0xffffffffu, a.v, off);
    b.i = __shfl_down_sync(0xffffffffu, a.i, off);
    a = argmax_pick(a, b);
  }
  return a;
}
// block-wide argmax; result valid in thread 0.  smem needs blockDim/32 entries.
__device__ __forceinline__ ArgMax block_argmax(ArgMax a, ArgMax* smem) {
  a = warp_argmax(a);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) smem[wid] = a;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (wid == 0) {
    ArgMax b = (lane < nw) ? smem[lane] : ArgMax{-1.0, 0x7fffffffffffffffLL};
    b = warp_argmax(b);
    if (lane == 0) smem[0] = b;
  }
  __syncthreads();
  ArgMax r = smem[0];
  __syncthreads();
  return r;
}

// Integer argmax keys.  For IEEE formats the bit pattern of |x| orders like |x|, so max-|x| searches
// run on the integer pipes instead of FP64 compares (GB300's FP64 pipe is 1/64 rate).  key = bits + 1
// for numbers, 0 for NaN (never preferred over a number, as with floating compares), -1 = empty.
__device__ __forceinline__ long long amax_key(double x) {
  const long long b = __double_as_longlong(x) & 0x7fffffffffffffffLL;
  return (b > 0x7ff0000000000000LL) ? 0 : b + 1;
}
__device__ __forceinline__ long long amax_key(float x) {
  const int b = __float_as_int(x) & 0x7fffffff;
  return (b > 0x7f800000) ? 0 : (long long)b + 1;
}
__device__ __forceinline__ long long amax_key(__half x) {
  const int b = __half_as_ushort(x) & 0x7fff;
  return (b > 0x7c00) ? 0 : (long long)b + 1;
}
__device__ __forceinline__ long long amax_key(__nv_bfloat16 x) {
  const int b = __bfloat16_as_ushort(x) & 0x7fff;
  return (b > 0x7f80) ? 0 : (long long)b + 1;
}
struct ArgMaxK {
  long long key;  // -1 means "empty"
  long long i;
};
__device__ __forceinline__ ArgMaxK argmaxk_pick(ArgMaxK a, ArgMaxK b) {
  if (b.key > a.key || (b.key == a.key && b.i < a.i && b.key >= 0)) return b;
  return a;
}
__device__ __forceinline__ ArgMaxK warp_argmaxk(ArgMaxK a) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ArgMaxK b;
    b.key = __shfl_down_sync(0xffffffffu, a.key, off);
    b.i = __shfl_down_sync(0xffffffffu, a.i, off);
    a = argmaxk_pick(a, b);
  }
  return a;
}
// Same result as warp_argmaxk, in every lane, from three warp-wide integer reductions (redux.sync):
// the larger key (as two 32-bit halves), then the lowest row among lanes holding it.  Rows must lie
// in [0, 2^32 - 2] for non-empty entries.
__device__ __forceinline__ ArgMaxK warp_argmaxk_all(ArgMaxK a) {
  const unsigned long long k1 = (unsigned long long)(a.key + 1);  // 0: empty
  const unsigned hi = (unsigned)(k1 >> 32), lo = (unsigned)k1;
  const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
  const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
  const bool win = (hi == mhi && lo == mlo);
  const unsigned mi = __reduce_min_sync(0xffffffffu, win ? (unsigned)a.i : 0xffffffffu);
  ArgMaxK r;
  r.key = (long long)(((unsigned long long)mhi << 32) | mlo) - 1;
  r.i = (r.key >= 0) ? (long long)mi : 0x7fffffffffffffffLL;
  return r;
}

// block-wide argmax, result returned to every thread.  smem needs blockDim/32 entries.
__device__ __forceinline__ ArgMaxK block_argmaxk(ArgMaxK a, ArgMaxK* smem) {
  a = warp_argmaxk(a);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) smem[wid] = a;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (wid == 0) {
    ArgMaxK b = (lane < nw) ? smem[lane] : ArgMaxK{-1, 0x7fffffffffffffffLL};
    b = warp_argmaxk(b);
    if (lane == 0) smem[0] = b;
  }
  __syncthreads();
  ArgMaxK r = smem[0];
  __syncthreads();
  return r;
}

// Per-column kernels over a cluster of CL CTAs of SCS_T threads (scale and split, split-K combine and
// scale): CTA r of a column's cluster holds rows [r SCS_T U, (r + 1) SCS_T U), U per thread.
constexpr int SCS_T = 1024;
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared-memory address of this CTA's variable p in CTA `rank` of the cluster
__device__ __forceinline__ unsigned cluster_map(const void* p, unsigned rank) {
  unsigned a = (unsigned)__cvta_generic_to_shared(p), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster_u64(unsigned addr, unsigned long long v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

// Launch of a per-column scaling kernel: ncols clusters of cl CTAs of SCS_T threads
template <typename... Exp, typename... Act>
static int launch_cols(ofrr_ctx* ctx, int cl, int64_t ncols, void (*k)(Exp...), Act&&... args) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(ncols * cl));
  cfg.blockDim = dim3(SCS_T);
  cfg.stream = ctx->stream;
  cfg.attrs = attr;
  cfg.numAttrs = cl > 1 ? 1 : 0;
  OFRR_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<Act>(args)...));
  return OFRR_SUCCESS;
}
// rows per thread U and CTAs per column CL for columns of m <= 8192 rows (every row of the padded
// column below CL SCS_T U)
template <class F>
static int scs_dispatch(int64_t m, F&& f) {
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  using I4 = std::integral_constant<int, 4>;
  if (m <= 1024) return f(I1(), I1());
  if (m <= 2048) return f(I2(), I1());
  if (m <= 4096) return f(I2(), I2());
  return f(I4(), I2());
}

// runtime dtype dispatch --------------------------------------------------------------
#define OFRR_DISPATCH_STORAGE(dt, T, ...)                         \
  switch (dt) {                                                   \
    case OFRR_F64: { using T = double; __VA_ARGS__; } break;      \
    case OFRR_F32: { using T = float; __VA_ARGS__; } break;       \
    case OFRR_F16: { using T = __half; __VA_ARGS__; } break;      \
    case OFRR_BF16: { using T = __nv_bfloat16; __VA_ARGS__; } break; \
    default: return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;               \
  }

#define OFRR_DISPATCH_COMPUTE(dt, TC, ...)                        \
  switch (dt) {                                                   \
    case OFRR_F64: { using TC = double; __VA_ARGS__; } break;     \
    case OFRR_F32: { using TC = float; __VA_ARGS__; } break;      \
    default: return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;               \
  }

inline int grid_for(long long n, int block, int cap = 152 * 16) {
  long long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

// Element-wise kernels over an m x n column-major matrix run on a 2-D grid (rows along x, columns
// along y) instead of dividing a flat 64-bit index (a 64-bit division is a long software sequence);
// about 4096 CTAs at most, each thread striding over rows.
inline dim3 grid_2d(long long m, long long n, int block) {
  long long gy = n < 1 ? 1 : (n > 65535 ? 65535 : n);
  long long gx = (m + block - 1) / block;
  long long cap = 4096 / gy;
  if (cap < 1) cap = 1;
  if (gx > cap) gx = cap;
  if (gx < 1) gx = 1;
  return dim3((unsigned)gx, (unsigned)gy);
}
#define OFRR_FOR_2D(i, j, m, n)                                                   \
  for (int64_t j = blockIdx.y; j < (int64_t)(n); j += gridDim.y)                  \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)(m); \
         i += (int64_t)gridDim.x * blockDim.x)

// ---- cross-file internal API ---------------------------------------------------------
// dense / sparse products into caller buffers (all on ctx->stream, no host sync)
int gemm_tc_scalecols(ofrr_ctx* ctx, ofrr_dtype t16, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                      const void* B, int64_t ldb, void* C, int64_t ldc, bool fast, bool* handled);
int gemm_impl(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype ta, ofrr_dtype tb, ofrr_dtype tc,
              ofrr_dtype tout, int64_t M, int64_t N, int64_t K, double alpha, const void* A,
              int64_t lda, const void* B, int64_t ldb, double beta, void* C, int64_t ldc);
int csrmm_impl(ofrr_ctx* ctx, const ofrr_csr* A, int trans, ofrr_dtype tx, ofrr_dtype tc, ofrr_dtype ty,
               int64_t nrhs, const void* X, int64_t ldx, void* Y, int64_t ldy);
// E4M3 copies with per-column power-of-two scales (rows past K up to ld8 zero) and their tcgen05 product
// C (M x N, FP32) = diag(sa) A8' B8 diag(sb) (K a multiple of 128, ld8 multiples of 16 bytes)
int quant_e4m3(ofrr_ctx* ctx, ofrr_dtype tin, int64_t K, int64_t M, const void* X, int64_t ldx, void* X8,
               int64_t ld8, float* scale);
int gemm_e4m3_tn(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const void* A8, int64_t lda8, const float* sa,
                 const void* B8, int64_t ldb8, const float* sb, float* C, int64_t ldc);
// A' as CSR (row pointers, rows sorted within each column, every value copy present in A), in ctx's
// current workspace scope; deterministic
int csr_transpose_impl(ofrr_ctx* ctx, const ofrr_csr* A, ofrr_csr* At);
int cast_transpose_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, int64_t m, int64_t n, const void* in,
                        int64_t ldin, void* out, int64_t ldout);
int cast_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, int64_t m, int64_t n, const void* in,
              int64_t ldin, void* out, int64_t ldout);
// fast = multiply by the reciprocal of the column's maximum (within an ulp of the quotient) for an
// FP64 compute type; fast = false keeps scalecols.m's correctly rounded division
int scalecols_impl(ofrr_ctx* ctx, ofrr_dtype po, ofrr_dtype pc, int64_t m, int64_t n, void* U, int64_t ldu,
                   int* piv, bool fast = false);
int fill_zero(ofrr_ctx* ctx, void* p, size_t bytes);

// Hessenberg basis on device: Q (m x n, tout) from A; outputs on device:
// R (n x n FP64, col-major), select (n ints, 1 = kept), perm (n ints, -1 if dropped)
// fast = FMA eliminations and reciprocal pivot scaling for an FP64 compute type (production
// refinement phases; not bit-identical to hessenberg.m's arithmetic, which fast = false keeps)
int hessenberg_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n,
                    const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol, double* R_dev,
                    int* select_dev, int* perm_dev, bool fast = false);
// column-pivoted LU basis (MATLAB/+src/+qr/lu.m), same contract as the Hessenberg basis
int lu_basis_impl(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n, const void* A,
                  int64_t lda, void* Q, int64_t ldq, double select_tol, double* R_dev, int* select_dev);
// Gram-Schmidt bases (orthogonal comparison path): MATLAB/+src/+qr/mgs.m, or cgs.m when classical
int gs_basis_impl(ofrr_ctx* ctx, bool classical, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m,
                  int64_t n, const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol, double* R_dev,
                  int* select_dev, double orth_tol = NAN, double reorth_tol = NAN);

// small dense FP64 solvers on device (one CTA); w ascending
int syev_dev(ofrr_ctx* ctx, int n, double* A, int lda, double* w);
int sygv_dev(ofrr_ctx* ctx, int n, double* A, int lda, double* B, int ldb, double* w);
// general real pencil eig(G, M) with M SPD: eigenvalues (real parts) and real parts of the
// eigenvectors, M-normalised; sorted descending by real part.  n <= 256.
int geig_dev(ofrr_ctx* ctx, int n, const double* G, int ldg, const double* M, int ldm, int symmetric,
             double* w, double* U, int ldu);

// production small solvers (FP32 Jacobi + FP64 refinement, multi-CTA FP64 products), n <= 128:
// eig(G, M + tau I) (M may be null) and the svd_rr pencil of B with Gram matrices UU, VV
// refine = number of Ogita-Aishima FP64 refinement steps after the FP32 Jacobi (each squares the
// vectors' error: 2 give FP64-accurate vectors; 16-bit bases use 1); the values are always FP64
// Rayleigh quotients of the final vectors
// eig(C) for a nonsymmetric n x n C (n <= 128), FP32 Hessenberg-QR: real/imaginary parts, eigenvectors
// (real parts, unit norm), unsorted
int nonsym_eig_dev(ofrr_ctx* ctx, int n, const double* C, double* wr, double* wi, double* X, bool refine,
                   bool pair_imag = false, bool values_only = false);
// eig(G, M) for nonsymmetric G, SPD M (or M null): real parts descending, unit real-part eigenvectors;
// refine = FP64 Newton steps on the real pairs (for FP32/FP64 bases)
// values_only: lam alone (FP32 Hessenberg-QR without vectors; U is not written)
int geig_nonsym(ofrr_ctx* ctx, int n, const double* G, const double* M, double* lam, double* U, bool refine,
                bool pair_imag = false, bool values_only = false);
// Y (n x p, ld n): basis of the invariant subspace of the pencil (G, M) (M SPD) for its p eigenvalues
// with real part above sigma (matrix sign function of L^-1 G L^-T - sigma I); n <= 96
int invariant_subspace_nonsym(ofrr_ctx* ctx, int n, const double* G, const double* M, double sigma, int p,
                              double* Y);
// the k leading Ritz pairs of (G, M) from a basis Y (n x p) of its invariant subspace for the p eigenvalues
// of largest real part: FP64 Hessenberg-QR of the restricted p x p pencil; lam (k), U (n x k, ld n)
int ritz_from_invariant(ofrr_ctx* ctx, int n, const double* G, const double* M, const double* Y, int p, int k,
                        double* lam, double* U);
int geig_fast(ofrr_ctx* ctx, int n, const double* G, const double* M, double tau, double* lam, double* U,
              int refine = 2);
int gsvd_fast(ofrr_ctx* ctx, int b, const double* B, const double* UU, const double* VV, double tau, double* sigma,
              double* Zf, double* Wf, int refine = 2);

// reductions
// ||AV(:,j) - s_j U(:,j)||_2 per column, FP64 (ld m; n <= 1024), over many CTAs per column
int residual_columns2(ofrr_ctx* ctx, int64_t m, int64_t n, const double* AV, const double* U, const double* s,
                      double* out);
int column_norms(ofrr_ctx* ctx, ofrr_dtype t, int64_t m, int64_t n, const void* X, int64_t ldx,
                 double* out_dev);
// exact-slice FP64 emulation (sliced.cu): digit stacks of a fixed K x M FP64 operand and the
// product C (M x N) = X' B with X the prepared operand and B (K x N) FP64
struct SlicedOperand {
  int64_t K = 0, Kp = 0, M = 0;
  __nv_bfloat16* stack = nullptr;
  int* expo = nullptr;
};
constexpr int kSliceDigits = 5;
int sliced_prepare(ofrr_ctx* ctx, int64_t K, int64_t M, const double* X, int64_t ldx, SlicedOperand* out);
int sliced_prepare_into(ofrr_ctx* ctx, int64_t K, int64_t M, const double* X, int64_t ldx, __nv_bfloat16* stack,
                        int* expo, SlicedOperand* out);
// scalecols (FAST, FP64) fused with the digit split of the scaled columns: U (m x n) is scaled in place
// and *out describes its digit stack in caller buffers (n * 5 * roundup(m, 64) bf16, n ints); m <= 8192
int scalecols_sliced(ofrr_ctx* ctx, int64_t m, int64_t n, double* U, int64_t ldu, __nv_bfloat16* stack, int* expo,
                     SlicedOperand* out);
// C (M x N) = A_op' B with both operands already split (B.K == A.K, N = B.M)
int sliced_gemm_tn_pre(ofrr_ctx* ctx, const SlicedOperand& A, const SlicedOperand& B, double* C, int64_t ldc);
int sliced_gemm_scalecols_pre(ofrr_ctx* ctx, const SlicedOperand& A, const SlicedOperand& B, double* U, int64_t ldu,
                              bool write_u, __nv_bfloat16* stack, int* expo, SlicedOperand* out);
int sliced_gemm_tn(ofrr_ctx* ctx, const SlicedOperand& A, int64_t N, const double* B, int64_t ldb, double* C,
                   int64_t ldc);

int residual_columns(ofrr_ctx* ctx, int64_t m, int64_t n, const double* AX, int64_t ldax,
                     const double* X, int64_t ldx, const double* lam_dev, double* out_dev);

// ---- thick-restart Krylov steps (krylov_tr.cu) ----------------------------------------------
// Device state of the Hessenberg-process Krylov steps of one solve: the basis V (ldv x nb, type t;
// ldv = n rounded up to 8 so every column starts 16-byte aligned), two staging vectors and the
// arithmetic (type te: FP32 for 16/32-bit bases, FP64 for FP64), pivot marks, the pivot rows and
// reciprocals, L = Q(perm, :) and its explicit inverse (row-major, nb x nb), the next coefficients,
// argmax partials, a ticket counter and the breakdown word (stop: -1 or the column that broke down).
constexpr int kKryMaxNb = 129;
struct KryState {
  const ofrr_csr* A = nullptr;
  ofrr_dtype t = OFRR_F16, te = OFRR_F32;
  int64_t n = 0, ldv = 0;
  int nb = 0, grid = 0;
  double stol = 0.0;
  void* V = nullptr;
  void* S[2] = {nullptr, nullptr};
  unsigned char* mark = nullptr;
  int* perm = nullptr;
  void *pvinv = nullptr, *coef = nullptr, *Lrows = nullptr, *Linv = nullptr, *partial = nullptr;
  unsigned int* counter = nullptr;
  int* stop = nullptr;
};
ofrr_dtype kry_arith_type(ofrr_dtype t);
int64_t kry_ld(int64_t n);
// allocates the state in ctx's current workspace scope; A's value copy of the arithmetic type is used
int kry_state_init(ofrr_ctx* ctx, KryState* s, const ofrr_csr* A, ofrr_dtype t, int nb, double stol);
// columns 0 .. q-1 of s.V final with pivot rows s.perm[0 .. q-1]: builds columns q .. nb-1
int kry_cycle_steps(ofrr_ctx* ctx, KryState& s, int q);
// Rayleigh-Ritz helpers: W = V Cf (FP32 arithmetic into an FP32 W for 16/32-bit V; FP64 through
// gemm_impl otherwise), w += a (one column), x = M^-1 g (SPD, nc <= 129),
// Cf = [U1(:, :k1), U2(:, :k2), -x], s = sum_j W(:, j) / nrm_j
int kry_backtransform(ofrr_ctx* ctx, ofrr_dtype t, int64_t n, int nc, const void* V, int64_t ldv, const double* Cf,
                      int k, ofrr_dtype tw, void* W, int64_t ldw, bool exact = false);
int kry_add_col(ofrr_ctx* ctx, ofrr_dtype tw, int64_t n, void* w, ofrr_dtype ta, const void* a);
int kry_spd_solve(ofrr_ctx* ctx, int nc, const double* M, const double* g, double* x);
int kry_coef_matrix(ofrr_ctx* ctx, int nc, int k1, const double* U1, int k2, const double* U2, const double* x,
                    double* Cf);
int kry_sum_unit_cols(ofrr_ctx* ctx, ofrr_dtype tw, int64_t n, int k, const void* W, int64_t ldw, const double* nrm,
                      double* s);
// C (M x N) = A' B for FP64 A (K x M), B (K x N), M, N <= 128, FP64 on the CUDA cores (fixed-order
// partial sums): the exact-arithmetic Gram products of a Rayleigh-Ritz step
int gram_f64(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
             int64_t ldb, double* C, int64_t ldc);
// C (M x N) = A (M x K) B (K x N), FP64 on the CUDA cores (K <= 256): exact-arithmetic back-transforms
int tsmm_f64(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
             int64_t ldb, double* C, int64_t ldc);
// G (nc x nc, FP64) = V' AV for a 16-bit V and an FP32 AV: hi/lo split of AV, two tensor-core products
int kry_gram16(ofrr_ctx* ctx, ofrr_dtype t, int64_t n, int nc, const void* V, int64_t ldv, const float* AV,
               int64_t ldav, double* G);

}  // namespace ofrr
