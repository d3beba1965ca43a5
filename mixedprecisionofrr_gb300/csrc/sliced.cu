// Exact-slice FP64 emulation of dense products on the tcgen05 tensor cores (Ozaki-style splitting).
//
// The refinement phase of the mixed solver needs A V and A' U in FP64 accuracy; GB300 runs FP64
// at 1/64 of its FP32 rate, while BF16 tensor cores run at ~1 PFLOP/s.  Each FP64 operand column is
// scaled by a power of two (x = 2^e y, |y| < 1) and split into S signed digits of BETA bits,
// y = sum_s d_s 2^{-BETA (s+1)}, every d_s an integer with |d_s| <= 2^BETA, stored exactly in BF16.
// The product of two columns is then sum_{s,t} 2^{e_a + e_b - BETA (s+t+2)} (d_s . d'_t).  Terms with
// s + t = L share one scale, so the digits are stacked along K ([d_0; d_1; ...] against
// [d'_L; d'_{L-1}; ...]) and every level L <= LMAX is ONE tensor-core GEMM of depth (L+1) K.
// Integer products summed in FP32 are exact while the partial sum stays below 2^24: the GEMM is
// split along K into ranges short enough for that on the two leading levels (where an FP32 rounding
// would show), and the exact FP32 partials are combined and scaled in FP64.  Dropped terms
// (s + t > LMAX) and the digit truncation are below 2^-(BETA (LMAX+1)) relative.
#include "ofrr_internal.cuh"
#include "tcgen05.cuh"

#include <algorithm>
#include <atomic>
#include <vector>

namespace ofrr {

namespace slice {
constexpr int BETA = 7;  // digit width: |leading digit| <= 128, later digits <= 64
constexpr int S = 5;     // digits per operand (35 bits)
constexpr int LMAX = 4;  // levels kept: pairs with s + t <= 4 (15 of 25), error ~ 2^-35

// Digits of every column of X (K x N, column-major).  Stacked layout: column n occupies
// stack[(n * S + s) * Kp + k] for digit s; rows k >= K are zero.  expo[n] = exponent e_n.
// Integer pipes only (GB300's FP64 pipe is 1/64 rate): the column maximum is taken on the bit
// patterns of |x|, e_n = frexp exponent of that maximum, and round(x 2^(BETA S - e_n)) is formed from
// the significand by a right shift with round-half-even (the same value __double2ll_rn gives).
// Columns of up to 8192 entries take one pass (k_slice_cols below); longer ones two passes over a
// (row chunk x column) grid: maxima by atomicMax on the bit patterns, then digits.
constexpr int SLICE_T = 256;
constexpr int SLICE_U = 4;
constexpr int64_t SLICE_CHUNK = (int64_t)SLICE_T * SLICE_U;  // rows per CTA

__global__ void __launch_bounds__(SLICE_T) k_slice_max(int64_t K, int64_t N, const double* __restrict__ X, int64_t ldx,
                                                       unsigned long long* __restrict__ colmax) {
  __shared__ unsigned long long red[SLICE_T / 32];
  const int64_t k0 = (int64_t)blockIdx.x * SLICE_CHUNK + threadIdx.x;
  for (int64_t n = blockIdx.y; n < N; n += gridDim.y) {
    const double* x = X + n * ldx;
    unsigned long long v[SLICE_U];
#pragma unroll
    for (int u = 0; u < SLICE_U; ++u) {
      const int64_t k = k0 + (int64_t)u * SLICE_T;
      v[u] = (k < K) ? ((unsigned long long)__double_as_longlong(x[k]) & 0x7fffffffffffffffull) : 0ull;
    }
    unsigned long long mx = 0;
#pragma unroll
    for (int u = 0; u < SLICE_U; ++u) mx = max(mx, v[u]);
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long m = 0;
      for (int w = 0; w < SLICE_T / 32; ++w) m = max(m, red[w]);
      if (m != 0) atomicMax(colmax + n, m);
    }
    __syncthreads();
  }
}

// s 2^e as a double, rounded once to nearest-even (the value (double)s then an exact power-of-two
// scaling gives), built on the integer pipes: GB300's FP64 pipe runs at 1/64 of the FP32 rate and a
// 64-bit integer conversion plus ldexp per element would bound the product's epilogue.  Results
// outside the normal range (never met by scaled operands of moderate range) take the FP64 path.
// |s| < 2^63 (the combined sums are bounded well below that).
__device__ __forceinline__ double i64_ldexp(long long s, int e) {
  if (s == 0) return 0.0;
  const unsigned long long sign = (s < 0) ? (1ull << 63) : 0ull;
  const unsigned long long u = (s < 0) ? (unsigned long long)(-s) : (unsigned long long)s;
  const int lz = __clzll((long long)u);
  const int be = (63 - lz) + e + 1023;  // biased exponent of the result (u in [2^(63-lz), 2^(64-lz)))
  if (be <= 0 || be >= 2047) return ldexp((double)s, e);
  const unsigned long long v = u << lz;  // leading one at bit 63
  unsigned long long mant = v >> 11;     // 53 significant bits
  const unsigned long long rem = v & 0x7ffull;
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ++mant;
  // the leading one (bit 52) lifts the exponent field from be - 1 to be; a rounding carry to 2^53
  // lifts it once more, and an exponent of 2047 with a zero fraction is the infinity RN gives
  return __longlong_as_double((long long)(sign | (((unsigned long long)(be - 1) << 52) + mant)));
}

// frexp exponent of a column maximum given as the bit pattern of |x|: m = f 2^e with f in [0.5, 1),
// so |x| 2^-e < 1 for every entry of the column (0 for an all-zero column)
__device__ __forceinline__ int colmax_expo(unsigned long long m) {
  const int bm = (int)(m >> 52);
  return (m == 0) ? 0 : (bm > 0) ? bm - 1022 : (64 - __clzll((long long)m)) - 1074;
}

// The S digits of one entry (bit pattern `bits`) of a column with exponent e, stored at col[s * Kp + k]
__device__ __forceinline__ void slice_store(unsigned long long bits, int e, __nv_bfloat16* __restrict__ col, int64_t Kp,
                                            int64_t k) {
  // x = M 2^(be' - 1075) with M the significand (implicit bit for normal numbers, be' = max(be, 1))
  const int be = (int)((bits >> 52) & 0x7ff);
  const unsigned long long M = (bits & 0x000fffffffffffffull) | (be > 0 ? (1ull << 52) : 0ull);
  const int sh = 1075 - (BETA * S) + e - (be > 0 ? be : 1);  // 18 or more unless the maximum is subnormal
  long long r = 0;
  if (sh <= 53 && M != 0) {
    unsigned long long q;
    if (sh <= 0) {
      q = M << (-sh);  // subnormal column maximum: exact scaling up
    } else {
      q = M >> sh;
      const unsigned long long rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
      if (rem > half || (rem == half && (q & 1ull))) ++q;
    }
    r = (bits >> 63) ? -(long long)q : (long long)q;
  }
#pragma unroll
  for (int s = S - 1; s > 0; --s) {  // centred base-2^BETA digits, least significant first
    const long long d = ((r + (1 << (BETA - 1))) & ((1 << BETA) - 1)) - (1 << (BETA - 1));
    r = (r - d) >> BETA;  // exact: r - d is a multiple of 2^BETA
    col[(size_t)s * Kp + k] = __float2bfloat16_rn((float)(int)d);  // |d| <= 64
  }
  col[k] = __float2bfloat16_rn((float)(int)r);  // leading digit, |r| <= 128: exact in bf16
}

__global__ void __launch_bounds__(SLICE_T) k_slice_digits(int64_t K, int64_t Kp, int64_t N, const double* __restrict__ X,
                                                          int64_t ldx, const unsigned long long* __restrict__ colmax,
                                                          __nv_bfloat16* __restrict__ stack, int* __restrict__ expo) {
  const int64_t k0 = (int64_t)blockIdx.x * SLICE_CHUNK + threadIdx.x;
  for (int64_t n = blockIdx.y; n < N; n += gridDim.y) {
    const int e = colmax_expo(colmax[n]);
    if (blockIdx.x == 0 && threadIdx.x == 0) expo[n] = e;
    const double* x = X + n * ldx;
    __nv_bfloat16* col = stack + (size_t)n * S * Kp;
    unsigned long long v[SLICE_U];
#pragma unroll
    for (int u = 0; u < SLICE_U; ++u) {
      const int64_t k = k0 + (int64_t)u * SLICE_T;
      v[u] = (k < K) ? (unsigned long long)__double_as_longlong(x[k]) : 0ull;
    }
#pragma unroll
    for (int u = 0; u < SLICE_U; ++u) {
      const int64_t k = k0 + (int64_t)u * SLICE_T;
      if (k >= Kp) break;
      slice_store(v[u], e, col, Kp, k);
    }
  }
}

// Single-pass form for columns of at most SC_T * U entries: one CTA per column keeps the column in
// registers, takes its maximum with a block reduction and writes the digits (no second read, no
// atomics, no zeroed scratch).
constexpr int SC_T = 512;
template <int U, int T = SC_T>
__global__ void __launch_bounds__(T) k_slice_cols(int64_t K, int64_t Kp, int64_t N, const double* __restrict__ X,
                                                  int64_t ldx, __nv_bfloat16* __restrict__ stack,
                                                  int* __restrict__ expo) {
  __shared__ unsigned long long red[T / 32];
  for (int64_t n = blockIdx.x; n < N; n += gridDim.x) {
    const double* x = X + n * ldx;
    unsigned long long v[U];
    unsigned long long mx = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = threadIdx.x + (int64_t)u * T;
      v[u] = (k < K) ? (unsigned long long)__double_as_longlong(x[k]) : 0ull;
      mx = max(mx, v[u] & 0x7fffffffffffffffull);
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < T / 32; ++w) mx = max(mx, red[w]);
    const int e = colmax_expo(mx);
    if (threadIdx.x == 0) expo[n] = e;
    __nv_bfloat16* col = stack + (size_t)n * S * Kp;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t k = threadIdx.x + (int64_t)u * T;
      if (k < Kp) slice_store(v[u], e, col, Kp, k);
    }
    __syncthreads();  // red is reused by the next column
  }
}

// scalecols (FP64, FAST: reciprocal multiply, pivot exactly 1) fused with the digit split of the
// scaled column, for columns of at most SCS_T U CL rows: a cluster of CL CTAs per column keeps the
// column in registers (CTA r holds rows [r SCS_T U, (r + 1) SCS_T U)), finds the pivot (integer
// argmax keys, lowest row on ties), scales, writes the FP64 column, takes the scaled column's maximum
// on the bit patterns and writes its digits -- the operand of the next exact-slice product, without
// reading the column again.  With CL = 2 the CTAs exchange their pivot candidates and maxima through
// distributed shared memory; the result is the same as one CTA over the whole column.
// Body shared by k_scalecols_slice and k_finish_scalecols_slice: v[u] holds row r0 + threadIdx.x +
// u SCS_T of column n (0 beyond m), r0 = this CTA's first row.  col != nullptr also stores the scaled
// column there.  For CL > 1 the caller has done cluster_arrive_relaxed() once on entry.
template <int U, int CL>
__device__ __forceinline__ void scalecols_slice_body(int64_t m, int64_t Kp, int n, int64_t r0, double (&v)[U],
                                                     double* __restrict__ col, __nv_bfloat16* __restrict__ stack,
                                                     int* __restrict__ expo) {
  __shared__ ArgMaxK red[SCS_T / 32];
  __shared__ unsigned long long redm[SCS_T / 32];
  __shared__ double s_t, s_y;
  __shared__ long long s_k;
  __shared__ bool s_pf;
  __shared__ unsigned long long s_ckey[CL], s_crow[CL], s_cval[CL], s_cmax[CL];  // filled by the cluster
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  ArgMaxK a{-1, 0x7fffffffffffffffLL};
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
    if (i < m) {
      const long long key = amax_key(v[u]);
      if (key > a.key) a = ArgMaxK{key, i};  // per-thread rows ascend: strict > keeps the lowest
    }
  }
  const ArgMaxK r = block_argmaxk(a, red);
  // the owner of this CTA's candidate row publishes its value (every column has a row 0, so the
  // first CTA always has a candidate)
  if (r.key >= 0 && threadIdx.x == (int)((r.i - r0) % SCS_T)) {
    const int ku = (int)((r.i - r0) / SCS_T);
    double pv = 0.0;
#pragma unroll
    for (int u = 0; u < U; ++u) pv = (u == ku) ? v[u] : pv;
    if (CL == 1) {
      s_t = pv;
      s_k = r.i;
      s_y = (pv != 0.0) ? pivot_recip(pv) : 0.0;  // once per column (1/64-rate FP64 pipe)
      s_pf = pivot_fast(pv);
    } else {
      s_t = pv;
    }
  }
  if (CL > 1) {
    __syncthreads();
    cluster_wait();  // every CTA of the cluster has started: its shared memory may be written
    const unsigned me = cluster_rank();
    if (threadIdx.x < CL) {
      st_cluster_u64(cluster_map(&s_ckey[me], threadIdx.x), (unsigned long long)r.key);
      st_cluster_u64(cluster_map(&s_crow[me], threadIdx.x), (unsigned long long)r.i);
      st_cluster_u64(cluster_map(&s_cval[me], threadIdx.x),
                     (unsigned long long)__double_as_longlong(r.key >= 0 ? s_t : 0.0));
    }
    cluster_arrive();
    cluster_wait();
    if (threadIdx.x == 0) {
      ArgMaxK g{-1, 0x7fffffffffffffffLL};
      double gv = 0.0;
#pragma unroll
      for (int q = 0; q < CL; ++q) {  // in row order: max key, lowest row on ties
        const ArgMaxK c{(long long)s_ckey[q], (long long)s_crow[q]};
        const ArgMaxK p = argmaxk_pick(g, c);
        if (p.key != g.key || p.i != g.i) gv = __longlong_as_double((long long)s_cval[q]);
        g = p;
      }
      s_t = gv;
      s_k = g.i;
      s_y = (gv != 0.0) ? pivot_recip(gv) : 0.0;
      s_pf = pivot_fast(gv);
    }
  }
  __syncthreads();
  const double t = s_t;
  const int64_t k = s_k;
  if (t != 0.0) {
    const double y = s_y;
    const bool pf = s_pf;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
      if (i < m) v[u] = scale_by<double, true>(v[u], t, y, pf, i == k);
    }
  }
  if (col) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
      if (i < m) col[i] = v[u];
    }
  }
  unsigned long long mx = 0;
#pragma unroll
  for (int u = 0; u < U; ++u) mx = max(mx, (unsigned long long)__double_as_longlong(v[u]) & 0x7fffffffffffffffull);
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) redm[wid] = mx;
  __syncthreads();
#pragma unroll
  for (int w = 0; w < SCS_T / 32; ++w) mx = max(mx, redm[w]);
  if (CL > 1) {
    const unsigned me = cluster_rank();
    if (threadIdx.x < CL) st_cluster_u64(cluster_map(&s_cmax[me], threadIdx.x), mx);
    cluster_arrive();
    cluster_wait();  // the last access to another CTA's shared memory is before this barrier
#pragma unroll
    for (int q = 0; q < CL; ++q) mx = max(mx, s_cmax[q]);
  }
  const int e = colmax_expo(mx);
  if (threadIdx.x == 0 && r0 == 0) expo[n] = e;
  __nv_bfloat16* dst = stack + (size_t)n * S * Kp;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
    if (i < Kp) slice_store((unsigned long long)__double_as_longlong(v[u]), e, dst, Kp, i);
  }
}

// CL CTAs per column (a cluster of CL along x): column blockIdx.x / CL, rows from (blockIdx.x % CL) SCS_T U
template <int U, int CL>
__global__ void __launch_bounds__(SCS_T) k_scalecols_slice(int64_t m, int64_t Kp, double* __restrict__ X,
                                                           int64_t ldx, __nv_bfloat16* __restrict__ stack,
                                                           int* __restrict__ expo) {
  if (CL > 1) cluster_arrive_relaxed();
  const int n = blockIdx.x / CL;
  const int64_t r0 = (int64_t)(blockIdx.x % CL) * SCS_T * U;
  double* col = X + (int64_t)n * ldx;
  double v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
    v[u] = (i < m) ? col[i] : 0.0;
  }
  scalecols_slice_body<U, CL>(m, Kp, n, r0, v, col, stack, expo);
}

// Fused exact-slice product.  One CTA owns a 128 x SBN tile of C and a range of at most 16 k-blocks
// (1024 entries of K, so that the level-0 and level-1 FP32 sums are exact).  Per k-block the B digits
// d'_0..d'_4 (5 tiles) are loaded once into a B slot, and the A digits d_0..d_4 stream through an
// A ring one tile at a time; for A digit s the MMA warp issues the pairs (s, t), t <= LMAX - s,
// into the TMEM accumulator of level L = s + t (5 accumulators of SBN columns), as one wide MMA.  A is therefore read
// once per product (not once per level).  The epilogue converts each level to an integer, combines
// acc = sum_L S_L 2^(BETA (LMAX - L)) exactly in 64 bits and writes it (one split) as
// C = 2^(ea + eb - BETA (LMAX + 2)) acc, or as an int64 partial for k_sliced_finish.
constexpr int SBN = 64;
constexpr int SL_ATILE = tc::BM * tc::BK * 2;  // 16 KB: one digit of a 128-row k-block
constexpr int SL_BTILE = SBN * tc::BK * 2;     // 8 KB
constexpr int SL_ASLOTS = 6;
constexpr int SL_BSLOTS = 2;
constexpr int SL_THREADS = 192;
constexpr int SL_KB_MAX = 16;
constexpr int SL_SHIFT = BETA * (LMAX + 2);
constexpr size_t SL_SMEM = (size_t)SL_ASLOTS * SL_ATILE + (size_t)SL_BSLOTS * S * SL_BTILE + 1024 + 256;
constexpr uint32_t SL_TMEM_COLS = 512;  // LMAX + 1 accumulators of SBN columns, rounded to a power of two
static_assert((LMAX + 1) * SBN <= (int)SL_TMEM_COLS, "TMEM columns");

// instruction descriptor with its N field (bits 17-22, N >> 3) replaced
__device__ __forceinline__ uint32_t idesc_with_n(uint32_t idesc, int n) {
  return (idesc & ~(0x3Fu << 17)) | ((uint32_t)(n >> 3) << 17);
}

__global__ void __launch_bounds__(SL_THREADS, 1)
    k_sliced_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
                int64_t Kp, int kb_total, int kb_per_split, uint32_t idesc, long long* __restrict__ partial,
                double* __restrict__ C, int64_t ldc, const int* __restrict__ ea, const int* __restrict__ eb,
                int* __restrict__ err) {
  using namespace tc;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = base;
  uint8_t* sB = base + SL_ASLOTS * SL_ATILE;
  uint64_t* bars = (uint64_t*)(sB + SL_BSLOTS * S * SL_BTILE);
  uint64_t* a_full = bars;
  uint64_t* a_empty = bars + SL_ASLOTS;
  uint64_t* b_full = bars + 2 * SL_ASLOTS;
  uint64_t* b_empty = b_full + SL_BSLOTS;
  uint64_t* accum = b_empty + SL_BSLOTS;
  uint32_t* tmem_slot = (uint32_t*)(accum + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * SBN;
  const int kb0 = blockIdx.z * kb_per_split;
  const int kb1 = min(kb0 + kb_per_split, kb_total);
  const int nkb = max(kb1 - kb0, 0);

  if (threadIdx.x == 0) {
    for (int i = 0; i < SL_ASLOTS; ++i) {
      mbar_init(&a_full[i], 1);
      mbar_init(&a_empty[i], 1);
    }
    for (int i = 0; i < SL_BSLOTS; ++i) {
      mbar_init(&b_full[i], 1);
      mbar_init(&b_empty[i], 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(SL_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
      int a_issued = 0, b_issued = 0;
      bool ok = true;
      for (int i = 0; i < nkb && ok; ++i) {
        const int bs = i % SL_BSLOTS;
        if (i >= SL_BSLOTS && !mbar_wait(&b_empty[bs], ((i / SL_BSLOTS) + 1) & 1, err, 21)) break;
        const int kx = (kb0 + i) * BK;
        mbar_expect_tx(&b_full[bs], S * SL_BTILE);
        for (int t = 0; t < S; ++t)
          tma_load_2d(&tmB, &b_full[bs], sB + (bs * S + t) * SL_BTILE, (int)(t * Kp) + kx, n0);
        b_issued = i + 1;
        for (int s = 0; s < S; ++s) {
          const int as = a_issued % SL_ASLOTS;
          if (a_issued >= SL_ASLOTS && !mbar_wait(&a_empty[as], ((a_issued / SL_ASLOTS) + 1) & 1, err, 22)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&a_full[as], SL_ATILE);
          tma_load_2d(&tmA, &a_full[as], sA + as * SL_ATILE, (int)(s * Kp) + kx, m0);
          ++a_issued;
        }
      }
      // drain: every issued copy must have landed before the CTA may exit
      for (int j = max(0, a_issued - SL_ASLOTS); j < a_issued; ++j)
        mbar_wait(&a_full[j % SL_ASLOTS], (j / SL_ASLOTS) & 1, err, 23);
      for (int j = max(0, b_issued - SL_BSLOTS); j < b_issued; ++j)
        mbar_wait(&b_full[j % SL_BSLOTS], (j / SL_BSLOTS) & 1, err, 24);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int a_used = 0;
      bool ok = true;
      for (int i = 0; i < nkb && ok; ++i) {
        const int bs = i % SL_BSLOTS;
        if (!mbar_wait(&b_full[bs], (i / SL_BSLOTS) & 1, err, 25)) break;
        fence_after();
        for (int s = 0; s < S; ++s) {
          const int as = a_used % SL_ASLOTS;
          if (!mbar_wait(&a_full[as], (a_used / SL_ASLOTS) & 1, err, 26)) {
            ok = false;
            break;
          }
          fence_after();
          // A digit s against the B digits 0..LMAX-s at once: the slot's B tiles are adjacent rows of
          // one K-major operand and the level accumulators s..LMAX adjacent TMEM columns, so one MMA
          // of N = (LMAX-s+1) SBN (at most 256; the rest in a second MMA) replaces LMAX-s+1 MMAs
          const uint32_t a0 = smem_u32(sA + as * SL_ATILE);
          const uint32_t b0 = smem_u32(sB + (bs * S) * SL_BTILE);
          const int nt = LMAX - s + 1;
          const int n1 = nt < 4 ? nt : 4;
          const uint32_t id1 = idesc_with_n(idesc, n1 * SBN), id2 = idesc_with_n(idesc, (nt - n1) * SBN);
          const uint32_t d = tmem + (uint32_t)(s * SBN);
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint32_t acc = (i > 0 || s > 0 || k > 0) ? 1u : 0u;
            umma_f16(d, desc_sw128(a0 + 32 * k), desc_sw128(b0 + 32 * k), id1, acc);
            if (nt > n1)
              umma_f16(d + (uint32_t)(n1 * SBN), desc_sw128(a0 + 32 * k), desc_sw128(b0 + n1 * SL_BTILE + 32 * k),
                       id2, acc);
          }
          umma_commit(&a_empty[as]);
          ++a_used;
        }
        umma_commit(&b_empty[bs]);
      }
      umma_commit(accum);
    }
    __syncwarp();
  } else {
    // epilogue warps 2..5 -> TMEM lane quarter (warp % 4)
    const int q = warp & 3;
    const bool ok = mbar_wait(accum, 0, err, 27);
    fence_after();
    const int row = m0 + 32 * q + lane;
    const int erow = (row < M) ? ea[row] : 0;
#pragma unroll 1
    for (int c = 0; c < SBN; c += 16) {
      long long acc[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[j] = 0;
#pragma unroll 1
      for (int L = 0; L <= LMAX; ++L) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(L * SBN + c), v);
        // every level sum is an integer below 2^25 in magnitude (at most 1024 terms of at most 2^14.3)
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j] += (long long)__float2int_rn(v[j]) * (1ll << (BETA * (LMAX - L)));
      }
      if (!ok || nkb == 0) {
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[j] = 0;
      }
      if (row < M) {
        if (partial != nullptr) {
          long long* P = partial + (size_t)blockIdx.z * (size_t)M * N;
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = n0 + c + j;
            if (n < N) P[row + (size_t)n * M] = acc[j];
          }
        } else {
#pragma unroll 4
          for (int j = 0; j < 16; ++j) {
            const int n = n0 + c + j;
            if (n < N) C[row + (size_t)n * ldc] = i64_ldexp(acc[j], erow + eb[n] - SL_SHIFT);
          }
        }
      }
    }
    fence_before();
  }
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(SL_TMEM_COLS) : "memory");
  }
}

// C = 2^(ea + eb - BETA (LMAX + 2)) * sum_z P_z  (64-bit integer partials, exact in any order).
// WIDE (many K ranges): eight independent accumulators keep eight loads in flight; otherwise the
// plain loop, whose low register count keeps more threads (and loads) resident.
template <bool WIDE>
__global__ void k_sliced_finish(int64_t M, int64_t N, int splits, const long long* __restrict__ P,
                                double* __restrict__ C, int64_t ldc, const int* __restrict__ ea,
                                const int* __restrict__ eb) {
  const int64_t total = M * N;
  OFRR_FOR_2D(m, n, M, N) {
    const int64_t e = m + n * M;
    long long s = 0;
    if (WIDE) {
      long long acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      int z = 0;
      for (; z + 8 <= splits; z += 8) {
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] += P[(size_t)(z + u) * total + e];
      }
      for (; z < splits; ++z) acc[0] += P[(size_t)z * total + e];
#pragma unroll
      for (int u = 0; u < 8; ++u) s += acc[u];
    } else {
      for (int z = 0; z < splits; ++z) s += P[(size_t)z * total + e];
    }
    C[m + n * ldc] = i64_ldexp(s, ea[m] + eb[n] - SL_SHIFT);
  }
}

// k_sliced_finish fused with k_scalecols_slice for a product C (m x N) that is only needed scaled and
// split: each CTA sums the int64 partials of its rows (same values as k_sliced_finish), then scales
// and splits them.  WRITE_U also stores the scaled FP64 column.
template <int U, int CL, bool WRITE_U>
__global__ void __launch_bounds__(SCS_T) k_finish_scalecols_slice(int64_t m, int64_t N, int64_t Kp, int splits,
                                                                  const long long* __restrict__ P,
                                                                  const int* __restrict__ ea,
                                                                  const int* __restrict__ eb, double* __restrict__ C,
                                                                  int64_t ldc, __nv_bfloat16* __restrict__ stack,
                                                                  int* __restrict__ expo) {
  if (CL > 1) cluster_arrive_relaxed();
  const int n = blockIdx.x / CL;
  const int64_t r0 = (int64_t)(blockIdx.x % CL) * SCS_T * U;
  const int64_t total = m * N;
  const long long* pc = P + (int64_t)n * m;
  long long s[U];
#pragma unroll
  for (int u = 0; u < U; ++u) s[u] = 0;
#pragma unroll 4
  for (int z = 0; z < splits; ++z) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
      if (i < m) s[u] += pc[(size_t)z * total + i];
    }
  }
  const int ebn = eb[n];
  double v[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int64_t i = r0 + threadIdx.x + (int64_t)u * SCS_T;
    v[u] = (i < m) ? i64_ldexp(s[u], ea[i] + ebn - SL_SHIFT) : 0.0;
  }
  scalecols_slice_body<U, CL>(m, Kp, n, r0, v, WRITE_U ? C + (int64_t)n * ldc : nullptr, stack, expo);
}

}  // namespace slice

static_assert(slice::S == kSliceDigits, "digit count");

// Digit stack of X (K x M, column-major FP64) into caller buffers (M * S * roundup(K, 64) bf16, M ints)
int sliced_prepare_into(ofrr_ctx* ctx, int64_t K, int64_t M, const double* X, int64_t ldx, __nv_bfloat16* stack,
                        int* expo, SlicedOperand* out) {
  out->K = K;
  out->Kp = (K + 63) / 64 * 64;
  out->M = M;
  out->stack = stack;
  out->expo = expo;
  if (out->Kp <= 128) {  // short columns (back-transform coefficients): 64 threads per column
    slice::k_slice_cols<2, 64><<<(unsigned)std::min<int64_t>(M, 65535), 64, 0, ctx->stream>>>(K, out->Kp, M, X, ldx,
                                                                                            stack, expo);
    OFRR_LAUNCHED(ctx, "k_slice_cols");
    return OFRR_SUCCESS;
  }
  if (out->Kp <= slice::SC_T * 16) {
    const unsigned grid = (unsigned)std::min<int64_t>(M, 65535);
    const int64_t u = (out->Kp + slice::SC_T - 1) / slice::SC_T;
    if (u <= 2)
      slice::k_slice_cols<2><<<grid, slice::SC_T, 0, ctx->stream>>>(K, out->Kp, M, X, ldx, stack, expo);
    else if (u <= 4)
      slice::k_slice_cols<4><<<grid, slice::SC_T, 0, ctx->stream>>>(K, out->Kp, M, X, ldx, stack, expo);
    else if (u <= 8)
      slice::k_slice_cols<8><<<grid, slice::SC_T, 0, ctx->stream>>>(K, out->Kp, M, X, ldx, stack, expo);
    else
      slice::k_slice_cols<16><<<grid, slice::SC_T, 0, ctx->stream>>>(K, out->Kp, M, X, ldx, stack, expo);
    OFRR_LAUNCHED(ctx, "k_slice_cols");
    return OFRR_SUCCESS;
  }
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  unsigned long long* colmax = ws_get<unsigned long long>(ctx, (size_t)M, &st);
  if (!colmax) return st;
  OFRR_CUDA(cudaMemsetAsync(colmax, 0, sizeof(unsigned long long) * (size_t)M, ctx->stream));
  const dim3 g1((unsigned)((K + slice::SLICE_CHUNK - 1) / slice::SLICE_CHUNK), (unsigned)std::min<int64_t>(M, 65535));
  slice::k_slice_max<<<g1, slice::SLICE_T, 0, ctx->stream>>>(K, M, X, ldx, colmax);
  OFRR_LAUNCHED(ctx, "k_slice_max");
  const dim3 g2((unsigned)((out->Kp + slice::SLICE_CHUNK - 1) / slice::SLICE_CHUNK), g1.y);
  slice::k_slice_digits<<<g2, slice::SLICE_T, 0, ctx->stream>>>(K, out->Kp, M, X, ldx, colmax, out->stack, out->expo);
  OFRR_LAUNCHED(ctx, "k_slice_digits");
  return OFRR_SUCCESS;
}

// Build the digit stack of X (K x M, column-major FP64) in the workspace.
int sliced_prepare(ofrr_ctx* ctx, int64_t K, int64_t M, const double* X, int64_t ldx, SlicedOperand* out) {
  int st = OFRR_SUCCESS;
  const int64_t Kp = (K + 63) / 64 * 64;
  __nv_bfloat16* stack = ws_get<__nv_bfloat16>(ctx, (size_t)M * slice::S * Kp, &st);
  if (!stack) return st;
  int* expo = ws_get<int>(ctx, (size_t)M, &st);
  if (!expo) return st;
  return sliced_prepare_into(ctx, K, M, X, ldx, stack, expo, out);
}

// C (M x N, FP64) = A_op' B with A_op the prepared stack (K x M) and B (K x N, FP64, column-major)
// C (M x N, FP64) = A_op' B with A_op the prepared stack (K x M) and B (K x N, FP64, column-major).
// reps > 1 (profiling) repeats the product kernel and reports its mean time per launch in *us.
// fs != nullptr (with several K ranges): the partial sums go straight to k_finish_scalecols_slice.
struct FusedScale {
  bool write_u;
  __nv_bfloat16* stack;
  int* expo;
  bool done = false;
};
static int sliced_gemm_run(ofrr_ctx* ctx, const SlicedOperand& A, int64_t N, const double* B, int64_t ldb, double* C,
                           int64_t ldc, int reps, double* us, double* bytes, const SlicedOperand* Bpre = nullptr,
                           FusedScale* fs = nullptr) {
  using namespace slice;
  const int64_t K = A.K, Kp = A.Kp, M = A.M;
  // the combined 64-bit integer is bounded by K 2^(2 BETA + BETA LMAX) (1 + 2^-6): K <= 2^20 keeps it below 2^63
  if (K > (1ll << 20) || M > (1ll << 30) || N > (1ll << 30)) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  SlicedOperand Bs;
  if (Bpre) {
    if (Bpre->K != K || Bpre->Kp != Kp || Bpre->M != N) return OFRR_ERR_INVALID_ARGUMENT;
    Bs = *Bpre;
  } else {
    OFRR_TRY(sliced_prepare(ctx, K, N, B, ldb, &Bs));
  }
  CUtensorMap ma, mb;
  if (!tc::make_map(&ma, OFRR_BF16, A.stack, S * Kp, M, S * Kp, tc::BM) ||
      !tc::make_map(&mb, OFRR_BF16, Bs.stack, S * Kp, N, S * Kp, SBN))
    return OFRR_ERR_INTERNAL;
  const int kbt = (int)(Kp / tc::BK);
  const int tiles = (int)(((M + tc::BM - 1) / tc::BM) * ((N + SBN - 1) / SBN));
  // K ranges of at most 16 k-blocks (exactness), and about one wave of CTAs
  int splits = std::max((kbt + SL_KB_MAX - 1) / SL_KB_MAX, std::min(kbt, std::max(1, 148 / tiles)));
  // few output tiles (Gram products): at most 32 K ranges, so the partial sums stay cheap to combine
  if (tiles <= 4) splits = std::min(splits, std::max((kbt + SL_KB_MAX - 1) / SL_KB_MAX, 32));
  const int kbps = (kbt + splits - 1) / splits;
  splits = (kbt + kbps - 1) / kbps;
  long long* P = nullptr;
  if (splits > 1) {
    P = ws_get<long long>(ctx, (size_t)splits * M * N, &st);
    if (!P) return st;
  }
  static std::atomic<bool> attr_set{false};
  if (!attr_set) {
    OFRR_TRY(allow_smem(k_sliced_tn));
    attr_set = true;
  }
  dim3 grid((unsigned)((M + tc::BM - 1) / tc::BM), (unsigned)((N + SBN - 1) / SBN), (unsigned)splits);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (reps > 1) {
    OFRR_CUDA(cudaEventCreate(&e0));
    OFRR_CUDA(cudaEventCreate(&e1));
    OFRR_CUDA(cudaEventRecord(e0, ctx->stream));
  }
  for (int r = 0; r < (reps > 1 ? reps : 1); ++r) {
    k_sliced_tn<<<grid, SL_THREADS, SL_SMEM, ctx->stream>>>(ma, mb, (int)M, (int)N, Kp, kbt, kbps,
                                                          tc::make_idesc(OFRR_BF16, SBN), P, C, ldc, A.expo, Bs.expo,
                                                          ctx->dev_flags + kFlagTcWait);
    OFRR_LAUNCHED(ctx, "k_sliced_tn");
  }
  if (reps > 1) {
    OFRR_CUDA(cudaEventRecord(e1, ctx->stream));
    OFRR_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    OFRR_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (us) *us = 1e3 * (double)ms / reps;
    if (bytes)  // digit stacks read once, int64 partials (or FP64 C) written once
      *bytes = (double)S * Kp * 2 * (double)(M + N) + (double)M * N * 8 * (splits > 1 ? splits : 1);
  }
  if (splits > 1 && fs) {
    const int64_t Kpc = (M + 63) / 64 * 64;
    OFRR_TRY(scs_dispatch(M, [&](auto u, auto cl) {
      constexpr int RU = decltype(u)::value, CL = decltype(cl)::value;
      if (fs->write_u)
        return launch_cols(ctx, CL, N, k_finish_scalecols_slice<RU, CL, true>, M, N, Kpc, splits, (const long long*)P,
                           (const int*)A.expo, (const int*)Bs.expo, C, ldc, fs->stack, fs->expo);
      return launch_cols(ctx, CL, N, k_finish_scalecols_slice<RU, CL, false>, M, N, Kpc, splits, (const long long*)P,
                         (const int*)A.expo, (const int*)Bs.expo, C, ldc, fs->stack, fs->expo);
    }));
    OFRR_LAUNCHED(ctx, "k_finish_scalecols_slice");
    fs->done = true;
  } else if (splits > 1) {
    if (splits >= 12)
      k_sliced_finish<true><<<grid_2d(M, N, 256), 256, 0, ctx->stream>>>(M, N, splits, P, C, ldc, A.expo, Bs.expo);
    else
      k_sliced_finish<false><<<grid_2d(M, N, 256), 256, 0, ctx->stream>>>(M, N, splits, P, C, ldc, A.expo, Bs.expo);
    OFRR_LAUNCHED(ctx, "k_sliced_finish");
  }
  return OFRR_SUCCESS;
}

int sliced_gemm_tn(ofrr_ctx* ctx, const SlicedOperand& A, int64_t N, const double* B, int64_t ldb, double* C,
                   int64_t ldc) {
  return sliced_gemm_run(ctx, A, N, B, ldb, C, ldc, 1, nullptr, nullptr);
}

int sliced_gemm_tn_pre(ofrr_ctx* ctx, const SlicedOperand& A, const SlicedOperand& B, double* C, int64_t ldc) {
  return sliced_gemm_run(ctx, A, B.M, nullptr, 0, C, ldc, 1, nullptr, nullptr, &B);
}

// U (m x N) = A_op' B, then scalecols and the digit split of the scaled block into stack / expo (out
// describes them), as sliced_gemm_tn_pre followed by scalecols_sliced and with the same results.  With
// several K ranges the partial sums are combined inside the scaling kernel, and write_u = false
// leaves U unwritten (a block that only feeds the next product through its digits).
int sliced_gemm_scalecols_pre(ofrr_ctx* ctx, const SlicedOperand& A, const SlicedOperand& B, double* U, int64_t ldu,
                              bool write_u, __nv_bfloat16* stack, int* expo, SlicedOperand* out) {
  const int64_t m = A.M, n = B.M;
  if (m < 1 || m > 8192 || n < 1 || n > 65535) return OFRR_ERR_BLAS_INVALID_SIZE;
  FusedScale fs{write_u, stack, expo};
  OFRR_TRY(sliced_gemm_run(ctx, A, n, nullptr, 0, U, ldu, 1, nullptr, nullptr, &B, &fs));
  if (!fs.done) return scalecols_sliced(ctx, m, n, U, ldu, stack, expo, out);
  out->K = m;
  out->Kp = (m + 63) / 64 * 64;
  out->M = n;
  out->stack = stack;
  out->expo = expo;
  return OFRR_SUCCESS;
}

int scalecols_sliced(ofrr_ctx* ctx, int64_t m, int64_t n, double* U, int64_t ldu, __nv_bfloat16* stack, int* expo,
                     SlicedOperand* out) {
  if (m < 1 || m > 8192 || n < 1 || n > 65535) return OFRR_ERR_BLAS_INVALID_SIZE;
  out->K = m;
  out->Kp = (m + 63) / 64 * 64;
  out->M = n;
  out->stack = stack;
  out->expo = expo;
  OFRR_TRY(scs_dispatch(m, [&](auto u, auto cl) {
    constexpr int RU = decltype(u)::value, CL = decltype(cl)::value;
    return launch_cols(ctx, CL, n, slice::k_scalecols_slice<RU, CL>, m, out->Kp, U, ldu, stack, expo);
  }));
  OFRR_LAUNCHED(ctx, "k_scalecols_slice");
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

// C ABI wrapper used by the tests: C = A' B in emulated FP64 (A: K x M, B: K x N, all FP64, column-major)
extern "C" int ofrr_gemm_f64_emulated(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                                      const double* B, int64_t ldb, double* C, int64_t ldc) {
  if (!ctx || M < 0 || N < 0 || K < 0) return OFRR_ERR_INVALID_ARGUMENT;
  if (M == 0 || N == 0) return OFRR_SUCCESS;
  if (!A || !B || !C || lda < K || ldb < K || ldc < M || K < 1) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  SlicedOperand As;
  OFRR_TRY(sliced_prepare(ctx, K, M, A, lda, &As));
  return sliced_gemm_tn(ctx, As, N, B, ldb, C, ldc);
}

// Profiling entry point: prepares the digit stacks of A and B once, then times `reps` launches of the
// fused exact-slice product kernel alone (CUDA events on the context's stream); C = A' B as above.
extern "C" int ofrr_profile_gemm_f64_emulated(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A,
                                              int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
                                              int reps, double* us_per_launch, double* bytes_per_launch) {
  if (!ctx || M < 1 || N < 1 || K < 1 || reps < 2 || !us_per_launch || !bytes_per_launch)
    return OFRR_ERR_INVALID_ARGUMENT;
  if (!A || !B || !C || lda < K || ldb < K || ldc < M) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  SlicedOperand As;
  OFRR_TRY(sliced_prepare(ctx, K, M, A, lda, &As));
  return sliced_gemm_run(ctx, As, N, B, ldb, C, ldc, reps, us_per_launch, bytes_per_launch);
}

// Self-test of the fused scale-and-split steps of the emulated FP64 power iteration.  mode 0: X (M x N)
// scaled in place (scalecols_sliced); mode 1: X = A' B (A: K x M, B: K x N) by the exact-slice product
// whose partial sums are combined inside the scaling kernel (sliced_gemm_scalecols_pre, X written);
// mode 2: the stand-alone slicer on X as it is.  All modes write the digit stack (N columns of
// 5 roundup(M, 64) BF16 values) and the column exponents.
extern "C" int ofrr_debug_scale_slice(ofrr_ctx* ctx, int mode, int64_t M, int64_t N, int64_t K, const double* A,
                                      int64_t lda, const double* B, int64_t ldb, double* X, int64_t ldx,
                                      void* digits, int* expo) {
  if (!ctx || mode < 0 || mode > 2 || M < 1 || M > 8192 || N < 1 || N > 65535 || !X || ldx < M || !digits || !expo)
    return OFRR_ERR_INVALID_ARGUMENT;
  __nv_bfloat16* stack = (__nv_bfloat16*)digits;
  SlicedOperand out;
  if (mode == 0) return scalecols_sliced(ctx, M, N, X, ldx, stack, expo, &out);
  if (mode == 2) return sliced_prepare_into(ctx, M, N, X, ldx, stack, expo, &out);
  if (K < 1 || !A || !B || lda < K || ldb < K) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  SlicedOperand As, Bs;
  OFRR_TRY(sliced_prepare(ctx, K, M, A, lda, &As));
  OFRR_TRY(sliced_prepare(ctx, K, N, B, ldb, &Bs));
  return sliced_gemm_scalecols_pre(ctx, As, Bs, X, ldx, true, stack, expo, &out);
}
