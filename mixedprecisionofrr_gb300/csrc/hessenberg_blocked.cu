// Blocked Hessenberg process on thread-block clusters.
//
// Same arithmetic as the per-column kernel in hessenberg.cu (MATLAB/+src/+qr/hessenberg.m:45-85,
// MGS order, one rounding to the output type per elimination), so results are bit-identical; only
// the schedule changes.  Columns are taken in blocks of HB_B = 16; for a block [c0, c1):
//   0. k_hess_blockcoef (one CTA): the coefficients r_{j,i}, j < c0, of every block column by a
//      forward substitution over the c0 pivot rows (one warp per block column), and R(j, i).  The
//      pivot rows are read from Q while the block columns are still untouched, before any update.
//   1. k_hess_blockupd (all SMs): every block column is eliminated against the final columns
//      0..c0-1 in order j = 0, 1, ..., c0-1; each thread owns one row and HB_CG block columns.
//   2. k_hess_inblock (one cluster of 8 or 16 CTAs): the block's columns one after another entirely
//      on chip, right-looking.  Each CTA keeps its slice of rows of the block in shared memory.  Per
//      column: each CTA publishes its candidate (local argmax and the block's values in that row);
//      after ONE cluster barrier every CTA reads all candidates through distributed shared memory,
//      takes the winner's row as the pivot row, scales the column and eliminates the later block
//      columns against it (their coefficients are the pivot row's values).
// For b = 64 columns this is 10 launches instead of 65.
#include <cooperative_groups.h>

#include <atomic>
#include <cstdlib>
#include <type_traits>

#include "ofrr_internal.cuh"
#include "tcgen05.cuh"

namespace cg = cooperative_groups;

namespace ofrr {

constexpr int HB_B = 16;     // block width (columns)
constexpr int HB_T = 512;    // threads per CTA of the in-block kernel (one row per thread at 8192 rows)
constexpr int HB_UT = 128;   // threads per CTA of the block update
constexpr int HB_CG = 2;     // block columns per CTA of the block update
constexpr size_t HB_SMEM_MAX = 200 * 1024;
constexpr int HBC_R = 8;  // block coefficients: entries per lane (c0 <= 256)

// One MGS elimination v - r q in the compute type.  Exact mode: the product rounded, then the
// difference (hessenberg.m's arithmetic, bit-identical to the per-column kernel).  FAST (FP64
// refinement phase of the mixed and FP64 solvers): one FMA, and pivot scaling by the correctly
// rounded reciprocal; GB300's FP64 pipe is 1/64 rate, so this halves the work that bounds the build.
template <bool FAST> __device__ __forceinline__ double elim(double v, double r, double q) {
  return FAST ? __fma_rn(-r, q, v) : __dsub_rn(v, __dmul_rn(r, q));
}
template <bool FAST> __device__ __forceinline__ float elim(float v, float r, float q) {
  return FAST ? __fmaf_rn(-r, q, v) : __fsub_rn(v, __fmul_rn(r, q));
}
__device__ __forceinline__ double mul_recip(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ float mul_recip(float x, float y) { return __fmul_rn(x, y); }

// Forward substitution of one block column over the c0 pivot rows, by one warp with the column's
// entries in registers (lane l holds entries l, l+32, .., NR of them): the coefficient of step j is a
// shuffle from its owner, then every later entry is updated; the same roundings as the shared-memory
// form (each update rounded to the storage type).
template <int NR, class TO, class TC, bool FAST>
__device__ __forceinline__ void blockcoef_subst(int c0, int n, int warp, int lane, const TO* x, const TO* s_L,
                                                const int* s_sel, TC* r, double* R) {
  TC xv[NR];
  bool sv[NR];
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const int jj = lane + 32 * q;
    xv[q] = (jj < c0) ? to_c<TC, TO>(x[jj]) : TC(0);
    sv[q] = (jj < c0) ? (s_sel[jj] != 0) : false;
  }
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    for (int jl = 0; jl < 32; ++jl) {
      const int j = 32 * q + jl;
      if (j >= c0) break;
      const bool selj = s_sel[j] != 0;
      const TC rc = __shfl_sync(0xffffffffu, xv[q], jl);
      if (lane == 0) {
        r[j] = selj ? rc : TC(0);
        R[j + (int64_t)(c0 + warp) * n] = selj ? to_c<double, TC>(rc) : 0.0;
      }
      if (!selj) continue;
#pragma unroll
      for (int w = q; w < NR; ++w) {
        const int jj = lane + 32 * w;
        if (jj > j && jj < c0 && sv[w])
          xv[w] = to_c<TC, TO>(from_c<TO, TC>(elim<FAST>(xv[w], rc, to_c<TC, TO>(s_L[jj * c0 + j]))));
      }
    }
  }
}

// ---- step 0: coefficients of the block columns against the final columns [0, c0) -----------------
template <class TO, class TC, bool FAST>
__global__ void __launch_bounds__(HB_B * 32) k_hess_blockcoef(int n, int c0, int c1, const TO* __restrict__ Q,
                                                              int64_t ldq, const int* __restrict__ select,
                                                              const int* __restrict__ perm, TC* __restrict__ rcoef,
                                                              double* __restrict__ R) {
  extern __shared__ unsigned char smem_raw[];
  const int nb = c1 - c0;
  TO* s_L = reinterpret_cast<TO*>(smem_raw);                                               // c0 x c0
  TO* s_x = s_L + (size_t)c0 * c0;                                                          // HB_B x c0
  int* s_sel = reinterpret_cast<int*>(((uintptr_t)(s_x + (size_t)HB_B * c0) + 15) & ~(uintptr_t)15);  // c0
  int* s_perm = s_sel + c0;                                                                 // c0
  const int tid = threadIdx.x;
  for (int j = tid; j < c0; j += blockDim.x) {
    s_sel[j] = select[j];
    s_perm[j] = perm[j];
  }
  __syncthreads();
  // pivot row jj of the final columns l < jj, and the (untouched) block columns at the pivot rows;
  // the gathers issued eight per thread at a time
  for (int e0 = tid; e0 < c0 * c0; e0 += 8 * blockDim.x) {
    TO v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * blockDim.x;
      const int jj = e / c0, l = e - jj * c0;
      v[u] = (e < c0 * c0 && l < jj && s_sel[jj]) ? Q[(int64_t)s_perm[jj] + (int64_t)l * ldq] : TO(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * blockDim.x;
      if (e < c0 * c0) s_L[e] = v[u];
    }
  }
  for (int e0 = tid; e0 < nb * c0; e0 += 8 * blockDim.x) {
    TO v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * blockDim.x;
      const int t = e / c0, j = e - t * c0;
      v[u] = (e < nb * c0 && s_sel[j]) ? Q[(int64_t)s_perm[j] + (int64_t)(c0 + t) * ldq] : TO(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = e0 + u * blockDim.x;
      if (e < nb * c0) s_x[e] = v[u];
    }
  }
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  if (warp < nb && c0 <= 32 * HBC_R) {
    const int nr = (c0 + 31) / 32;  // registers per lane actually used: predicated-off FP64 slots would
                                    // still occupy the 1/64-rate pipe, so the width is a template
    TO* x = s_x + warp * c0;
    TC* r = rcoef + (size_t)warp * c0;
    switch (nr) {
      case 1: blockcoef_subst<1, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      case 2: blockcoef_subst<2, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      case 3: blockcoef_subst<3, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      case 4: blockcoef_subst<4, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      case 5: blockcoef_subst<5, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      case 6: blockcoef_subst<6, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      case 7: blockcoef_subst<7, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
      default: blockcoef_subst<8, TO, TC, FAST>(c0, n, warp, lane, x, s_L, s_sel, r, R); break;
    }
  } else if (warp < nb) {
    TO* x = s_x + warp * c0;
    TC* r = rcoef + (size_t)warp * c0;
    for (int j = 0; j < c0; ++j) {
      __syncwarp();
      if (!s_sel[j]) {
        if (lane == 0) {
          r[j] = TC(0);
          R[j + (int64_t)(c0 + warp) * n] = 0.0;
        }
        continue;
      }
      const TC rc = to_c<TC, TO>(x[j]);
      for (int jj = j + 1 + lane; jj < c0; jj += 32) {
        if (s_sel[jj]) x[jj] = from_c<TO, TC>(elim<FAST>(to_c<TC, TO>(x[jj]), rc, to_c<TC, TO>(s_L[jj * c0 + j])));
      }
      if (lane == 0) {
        r[j] = rc;
        R[j + (int64_t)(c0 + warp) * n] = to_c<double, TC>(rc);
      }
    }
  }
}

// ---- step 1: eliminate block columns against the final columns [0, c0) ----------------------------
template <class TO, class TC, bool FAST>
__global__ void __launch_bounds__(HB_UT) k_hess_blockupd(int64_t m, int c0, int c1, TO* __restrict__ Q, int64_t ldq,
                                                         const int* __restrict__ select,
                                                         const TC* __restrict__ rcoef) {
  extern __shared__ unsigned char smem_raw[];
  TC* s_r = reinterpret_cast<TC*>(smem_raw);                // HB_CG x c0
  int* s_sel = reinterpret_cast<int*>(s_r + HB_CG * c0);   // c0
  const int tid = threadIdx.x;
  const int t0 = c0 + blockIdx.y * HB_CG;
  const int nl = min(HB_CG, c1 - t0);
  for (int e = tid; e < nl * c0; e += blockDim.x) s_r[e] = rcoef[(size_t)(t0 - c0) * c0 + e];
  for (int j = tid; j < c0; j += blockDim.x) s_sel[j] = select[j];
  __syncthreads();
  const int64_t row = blockIdx.x * (int64_t)HB_UT + tid;
  if (row >= m) return;
  TC v[HB_CG];
  TO vo[HB_CG];
#pragma unroll
  for (int t = 0; t < HB_CG; ++t) {
    vo[t] = (t < nl) ? Q[row + (int64_t)(t0 + t) * ldq] : TO(0);
    v[t] = to_c<TC, TO>(vo[t]);
  }
  constexpr int U = 8;  // loads of Q(row, j) issued ahead of their use
  for (int j0 = 0; j0 < c0; j0 += U) {
    TO q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) q[u] = (j0 + u < c0) ? Q[row + (int64_t)(j0 + u) * ldq] : TO(0);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = j0 + u;
      if (j < c0 && s_sel[j]) {
        const TC qc = to_c<TC, TO>(q[u]);
#pragma unroll
        for (int t = 0; t < HB_CG; ++t) {
          vo[t] = from_c<TO, TC>(elim<FAST>(v[t], s_r[t * c0 + j], qc));
          v[t] = to_c<TC, TO>(vo[t]);
        }
      }
    }
  }
#pragma unroll
  for (int t = 0; t < HB_CG; ++t)
    if (t < nl) Q[row + (int64_t)(t0 + t) * ldq] = vo[t];
}

// ---- step 2: the block's columns on one cluster ---------------------------------------------------
// Right-looking within the block: when column t's pivot row k is known, the coefficients r_{t,u} of
// the later block columns are simply their current values in row k (they have been eliminated against
// the columns before t), so no substitution is needed.  Every element still sees its eliminations in
// the order j = 0, 1, ..., u-1 with the same operands, so the result is bit-identical to the
// left-looking per-column kernel.
template <class TO>
struct __align__(16) HbCand {
  long long key;  // argmax key of the local max |value| (-1: the CTA has no rows)
  long long i;    // its row
  TO vals[HB_B];  // the block's current values in that row
};
constexpr int HB_CL_MAX = 16;

__device__ __forceinline__ uint32_t cluster_addr(const void* p, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(tc::smem_u32(p)), "r"(rank));
  return r;
}

// Candidates travel by push: each CTA stores its candidate for column t into slot [rank] of every
// CTA's receive buffer t & 1 with st.async (16-byte remote stores completing on the receiver's
// mbarrier), so a column costs one one-way DSMEM transfer instead of a cluster barrier plus remote
// reads.  Buffer / barrier t & 1 is reused for column t + 2 only after every CTA has received all
// candidates of column t + 1, which each CTA sends after it finished reading column t's buffer.
// Within a CTA the argmax of column t + 1 takes one barrier: every warp leaves its (key, row) in
// shared memory and warp 0 alone combines them and sends.
template <class TO, class TC, bool FAST>
__global__ void __launch_bounds__(HB_T) k_hess_inblock(int64_t m, int n, int c0, int c1, TO* __restrict__ Q,
                                                       int64_t ldq, int* __restrict__ select, int* __restrict__ perm,
                                                       double* __restrict__ R, double select_tol,
                                                       int64_t rows_per_cta, int* __restrict__ err) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int ncl = (int)cluster.num_blocks();
  const int nb = c1 - c0;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t RR = rows_per_cta;
  const int64_t r0 = (int64_t)rank * RR;
  const int64_t r1 = (r0 + RR < m) ? r0 + RR : m;
  const int nloc = (r1 > r0) ? (int)(r1 - r0) : 0;
  constexpr uint32_t CB = sizeof(HbCand<TO>);
  constexpr int NCH = (int)(CB / 16);  // 16-byte chunks per candidate
  static_assert(CB % 16 == 0, "candidates move in 16-byte stores");
  extern __shared__ unsigned char smem_raw[];
  TO* s_blk = reinterpret_cast<TO*>(smem_raw);  // HB_B columns x RR rows (column t at t * RR)
  __shared__ HbCand<TO> s_recv[2][HB_CL_MAX];   // candidates of column t in [t & 1][source rank]
  __shared__ HbCand<TO> s_send;                 // this CTA's candidate, staged for the stores
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ ArgMaxK red[HB_T / 32];
  __shared__ int s_abort;
  __shared__ TC s_y;
  __shared__ bool s_pf;

  if (tid == 0) {
    tc::mbar_init(&s_bar[0], 1);
    tc::mbar_init(&s_bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc::mbar_expect_tx(&s_bar[0], ncl * CB);
    if (nb > 1) tc::mbar_expect_tx(&s_bar[1], ncl * CB);
    s_abort = 0;
  }
  for (int lr = tid; lr < nloc; lr += HB_T) {
    TO v[HB_B];
#pragma unroll
    for (int t = 0; t < HB_B; ++t) v[t] = (t < nb) ? Q[r0 + lr + (int64_t)(c0 + t) * ldq] : TO(0);
#pragma unroll
    for (int t = 0; t < HB_B; ++t) s_blk[(size_t)t * RR + lr] = v[t];
  }
  cluster.sync();  // every CTA's barriers are armed before the first push

  // Warp argmax `a` of every warp -> this CTA's candidate for column t, sent to all CTAs.  Called by
  // all threads; the caller's writes to s_blk precede the barrier here.
  auto publish = [&](int t, ArgMaxK a) {
    a = warp_argmaxk_all(a);
    if (lane == 0) red[wid] = a;
    __syncthreads();
    if (wid == 0) {
      ArgMaxK loc = (lane < HB_T / 32) ? red[lane] : ArgMaxK{-1, 0x7fffffffffffffffLL};
      loc = warp_argmaxk_all(loc);
      if (lane < HB_B) {
        s_send.vals[lane] = (loc.key >= 0 && lane < nb) ? s_blk[(size_t)lane * RR + (loc.i - r0)] : TO(0);
        if (lane == 0) {
          s_send.key = loc.key;
          s_send.i = loc.i;
        }
      }
      __syncwarp();
      const uint64_t* src = reinterpret_cast<const uint64_t*>(&s_send);
      for (int x = lane; x < ncl * NCH; x += 32) {
        const int d = x / NCH, c = x - d * NCH;
        asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b64 [%0], {%1, %2}, [%3];" ::"r"(
                         cluster_addr(reinterpret_cast<const char*>(&s_recv[t & 1][rank]) + 16 * c, d)),
                     "l"(src[2 * c]), "l"(src[2 * c + 1]), "r"(cluster_addr(&s_bar[t & 1], d))
                     : "memory");
      }
    }
  };

  const double tol_o = to_c<double, TO>(from_c<TO, double>(select_tol));
  {  // candidate for column 0 (already eliminated against the columns before the block)
    ArgMaxK a{-1, 0x7fffffffffffffffLL};
    for (int lr = tid; lr < nloc; lr += HB_T) {
      const long long key = amax_key(s_blk[lr]);
      if (key > a.key) a = ArgMaxK{key, r0 + lr};
    }
    publish(0, a);
  }

  for (int t = 0; t < nb; ++t) {
    // (1) all candidates of column t; the winner (lowest row among equal maxima), in every warp
    const int b = t & 1;
    if (!tc::mbar_wait(&s_bar[b], (uint32_t)((t >> 1) & 1), err, 41)) s_abort = 1;
    if (tid == 0 && t + 2 < nb) tc::mbar_expect_tx(&s_bar[b], ncl * CB);  // re-arm for column t + 2
    const HbCand<TO>* rc = s_recv[b];
    ArgMaxK w{-1, 0x7fffffffffffffffLL};
    if (lane < ncl) w = ArgMaxK{rc[lane].key, rc[lane].i};
    const ArgMaxK mine = w;
    w = warp_argmaxk_all(w);
    const long long bk = w.key, bi = w.i;
    const unsigned hit = __ballot_sync(0xffffffffu, lane < ncl && mine.key == bk && mine.i == bi);
    const TO* pr = rc[hit ? __ffs(hit) - 1 : 0].vals;  // the pivot row's current values
    const long long k = (bk < 0) ? 0 : bi;
    const TO pv = pr[t];
    const bool keep = !(absd(pv) < tol_o);  // a NaN pivot keeps the column (hessenberg.m)
    // (2) bookkeeping (rank 0): pivot, selection, row i of R (R(i, c0+u) = r_{t,u} for u > t)
    if (rank == 0) {
      const int i = c0 + t;
      if (tid == 0) {
        select[i] = keep ? 1 : 0;
        perm[i] = keep ? (int)k : -1;
        R[i + (int64_t)i * n] = to_c<double, TO>(pv);
      }
      for (int u = t + 1 + tid; u < nb; u += blockDim.x)
        R[i + (int64_t)(c0 + u) * n] = keep ? to_c<double, TC>(to_c<TC, TO>(pr[u])) : 0.0;
    }
    // (3) scale (or zero) column t, eliminate the later block columns against it, argmax of column t+1
    const TC pc = to_c<TC, TO>(pv);
    TC y;
    bool pf;
    if constexpr (std::is_same<TC, double>::value) {
      // one FP64 reciprocal per column (a sequence of 1/64-rate instructions), shared through
      // shared memory: s_y is rewritten only after the next column's exchange, past every read
      if (tid == 0) {
        s_y = pivot_recip(pc);
        s_pf = pivot_fast(pc);
      }
      __syncthreads();
      y = s_y;
      pf = s_pf;
    } else {
      y = pivot_recip(pc);
      pf = pivot_fast(pc);
    }
    const bool has_next = t + 1 < nb;
    ArgMaxK a{-1, 0x7fffffffffffffffLL};
    for (int lr = tid; lr < nloc; lr += HB_T) {
      TO* row = s_blk + lr;
      if (keep) {
        const TC q = to_c<TC, TO>(row[(size_t)t * RR]);
        // FAST: x * RN(1/p) (within an ulp of x / p), the pivot itself exactly 1
        const TC sq = (FAST && pf) ? ((r0 + lr == k) ? TC(1) : mul_recip(q, y)) : pivot_div(q, pc, y, pf);
        const TO so = from_c<TO, TC>(sq);
        row[(size_t)t * RR] = so;
        const TC qs = to_c<TC, TO>(so);
        for (int u = t + 1; u < nb; ++u) {
          TO* e = row + (size_t)u * RR;
          *e = from_c<TO, TC>(elim<FAST>(to_c<TC, TO>(*e), to_c<TC, TO>(pr[u]), qs));
        }
      } else {
        row[(size_t)t * RR] = TO(0);
      }
      if (has_next) {
        const long long key = amax_key(row[(size_t)(t + 1) * RR]);
        if (key > a.key) a = ArgMaxK{key, r0 + lr};
      }
    }
    if (!has_next) break;
    publish(t + 1, a);  // its barrier also makes s_abort visible to every thread
    if (s_abort) break;  // a peer stopped answering: leave (the status word is set)
  }
  __syncthreads();
  for (int lr = tid; lr < nloc; lr += HB_T) {
#pragma unroll
    for (int t = 0; t < HB_B; ++t)
      if (t < nb) Q[r0 + lr + (int64_t)(c0 + t) * ldq] = s_blk[(size_t)t * RR + lr];
  }
  cluster.sync();  // every push into this CTA has landed before any CTA leaves
}

// shared memory the in-block kernel needs for m rows on ncl CTAs (0 if it does not fit)
size_t hess_blocked_smem(int64_t m, size_t es, int ncl) {
  const int64_t RR = (m + ncl - 1) / ncl;
  const size_t bytes = (size_t)HB_B * RR * es;
  return bytes <= HB_SMEM_MAX ? bytes : 0;
}

// Cluster size for the in-block kernel: 16 CTAs (non-portable) when the device can co-schedule
// them with this much shared memory and every CTA gets at least 64 rows, else the portable 8.
template <class TO, class TC, bool FAST>
static int inblock_cluster(int64_t m, size_t smem16) {
  static std::atomic<long long> cache{-1};  // (smem << 8) | ncl of the last query
  if (m < 16 * 64 || !smem16) return 8;
  const char* env = getenv("OFRR_HESS_CLUSTER");
  if (env && atoi(env) == 8) return 8;
  const long long c = cache.load(std::memory_order_relaxed);
  if (c >= 0 && (size_t)(c >> 8) == smem16) return (int)(c & 0xff);
  int ncl = 8;
  if (cudaFuncSetAttribute(k_hess_inblock<TO, TC, FAST>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
          cudaSuccess &&
      allow_smem(k_hess_inblock<TO, TC, FAST>) == OFRR_SUCCESS) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 16;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(HB_T);
    cfg.dynamicSmemBytes = smem16;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_hess_inblock<TO, TC, FAST>, &cfg) == cudaSuccess && nclusters >= 1)
      ncl = 16;
  }
  (void)cudaGetLastError();  // a refused query leaves the portable size
  cache.store(((long long)smem16 << 8) | ncl, std::memory_order_relaxed);
  return ncl;
}

template <class TO, class TC, bool FAST>
int hess_run_blocked_t(ofrr_ctx* ctx, int64_t m, int n, TO* Q, int64_t ldq, double select_tol, double* R, int* select,
                       int* perm, bool* done) {
  const size_t smem16 = hess_blocked_smem(m, sizeof(TO), 16);
  if (!smem16) return OFRR_SUCCESS;
  const int ncl = inblock_cluster<TO, TC, FAST>(m, smem16);
  const size_t smem2 = hess_blocked_smem(m, sizeof(TO), ncl);
  if (!smem2) return OFRR_SUCCESS;  // needs 16 CTAs, and the device cannot co-schedule them
  *done = true;
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  TC* rcoef = ws_get<TC>(ctx, (size_t)HB_B * n, &st);
  if (!rcoef) return st;
  OFRR_TRY(fill_zero(ctx, R, sizeof(double) * (size_t)n * n));
  const int64_t RR = (m + ncl - 1) / ncl;
  if (ncl > 8)
    OFRR_CUDA(cudaFuncSetAttribute(k_hess_inblock<TO, TC, FAST>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  OFRR_TRY(allow_smem(k_hess_inblock<TO, TC, FAST>));
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ncl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ncl);
  cfg.blockDim = dim3(HB_T);
  cfg.dynamicSmemBytes = smem2;
  cfg.stream = ctx->stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  for (int c0 = 0; c0 < n; c0 += HB_B) {
    const int c1 = (c0 + HB_B < n) ? c0 + HB_B : n;
    const int nb = c1 - c0;
    if (c0 > 0) {
      const size_t smem0 = (size_t)c0 * c0 * sizeof(TO) + (size_t)HB_B * c0 * sizeof(TO) + 16 + 2 * (size_t)c0 * 4;
      if (smem0 > 48 * 1024)
        OFRR_TRY(allow_smem(k_hess_blockcoef<TO, TC, FAST>));
      k_hess_blockcoef<TO, TC, FAST><<<1, HB_B * 32, smem0, ctx->stream>>>(n, c0, c1, Q, ldq, select, perm, rcoef, R);
      OFRR_LAUNCHED(ctx, "k_hess_blockcoef");
      const size_t smem1 = (size_t)HB_CG * c0 * sizeof(TC) + (size_t)c0 * sizeof(int);
      const dim3 grid1((unsigned)((m + HB_UT - 1) / HB_UT), (unsigned)((nb + HB_CG - 1) / HB_CG));
      k_hess_blockupd<TO, TC, FAST><<<grid1, HB_UT, smem1, ctx->stream>>>(m, c0, c1, Q, ldq, select, rcoef);
      OFRR_LAUNCHED(ctx, "k_hess_blockupd");
    }
    OFRR_CUDA(cudaLaunchKernelEx(&cfg, k_hess_inblock<TO, TC, FAST>, m, n, c0, c1, Q, ldq, select, perm, R, select_tol,
                                 RR, ctx->dev_flags + kFlagHessWait));
    OFRR_LAUNCHED(ctx, "k_hess_inblock");
  }
  return OFRR_SUCCESS;
}

// Blocked build when it fits (m rows of the block in the cluster's shared memory, n <= 256);
// *done = false leaves the call to the per-column path.  fast selects the FMA / reciprocal arithmetic
// for an FP64 compute type (the production refinement phases); the exact arithmetic otherwise.
int hess_run_blocked(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n, void* Q, int64_t ldq,
                     double select_tol, double* R, int* select, int* perm, bool fast, bool* done) {
  *done = false;
  if (n > 256 || m < 2 * 8 || getenv("OFRR_HESS_PER_COLUMN")) return OFRR_SUCCESS;
  // step-0 shared memory at the last block: the c0 x c0 pivot block and the block's pivot-row values
  const int64_t c0max = ((n - 1) / HB_B) * HB_B;
  const size_t es = dtype_size(tout);
  if ((size_t)c0max * c0max * es + (size_t)HB_B * c0max * es + 16 + 2 * (size_t)c0max * 4 > HB_SMEM_MAX)
    return OFRR_SUCCESS;
  if (fast && tc == OFRR_F64) {
    OFRR_DISPATCH_STORAGE(tout, TO, {
      OFRR_TRY((hess_run_blocked_t<TO, double, true>(ctx, m, (int)n, (TO*)Q, ldq, select_tol, R, select, perm, done)));
    });
    return OFRR_SUCCESS;
  }
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    OFRR_TRY((hess_run_blocked_t<TO, TC, false>(ctx, m, (int)n, (TO*)Q, ldq, select_tol, R, select, perm, done)));
  }));
  return OFRR_SUCCESS;
}

}  // namespace ofrr
