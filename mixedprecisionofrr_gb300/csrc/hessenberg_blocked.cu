// Blocked Hessenberg process on thread-block clusters.
//
// Same arithmetic as the per-column kernel in hessenberg.cu (MATLAB/+src/+qr/hessenberg.m:45-85,
// MGS order, one rounding to the output type per elimination), so results are bit-identical; only
// the schedule changes.  Columns are taken in blocks of HB_B = 16:
//   1. k_hess_blockupd (one launch per block, all SMs): every column of the block is eliminated
//      against the already final columns 0..c0-1 in order j = 0, 1, ..., c0-1.  The coefficients
//      r_{j,i} come from a forward substitution over the c0 pivot rows (one warp per column of the
//      block).  Each thread loads q_j(row) once per j and applies it to all block columns.
//   2. k_hess_inblock (one launch per block, one 8-CTA cluster): the block's columns are processed
//      one after another entirely on chip.  Each CTA keeps its slice of rows of the block in shared
//      memory; the grid-wide argmax of a column is a cluster barrier plus reads of the other CTAs'
//      partials through distributed shared memory; every CTA then reads the pivot row of the block
//      from its owner (DSMEM), which holds exactly the values the later columns' substitutions need.
// For b = 64 columns this is 7 launches instead of 65.  Used when the block's rows fit in the
// cluster's shared memory; larger problems keep the per-column kernel.
#include <cooperative_groups.h>

#include <cstdlib>

#include "ofrr_internal.cuh"

namespace cg = cooperative_groups;

namespace ofrr {

constexpr int HB_B = 16;        // block width (columns)
constexpr int HB_CL = 8;        // CTAs per cluster (portable cluster size)
constexpr int HB_T = 256;       // threads per CTA
constexpr size_t HB_SMEM_MAX = 200 * 1024;

// ---- step 1: eliminate block columns [c0, c1) against final columns [0, c0) -----------------------
template <class TO, class TC>
__global__ void __launch_bounds__(HB_T) k_hess_blockupd(int64_t m, int n, int c0, int c1, TO* __restrict__ Q,
                                                        int64_t ldq, const int* __restrict__ select,
                                                        const int* __restrict__ perm, const TO* __restrict__ pivrows,
                                                        double* __restrict__ R) {
  extern __shared__ unsigned char smem_raw[];
  const int nb = c1 - c0;
  TC* s_r = reinterpret_cast<TC*>(smem_raw);                                // HB_B x c0
  TO* s_x = reinterpret_cast<TO*>(s_r + HB_B * c0);                         // HB_B x c0
  TO* s_L = reinterpret_cast<TO*>(((uintptr_t)(s_x + HB_B * c0) + 15) & ~(uintptr_t)15);  // c0 x c0
  int* s_sel = reinterpret_cast<int*>(((uintptr_t)(s_L + c0 * c0) + 15) & ~(uintptr_t)15); // c0
  const int tid = threadIdx.x;
  for (int j = tid; j < c0; j += blockDim.x) s_sel[j] = select[j];
  for (int e = tid; e < c0 * c0; e += blockDim.x) {
    const int jj = e / c0, l = e % c0;
    if (l < jj) s_L[e] = pivrows[(int64_t)jj * n + l];
  }
  __syncthreads();
  for (int e = tid; e < nb * c0; e += blockDim.x) {
    const int t = e / c0, j = e % c0;
    s_x[t * c0 + j] = s_sel[j] ? Q[(int64_t)perm[j] + (int64_t)(c0 + t) * ldq] : TO(0);
  }
  __syncthreads();
  // forward substitution per block column (warp w handles columns w, w + 8, ...)
  const int warp = tid >> 5, lane = tid & 31;
  for (int t = warp; t < nb; t += (blockDim.x >> 5)) {
    TO* x = s_x + t * c0;
    TC* r = s_r + t * c0;
    for (int j = 0; j < c0; ++j) {
      __syncwarp();
      if (!s_sel[j]) {
        if (lane == 0) r[j] = TC(0);
        continue;
      }
      const TC rc = to_c<TC, TO>(x[j]);
      for (int jj = j + 1 + lane; jj < c0; jj += 32) {
        if (s_sel[jj]) x[jj] = from_c<TO, TC>(sub_rn(to_c<TC, TO>(x[jj]), mul_rn(rc, to_c<TC, TO>(s_L[jj * c0 + j]))));
      }
      if (lane == 0) r[j] = rc;
    }
    __syncwarp();
  }
  __syncthreads();
  if (blockIdx.x == 0) {  // R(j, i) for j < c0
    for (int e = tid; e < nb * c0; e += blockDim.x) {
      const int t = e / c0, j = e % c0;
      R[j + (int64_t)(c0 + t) * n] = s_sel[j] ? to_c<double, TC>(s_r[t * c0 + j]) : 0.0;
    }
  }
  // eliminations, MGS order j = 0 .. c0-1 for every block column of this thread's rows
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + tid; row < m; row += stride) {
    TC v[HB_B];
    TO vo[HB_B];
#pragma unroll
    for (int t = 0; t < HB_B; ++t) {
      vo[t] = (t < nb) ? Q[row + (int64_t)(c0 + t) * ldq] : TO(0);
      v[t] = to_c<TC, TO>(vo[t]);
    }
    for (int j = 0; j < c0; ++j) {
      if (!s_sel[j]) continue;
      const TC q = to_c<TC, TO>(Q[row + (int64_t)j * ldq]);
#pragma unroll
      for (int t = 0; t < HB_B; ++t) {
        if (t < nb) {
          vo[t] = from_c<TO, TC>(sub_rn(v[t], mul_rn(s_r[t * c0 + j], q)));
          v[t] = to_c<TC, TO>(vo[t]);
        }
      }
    }
#pragma unroll
    for (int t = 0; t < HB_B; ++t)
      if (t < nb) Q[row + (int64_t)(c0 + t) * ldq] = vo[t];
  }
}

// ---- step 2: the block's columns on one cluster ---------------------------------------------------
template <class TO, class TC>
__global__ void __cluster_dims__(HB_CL, 1, 1) __launch_bounds__(HB_T)
    k_hess_inblock(int64_t m, int n, int c0, int c1, TO* __restrict__ Q, int64_t ldq, int* __restrict__ select,
                   int* __restrict__ perm, TO* __restrict__ pivrows, TO* __restrict__ pvals, double* __restrict__ R,
                   double select_tol, int64_t rows_per_cta) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int nb = c1 - c0;
  const int tid = threadIdx.x;
  const int64_t RR = rows_per_cta;
  const int64_t r0 = (int64_t)rank * RR;
  const int64_t r1 = (r0 + RR < m) ? r0 + RR : m;
  extern __shared__ unsigned char smem_raw[];
  TO* s_blk = reinterpret_cast<TO*>(smem_raw);             // HB_B columns x RR rows (column t at t * RR)
  TO* s_prow = s_blk + (size_t)HB_B * RR;                  // HB_B x HB_B: pivot row of block column t'
  __shared__ ArgMax s_part;
  __shared__ ArgMax red[32];
  __shared__ TC s_r[HB_B];
  __shared__ TO s_x[HB_B];
  __shared__ int s_sel[HB_B];
  __shared__ int64_t s_k;
  __shared__ int s_keep;

  for (int64_t row = r0 + tid; row < r1; row += blockDim.x)
    for (int t = 0; t < nb; ++t) s_blk[(size_t)t * RR + (row - r0)] = Q[row + (int64_t)(c0 + t) * ldq];
  __syncthreads();
  const double tol_o = to_c<double, TO>(from_c<TO, double>(select_tol));

  for (int t = 0; t < nb; ++t) {
    // (1) forward substitution over the in-block pivot rows t' < t (warp 0; every CTA alike)
    if (tid < 32) {
      for (int tp = tid; tp < t; tp += 32) s_x[tp] = s_prow[tp * HB_B + t];
      __syncwarp();
      for (int tp = 0; tp < t; ++tp) {
        __syncwarp();
        if (!s_sel[tp]) {
          if (tid == 0) s_r[tp] = TC(0);
          continue;
        }
        const TC rc = to_c<TC, TO>(s_x[tp]);
        for (int tq = tp + 1 + tid; tq < t; tq += 32) {
          if (s_sel[tq])
            s_x[tq] = from_c<TO, TC>(sub_rn(to_c<TC, TO>(s_x[tq]), mul_rn(rc, to_c<TC, TO>(s_prow[tq * HB_B + tp]))));
        }
        if (tid == 0) s_r[tp] = rc;
      }
    }
    __syncthreads();
    // (2) eliminations of this CTA's rows against the in-block columns t' < t (MGS order continues
    //     after the j < c0 eliminations of step 1), local argmax
    ArgMax a{-1.0, 0x7fffffffffffffffLL};
    for (int64_t row = r0 + tid; row < r1; row += blockDim.x) {
      const int64_t lr = row - r0;
      TO vo = s_blk[(size_t)t * RR + lr];
      TC v = to_c<TC, TO>(vo);
      for (int tp = 0; tp < t; ++tp) {
        if (!s_sel[tp]) continue;
        vo = from_c<TO, TC>(sub_rn(v, mul_rn(s_r[tp], to_c<TC, TO>(s_blk[(size_t)tp * RR + lr]))));
        v = to_c<TC, TO>(vo);
      }
      s_blk[(size_t)t * RR + lr] = vo;
      const double av = absd(vo);
      if (av > a.v) a = ArgMax{av, row};
    }
    ArgMax r = block_argmax(a, red);
    if (tid == 0) s_part = r;
    // (3) cluster-wide argmax through distributed shared memory
    cluster.sync();
    if (tid == 0) {
      ArgMax b{-1.0, 0x7fffffffffffffffLL};
      for (int q = 0; q < HB_CL; ++q) {
        const ArgMax* pq = cluster.map_shared_rank(&s_part, q);
        ArgMax p;
        p.v = pq->v;
        p.i = pq->i;
        b = argmax_pick(b, p);
      }
      s_k = (b.v < 0.0) ? 0 : b.i;
    }
    __syncthreads();
    // (4) the pivot row of the block, read from the CTA that owns it
    const int64_t k = s_k;
    const int owner = (int)(k / RR);
    if (tid < HB_B) {
      const TO* ob = cluster.map_shared_rank(s_blk, owner);
      s_prow[t * HB_B + tid] = (tid < nb) ? ob[(size_t)tid * RR + (k - (int64_t)owner * RR)] : TO(0);
    }
    __syncthreads();
    const TO pv = s_prow[t * HB_B + t];
    const bool keep = absd(pv) >= tol_o && s_k >= 0;
    if (tid == 0) {
      s_keep = keep ? 1 : 0;
      s_sel[t] = keep ? 1 : 0;
    }
    cluster.sync();  // every CTA has read the owner's row before anyone scales it
    // (5) scale (or zero) this CTA's rows of column t
    const TC pc = to_c<TC, TO>(pv);
    for (int64_t row = r0 + tid; row < r1; row += blockDim.x) {
      const int64_t lr = row - r0;
      const TO q = s_blk[(size_t)t * RR + lr];
      s_blk[(size_t)t * RR + lr] = keep ? from_c<TO, TC>(div_rn(to_c<TC, TO>(q), pc)) : TO(0);
    }
    // (6) bookkeeping (rank 0): pivot, selection, R(:, i), pivot row of Q for later blocks
    if (rank == 0) {
      const int i = c0 + t;
      if (tid == 0) {
        select[i] = keep ? 1 : 0;
        perm[i] = keep ? (int)k : -1;
        pvals[i] = keep ? pv : TO(0);
        R[i + (int64_t)i * n] = to_c<double, TO>(pv);
      }
      for (int tp = tid; tp < t; tp += blockDim.x)
        R[(c0 + tp) + (int64_t)i * n] = s_sel[tp] ? to_c<double, TC>(s_r[tp]) : 0.0;
      if (keep) {
        for (int l = tid; l < i; l += blockDim.x)
          pivrows[(int64_t)i * n + l] = (l < c0) ? Q[k + (int64_t)l * ldq] : s_prow[t * HB_B + (l - c0)];
      }
    }
    __syncthreads();
  }
  for (int64_t row = r0 + tid; row < r1; row += blockDim.x)
    for (int t = 0; t < nb; ++t) Q[row + (int64_t)(c0 + t) * ldq] = s_blk[(size_t)t * RR + (row - r0)];
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// shared memory the in-block kernel needs for m rows (0 if it does not fit)
size_t hess_blocked_smem(int64_t m, size_t es) {
  const int64_t RR = (m + HB_CL - 1) / HB_CL;
  const size_t bytes = (size_t)HB_B * RR * es + (size_t)HB_B * HB_B * es + 64;
  return bytes <= HB_SMEM_MAX ? bytes : 0;
}

template <class TO, class TC>
int hess_run_blocked_t(ofrr_ctx* ctx, int64_t m, int n, TO* Q, int64_t ldq, double select_tol, double* R, int* select,
                       int* perm) {
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  TO* pivrows = ws_get<TO>(ctx, (size_t)n * n, &st);
  if (!pivrows) return st;
  TO* pvals = ws_get<TO>(ctx, (size_t)n, &st);
  if (!pvals) return st;
  OFRR_TRY(fill_zero(ctx, R, sizeof(double) * (size_t)n * n));
  OFRR_TRY(fill_zero(ctx, pivrows, sizeof(TO) * (size_t)n * n));
  const int64_t RR = (m + HB_CL - 1) / HB_CL;
  const size_t smem2 = hess_blocked_smem(m, sizeof(TO));
  if (!smem2) return OFRR_ERR_BLAS_INVALID_SIZE;
  OFRR_CUDA(cudaFuncSetAttribute(k_hess_inblock<TO, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
  const int grid1 = grid_for(m, HB_T, 152 * 2);
  for (int c0 = 0; c0 < n; c0 += HB_B) {
    const int c1 = (c0 + HB_B < n) ? c0 + HB_B : n;
    if (c0 > 0) {
      const size_t smem1 = (size_t)HB_B * c0 * (sizeof(TC) + sizeof(TO)) + 32 + (size_t)c0 * c0 * sizeof(TO) +
                           (size_t)c0 * sizeof(int);
      if (smem1 > 48 * 1024)
        OFRR_CUDA(cudaFuncSetAttribute(k_hess_blockupd<TO, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem1));
      k_hess_blockupd<TO, TC><<<grid1, HB_T, smem1, ctx->stream>>>(m, n, c0, c1, Q, ldq, select, perm, pivrows, R);
      OFRR_LAUNCHED(ctx, "k_hess_blockupd");
    }
    k_hess_inblock<TO, TC><<<HB_CL, HB_T, smem2, ctx->stream>>>(m, n, c0, c1, Q, ldq, select, perm, pivrows, pvals, R,
                                                               select_tol, RR);
    OFRR_LAUNCHED(ctx, "k_hess_inblock");
  }
  return OFRR_SUCCESS;
}

// Blocked build when it fits (m rows of the block in the cluster's shared memory, n <= 256);
// *done = false leaves the call to the per-column path.
int hess_run_blocked(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n, void* Q, int64_t ldq,
                     double select_tol, double* R, int* select, int* perm, bool* done) {
  *done = false;
  if (n > 256 || m < 2 * HB_CL || getenv("OFRR_HESS_PER_COLUMN")) return OFRR_SUCCESS;
  if (!hess_blocked_smem(m, dtype_size(tout))) return OFRR_SUCCESS;
  // step-1 shared memory at the last block: coefficients, working values and the c0 x c0 pivot block
  const int64_t c0max = ((n - 1) / HB_B) * HB_B;
  const size_t es = dtype_size(tout), ec = dtype_size(tc);
  if ((size_t)HB_B * c0max * (es + ec) + 32 + (size_t)c0max * c0max * es + (size_t)c0max * 4 > HB_SMEM_MAX)
    return OFRR_SUCCESS;
  OFRR_DISPATCH_STORAGE(tout, TO, OFRR_DISPATCH_COMPUTE(tc, TC, {
    OFRR_TRY((hess_run_blocked_t<TO, TC>(ctx, m, (int)n, (TO*)Q, ldq, select_tol, R, select, perm)));
  }));
  *done = true;
  return OFRR_SUCCESS;
}

}  // namespace ofrr
