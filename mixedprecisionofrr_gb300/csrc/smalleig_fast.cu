// Fast small projected eigenproblems for the production modes (mixed and FP64).
//
// GB300 runs FP64 at about 2 FMA/clock per SM, 1/64 of its FP32 rate, so an FP64 Jacobi on one CTA
// (the reference-semantics solver in smalleig.cu) costs milliseconds for n = 64..128.  This solver
// keeps FP64 accuracy with almost no FP64 work on any single SM:
//   1. Cholesky of the Gram matrix M + tau I (FP64, one CTA, n^3/6);
//   2. reduction C = L^-1 G L^-T by two column-parallel triangular solves (one warp per column);
//   3. cyclic Jacobi on C in FP32 (one CTA, shared memory) -> eigenvectors W accurate to ~1e-7;
//   4. two steps of the Ogita-Aishima refinement for symmetric eigenproblems (Ogita & Aishima,
//      "Iterative refinement for symmetric eigenvalue decomposition", JJIAM 2018): with
//      P = W'W, T = W'CW (FP64), lambda_i = T_ii / P_ii (Rayleigh quotient) and, for |lambda_j - lambda_i| above a
//      cluster threshold, E_ij = (T_ij + lambda_j (delta_ij - P_ij)) / (lambda_j - lambda_i), else
//      E_ij = (delta_ij - P_ij) / 2; W <- W (I + E).  Each step is quadratically convergent, so two
//      steps take FP32-accurate vectors to FP64 accuracy.  Its products are small FP64 GEMMs spread
//      over many CTAs (one thread per output entry);
//   5. sort by descending eigenvalue and back-transform U = L^-T W (M-orthonormal eigenvectors).
// The SVD form (svd_rr.m's pencil [[0,B],[B',0]] vs blkdiag(U'U, V'V) + tau I) reduces with two
// Cholesky factors to the SVD of C = Lu^-1 B Lv^-T; its right singular vectors are the eigenvectors
// of C'C (refined as above), the left ones Y = C W diag(1/sigma).
#include "ofrr_internal.cuh"

#include <algorithm>

namespace ofrr {

// ---- 1. Cholesky (lower) of M + tau I; batched over blockIdx.x ------------------------------------
// Right-looking; per column one reciprocal square root, the column scaled by it, and the lower
// triangle of the trailing block updated with one warp per column (no index division).
__global__ void __launch_bounds__(256) k_chol_f64(int n, const double* const* Ms, int ldm, double tau,
                                                  double* const* Ls, int* flag) {
  extern __shared__ double S[];
  const double* M = Ms[blockIdx.x];
  double* L = Ls[blockIdx.x];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  __shared__ double s_maxd, s_rinv2[2];
  // stage M + tau I (lower triangle) with 16 loads per thread in flight (the kernel is latency-bound)
  const int nn = n * n;
  for (int e0 = tid; e0 < nn; e0 += 16 * nt) {
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * nt;
      const int j = e / n, i = e - j * n;
      v[u] = (e < nn && i >= j) ? M[i + (size_t)j * ldm] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * nt;
      const int j = e / n, i = e - j * n;
      if (e < nn) S[e] = v[u] + ((i == j) ? tau : 0.0);
    }
  }
  __syncthreads();
  if (tid < 32) {
    long long kmax = -1;
    for (int k = lane; k < n; k += 32) kmax = max(kmax, amax_key(S[k + k * n]));
    for (int o = 16; o > 0; o >>= 1) kmax = max(kmax, (long long)__shfl_xor_sync(0xffffffffu, kmax, o));
    if (lane == 0) s_maxd = (kmax > 0) ? __longlong_as_double(kmax - 1) : 0.0;
  }
  __syncthreads();
  // The pivot's reciprocal square root (~430 cycles of dependent 1/64-rate FP64 instructions) is the
  // serial part of each column.  It is pipelined: while warps 0..nw-2 apply column k to the trailing
  // block, the last warp updates the next diagonal entry S(k+1, k+1) itself and computes its
  // reciprocal square root, so the two overlap.  The arithmetic and its order are unchanged.
  const double floor_d = s_maxd * 1e-15 + 1e-300;
  auto pivot = [&](int k) {  // one thread: floor, reciprocal square root, L_kk = sqrt(d)
    double d = S[k + k * n];
    if (!(d > floor_d)) {
      d = floor_d;
      if (flag) *flag = 1;
    }
    const double r = rsqrt(d);
    S[k + k * n] = d * r;
    s_rinv2[k & 1] = r;
  };
  if (tid == 0 && n > 0) pivot(0);
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const double rinv = s_rinv2[k & 1];
    for (int i = k + 1 + tid; i < n; i += nt) S[i + k * n] *= rinv;
    __syncthreads();
    if (warp == nw - 1) {
      if (lane == 0 && k + 1 < n) {
        const double l = S[k + 1 + k * n];
        S[k + 1 + (k + 1) * n] = fma(-l, l, S[k + 1 + (k + 1) * n]);
        pivot(k + 1);
      }
    } else {
      for (int j = k + 1 + warp; j < n; j += nw - 1) {
        const double ljk = S[j + k * n];
        for (int i = (j == k + 1 ? j + 1 : j) + lane; i < n; i += 32)
          S[i + j * n] = fma(-S[i + k * n], ljk, S[i + j * n]);
      }
    }
    __syncthreads();
  }
  for (int j = warp; j < n; j += nw)
    for (int i = lane; i < n; i += 32) L[i + j * n] = (i >= j) ? S[i + j * n] : 0.0;
}

// ---- 2. triangular solves, one warp per right-hand side ------------------------------------------
// upper == 0: L X = B (forward); upper == 1: L' X = B (backward).  transB: right-hand side j is row j.
// Column-oriented: lane l holds rows l, l+32, l+64, l+96 of its right-hand side in registers; for each
// i the owner broadcasts x_i = x_i / L_ii (multiplied by the staged reciprocal) and every lane
// updates its rows with one FMA each -- about three FP64 warp instructions per row (GB300's FP64 pipe
// is 1/64 rate, so a shuffle-reduced dot product per row would cost several times more).
// TRSM_R: rows per lane (n <= 32 TRSM_R), a template so that no predicated-off FP64 instruction
// occupies the 1/64-rate pipe.
template <int TRSM_R>
// blockIdx.y selects one of up to two independent systems (L, B, X), (L2, B2, X2) of the same shape
__global__ void __launch_bounds__(128) k_trsm_f64(int n, int nrhs, const double* __restrict__ L1, int ldl,
                                                  const double* __restrict__ B1, int ldb, int transB,
                                                  double* __restrict__ X1, int ldx, int upper,
                                                  const double* __restrict__ L2, const double* __restrict__ B2,
                                                  double* __restrict__ X2) {
  const double* __restrict__ L = blockIdx.y ? L2 : L1;
  const double* __restrict__ B = blockIdx.y ? B2 : B1;
  double* __restrict__ X = blockIdx.y ? X2 : X1;
  extern __shared__ double sm_trsm[];  // L (n x n, padded ld n+1), then the n diagonal reciprocals
  const int ld = n + 1;
  double* Ls = sm_trsm;
  double* rd = sm_trsm + (size_t)n * ld;
  const int nn = n * n;
  for (int e0 = threadIdx.x; e0 < nn; e0 += 16 * blockDim.x) {  // 16 loads per thread in flight
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * blockDim.x;
      const int j = e / n, i = e - j * n;
      v[u] = (e < nn) ? L[i + (size_t)j * ldl] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * blockDim.x;
      const int j = e / n, i = e - j * n;
      if (e < nn) Ls[i + j * ld] = v[u];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) rd[i] = 1.0 / Ls[i + i * ld];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = blockIdx.x * 4 + w;
  if (col >= nrhs) return;
  double x[TRSM_R];
#pragma unroll
  for (int u = 0; u < TRSM_R; ++u) {
    const int i = lane + 32 * u;
    x[u] = (i < n) ? (transB ? B[col + (size_t)i * ldb] : B[i + (size_t)col * ldb]) : 0.0;
  }
  if (!upper) {
#pragma unroll
    for (int u = 0; u < TRSM_R; ++u) {
      for (int il = 0; il < 32; ++il) {
        const int i = 32 * u + il;
        if (i >= n) break;
        const double xi = __shfl_sync(0xffffffffu, x[u], il) * rd[i];
        if (lane == il) x[u] = xi;
#pragma unroll
        for (int v = u; v < TRSM_R; ++v) {
          const int k = lane + 32 * v;
          if (k > i && k < n) x[v] = fma(-Ls[k + i * ld], xi, x[v]);
        }
      }
    }
  } else {
#pragma unroll
    for (int u = TRSM_R - 1; u >= 0; --u) {
      for (int il = 31; il >= 0; --il) {
        const int i = 32 * u + il;
        if (i >= n) continue;
        const double xi = __shfl_sync(0xffffffffu, x[u], il) * rd[i];
        if (lane == il) x[u] = xi;
#pragma unroll
        for (int v = 0; v <= u; ++v) {
          const int k = lane + 32 * v;
          if (k < i) x[v] = fma(-Ls[i + k * ld], xi, x[v]);  // (L')(k, i) = L(i, k)
        }
      }
    }
  }
#pragma unroll
  for (int u = 0; u < TRSM_R; ++u) {
    const int i = lane + 32 * u;
    if (i < n) X[i + (size_t)col * ldx] = x[u];
  }
}

// ---- small FP64 GEMM: C = alpha op(A) op(B) + beta C, one thread per output entry -----------------
// 32-thread CTAs (one output column segment each, so the B loads are broadcasts and the A loads
// coalesced for op(A) = A) spread the FP64 work over many SMs; K is consumed in chunks of GS_K with all
// of a chunk's loads issued before its FMAs, so a 64-deep product waits for two rounds of L2 latency.
constexpr int GS_K = 32;
struct GemmSmall {
  int M, N, K;
  double alpha;
  const double* A;
  int lda, tA;
  const double* B;
  int ldb, tB;
  double beta;
  double* C;
  int ldc;
};
__device__ __forceinline__ void gemm_small_entry(const GemmSmall& g, int i, int j);

// up to two independent products in one launch (blockIdx.z selects), so that the ones that do not
// depend on each other share a launch
__global__ void __launch_bounds__(32) k_gemm_small2_f64(GemmSmall g0, GemmSmall g1) {
  const GemmSmall& g = blockIdx.z ? g1 : g0;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y;
  if (i >= g.M || j >= g.N) return;
  gemm_small_entry(g, i, j);
}

__device__ __forceinline__ void gemm_small_entry(const GemmSmall& g, int i, int j) {
  const int K = g.K, lda = g.lda, ldb = g.ldb, tA = g.tA, tB = g.tB;
  const double* __restrict__ A = g.A;
  const double* __restrict__ B = g.B;
  double s0 = 0.0, s1 = 0.0;
  for (int k0 = 0; k0 < K; k0 += GS_K) {
    double a[GS_K], b[GS_K];
#pragma unroll
    for (int u = 0; u < GS_K; ++u) {
      const int k = k0 + u;
      a[u] = (k < K) ? (tA ? A[k + (size_t)i * lda] : A[i + (size_t)k * lda]) : 0.0;
      b[u] = (k < K) ? (tB ? B[j + (size_t)k * ldb] : B[k + (size_t)j * ldb]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < GS_K; u += 2) {
      s0 = fma(a[u], b[u], s0);
      s1 = fma(a[u + 1], b[u + 1], s1);
    }
  }
  const double s = s0 + s1;
  g.C[i + (size_t)j * g.ldc] = (g.beta == 0.0) ? g.alpha * s : fma(g.alpha, s, g.beta * g.C[i + (size_t)j * g.ldc]);
}

__global__ void __launch_bounds__(32) k_gemm_small_f64(int M, int N, int K, double alpha, const double* __restrict__ A,
                                                       int lda, int tA, const double* __restrict__ B, int ldb, int tB,
                                                       double beta, double* __restrict__ C, int ldc) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y;
  if (i >= M || j >= N) return;
  double s0 = 0.0, s1 = 0.0;
  for (int k0 = 0; k0 < K; k0 += GS_K) {
    double a[GS_K], b[GS_K];
#pragma unroll
    for (int u = 0; u < GS_K; ++u) {
      const int k = k0 + u;
      a[u] = (k < K) ? (tA ? A[k + (size_t)i * lda] : A[i + (size_t)k * lda]) : 0.0;
      b[u] = (k < K) ? (tB ? B[j + (size_t)k * ldb] : B[k + (size_t)j * ldb]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < GS_K; u += 2) {
      s0 = fma(a[u], b[u], s0);
      s1 = fma(a[u + 1], b[u + 1], s1);
    }
  }
  const double s = s0 + s1;
  C[i + (size_t)j * ldc] = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * C[i + (size_t)j * ldc]);
}

// ---- 3. FP32 cyclic Jacobi (round-robin parallel ordering), one CTA --------------------------------
__device__ __forceinline__ int rr_idx(int i, int r, int N) { return i == 0 ? 0 : ((i - 1 + r) % (N - 1)) + 1; }

// Each round applies n/2 disjoint rotations J.  C <- J' C J is done block-wise: the 2 x 2 block of C
// on the rows of pair a and the columns of pair b depends only on that block, so one pass updates all
// blocks (and W <- W J) between two barriers.
__global__ void __launch_bounds__(512) k_jacobi_f32(int n, const double* __restrict__ Cin, int ldc,
                                                    double* __restrict__ Wout, double* __restrict__ lam) {
  extern __shared__ float smf[];
  const int ld = n + 1;  // padded: row-wise accesses at stride ld spread over the 32 banks
  float* C = smf;
  float* W = smf + n * ld;
  __shared__ float s_c[64], s_s[64];
  __shared__ int s_p[64], s_q[64];  // the pair's indices (q may be n: the padding index for odd n)
  __shared__ float s_red[32];
  __shared__ int s_stop;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < n * n; e += nt) {
    const int i = e % n, j = e / n;
    C[i + j * ld] = (float)(0.5 * (Cin[i + (size_t)j * ldc] + Cin[j + (size_t)i * ldc]));
    W[i + j * ld] = (i == j) ? 1.f : 0.f;
  }
  __syncthreads();
  const int N = n + (n & 1), npair = N / 2;
  for (int sweep = 0; sweep < 10 && n > 1; ++sweep) {
    float off = 0.f, tot = 0.f;
    for (int e = tid; e < n * n; e += nt) {
      const int i = e % n, j = e / n;
      const float v = C[i + j * ld] * C[i + j * ld];
      tot += v;
      if (i != j) off += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_down_sync(0xffffffffu, off, o);
      tot += __shfl_down_sync(0xffffffffu, tot, o);
    }
    if ((tid & 31) == 0) s_red[tid >> 5] = off;
    __syncthreads();
    float offs = 0.f;
    if (tid == 0)
      for (int w = 0; w < (nt >> 5); ++w) offs += s_red[w];
    __syncthreads();
    if ((tid & 31) == 0) s_red[tid >> 5] = tot;
    __syncthreads();
    if (tid == 0) {
      float tots = 0.f;
      for (int w = 0; w < (nt >> 5); ++w) tots += s_red[w];
      // off(C) <= 3e-5 ||C|| (FP32 stalls near n eps ||C||); the FP64 refinement does the rest
      s_stop = (offs <= 1e-9f * tots) ? 1 : 0;
    }
    __syncthreads();
    if (s_stop) break;
    for (int r = 0; r < N - 1; ++r) {
      for (int k = tid; k < npair; k += nt) {
        int p = rr_idx(k, r, N), q = rr_idx(N - 1 - k, r, N);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        float c = 1.f, s = 0.f;
        if (q < n) {
          const float apq = C[p + q * ld];
          if (apq != 0.f) {
            const float tau = (C[q + q * ld] - C[p + p * ld]) / (2.f * apq);
            const float t = (tau >= 0.f) ? 1.f / (tau + sqrtf(1.f + tau * tau)) : -1.f / (-tau + sqrtf(1.f + tau * tau));
            c = rsqrtf(1.f + t * t);
            s = t * c;
          }
        }
        s_p[k] = p;
        s_q[k] = q;
        s_c[k] = c;
        s_s[k] = s;
      }
      __syncthreads();
      // rows of pair a rotated by J_a', then columns of pair b by J_b; diagonal blocks lose their
      // off-diagonal pair entries exactly
      for (int e = tid; e < npair * npair; e += nt) {
        const int ka = e % npair, kb = e / npair;
        const int pa = s_p[ka], qa = s_q[ka], pb = s_p[kb], qb = s_q[kb];
        const float ca = s_c[ka], sa = s_s[ka], cb = s_c[kb], sb = s_s[kb];
        if (sa == 0.f && sb == 0.f) continue;
        const bool qav = qa < n, qbv = qb < n;
        const float x11 = C[pa + pb * ld];
        const float x12 = qbv ? C[pa + qb * ld] : 0.f;
        const float x21 = qav ? C[qa + pb * ld] : 0.f;
        const float x22 = (qav && qbv) ? C[qa + qb * ld] : 0.f;
        const float y11 = ca * x11 - sa * x21, y12 = ca * x12 - sa * x22;
        const float y21 = sa * x11 + ca * x21, y22 = sa * x12 + ca * x22;
        float z11 = cb * y11 - sb * y12, z12 = sb * y11 + cb * y12;
        float z21 = cb * y21 - sb * y22, z22 = sb * y21 + cb * y22;
        if (ka == kb) {
          z12 = 0.f;
          z21 = 0.f;
        }
        C[pa + pb * ld] = z11;
        if (qbv) C[pa + qb * ld] = z12;
        if (qav) C[qa + pb * ld] = z21;
        if (qav && qbv) C[qa + qb * ld] = z22;
      }
      for (int e = tid; e < npair * n; e += nt) {
        const int k = e / n, i = e % n;
        const float s = s_s[k];
        if (s == 0.f) continue;
        const int p = s_p[k], q = s_q[k];
        const float c = s_c[k];
        const float ap = W[i + p * ld], aq = W[i + q * ld];
        W[i + p * ld] = c * ap - s * aq;
        W[i + q * ld] = s * ap + c * aq;
      }
      __syncthreads();
    }
  }
  for (int e = tid; e < n * n; e += nt) Wout[e] = (double)W[(e % n) + (e / n) * ld];
  for (int i = tid; i < n; i += nt) lam[i] = (double)C[i + i * ld];
}

// ---- 3b. FP32 one-sided (Hestenes) Jacobi on the columns of G: G V = U Sigma ------------------------
// The SVD form's starting vectors: the right singular vectors of C directly (better conditioned than
// an eigen-solve of C'C).  Round-robin pairs: the pair's dot product reduced with shuffles (the squared
// column norms are kept in shared memory, updated with each rotation and recomputed every sweep), then
// the two columns of G and of V rotated; one barrier per round.  A pair rotates when
// |g_p . g_q| > 3e-5 ||g_p|| ||g_q|| (above FP32 rounding noise); sweeps stop when no pair rotates (at
// most 12).
// Round-robin partner of position i in round r for N positions (position 0 fixed), without a division.
__device__ __forceinline__ int rr_pos(int i, int r, int N) {
  if (i == 0) return 0;
  int x = i - 1 + r;
  if (x >= N - 1) x -= N - 1;
  return x + 1;
}

// Eight lanes per column pair (each lane holds rows sl, sl + 8, ... of both columns in registers), four
// pairs per warp: the kernel is bound by instruction issue, and the per-pair scalar work (the angle, the
// threshold test, the norm update) is then shared by four pairs in one warp instruction stream.  The
// angle need not be exact, only the rotation orthogonal: c = 1/sqrt(1 + t^2) is refined by one Newton
// step so that c^2 + s^2 = 1 to rounding (the accumulated V stays orthogonal to FP32 accuracy).
// Column stride of G and V in shared memory: ld = 8 (mod 32), so that the columns of the four pairs a
// warp handles (adjacent positions of the round-robin order, mostly adjacent column indices) fall in
// disjoint groups of eight banks.
__host__ __device__ __forceinline__ int j1_ld(int n) { return n + (40 - n % 32) % 32; }

template <int R>  // rows per lane: n <= 8 R
__global__ void __launch_bounds__(256, 1) k_jacobi1_f32(int n, const double* __restrict__ Gin, int ldg, int trans,
                                                     double* __restrict__ Vout) {
  extern __shared__ float sm1[];
  const int ld = j1_ld(n);
  float* G = sm1;
  float* V = sm1 + n * ld;
  __shared__ int s_any;
  __shared__ float nrm[8 * R];  // squared column norms, updated with each rotation, recomputed per sweep
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e0 = tid; e0 < n * n; e0 += 16 * nt) {  // 16 loads per thread in flight
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * nt;
      const int j = e / n, i = e - j * n;
      v[u] = (e < n * n) ? (trans ? Gin[j + (size_t)i * ldg] : Gin[i + (size_t)j * ldg]) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * nt;
      const int j = e / n, i = e - j * n;
      if (e < n * n) {
        G[i + j * ld] = (float)v[u];
        V[i + j * ld] = (i == j) ? 1.f : 0.f;
      }
    }
  }
  const int N = n + (n & 1), npair = N / 2;
  const int grp = tid >> 3, sl = tid & 7, ngrp = nt >> 3;
  for (int sweep = 0; sweep < 12 && n > 1; ++sweep) {
    if (tid == 0) s_any = 0;
    __syncthreads();
    for (int jb = 0; jb < n; jb += ngrp) {  // uniform trip count: the shuffles need whole warps
      const int j = jb + grp;
      float s2 = 0.f;
#pragma unroll
      for (int u = 0; u < R; ++u) {
        const int i = sl + 8 * u;
        const float x = (j < n && i < n) ? G[i + j * ld] : 0.f;
        s2 = fmaf(x, x, s2);
      }
      s2 += __shfl_xor_sync(0xffffffffu, s2, 4);
      s2 += __shfl_xor_sync(0xffffffffu, s2, 2);
      s2 += __shfl_xor_sync(0xffffffffu, s2, 1);
      if (sl == 0 && j < n) nrm[j] = s2;
    }
    __syncthreads();
    int any = 0;
    for (int r = 0; r < N - 1; ++r) {
      for (int kb = 0; kb < npair; kb += ngrp) {
        const int k = kb + grp;
        int p = rr_pos(k, r, N), q = rr_pos(N - 1 - k, r, N);
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        const bool live = k < npair && q < n;
        float gp[R], gq[R];
        float g = 0.f;
#pragma unroll
        for (int u = 0; u < R; ++u) {
          const int i = sl + 8 * u;
          const bool in = live && i < n;
          gp[u] = in ? G[i + p * ld] : 0.f;
          gq[u] = in ? G[i + q * ld] : 0.f;
          g = fmaf(gp[u], gq[u], g);
        }
        g += __shfl_xor_sync(0xffffffffu, g, 4);
        g += __shfl_xor_sync(0xffffffffu, g, 2);
        g += __shfl_xor_sync(0xffffffffu, g, 1);
        if (!live || g == 0.f) continue;
        const float a = nrm[p], b = nrm[q];
        if (fabsf(g) * rsqrtf(a) * rsqrtf(b) > 3e-5f) {
          any = 1;
          const float zeta = __fdividef(b - a, 2.f * g);
          const float z1 = fmaf(zeta, zeta, 1.f);
          const float t = __fdividef(copysignf(1.f, zeta), fabsf(zeta) + z1 * rsqrtf(z1));
          const float x = fmaf(t, t, 1.f);
          float c = rsqrtf(x);
          c = c * fmaf(-0.5f * x * c, c, 1.5f);  // Newton step for 1/sqrt(x)
          const float sn = t * c;
#pragma unroll
          for (int u = 0; u < R; ++u) {
            const int i = sl + 8 * u;
            if (i < n) {
              G[i + p * ld] = c * gp[u] - sn * gq[u];
              G[i + q * ld] = sn * gp[u] + c * gq[u];
              const float vp = V[i + p * ld], vq = V[i + q * ld];
              V[i + p * ld] = c * vp - sn * vq;
              V[i + q * ld] = sn * vp + c * vq;
            }
          }
          if (sl == 0) {  // norms after the rotation (exact arithmetic; drift is reset each sweep)
            const float cc = c * c, ss = sn * sn, cs2 = 2.f * c * sn * g;
            nrm[p] = cc * a + ss * b - cs2;
            nrm[q] = ss * a + cc * b + cs2;
          }
        }
      }
      __syncthreads();
    }
    if (any) s_any = 1;
    __syncthreads();
    if (!s_any) break;
  }
  __syncthreads();
  for (int j = tid >> 5; j < n; j += nt >> 5)
    for (int i = tid & 31; i < n; i += 32) Vout[i + (size_t)j * n] = (double)V[i + j * ld];
}

// ---- 4. Ogita-Aishima correction: from P = W'W and T = W'CW build lambda and F = I + E ------------
// One thread per entry of F over a grid of CTAs; every CTA forms the n Rayleigh quotients itself.
__global__ void __launch_bounds__(256) k_oa_correction(int n, const double* __restrict__ P, const double* __restrict__ T,
                                                       double* __restrict__ lam, double* __restrict__ F,
                                                       double rel_cluster) {
  extern __shared__ double sl[];
  __shared__ double s_scale;
  for (int i = threadIdx.x; i < n; i += blockDim.x) sl[i] = T[i + (size_t)i * n] / P[i + (size_t)i * n];
  __syncthreads();
  if (threadIdx.x < 32) {
    long long kmax = -1;
    for (int i = threadIdx.x; i < n; i += 32) kmax = max(kmax, amax_key(sl[i]));
    for (int o = 16; o > 0; o >>= 1) kmax = max(kmax, (long long)__shfl_xor_sync(0xffffffffu, kmax, o));
    if (threadIdx.x == 0) {
      const double m = (kmax > 1) ? __longlong_as_double(kmax - 1) : 0.0;
      s_scale = (m > 0 ? m : 1.0) * rel_cluster;
    }
  }
  __syncthreads();
  const double delta = s_scale;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n * n) {
    const int i = e % n, j = e / n;
    const double r = (i == j ? 1.0 : 0.0) - P[e];
    double f;
    if (i == j) {
      f = 1.0 + 0.5 * r;
    } else {
      const double gap = sl[j] - sl[i];
      f = (fabs(gap) > delta) ? (T[e] + sl[j] * r) / gap : 0.5 * r;
    }
    F[e] = f;
  }
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) lam[i] = sl[i];
}

// ---- 5. sort descending, gather columns --------------------------------------------------------------
// Ranks from order-preserving integer keys of the doubles (no FP64 compares); then a parallel gather.
__device__ __forceinline__ long long order_key(double x) {
  const long long b = __double_as_longlong(x);
  return (b < 0) ? (b ^ 0x7fffffffffffffffLL) : b;
}
__global__ void __launch_bounds__(256) k_sort_desc(int n, const double* __restrict__ lam, const double* __restrict__ W,
                                                   double* __restrict__ lam_out, double* __restrict__ Wout) {
  __shared__ long long s_key[256];
  __shared__ int s_rank[256];
  for (int i = threadIdx.x; i < n; i += blockDim.x) s_key[i] = order_key(lam[i]);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long ki = s_key[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const long long kj = s_key[j];
      rank += (kj > ki || (kj == ki && j < i)) ? 1 : 0;
    }
    s_rank[i] = rank;
    lam_out[rank] = lam[i];
  }
  __syncthreads();
  if (!W) return;  // values only
  for (int e0 = threadIdx.x; e0 < n * n; e0 += 16 * blockDim.x) {  // 16 loads per thread in flight
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * blockDim.x;
      v[u] = (e < n * n) ? W[e] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = e0 + u * blockDim.x;
      const int i = e / n, r = e - i * n;
      if (e < n * n) Wout[r + (size_t)s_rank[i] * n] = v[u];
    }
  }
}

// Y(:,j) = C W(:,j) / sigma_j (sigma_j = sqrt(max(lam_j, 0))), then the sigmas themselves
__global__ void k_svd_left(int n, const double* __restrict__ CW, const double* __restrict__ lam, double* __restrict__ Y,
                           double* __restrict__ sig) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n * n) {
    const int j = e / n;
    const double s = sqrt(fmax(lam[j], 0.0));
    Y[e] = (s > 0.0) ? CW[e] / s : 0.0;
    if (e % n == 0) sig[j] = s;
  }
}

// ---- host helpers ----------------------------------------------------------------------------------
static int gemm_small(ofrr_ctx* ctx, int M, int N, int K, double alpha, const double* A, int lda, int tA,
                      const double* B, int ldb, int tB, double beta, double* C, int ldc) {
  if (M <= 0 || N <= 0) return OFRR_SUCCESS;
  k_gemm_small_f64<<<dim3((unsigned)((M + 31) / 32), (unsigned)N), 32, 0, ctx->stream>>>(M, N, K, alpha, A, lda, tA, B,
                                                                                       ldb, tB, beta, C, ldc);
  OFRR_LAUNCHED(ctx, "k_gemm_small_f64");
  return OFRR_SUCCESS;
}

static int gemm_small2(ofrr_ctx* ctx, const GemmSmall& g0, const GemmSmall& g1) {
  const int M = std::max(g0.M, g1.M), N = std::max(g0.N, g1.N);
  if (M <= 0 || N <= 0) return OFRR_SUCCESS;
  k_gemm_small2_f64<<<dim3((unsigned)((M + 31) / 32), (unsigned)N, 2), 32, 0, ctx->stream>>>(g0, g1);
  OFRR_LAUNCHED(ctx, "k_gemm_small2_f64");
  return OFRR_SUCCESS;
}

template <int R>
static int trsm_r(ofrr_ctx* ctx, int n, int nrhs, const double* L, const double* B, int ldb, int transB, double* X,
                  int upper, const double* L2, const double* B2, double* X2) {
  const size_t smem = ((size_t)n * (n + 1) + (size_t)n) * sizeof(double);
  OFRR_TRY(allow_smem(k_trsm_f64<R>));
  const dim3 grid((unsigned)((nrhs + 3) / 4), L2 ? 2u : 1u);
  k_trsm_f64<R><<<grid, 128, smem, ctx->stream>>>(n, nrhs, L, n, B, ldb, transB, X, n, upper, L2, B2, X2);
  OFRR_LAUNCHED(ctx, "k_trsm_f64");
  return OFRR_SUCCESS;
}

// X = L^-1 B (upper == 0) or L^-T B (upper == 1); with L2 set, X2 = (same op of L2) B2 in the same launch
static int trsm(ofrr_ctx* ctx, int n, int nrhs, const double* L, const double* B, int ldb, int transB, double* X,
                int upper, const double* L2 = nullptr, const double* B2 = nullptr, double* X2 = nullptr) {
  if (n <= 32) return trsm_r<1>(ctx, n, nrhs, L, B, ldb, transB, X, upper, L2, B2, X2);
  if (n <= 64) return trsm_r<2>(ctx, n, nrhs, L, B, ldb, transB, X, upper, L2, B2, X2);
  if (n <= 96) return trsm_r<3>(ctx, n, nrhs, L, B, ldb, transB, X, upper, L2, B2, X2);
  return trsm_r<4>(ctx, n, nrhs, L, B, ldb, transB, X, upper, L2, B2, X2);
}

static int chol(ofrr_ctx* ctx, int n, int count, const double* const* Ms_host, int ldm, double tau,
                double* const* Ls_host) {
  int st = OFRR_SUCCESS;
  const double** Md = ws_get<const double*>(ctx, 4, &st);
  if (!Md) return st;
  double** Ld = (double**)(Md + 2);
  const void* hp[4] = {Ms_host[0], count > 1 ? Ms_host[1] : Ms_host[0], Ls_host[0], count > 1 ? Ls_host[1] : Ls_host[0]};
  OFRR_CUDA(cudaMemcpyAsync(Md, hp, sizeof(hp), cudaMemcpyHostToDevice, ctx->stream));
  const size_t smem = (size_t)n * n * sizeof(double);
  OFRR_TRY(allow_smem(k_chol_f64));
  k_chol_f64<<<count, 256, smem, ctx->stream>>>(n, Md, ldm, tau, Ld, ctx->dev_flags + 1);
  OFRR_LAUNCHED(ctx, "k_chol_f64");
  return OFRR_SUCCESS;
}

// Ogita-Aishima refinement of approximate eigenvectors W0 (n x n, overwritten) of a symmetric C
// (FP64): W (orthonormal, columns sorted by descending eigenvalue) and lam (descending)
static int eig_refine(ofrr_ctx* ctx, int n, const double* C, double* W0, double* W, double* lam, int steps) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *W1 = ws_get<double>(ctx, (size_t)n * n, &st), *P = ws_get<double>(ctx, (size_t)n * n, &st),
         *CW = ws_get<double>(ctx, (size_t)n * n, &st), *T = ws_get<double>(ctx, (size_t)n * n, &st),
         *F = ws_get<double>(ctx, (size_t)n * n, &st), *l0 = ws_get<double>(ctx, (size_t)n, &st);
  if (!W1 || !P || !CW || !T || !F || !l0) return st;
  double* Wc = W0;
  double* Wn = W1;
  for (int it = 0; it < steps; ++it) {
    OFRR_TRY(gemm_small2(ctx, GemmSmall{n, n, n, 1.0, Wc, n, 1, Wc, n, 0, 0.0, P, n},     // P = W'W
                         GemmSmall{n, n, n, 1.0, C, n, 0, Wc, n, 0, 0.0, CW, n}));     // CW
    OFRR_TRY(gemm_small(ctx, n, n, n, 1.0, Wc, n, 1, CW, n, 0, 0.0, T, n));   // T = W'CW
    k_oa_correction<<<(n * n + 255) / 256, 256, n * sizeof(double), ctx->stream>>>(n, P, T, l0, F, 1e-5);
    OFRR_LAUNCHED(ctx, "k_oa_correction");
    OFRR_TRY(gemm_small(ctx, n, n, n, 1.0, Wc, n, 0, F, n, 0, 0.0, Wn, n));   // W <- W (I + E)
    std::swap(Wc, Wn);
  }
  // final Rayleigh quotients with the refined vectors
  OFRR_TRY(gemm_small2(ctx, GemmSmall{n, n, n, 1.0, Wc, n, 1, Wc, n, 0, 0.0, P, n},
                       GemmSmall{n, n, n, 1.0, C, n, 0, Wc, n, 0, 0.0, CW, n}));
  OFRR_TRY(gemm_small(ctx, n, n, n, 1.0, Wc, n, 1, CW, n, 0, 0.0, T, n));
  k_oa_correction<<<(n * n + 255) / 256, 256, n * sizeof(double), ctx->stream>>>(n, P, T, l0, F, 1e-5);
  OFRR_LAUNCHED(ctx, "k_oa_correction");
  k_sort_desc<<<1, 256, 0, ctx->stream>>>(n, l0, Wc, lam, W);
  OFRR_LAUNCHED(ctx, "k_sort_desc");
  return OFRR_SUCCESS;
}

// eigen-decomposition of a symmetric C (n x n, FP64): W (orthonormal, columns sorted by descending
// eigenvalue) and lam (descending); FP32 two-sided Jacobi, then the FP64 refinement
static int sym_eig_refined(ofrr_ctx* ctx, int n, const double* C, double* W, double* lam, int steps) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *W0 = ws_get<double>(ctx, (size_t)n * n, &st), *l0 = ws_get<double>(ctx, (size_t)n, &st);
  if (!W0 || !l0) return st;
  const size_t smem = (size_t)2 * n * (n + 1) * sizeof(float);
  OFRR_TRY(allow_smem(k_jacobi_f32));
  k_jacobi_f32<<<1, 512, smem, ctx->stream>>>(n, C, n, W0, l0);
  OFRR_LAUNCHED(ctx, "k_jacobi_f32");
  return eig_refine(ctx, n, C, W0, W, lam, steps);
}

// unit 2-norm columns (n x n, ld n), one warp per column
__global__ void k_unit_cols(int n, double* __restrict__ U) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= n) return;
  double* u = U + (size_t)w * n;
  double s = 0.0;
  for (int i = lane; i < n; i += 32) s = fma(u[i], u[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const double inv = (s > 0.0) ? 1.0 / sqrt(s) : 0.0;
  for (int i = lane; i < n; i += 32) u[i] *= inv;
}

// ---- invariant subspace of a nonsymmetric pencil (the thick restart of the Krylov eigensolver) ----
// The restart keeps span{Ritz vectors of the wanted Ritz values}; for a non-normal projected matrix two
// close Ritz values can have nearly parallel eigenvectors, whose span then carries rounding noise of the
// size eps / angle.  The invariant subspace itself is well conditioned when the wanted values are
// separated from the others, and the matrix sign function gives it without eigenvectors:
// S = sign(C - sigma I) (Newton, X <- (mu X + (mu X)^-1) / 2 with determinant scaling mu), P = (I + S) / 2
// projects onto the eigenvalues with real part above sigma [N. J. Higham, Functions of Matrices,
// SIAM 2008, ch. 5].  One CTA, FP64; Gauss-Jordan inversion with partial pivoting in shared memory.
constexpr int kSignMaxN = 96;

template <class T>
__global__ void __launch_bounds__(256) k_sign_newton(int n, double* __restrict__ Xg, int maxit, double tol,
                                                     int* __restrict__ flag) {
  extern __shared__ unsigned char sgn_raw[];
  T* X = reinterpret_cast<T*>(sgn_raw);  // n x n, column-major
  T* Y = X + (size_t)n * n;              // its inverse (Gauss-Jordan in place)
  __shared__ int piv[kSignMaxN];
  __shared__ T s_col[kSignMaxN];
  __shared__ int s_p;
  __shared__ double s_logdet, s_num, s_den;
  const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31;
  const int nn = n * n;
  if (*flag) return;  // an earlier stage met a singular matrix
  for (int e = tid; e < nn; e += nthr) X[e] = (T)Xg[e];
  __syncthreads();
  for (int it = 0; it < maxit; ++it) {
    for (int e = tid; e < nn; e += nthr) Y[e] = X[e];
    if (tid == 0) s_logdet = 0.0;
    __syncthreads();
    bool singular = false;
    for (int k = 0; k < n; ++k) {
      if (tid < 32) {  // pivot: first largest |Y(i, k)|, i >= k
        T best = T(-1);
        int bi = k;
        for (int i = k + lane; i < n; i += 32) {
          const T a = fabs(Y[i + (size_t)k * n]);
          if (a > best) {
            best = a;
            bi = i;
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const T ob = __shfl_down_sync(0xffffffffu, best, off);
          const int oi = __shfl_down_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
          }
        }
        if (lane == 0) s_p = bi;
      }
      __syncthreads();
      const int p = s_p;
      if (p != k)
        for (int j = tid; j < n; j += nthr) {
          const T t = Y[k + (size_t)j * n];
          Y[k + (size_t)j * n] = Y[p + (size_t)j * n];
          Y[p + (size_t)j * n] = t;
        }
      if (tid == 0) piv[k] = p;
      __syncthreads();
      const T d = Y[k + (size_t)k * n];
      if (!(fabs(d) > T(0))) {  // zero or NaN pivot: every thread sees the same value
        singular = true;
        break;
      }
      const T dinv = T(1) / d;
      if (tid == 0) s_logdet += log(fabs((double)d));
      for (int i = tid; i < n; i += nthr) s_col[i] = (i == k) ? T(0) : Y[i + (size_t)k * n];
      __syncthreads();
      for (int j = tid; j < n; j += nthr) Y[k + (size_t)j * n] = (j == k) ? dinv : Y[k + (size_t)j * n] * dinv;
      for (int i = tid; i < n; i += nthr)
        if (i != k) Y[i + (size_t)k * n] = T(0);
      __syncthreads();
      for (int e = tid; e < nn; e += nthr) {
        const int i = e % n, j = e / n;
        if (i != k) Y[e] -= s_col[i] * Y[k + (size_t)j * n];
      }
      __syncthreads();
    }
    if (singular) {
      if (tid == 0) *flag = 1;
      return;
    }
    for (int k = n - 1; k >= 0; --k) {  // undo the row interchanges as column interchanges of the inverse
      const int p = piv[k];
      if (p != k)
        for (int i = tid; i < n; i += nthr) {
          const T t = Y[i + (size_t)k * n];
          Y[i + (size_t)k * n] = Y[i + (size_t)p * n];
          Y[i + (size_t)p * n] = t;
        }
      __syncthreads();
    }
    const double mu = (it < 4) ? exp(-s_logdet / n) : 1.0;  // determinant scaling in the first steps
    if (tid == 0) {
      s_num = 0.0;
      s_den = 0.0;
    }
    __syncthreads();
    double num = 0.0, den = 0.0;
    for (int e = tid; e < nn; e += nthr) {
      const T xn = (T)(0.5 * (mu * (double)X[e] + (double)Y[e] / mu));
      num += ((double)xn - (double)X[e]) * ((double)xn - (double)X[e]);
      den += (double)xn * (double)xn;
      X[e] = xn;
    }
    atomicAdd(&s_num, num);
    atomicAdd(&s_den, den);
    __syncthreads();
    const bool done = s_num <= tol * tol * s_den;
    __syncthreads();
    if (done && it >= 1) break;
  }
  for (int e = tid; e < nn; e += nthr) Xg[e] = (double)X[e];
}

__global__ void k_shift_copy(int n, const double* __restrict__ C, double sigma, double* __restrict__ X) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x)
    X[e] = C[e] - ((e % n == e / n) ? sigma : 0.0);
}

// Q (n x p) = orthonormal basis of range((I + S) / 2): the projector applied to a fixed pseudo-random
// block (splitmix64 hashes), then modified Gram-Schmidt twice (FP64, one CTA)
__global__ void __launch_bounds__(256) k_proj_basis(int n, int p, const double* __restrict__ S, double* __restrict__ Q) {
  extern __shared__ double pb[];  // n x p
  __shared__ double s_red[8];
  __shared__ double s_dot;
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int e = tid; e < n * p; e += nthr) {
    const int i = e % n, c = e / n;
    double acc = 0.0;
    for (int k = 0; k < n; ++k) {
      unsigned long long h = 0x9e3779b97f4a7c15ULL * (unsigned long long)(k + 1) + 0xbf58476d1ce4e5b9ULL * (c + 1);
      h ^= h >> 31;
      h *= 0x94d049bb133111ebULL;
      h ^= h >> 29;
      const double om = (double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5;
      const double pik = 0.5 * (S[i + (size_t)k * n] + ((i == k) ? 1.0 : 0.0));
      acc += pik * om;
    }
    pb[e] = acc;
  }
  __syncthreads();
  auto block_sum = [&](double v) -> double {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((tid & 31) == 0) s_red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < (nthr + 31) / 32; ++w) t += s_red[w];
      s_dot = t;
    }
    __syncthreads();
    const double r = s_dot;
    __syncthreads();
    return r;
  };
  for (int c = 0; c < p; ++c) {
    double* qc = pb + (size_t)c * n;
    for (int pass = 0; pass < 2; ++pass) {
      for (int c2 = 0; c2 < c; ++c2) {
        const double* q2 = pb + (size_t)c2 * n;
        double v = 0.0;
        for (int i = tid; i < n; i += nthr) v += q2[i] * qc[i];
        const double dt = block_sum(v);
        for (int i = tid; i < n; i += nthr) qc[i] -= dt * q2[i];
        __syncthreads();
      }
    }
    double v = 0.0;
    for (int i = tid; i < n; i += nthr) v += qc[i] * qc[i];
    const double t = block_sum(v);
    const double sc = (t > 0.0) ? 1.0 / sqrt(t) : 0.0;
    for (int i = tid; i < n; i += nthr) qc[i] *= sc;
    __syncthreads();
  }
  for (int e = tid; e < n * p; e += nthr) Q[e] = pb[e];
}

// Y (n x p, ld n) spanning the invariant subspace of the pencil (G, M) for its p eigenvalues with real
// part above sigma: C = L^-1 G L^-T (M = L L'), Q = orth((I + sign(C - sigma I)) / 2), Y = L^-T Q.
// Returns OFRR_ERR_SINGULAR_MATRIX when a Newton step meets a singular matrix (sigma an eigenvalue).
int invariant_subspace_nonsym(ofrr_ctx* ctx, int n, const double* G, const double* M, double sigma, int p,
                              double* Y) {
  if (n <= 0 || p <= 0) return OFRR_SUCCESS;
  if (n > kSignMaxN || p > n) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *L = ws_get<double>(ctx, (size_t)n * n, &st), *Z = ws_get<double>(ctx, (size_t)n * n, &st),
         *C = ws_get<double>(ctx, (size_t)n * n, &st), *X = ws_get<double>(ctx, (size_t)n * n, &st),
         *Q = ws_get<double>(ctx, (size_t)n * p, &st);
  int* flag = ws_get<int>(ctx, 1, &st);
  if (!L || !Z || !C || !X || !Q || !flag) return st;
  const double* Ms[1] = {M};
  double* Ls[1] = {L};
  OFRR_TRY(chol(ctx, n, 1, Ms, n, 0.0, Ls));
  OFRR_TRY(trsm(ctx, n, n, L, G, n, 1, Z, 0));  // Z = L^-1 G'
  OFRR_TRY(trsm(ctx, n, n, L, Z, n, 1, C, 0));  // C = L^-1 Z' = L^-1 G L^-T
  k_shift_copy<<<(n * n + 255) / 256, 256, 0, ctx->stream>>>(n, C, sigma, X);
  OFRR_LAUNCHED(ctx, "k_shift_copy");
  OFRR_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
  // FP64 throughout: the iteration converges to the sign of the matrix it is given, so rounding errors of
  // a lower-precision start are not corrected by later FP64 steps (they change the matrix, not the path)
  const size_t sm64 = 2 * (size_t)n * n * sizeof(double);
  OFRR_TRY(allow_smem(k_sign_newton<double>));
  k_sign_newton<double><<<1, 256, sm64, ctx->stream>>>(n, X, 80, 1e-14, flag);
  OFRR_LAUNCHED(ctx, "k_sign_newton");
  OFRR_TRY(allow_smem(k_proj_basis));
  k_proj_basis<<<1, 256, (size_t)n * p * sizeof(double), ctx->stream>>>(n, p, X, Q);
  OFRR_LAUNCHED(ctx, "k_proj_basis");
  OFRR_TRY(trsm(ctx, n, p, L, Q, n, 0, Y, 1));  // Y = L^-T Q
  int hf = 0;
  OFRR_CUDA(cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  return hf ? OFRR_ERR_SINGULAR_MATRIX : OFRR_SUCCESS;
}

// unit 2-norm columns of U (n x k, ld n), one warp per column
__global__ void k_unit_cols_nk(int n, int k, double* __restrict__ U) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= k) return;
  double* u = U + (size_t)w * n;
  double s = 0.0;
  for (int i = lane; i < n; i += 32) s = fma(u[i], u[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const double inv = (s > 0.0) ? 1.0 / sqrt(s) : 0.0;
  for (int i = lane; i < n; i += 32) u[i] *= inv;
}

// The k leading Ritz pairs of the pencil (G, M) from a basis Y (n x p, ld n) of its invariant subspace for
// the p eigenvalues of largest real part: the restricted pencil (Y'GY, Y'MY) has exactly those
// eigenvalues, so its p x p FP64 Hessenberg-QR replaces the one of the whole n x n pencil (the QR's cost
// grows as the cube of the order, and on one warp in FP64 it was the largest part of a restart).
// lam: the k leading values (real parts, descending; the imaginary part for the second member of a
// complex pair, as geig_nonsym with pair_imag); U (n x k, ld n): unit 2-norm coefficient vectors.
int ritz_from_invariant(ofrr_ctx* ctx, int n, const double* G, const double* M, const double* Y, int p, int k,
                        double* lam, double* U) {
  if (k <= 0 || p <= 0) return OFRR_SUCCESS;
  if (k > p || p > n || n > 128) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *GY = ws_get<double>(ctx, (size_t)n * p, &st), *MY = ws_get<double>(ctx, (size_t)n * p, &st),
         *Gr = ws_get<double>(ctx, (size_t)p * p, &st), *Mr = ws_get<double>(ctx, (size_t)p * p, &st),
         *lr = ws_get<double>(ctx, (size_t)p, &st), *Zr = ws_get<double>(ctx, (size_t)p * p, &st);
  if (!GY || !MY || !Gr || !Mr || !lr || !Zr) return st;
  OFRR_TRY(gemm_small2(ctx, GemmSmall{n, p, n, 1.0, G, n, 0, Y, n, 0, 0.0, GY, n},
                       GemmSmall{n, p, n, 1.0, M, n, 0, Y, n, 0, 0.0, MY, n}));
  OFRR_TRY(gemm_small2(ctx, GemmSmall{p, p, n, 1.0, Y, n, 1, GY, n, 0, 0.0, Gr, p},
                       GemmSmall{p, p, n, 1.0, Y, n, 1, MY, n, 0, 0.0, Mr, p}));
  OFRR_TRY(geig_nonsym(ctx, p, Gr, Mr, lr, Zr, true, true));
  OFRR_TRY(gemm_small(ctx, n, k, p, 1.0, Y, n, 0, Zr, p, 0, 0.0, U, n));
  k_unit_cols_nk<<<(k + 3) / 4, 128, 0, ctx->stream>>>(n, k, U);
  OFRR_LAUNCHED(ctx, "k_unit_cols_nk");
  OFRR_CUDA(cudaMemcpyAsync(lam, lr, sizeof(double) * k, cudaMemcpyDeviceToDevice, ctx->stream));
  return OFRR_SUCCESS;
}

// eig(G, M) for a nonsymmetric G and SPD M (M null: eig(G)): lam = real parts, descending (stable);
// U (ld n) the real parts of the eigenvectors, unit 2-norm.  M is reduced away with its FP64
// Cholesky factor (C = L^-1 G L^-T, U = L^-T X); C is solved in FP32 (smalleig_nonsym.cu).
int geig_nonsym(ofrr_ctx* ctx, int n, const double* G, const double* M, double* lam, double* U, bool refine,
                bool pair_imag, bool values_only) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 128) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *L = ws_get<double>(ctx, (size_t)n * n, &st), *Z = ws_get<double>(ctx, (size_t)n * n, &st),
         *C = ws_get<double>(ctx, (size_t)n * n, &st), *X = ws_get<double>(ctx, (size_t)n * n, &st),
         *W = ws_get<double>(ctx, (size_t)n * n, &st), *wr = ws_get<double>(ctx, (size_t)n, &st),
         *wi = ws_get<double>(ctx, (size_t)n, &st);
  if (!L || !Z || !C || !X || !W || !wr || !wi) return st;
  const double* Cs = G;
  if (M) {
    const double* Ms[1] = {M};
    double* Ls[1] = {L};
    OFRR_TRY(chol(ctx, n, 1, Ms, n, 0.0, Ls));
    OFRR_TRY(trsm(ctx, n, n, L, G, n, 1, Z, 0));  // Z = L^-1 G'
    OFRR_TRY(trsm(ctx, n, n, L, Z, n, 1, C, 0));  // C = L^-1 Z' = L^-1 G L^-T
    Cs = C;
  }
  OFRR_TRY(nonsym_eig_dev(ctx, n, Cs, wr, wi, X, refine, pair_imag, values_only));
  if (values_only) {
    k_sort_desc<<<1, 256, 0, ctx->stream>>>(n, wr, nullptr, lam, nullptr);
    OFRR_LAUNCHED(ctx, "k_sort_desc");
    return OFRR_SUCCESS;
  }
  if (M) {
    OFRR_TRY(trsm(ctx, n, n, L, X, n, 0, W, 1));  // W = L^-T X
    k_unit_cols<<<(n + 3) / 4, 128, 0, ctx->stream>>>(n, W);
    OFRR_LAUNCHED(ctx, "k_unit_cols");
  } else {
    OFRR_CUDA(cudaMemcpyAsync(W, X, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  k_sort_desc<<<1, 256, 0, ctx->stream>>>(n, wr, W, lam, U);
  OFRR_LAUNCHED(ctx, "k_sort_desc");
  return OFRR_SUCCESS;
}

// eig(G, M + tau I) for symmetric G and SPD M: lam descending, U M-orthonormal (ldu = n)
int geig_fast(ofrr_ctx* ctx, int n, const double* G, const double* M, double tau, double* lam, double* U,
              int refine) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 128) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *L = ws_get<double>(ctx, (size_t)n * n, &st), *Y = ws_get<double>(ctx, (size_t)n * n, &st),
         *C = ws_get<double>(ctx, (size_t)n * n, &st), *W = ws_get<double>(ctx, (size_t)n * n, &st);
  if (!L || !Y || !C || !W) return st;
  if (M) {
    const double* Ms[1] = {M};
    double* Ls[1] = {L};
    OFRR_TRY(chol(ctx, n, 1, Ms, n, tau, Ls));
    OFRR_TRY(trsm(ctx, n, n, L, G, n, 0, Y, 0));  // Y = L^-1 G
    OFRR_TRY(trsm(ctx, n, n, L, Y, n, 1, C, 0));  // C = L^-1 Y'  (= L^-1 G L^-T)
  } else {
    OFRR_CUDA(cudaMemcpyAsync(C, G, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  OFRR_TRY(sym_eig_refined(ctx, n, C, W, lam, refine));
  if (M) {
    OFRR_TRY(trsm(ctx, n, n, L, W, n, 0, U, 1));  // U = L^-T W
  } else {
    OFRR_CUDA(cudaMemcpyAsync(U, W, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return OFRR_SUCCESS;
}

// SVD pencil of svd_rr.m: returns sigma (descending) and the coefficient matrices Zf = Lu^-T Y,
// Wf = Lv^-T X such that U Zf, V Wf are the (unit-norm in the Gram metrics) singular vectors.
int gsvd_fast(ofrr_ctx* ctx, int b, const double* B, const double* UU, const double* VV, double tau, double* sigma,
              double* Zf, double* Wf, int refine) {
  if (b <= 0) return OFRR_SUCCESS;
  if (b > 128) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double *Lu = ws_get<double>(ctx, (size_t)b * b, &st), *Lv = ws_get<double>(ctx, (size_t)b * b, &st),
         *T1 = ws_get<double>(ctx, (size_t)b * b, &st), *C = ws_get<double>(ctx, (size_t)b * b, &st),
         *S = ws_get<double>(ctx, (size_t)b * b, &st), *X = ws_get<double>(ctx, (size_t)b * b, &st),
         *lam = ws_get<double>(ctx, (size_t)b, &st), *CX = ws_get<double>(ctx, (size_t)b * b, &st),
         *Y = ws_get<double>(ctx, (size_t)b * b, &st);
  if (!Lu || !Lv || !T1 || !C || !S || !X || !lam || !CX || !Y) return st;
  const double* Ms[2] = {UU, VV};
  double* Ls[2] = {Lu, Lv};
  OFRR_TRY(chol(ctx, b, 2, Ms, b, tau, Ls));
  OFRR_TRY(trsm(ctx, b, b, Lu, B, b, 0, T1, 0));   // T1 = Lu^-1 B
  OFRR_TRY(trsm(ctx, b, b, Lv, T1, b, 1, C, 0));   // C' = Lv^-1 T1'  -> C holds (Lu^-1 B Lv^-T)'
  // S = C'C with C = (stored)' : S = stored * stored'
  OFRR_TRY(gemm_small(ctx, b, b, b, 1.0, C, b, 0, C, b, 1, 0.0, S, b));
  {  // starting vectors: FP32 one-sided Jacobi on the columns of C (= rows of the stored matrix)
    double* X0 = ws_get<double>(ctx, (size_t)b * b, &st);
    if (!X0) return st;
    const size_t smem = (size_t)2 * b * j1_ld(b) * sizeof(float);
    if (b <= 64) {
      OFRR_TRY(allow_smem(k_jacobi1_f32<8>));
      k_jacobi1_f32<8><<<1, 256, smem, ctx->stream>>>(b, C, b, 1, X0);
    } else {
      OFRR_TRY(allow_smem(k_jacobi1_f32<16>));
      k_jacobi1_f32<16><<<1, 256, smem, ctx->stream>>>(b, C, b, 1, X0);
    }
    OFRR_LAUNCHED(ctx, "k_jacobi1_f32");
    OFRR_TRY(eig_refine(ctx, b, S, X0, X, lam, refine));  // right singular vectors X, sigma^2 (FP64)
  }
  OFRR_TRY(gemm_small(ctx, b, b, b, 1.0, C, b, 1, X, b, 0, 0.0, CX, b));  // (true C) X
  k_svd_left<<<(b * b + 255) / 256, 256, 0, ctx->stream>>>(b, CX, lam, Y, sigma);
  OFRR_LAUNCHED(ctx, "k_svd_left");
  OFRR_TRY(trsm(ctx, b, b, Lu, Y, b, 0, Zf, 1, Lv, X, Wf));  // Zf = Lu^-T Y, Wf = Lv^-T X (one launch)
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

// Self-test of the restart block of the nonsymmetric thick-restart Krylov path (no reference
// counterpart): Y (n x p, ld n) spanning the invariant subspace of (G, M) for the eigenvalues with real
// part above sigma.  G, M, Y: device FP64, column-major, ld n; n <= 96.
extern "C" int ofrr_debug_invariant_subspace(ofrr_ctx* ctx, int n, const double* G, const double* M, double sigma,
                                             int p, double* Y) {
  if (!ctx || !G || !M || !Y || n < 1 || p < 1 || p > n) return OFRR_ERR_INVALID_ARGUMENT;
  return invariant_subspace_nonsym(ctx, n, G, M, sigma, p, Y);
}
