// Batched dense symmetric eigensolves in one persistent launch (the batched workload: thousands of
// matrices of different sizes, a few leading eigenpairs each).
//
// Behaviour followed per matrix: MATLAB/+src/+subspace/subspace_iter_eig.m:50-68 -- step_size power
// steps with scalecols (scalecols.m:21-34), the Hessenberg basis of the block (hessenberg.m:45-85, MGS
// order, pivot on the first largest entry), generalized Rayleigh-Ritz (eig_rr.m:46-57) -- plus the
// library's convergence test on the leading nev pairs and a precision schedule.
//
// Design:
//  * k_batch_si: a persistent grid (one 512-thread CTA per SM) pulls matrices from an atomic queue, the
//    largest first.  A CTA keeps its matrix's block (n x b, b <= 16, FP32) and the product block in
//    shared memory (row-major, 2 x 64 KB at n = 1024) and streams A from HBM for every product: phase 1
//    reads a 16-bit copy of A (half the bytes), phase 2 (once the 16-bit residuals stop improving) the
//    FP32 copy; products accumulate in FP32 on the CUDA cores (16 FMAs per element of A streamed, so the
//    16-bit phase is bound by HBM, not by the FP32 pipe).  Rows are split over thread groups when n is
//    small (each group a slice of k, partial sums added in a fixed order: results do not depend on the
//    schedule).  The Gram matrices sum 64-row chunks in FP32 and the chunks in FP64; the 16 x 16 pencil
//    is reduced by an FP64 Cholesky factor and solved by an FP32 Jacobi method.
//  * k_batch_refine: FP32 arithmetic cannot certify residuals near 1e-7 (its own rounding is ~1e-7 of
//    ||A||), so a second persistent pass takes each matrix's FP32 block (the nev wanted vectors and the
//    guard columns) to FP64 accuracy: block steps of Rayleigh-Ritz on [X, A X - X diag(l)] with FP64
//    products from the FP64 input until the FP64 residuals of the nev leading pairs meet tol (usually one
//    or two steps; at most 8).
// No spin waits: the queue is one atomic counter per kernel.
#include "ofrr_internal.cuh"

namespace ofrr {
namespace {

constexpr int BE_T = 512;      // threads per CTA
constexpr int BE_B = 16;       // block width (columns)
constexpr int BE_NMAX = 1024;  // largest matrix dimension held in shared memory
constexpr int BE_NEV = 8;      // leading pairs certified by the refinement

struct BatchDev {
  const int64_t* n;        // count
  const int64_t* off;      // element offset of matrix i in the FP64 / FP32 / 16-bit copies
  const int* order;        // processing order (largest first)
  const double* A64;
  const float* A32;
  const void* A16;         // __half or __nv_bfloat16
  float* X;                // count blocks of n x BE_B (FP32 Ritz vectors out), at 16 * off[i] / n[i]... (xoff)
  const int64_t* xoff;     // element offset of matrix i's n x BE_B block in X
  float* lam;              // count x BE_B Ritz values (descending)
  int* iters;              // count: outer iterations
  int* phase2;             // count: outer iteration at which the FP32 phase began (-1: never)
  unsigned long long* tstart;  // count: global timer when the matrix was taken from the queue
  unsigned int* queue;
  int count, b, nev, step, maxit;
  float tol16, tol32;      // residual targets that end the 16-bit and the FP32 phase
  uint64_t seed;
};

__device__ __forceinline__ float be_ld(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float be_ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float be_ld(const float* p) { return *p; }

__device__ __forceinline__ unsigned long long tc_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint64_t be_mix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// block sum of one float per thread (all threads get the result); red: BE_T / 32 floats
__device__ __forceinline__ float be_block_sum(float v, float* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = 0.f;
  for (int w = 0; w < BE_T / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

// W (n x b, row-major, shared) = A (n x n, column-major, global, type TA) V (n x b, row-major, shared).
// G thread groups split k; group g's partial sums land in P (G x n x b) and are added in group order.
template <class TA>
__device__ void be_matmul(int n, int b, const TA* __restrict__ A, const float* V, float* W, float* P) {
  const int tid = threadIdx.x;
  const int npad = (n + 31) & ~31;
  const int G = max(1, min(BE_T / npad, 16));
  const int g = tid / npad, i0 = tid % npad;
  const int kper = (n + G - 1) / G;
  if (g < G) {
    const int k0 = g * kper, k1 = min(n, k0 + kper);
    for (int i = i0; i < n; i += (G == 1 ? BE_T : n + 1)) {  // G > 1: one row per thread
      float acc[BE_B];
#pragma unroll
      for (int c = 0; c < BE_B; ++c) acc[c] = 0.f;
      const TA* Ai = A + i;
#pragma unroll 4
      for (int k = k0; k < k1; ++k) {
        const float a = be_ld(Ai + (int64_t)k * n);
        const float* vk = V + k * BE_B;
#pragma unroll
        for (int c = 0; c < BE_B; ++c) acc[c] = fmaf(a, vk[c], acc[c]);
      }
      float* dst = (G == 1) ? (W + i * BE_B) : (P + ((size_t)g * n + i) * BE_B);
#pragma unroll
      for (int c = 0; c < BE_B; ++c) dst[c] = (c < b) ? acc[c] : 0.f;
      if (G > 1) break;
    }
  }
  __syncthreads();
  if (G > 1) {
    for (int e = tid; e < n * BE_B; e += BE_T) {
      float s = 0.f;
      for (int gg = 0; gg < G; ++gg) s += P[(size_t)gg * n * BE_B + e];
      W[e] = s;
    }
    __syncthreads();
  }
}

// per column of X (n x b, row-major): the signed value of largest magnitude (first row on ties)
__device__ void be_colmax(int n, int b, const float* X, float* out, float* redv, int* redi) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int c = 0; c < b; ++c) {
    float best = -1.f;
    int bi = 0x7fffffff;
    for (int i = tid; i < n; i += BE_T) {
      const float a = fabsf(X[i * BE_B + c]);
      if (a > best) {
        best = a;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      redv[wid] = best;
      redi[wid] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      float bb = -1.f;
      int ii = 0x7fffffff;
      for (int w = 0; w < BE_T / 32; ++w)
        if (redv[w] > bb || (redv[w] == bb && redi[w] < ii)) {
          bb = redv[w];
          ii = redi[w];
        }
      out[c] = (ii < n) ? X[ii * BE_B + c] : 0.f;
    }
    __syncthreads();
  }
}

// Symmetric 16 x 16 Jacobi eigensolver in FP32 on one warp, parallel (round-robin) ordering: every round
// rotates 8 disjoint pairs at once, lane m < 8 computing pair m's rotation, lane k < 16 applying all 8 to
// row / column k.  S (ld BE_B) is overwritten, U holds the eigenvectors (columns), w the eigenvalues.
// Rows and columns past b must be zero off the diagonal (their diagonal sorts them last).
__device__ void be_jacobi(float* S, float* U, float* w, float* cs, int* pq) {
  const int lane = threadIdx.x & 31;
  for (int e = lane; e < BE_B * BE_B; e += 32) U[e] = ((e / BE_B) == (e % BE_B)) ? 1.f : 0.f;
  __syncwarp();
  for (int sweep = 0; sweep < 20; ++sweep) {
    float off = 0.f, dn = 0.f;
    for (int e = lane; e < BE_B * BE_B; e += 32) {
      const float v = S[e] * S[e];
      if (e / BE_B != e % BE_B) off += v;
      else dn += (fabsf(S[e]) < 1e29f) ? v : 0.f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dn += __shfl_xor_sync(0xffffffffu, dn, o);
    }
    if (off <= 1e-14f * dn || off == 0.f) break;
    for (int round = 0; round < BE_B - 1; ++round) {
      if (lane < BE_B / 2) {  // round-robin pairs: position 0 fixed, the others rotate
        const int a = (lane == 0) ? 0 : 1 + (lane - 1 + round) % (BE_B - 1);
        const int bb = 1 + (BE_B - 2 - lane + round) % (BE_B - 1);
        const int p = min(a, bb), q = max(a, bb);
        const float apq = S[p * BE_B + q];
        float c = 1.f, sn = 0.f;
        if (fabsf(apq) > 1e-30f) {
          const float theta = (S[q * BE_B + q] - S[p * BE_B + p]) / (2.f * apq);
          const float t = copysignf(1.f, theta) / (fabsf(theta) + sqrtf(fmaf(theta, theta, 1.f)));
          c = rsqrtf(fmaf(t, t, 1.f));
          sn = t * c;
        }
        cs[2 * lane] = c;
        cs[2 * lane + 1] = sn;
        pq[2 * lane] = p;
        pq[2 * lane + 1] = q;
      }
      __syncwarp();
      if (lane < BE_B) {  // columns: S = S J, U = U J (row `lane`)
        for (int m = 0; m < BE_B / 2; ++m) {
          const int p = pq[2 * m], q = pq[2 * m + 1];
          const float c = cs[2 * m], sn = cs[2 * m + 1];
          const float sp = S[lane * BE_B + p], sq = S[lane * BE_B + q];
          S[lane * BE_B + p] = c * sp - sn * sq;
          S[lane * BE_B + q] = sn * sp + c * sq;
          const float up = U[lane * BE_B + p], uq = U[lane * BE_B + q];
          U[lane * BE_B + p] = c * up - sn * uq;
          U[lane * BE_B + q] = sn * up + c * uq;
        }
      }
      __syncwarp();
      if (lane < BE_B) {  // rows: S = J' S (column `lane`)
        for (int m = 0; m < BE_B / 2; ++m) {
          const int p = pq[2 * m], q = pq[2 * m + 1];
          const float c = cs[2 * m], sn = cs[2 * m + 1];
          const float sp = S[p * BE_B + lane], sq = S[q * BE_B + lane];
          S[p * BE_B + lane] = c * sp - sn * sq;
          S[q * BE_B + lane] = sn * sp + c * sq;
        }
      }
      __syncwarp();
    }
  }
  if (lane < BE_B) w[lane] = S[lane * BE_B + lane];
  __syncwarp();
}

template <class T16>
__global__ void __launch_bounds__(BE_T, 1) k_batch_si(BatchDev d) {
  extern __shared__ float be_sm[];
  float* V = be_sm;                  // BE_NMAX x BE_B
  float* W = V + BE_NMAX * BE_B;     // BE_NMAX x BE_B
  float* P = W + BE_NMAX * BE_B;     // partial sums of small matrices: 16 x 32 x BE_B (also Gram chunks)
  __shared__ float s_red[BE_T / 32];
  __shared__ int s_redi[BE_T / 32];
  __shared__ float s_piv[BE_B];
  __shared__ int s_perm[BE_B];
  __shared__ int s_sel[BE_B];
  __shared__ double s_G[BE_B * BE_B], s_M[BE_B * BE_B], s_L[BE_B * BE_B], s_T[BE_B * BE_B];
  __shared__ float s_S[BE_B * BE_B], s_U[BE_B * BE_B], s_w[BE_B];
  __shared__ float s_Z[BE_B * BE_B];
  __shared__ float s_lam[BE_B];
  __shared__ float s_cs[BE_B];
  __shared__ int s_pq[BE_B];
  __shared__ int s_job;
  const int tid = threadIdx.x;
  const int b = d.b;
  while (true) {
    if (tid == 0) s_job = (int)atomicAdd(d.queue, 1u);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= d.count) return;
    const int mi = d.order[job];
    if (tid == 0) d.tstart[mi] = tc_globaltimer();
    const int n = (int)d.n[mi];
    const int64_t off = d.off[mi];
    const T16* A16 = reinterpret_cast<const T16*>(d.A16) + off;
    const float* A32 = d.A32 + off;
    // start block: Gaussian-like draws (sum of uniforms) from the matrix's key, scaled to unit maximum
    for (int e = tid; e < n * BE_B; e += BE_T) {
      const int i = e / BE_B, c = e % BE_B;
      const uint64_t h = be_mix(d.seed ^ be_mix((uint64_t)mi * 0x100000001b3ull + (uint64_t)(i * BE_B + c)));
      V[e] = (c < b) ? ((float)(h >> 40) * (1.f / 16777216.f) - 0.5f) : 0.f;
    }
    __syncthreads();
    int phase = 0, it = 0, p2 = -1;
    float best = INFINITY, prev = INFINITY;
    int stall = 0;
    for (; it < d.maxit; ++it) {
      // ---- power steps: V = scalecols(A V) ----
      for (int s = 0; s < d.step; ++s) {
        if (phase == 0) be_matmul<T16>(n, b, A16, V, W, P);
        else be_matmul<float>(n, b, A32, V, W, P);
        be_colmax(n, b, W, s_piv, s_red, s_redi);
        for (int e = tid; e < n * BE_B; e += BE_T) {
          const int c = e % BE_B;
          const float pv = s_piv[c];
          V[e] = (c < b && pv != 0.f) ? W[e] / pv : 0.f;
        }
        __syncthreads();
      }
      // ---- Hessenberg basis of V (in place): MGS order, pivot on the first largest entry ----
      for (int j = 0; j < b; ++j) {
        for (int l = 0; l < j; ++l) {
          if (!s_sel[l]) continue;
          const float cl = V[s_perm[l] * BE_B + j];
          __syncthreads();
          for (int i = tid; i < n; i += BE_T) V[i * BE_B + j] -= cl * V[i * BE_B + l];
          __syncthreads();
        }
        // pivot of column j
        float bv = -1.f;
        int bi = 0x7fffffff;
        for (int i = tid; i < n; i += BE_T) {
          const float a = fabsf(V[i * BE_B + j]);
          if (a > bv) {
            bv = a;
            bi = i;
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ob = __shfl_xor_sync(0xffffffffu, bv, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ob > bv || (ob == bv && oi < bi)) {
            bv = ob;
            bi = oi;
          }
        }
        if ((tid & 31) == 0) {
          s_red[tid >> 5] = bv;
          s_redi[tid >> 5] = bi;
        }
        __syncthreads();
        if (tid == 0) {
          float bb = -1.f;
          int ii = 0x7fffffff;
          for (int w = 0; w < BE_T / 32; ++w)
            if (s_red[w] > bb || (s_red[w] == bb && s_redi[w] < ii)) {
              bb = s_red[w];
              ii = s_redi[w];
            }
          const bool keep = ii < n && bb >= 1e-5f;  // columns enter with unit maximum
          s_sel[j] = keep ? 1 : 0;
          s_perm[j] = keep ? ii : 0;
          s_piv[j] = keep ? V[ii * BE_B + j] : 0.f;
        }
        __syncthreads();
        const float pv = s_piv[j];
        for (int i = tid; i < n; i += BE_T) V[i * BE_B + j] = (pv != 0.f) ? V[i * BE_B + j] / pv : 0.f;
        __syncthreads();
      }
      // ---- Rayleigh-Ritz: W = A Q, G = Q' W, M = Q' Q (64-row FP32 chunks summed in FP64) ----
      if (phase == 0) be_matmul<T16>(n, b, A16, V, W, P);
      else be_matmul<float>(n, b, A32, V, W, P);
      {
        const int pairs = BE_B * BE_B;
        const int nch = (n + 63) / 64;
        for (int e = tid; e < 2 * pairs; e += BE_T) {
          const int which = e / pairs, pr = e % pairs, r = pr / BE_B, c = pr % BE_B;
          double acc = 0.0;
          if (r < b && c < b) {
            for (int ch = 0; ch < nch; ++ch) {
              float s = 0.f;
              const int i1 = min(n, ch * 64 + 64);
              for (int i = ch * 64; i < i1; ++i) s = fmaf(V[i * BE_B + r], which ? V[i * BE_B + c] : W[i * BE_B + c], s);
              acc += (double)s;
            }
          }
          if (which) s_M[pr] = acc;
          else s_G[pr] = acc;
        }
        __syncthreads();
      }
      // ---- the b x b pencil on warp 0: M + tau I = L L' (FP64), C = L^-1 sym(G) L^-T, Jacobi (FP32) ----
      if (tid < 32) {
        const int lane = tid;
        if (lane == 0) {
          double mx = 0.0;
          for (int i = 0; i < b; ++i) mx = fmax(mx, s_M[i * BE_B + i]);
          for (int i = 0; i < b; ++i) s_M[i * BE_B + i] += 1e-12 * mx + 1e-300;
          for (int j = 0; j < b; ++j) {  // Cholesky, row-major lower factor in s_L
            double dj = s_M[j * BE_B + j];
            for (int k = 0; k < j; ++k) dj -= s_L[j * BE_B + k] * s_L[j * BE_B + k];
            dj = sqrt(fmax(dj, 1e-300));
            s_L[j * BE_B + j] = dj;
            for (int i = j + 1; i < b; ++i) {
              double v = s_M[i * BE_B + j];
              for (int k = 0; k < j; ++k) v -= s_L[i * BE_B + k] * s_L[j * BE_B + k];
              s_L[i * BE_B + j] = v / dj;
            }
            for (int i = 0; i < j; ++i) s_L[i * BE_B + j] = 0.0;
          }
        }
        __syncwarp();
        // T = L^-1 sym(G) (column c by forward substitution, lanes over columns)
        for (int c = lane; c < b; c += 32) {
          for (int i = 0; i < b; ++i) {
            double v = 0.5 * (s_G[i * BE_B + c] + s_G[c * BE_B + i]);
            for (int k = 0; k < i; ++k) v -= s_L[i * BE_B + k] * s_T[k * BE_B + c];
            s_T[i * BE_B + c] = v / s_L[i * BE_B + i];
          }
        }
        __syncwarp();
        // C = T L^-T: row r of C solves L (C row r)' = (T row r)'
        for (int r = lane; r < b; r += 32) {
          double y[BE_B];
          for (int i = 0; i < b; ++i) {
            double v = s_T[r * BE_B + i];
            for (int k = 0; k < i; ++k) v -= s_L[i * BE_B + k] * y[k];
            y[i] = v / s_L[i * BE_B + i];
          }
          for (int i = 0; i < b; ++i) s_S[r * BE_B + i] = (float)y[i];
        }
        __syncwarp();
        for (int e = lane; e < BE_B * BE_B; e += 32) {  // symmetrise; pad rows / columns past b
          const int i = e / BE_B, j = e % BE_B;
          if (i >= b || j >= b) {
            s_S[e] = (i == j) ? -1e30f : 0.f;
          } else if (i < j) {
            const float a = 0.5f * (s_S[i * BE_B + j] + s_S[j * BE_B + i]);
            s_S[i * BE_B + j] = a;
            s_S[j * BE_B + i] = a;
          }
        }
        __syncwarp();
        be_jacobi(s_S, s_U, s_w, s_cs, s_pq);
        // sort descending (lane 0), Z = L^-T U (FP64 back substitution, lanes over columns)
        if (lane == 0) {
          for (int i = 0; i < b; ++i) s_lam[i] = s_w[i];
          int idx[BE_B];
          for (int i = 0; i < b; ++i) idx[i] = i;
          for (int i = 1; i < b; ++i) {
            const int v = idx[i];
            int j = i - 1;
            while (j >= 0 && s_w[idx[j]] < s_w[v]) {
              idx[j + 1] = idx[j];
              --j;
            }
            idx[j + 1] = v;
          }
          for (int i = 0; i < b; ++i) s_redi[i] = idx[i];
          for (int i = 0; i < b; ++i) s_lam[i] = s_w[idx[i]];
        }
        __syncwarp();
        for (int c = lane; c < b; c += 32) {
          const int src = s_redi[c];
          double y[BE_B];
          for (int i = b - 1; i >= 0; --i) {
            double v = (double)s_U[i * BE_B + src];
            for (int k = i + 1; k < b; ++k) v -= s_L[k * BE_B + i] * y[k];
            y[i] = v / s_L[i * BE_B + i];
          }
          for (int i = 0; i < b; ++i) s_Z[i * BE_B + c] = (float)y[i];
        }
      }
      __syncthreads();
      // ---- Ritz vectors X = Q Z (into P as scratch rows), A X = W Z, residuals of the nev leading ----
      for (int i = tid; i < n; i += BE_T) {
        float q[BE_B], a[BE_B];
#pragma unroll
        for (int c = 0; c < BE_B; ++c) {
          q[c] = V[i * BE_B + c];
          a[c] = W[i * BE_B + c];
        }
#pragma unroll
        for (int c = 0; c < BE_B; ++c) {
          float x = 0.f, ax = 0.f;
#pragma unroll
          for (int r = 0; r < BE_B; ++r) {
            x = fmaf(q[r], s_Z[r * BE_B + c], x);
            ax = fmaf(a[r], s_Z[r * BE_B + c], ax);
          }
          V[i * BE_B + c] = (c < b) ? x : 0.f;
          W[i * BE_B + c] = (c < b) ? ax : 0.f;
        }
      }
      __syncthreads();
      float maxres = 0.f;
      const float lmax = fmaxf(fabsf(s_lam[0]), 1e-30f);
      for (int c = 0; c < d.nev; ++c) {
        float rr = 0.f, xx = 0.f;
        for (int i = tid; i < n; i += BE_T) {
          const float x = V[i * BE_B + c];
          const float r = W[i * BE_B + c] - s_lam[c] * x;
          rr = fmaf(r, r, rr);
          xx = fmaf(x, x, xx);
        }
        rr = be_block_sum(rr, s_red);
        xx = be_block_sum(xx, s_red);
        const float res = (xx > 0.f) ? sqrtf(rr / xx) / lmax : INFINITY;
        maxres = fmaxf(maxres, res);
      }
      // ---- phase and stop decisions (uniform across the CTA): a phase ends at its target or when the
      //      residual has not improved by 10 % over 8 iterations (its rounding floor) ----
      if (maxres < 0.9f * best) {
        best = maxres;
        stall = 0;
      } else {
        ++stall;
      }
      prev = maxres;
      if (phase == 0 && (maxres <= d.tol16 || stall >= 8)) {
        phase = 1;
        p2 = it + 1;
        best = INFINITY;
        stall = 0;
      } else if (phase == 1 && (maxres <= d.tol32 || stall >= 8)) {
        ++it;
        break;
      }
      // the Ritz vectors, scaled to a unit maximum, start the next iteration; a column that vanished
      // (deselected by the basis) restarts from fresh draws
      be_colmax(n, b, V, s_piv, s_red, s_redi);
      for (int e = tid; e < n * BE_B; e += BE_T) {
        const int i = e / BE_B, c = e % BE_B;
        const float pv = s_piv[c];
        float v = 0.f;
        if (c < b) {
          if (pv != 0.f) {
            v = V[e] / pv;
          } else {
            const uint64_t h = be_mix(d.seed ^ be_mix(((uint64_t)mi << 32) + (uint64_t)(it + 1) * 1315423911ull +
                                                      (uint64_t)(i * BE_B + c)));
            v = (float)(h >> 40) * (1.f / 16777216.f) - 0.5f;
          }
        }
        V[e] = v;
      }
      __syncthreads();
    }
    (void)prev;
    // ---- outputs: Ritz vectors (FP32, n x BE_B), values, counts ----
    float* X = d.X + d.xoff[mi];
    for (int e = tid; e < n * BE_B; e += BE_T) {
      const int i = e / BE_B, c = e % BE_B;
      X[i + (int64_t)c * n] = V[e];
    }
    if (tid < BE_B) d.lam[(int64_t)mi * BE_B + tid] = (tid < b) ? s_lam[tid] : 0.f;
    if (tid == 0) {
      d.iters[mi] = it;
      d.phase2[mi] = p2;
    }
    __syncthreads();
  }
}

// ---- FP64 refinement of the nev leading Ritz pairs of every matrix ------------------------------------
struct RefineDev {
  const int64_t* n;
  const int64_t* off;
  const int* order;
  const double* A64;
  const float* X32;     // from k_batch_si (n x BE_B per matrix at xoff)
  const int64_t* xoff;
  const float* lam32;
  double* X64;          // out: n x nev per matrix at xoff64
  const int64_t* xoff64;
  double* lam;          // out: count x nev
  double* res;          // out: count x nev (FP64 residuals / max|l|)
  double* scratch;      // per CTA: 3 x BE_NMAX x 2 BE_B doubles
  unsigned long long* tend;  // count: global timer when the matrix's refinement finished
  unsigned int* queue;
  int count, nev, b, steps;
  double tol;
};

constexpr int BR_K2 = 2 * BE_B;  // width of [X, R]

// Y (n x k, ld n, FP64) = A (n x n) X (n x k, ld n) in FP64, threads over rows
__device__ void br_matmul(int n, int k, const double* __restrict__ A, const double* X, double* Y) {
  for (int i = threadIdx.x; i < n; i += BE_T) {
    double acc[BE_B];
#pragma unroll
    for (int c = 0; c < BE_B; ++c) acc[c] = 0.0;
    for (int kk = 0; kk < n; ++kk) {
      const double a = A[i + (int64_t)kk * n];
#pragma unroll
      for (int c = 0; c < BE_B; ++c)
        if (c < k) acc[c] = fma(a, X[kk + (int64_t)c * n], acc[c]);
    }
    for (int c = 0; c < k; ++c) Y[i + (int64_t)c * n] = acc[c];
  }
  __syncthreads();
}

__device__ double br_block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < BE_T / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

// Rayleigh-Ritz of the symmetric pencil (G, M) of k2 unit columns, on one thread in FP64: M + tiny I = L L'
// with columns whose part outside the span of the earlier ones is below 1e-4 of their norm dropped (their
// row and column of the pencil removed), C = L^-1 sym(G) L^-T by a cyclic Jacobi method, and the kb largest
// eigenvalues' vectors Z = L^-T U (k2 x kb, row-major, into Zout).  L, T, U are k2 x k2 scratch arrays.
__device__ void br_rayleigh_ritz(int k2, int kb, double* G, double* M, double* L, double* T, double* Zout) {
  bool drop[BR_K2];
  double mx = 0.0;
  for (int i = 0; i < k2; ++i) mx = fmax(mx, M[i * k2 + i]);
  for (int j = 0; j < k2; ++j) {
    double dj = M[j * k2 + j] + 1e-14 * mx;
    for (int q = 0; q < j; ++q) dj -= L[j * k2 + q] * L[j * k2 + q];
    drop[j] = !(dj > 1e-8 * M[j * k2 + j]);
    for (int i = 0; i < j; ++i) L[i * k2 + j] = 0.0;
    if (drop[j]) {
      for (int q = 0; q < k2; ++q) L[j * k2 + q] = (q == j) ? 1.0 : 0.0;
      for (int i = j + 1; i < k2; ++i) L[i * k2 + j] = 0.0;
      for (int q = 0; q < k2; ++q) G[j * k2 + q] = G[q * k2 + j] = 0.0;
      continue;
    }
    dj = sqrt(dj);
    L[j * k2 + j] = dj;
    for (int i = j + 1; i < k2; ++i) {
      double v = M[i * k2 + j];
      for (int q = 0; q < j; ++q) v -= L[i * k2 + q] * L[j * k2 + q];
      L[i * k2 + j] = v / dj;
    }
  }
  // rows of L for columns after a dropped one: entries L[i][j] of a dropped j are already zero
  for (int c = 0; c < k2; ++c)
    for (int i = 0; i < k2; ++i) {
      double v = 0.5 * (G[i * k2 + c] + G[c * k2 + i]);
      for (int q = 0; q < i; ++q) v -= L[i * k2 + q] * T[q * k2 + c];
      T[i * k2 + c] = v / L[i * k2 + i];
    }
  double* Cm = M;  // C = T L^-T
  for (int r = 0; r < k2; ++r)
    for (int i = 0; i < k2; ++i) {
      double v = T[r * k2 + i];
      for (int q = 0; q < i; ++q) v -= L[i * k2 + q] * Cm[r * k2 + q];
      Cm[r * k2 + i] = v / L[i * k2 + i];
    }
  double* U = G;
  for (int e = 0; e < k2 * k2; ++e) U[e] = (e / k2 == e % k2) ? 1.0 : 0.0;
  for (int i = 0; i < k2; ++i)
    for (int j = i + 1; j < k2; ++j) {
      const double a = 0.5 * (Cm[i * k2 + j] + Cm[j * k2 + i]);
      Cm[i * k2 + j] = a;
      Cm[j * k2 + i] = a;
    }
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0.0, dn = 0.0;
    for (int i = 0; i < k2; ++i)
      for (int j = 0; j < k2; ++j) (i == j ? dn : off) += Cm[i * k2 + j] * Cm[i * k2 + j];
    if (off <= 1e-30 * dn) break;
    for (int p = 0; p < k2 - 1; ++p)
      for (int q = p + 1; q < k2; ++q) {
        const double apq = Cm[p * k2 + q];
        if (fabs(apq) < 1e-300) continue;
        const double theta = (Cm[q * k2 + q] - Cm[p * k2 + p]) / (2.0 * apq);
        const double t = copysign(1.0, theta) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int q2 = 0; q2 < k2; ++q2) {
          const double a1 = Cm[q2 * k2 + p], a2 = Cm[q2 * k2 + q];
          Cm[q2 * k2 + p] = c * a1 - s * a2;
          Cm[q2 * k2 + q] = s * a1 + c * a2;
        }
        for (int q2 = 0; q2 < k2; ++q2) {
          const double a1 = Cm[p * k2 + q2], a2 = Cm[q * k2 + q2];
          Cm[p * k2 + q2] = c * a1 - s * a2;
          Cm[q * k2 + q2] = s * a1 + c * a2;
          const double u1 = U[q2 * k2 + p], u2 = U[q2 * k2 + q];
          U[q2 * k2 + p] = c * u1 - s * u2;
          U[q2 * k2 + q] = s * u1 + c * u2;
        }
      }
  }
  // the kb largest eigenvalues among the kept directions (a dropped index keeps U = e_j, C_jj = 0)
  int idx[BR_K2];
  int nk = 0;
  for (int i = 0; i < k2; ++i)
    if (!drop[i]) idx[nk++] = i;
  for (int i = 1; i < nk; ++i) {
    const int v = idx[i];
    int j = i - 1;
    while (j >= 0 && Cm[idx[j] * k2 + idx[j]] < Cm[v * k2 + v]) {
      idx[j + 1] = idx[j];
      --j;
    }
    idx[j + 1] = v;
  }
  for (int c = 0; c < kb; ++c) {
    const int src = idx[c < nk ? c : nk - 1];
    for (int i = k2 - 1; i >= 0; --i) {
      double v = U[i * k2 + src];
      for (int q = i + 1; q < k2; ++q) v -= L[q * k2 + i] * T[q * k2 + c];
      T[i * k2 + c] = v / L[i * k2 + i];
    }
  }
  for (int e = 0; e < k2 * kb; ++e) Zout[e] = T[(e / kb) * k2 + (e % kb)];
}

// The whole FP32 block (b columns, the nev wanted plus guard vectors) is refined: block steps of
// Rayleigh-Ritz on [X, A X - X diag(l)] with FP64 products from the FP64 input, until the FP64 residuals of
// the nev leading pairs meet tol (or `steps` steps).  The guard columns keep the nearby part of the
// spectrum inside the search space, so each step removes the error along it instead of only damping it.
__global__ void __launch_bounds__(BE_T, 1) k_batch_refine(RefineDev d) {
  __shared__ double s_red[BE_T / 32];
  __shared__ double s_G[BR_K2 * BR_K2], s_M[BR_K2 * BR_K2], s_L[BR_K2 * BR_K2], s_T[BR_K2 * BR_K2];
  __shared__ double s_Z[BR_K2 * BE_B];
  __shared__ double s_lam[2 * BE_B];
  __shared__ int s_job;
  const int tid = threadIdx.x;
  const int kb = d.b, k2 = 2 * d.b, nev = d.nev;
  double* Sx = d.scratch + (size_t)blockIdx.x * 3 * BE_NMAX * BR_K2;  // [X | R] (n x 2 kb)
  double* Sa = Sx + (size_t)BE_NMAX * BR_K2;                          // A [X | R]
  double* Sy = Sa + (size_t)BE_NMAX * BR_K2;                          // new X, A X
  while (true) {
    if (tid == 0) s_job = (int)atomicAdd(d.queue, 1u);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= d.count) return;
    const int mi = d.order[job];
    const int n = (int)d.n[mi];
    const double* A = d.A64 + d.off[mi];
    const float* X32 = d.X32 + d.xoff[mi];
    for (int e = tid; e < n * kb; e += BE_T) Sx[e] = (double)X32[e];
    __syncthreads();
    br_matmul(n, kb, A, Sx, Sa);
    for (int step = 0;; ++step) {
      // Rayleigh quotients and residuals R = A X - X diag(l) (into columns kb .. 2kb-1 of Sx)
      for (int c = 0; c < kb; ++c) {
        double xax = 0.0, xx = 0.0;
        for (int i = tid; i < n; i += BE_T) {
          xax = fma(Sx[i + c * n], Sa[i + c * n], xax);
          xx = fma(Sx[i + c * n], Sx[i + c * n], xx);
        }
        xax = br_block_sum(xax, s_red);
        xx = br_block_sum(xx, s_red);
        if (tid == 0) s_lam[c] = (xx > 0.0) ? xax / xx : 0.0;
        if (tid == 0) s_lam[kb + c] = xx;
        __syncthreads();
      }
      double lmax = 0.0;
      for (int c = 0; c < nev; ++c) lmax = fmax(lmax, fabs(s_lam[c]));
      if (lmax == 0.0) lmax = 1.0;
      double maxres = 0.0;
      for (int c = 0; c < kb; ++c) {
        double rr = 0.0;
        for (int i = tid; i < n; i += BE_T) {
          const double r = Sa[i + c * n] - s_lam[c] * Sx[i + c * n];
          Sx[i + (c + kb) * n] = r;
          rr = fma(r, r, rr);
        }
        rr = br_block_sum(rr, s_red);
        if (c < nev) {
          const double res = (s_lam[kb + c] > 0.0) ? sqrt(rr / s_lam[kb + c]) / lmax : INFINITY;
          if (tid == 0) d.res[(int64_t)mi * nev + c] = res;
          maxres = fmax(maxres, res);
        }
        // unit columns for the block step: X (and A X) and the residual direction (the span is unchanged,
        // and the Gram matrix of [X, R] stays well scaled however small the residuals are)
        const double sx = (s_lam[kb + c] > 0.0) ? 1.0 / sqrt(s_lam[kb + c]) : 0.0;
        const double sr = (rr > 0.0) ? 1.0 / sqrt(rr) : 0.0;
        for (int i = tid; i < n; i += BE_T) {
          Sx[i + c * n] *= sx;
          Sa[i + c * n] *= sx;
          Sx[i + (c + kb) * n] *= sr;
        }
      }
      __syncthreads();
      if (step >= d.steps || maxres <= d.tol) {
        if (tid < kb) s_lam[kb + tid] = 1.0;  // the columns are unit now
        __syncthreads();
        break;
      }
      // block step: Rayleigh-Ritz on [X, R] (FP64 products)
      br_matmul(n, kb, A, Sx + (size_t)kb * n, Sa + (size_t)kb * n);
      for (int e = tid; e < 2 * k2 * k2; e += BE_T) {
        const int which = e / (k2 * k2), pr = e % (k2 * k2), r = pr / k2, c = pr % k2;
        if (c < r) continue;  // both matrices are symmetric: upper triangle, mirrored below
        double acc = 0.0;
        const double* Bc = which ? Sx : Sa;
        for (int i = 0; i < n; ++i) acc = fma(Sx[i + r * n], Bc[i + c * n], acc);
        double* D = which ? s_M : s_G;
        D[pr] = acc;
        D[c * k2 + r] = acc;
      }
      __syncthreads();
      if (tid == 0) br_rayleigh_ritz(k2, kb, s_G, s_M, s_L, s_T, s_Z);
      __syncthreads();
      // X <- [X R] Z, A X <- [AX AR] Z
      for (int e = tid; e < 2 * n; e += BE_T) {
        const int i = e % n, which = e / n;
        const double* src = which ? Sa : Sx;
        double vr[BR_K2];
#pragma unroll
        for (int r = 0; r < BR_K2; ++r) vr[r] = (r < k2) ? src[i + r * n] : 0.0;
        for (int c = 0; c < kb; ++c) {
          double x = 0.0;
#pragma unroll
          for (int r = 0; r < BR_K2; ++r)
            if (r < k2) x = fma(vr[r], s_Z[r * kb + c], x);
          Sy[i + (c + which * kb) * n] = x;
        }
      }
      __syncthreads();
      for (int e = tid; e < n * kb; e += BE_T) {
        Sx[e] = Sy[e];
        Sa[e] = Sy[e + (size_t)kb * n];
      }
      __syncthreads();
    }
    // outputs: unit-norm FP64 Ritz vectors of the nev leading pairs, their Rayleigh quotients
    double* Xo = d.X64 + d.xoff64[mi];
    for (int c = 0; c < nev; ++c) {
      const double inv = 1.0 / sqrt(fmax(s_lam[kb + c], 1e-300));
      for (int i = tid; i < n; i += BE_T) Xo[i + (int64_t)c * n] = Sx[i + c * n] * inv;
      if (tid == 0) d.lam[(int64_t)mi * nev + c] = s_lam[c];
    }
    __syncthreads();
    if (tid == 0) d.tend[mi] = tc_globaltimer();
  }
}

template <class TI, class TO>
__global__ void k_be_convert(int64_t count, const TI* __restrict__ in, TO* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = from_c<TO, double>(to_c<double, TI>(in[e]));
}

}  // namespace
}  // namespace ofrr

using namespace ofrr;

static int batch_sym_eig_impl(ofrr_ctx* ctx, int count, const int64_t* n_host, const int64_t* offset_host,
                              const double* A, const ofrr_options* opt, double* X, const int64_t* xoffset_host,
                              double* evals, double* resid, int* iterations, int* statuses, double* latency_ms) {
  if (!ctx || count < 0 || !n_host || !offset_host || !A || !opt || !X || !xoffset_host || !evals || !statuses)
    return OFRR_ERR_INVALID_ARGUMENT;
  if (count == 0) return OFRR_SUCCESS;
  const int nev = opt->nev > 0 ? opt->nev : BE_NEV;
  const int b = std::min(opt->block > 0 ? opt->block : BE_B, BE_B);
  if (nev > BE_NEV || nev > b || b < 2) return OFRR_ERR_INVALID_ARGUMENT;
  const ofrr_dtype t16 = (opt->p_output == OFRR_F16) ? OFRR_F16 : OFRR_BF16;
  int64_t total = 0, xtot = 0;
  std::vector<int> order(count);
  for (int i = 0; i < count; ++i) {
    if (n_host[i] < b || n_host[i] > BE_NMAX || offset_host[i] < 0) return OFRR_ERR_BLAS_INVALID_SIZE;
    total = std::max(total, offset_host[i] + n_host[i] * n_host[i]);
    order[i] = i;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return n_host[a] > n_host[c]; });
  std::vector<int64_t> xo32(count), xo64(count);
  for (int i = 0; i < count; ++i) {
    xo32[i] = xtot;
    xtot += n_host[i] * BE_B;
    xo64[i] = xoffset_host[i];
  }
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  float* A32 = ws_get<float>(ctx, (size_t)total, &st);
  void* A16 = ws_alloc(ctx, (size_t)total * 2, &st);
  float* X32 = ws_get<float>(ctx, (size_t)xtot, &st);
  float* lam32 = ws_get<float>(ctx, (size_t)count * BE_B, &st);
  int64_t* dn = ws_get<int64_t>(ctx, (size_t)count, &st);
  int64_t* doff = ws_get<int64_t>(ctx, (size_t)count, &st);
  int64_t* dxo = ws_get<int64_t>(ctx, (size_t)count, &st);
  int64_t* dxo64 = ws_get<int64_t>(ctx, (size_t)count, &st);
  int* dorder = ws_get<int>(ctx, (size_t)count, &st);
  int* dit = ws_get<int>(ctx, (size_t)2 * count, &st);
  double* dlam = ws_get<double>(ctx, (size_t)count * nev, &st);
  double* dres = ws_get<double>(ctx, (size_t)count * nev, &st);
  unsigned int* queues = ws_get<unsigned int>(ctx, 2, &st);
  unsigned long long* times = ws_get<unsigned long long>(ctx, (size_t)2 * count, &st);
  int dev = 0, sms = 0;
  OFRR_CUDA(cudaGetDevice(&dev));
  OFRR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = std::max(1, std::min(sms, count));
  double* scratch = ws_get<double>(ctx, (size_t)grid * 3 * BE_NMAX * BR_K2, &st);
  if (!A32 || !A16 || !X32 || !lam32 || !dn || !doff || !dxo || !dxo64 || !dorder || !dit || !dlam || !dres ||
      !queues || !scratch || !times)
    return st;
  OFRR_CUDA(cudaMemcpyAsync(dn, n_host, sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(doff, offset_host, sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(dxo, xo32.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(dxo64, xo64.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(dorder, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(queues, 0, 2 * sizeof(unsigned int), ctx->stream));
  // the FP32 and 16-bit copies of every matrix (one pass over the FP64 input)
  const int gc = grid_for(total, 256, 152 * 16);
  k_be_convert<double, float><<<gc, 256, 0, ctx->stream>>>(total, A, A32);
  OFRR_LAUNCHED(ctx, "k_be_convert");
  if (t16 == OFRR_F16) k_be_convert<double, __half><<<gc, 256, 0, ctx->stream>>>(total, A, (__half*)A16);
  else k_be_convert<double, __nv_bfloat16><<<gc, 256, 0, ctx->stream>>>(total, A, (__nv_bfloat16*)A16);
  OFRR_LAUNCHED(ctx, "k_be_convert");
  BatchDev d{};
  d.n = dn;
  d.off = doff;
  d.order = dorder;
  d.A64 = A;
  d.A32 = A32;
  d.A16 = A16;
  d.X = X32;
  d.xoff = dxo;
  d.lam = lam32;
  d.iters = dit;
  d.phase2 = dit + count;
  d.tstart = times;
  d.queue = queues;
  d.count = count;
  d.b = b;
  d.nev = nev;
  d.step = std::max(1, opt->step_size);
  d.maxit = opt->maxiter > 0 ? opt->maxiter : 500;
  d.tol16 = (t16 == OFRR_F16) ? 2e-3f : 1e-2f;
  d.tol32 = (float)std::max(opt->tol, 1e-7);
  d.seed = opt->seed;
  const size_t smem = (size_t)(2 * BE_NMAX * BE_B + 16 * 32 * BE_B) * sizeof(float);
  if (t16 == OFRR_F16) {
    OFRR_TRY(allow_smem(k_batch_si<__half>));
    k_batch_si<__half><<<grid, BE_T, smem, ctx->stream>>>(d);
  } else {
    OFRR_TRY(allow_smem(k_batch_si<__nv_bfloat16>));
    k_batch_si<__nv_bfloat16><<<grid, BE_T, smem, ctx->stream>>>(d);
  }
  OFRR_LAUNCHED(ctx, "k_batch_si");
  RefineDev r{};
  r.n = dn;
  r.off = doff;
  r.order = dorder;
  r.A64 = A;
  r.X32 = X32;
  r.xoff = dxo;
  r.lam32 = lam32;
  r.X64 = X;
  r.xoff64 = dxo64;
  r.lam = dlam;
  r.res = dres;
  r.scratch = scratch;
  r.tend = times + count;
  r.queue = queues + 1;
  r.count = count;
  r.nev = nev;
  r.b = b;
  r.steps = 8;
  r.tol = opt->tol > 0 ? opt->tol : 1e-7;
  k_batch_refine<<<grid, BE_T, 0, ctx->stream>>>(r);
  OFRR_LAUNCHED(ctx, "k_batch_refine");
  std::vector<double> hres((size_t)count * nev);
  std::vector<int> hit(2 * (size_t)count);
  OFRR_CUDA(cudaMemcpyAsync(evals, dlam, sizeof(double) * count * nev, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(hres.data(), dres, sizeof(double) * count * nev, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(hit.data(), dit, sizeof(int) * 2 * count, cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<unsigned long long> ht(2 * (size_t)count);
  OFRR_CUDA(cudaMemcpyAsync(ht.data(), times, sizeof(unsigned long long) * 2 * count, cudaMemcpyDeviceToHost,
                            ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  if (latency_ms)
    for (int i = 0; i < count; ++i) latency_ms[i] = 1e-6 * (double)(ht[count + i] - ht[i]);
  for (int i = 0; i < count; ++i) {
    double mr = 0.0;
    for (int j = 0; j < nev; ++j) mr = std::max(mr, hres[(size_t)i * nev + j]);
    statuses[i] = (opt->tol > 0 && !(mr <= opt->tol)) ? OFRR_ERR_SOLVER_MAX_ITERATIONS : OFRR_SUCCESS;
    if (iterations) iterations[i] = hit[i];
  }
  if (resid) std::copy(hres.begin(), hres.end(), resid);
  return OFRR_SUCCESS;
}

extern "C" int ofrr_batch_sym_eig(ofrr_ctx* ctx, int count, const int64_t* n_host, const int64_t* offset_host,
                                  const double* A, const ofrr_options* opt, double* X, const int64_t* xoffset_host,
                                  double* evals, double* resid, int* iterations, int* statuses) {
  return batch_sym_eig_impl(ctx, count, n_host, offset_host, A, opt, X, xoffset_host, evals, resid, iterations,
                            statuses, nullptr);
}

// Same, also returning each matrix's time from leaving the queue to its certified result (ms), for the
// per-matrix latency of the batch (no reference counterpart).
extern "C" int ofrr_batch_sym_eig_timed(ofrr_ctx* ctx, int count, const int64_t* n_host, const int64_t* offset_host,
                                        const double* A, const ofrr_options* opt, double* X,
                                        const int64_t* xoffset_host, double* evals, double* resid, int* iterations,
                                        int* statuses, double* latency_ms) {
  return batch_sym_eig_impl(ctx, count, n_host, offset_host, A, opt, X, xoffset_host, evals, resid, iterations,
                            statuses, latency_ms);
}
