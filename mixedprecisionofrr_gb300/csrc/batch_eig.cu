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
//    shared memory (row-major, 2 x 64 KB at n = 1024) and streams A through a ring of bulk asynchronous
//    copies for every product: phase 1 reads a 16-bit copy of A (half the bytes), phase 2 (once the
//    16-bit residuals stop improving) the FP32 copy; products accumulate in FP32 on the CUDA cores (16
//    FMAs per element of A streamed).  Rows are split over thread groups when n is small (each group a
//    slice of k, partial sums added in a fixed order: results do not depend on the schedule).  The Gram
//    matrices sum 64-row chunks in FP32 and the chunks in FP64; the 16 x 16 pencil is reduced by an FP64
//    Cholesky factor and solved by an FP32 Jacobi method.
//  * FP64 refinement (be_refine_one, same CTA, right after the matrix's FP32 phase, so a matrix's latency
//    is its own work): FP32 arithmetic cannot certify residuals near 1e-7 (its own rounding is ~1e-7 of
//    ||A||), so the CTA takes the FP32 block (the nev wanted vectors and the guard columns) to FP64
//    accuracy: block steps of Rayleigh-Ritz on [X, A X - X diag(l)] with FP64 products from the FP64
//    input until the FP64 residuals of the nev leading pairs meet tol (usually one step; at most 12).
// Bounded waits only: the queue is one atomic counter; the copy ring's mbarrier waits give up after ~2 s
// (status word, then the CTA leaves).
#include "ofrr_internal.cuh"
#include "tcgen05.cuh"

namespace ofrr {
namespace {

constexpr int BE_T = 512;      // threads per CTA
constexpr int BE_B = 16;       // block width (columns)
constexpr int BE_NMAX = 1024;  // largest matrix dimension held in shared memory
constexpr int BE_NEV = 8;      // leading pairs certified by the refinement

// The n x BE_B blocks in shared memory are row-major with the four float4 quads of row i stored at quad
// position q ^ (i & 3): a column is then spread over 8 bank groups instead of 2 (column-wise passes,
// one row per lane, had 16-way bank conflicts), while whole quads stay aligned for 16-byte accesses.
__device__ __forceinline__ int be_at(int i, int c) { return i * BE_B + ((((c >> 2) ^ (i & 3))) << 2) + (c & 3); }
// logical column of the element stored at physical offset e of the block
__device__ __forceinline__ int be_col(int e) {
  const int i = e / BE_B, p = e % BE_B;
  return ((((p >> 2) ^ (i & 3))) << 2) + (p & 3);
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
  int count, nev, b, steps;
  double tol;
};

struct BatchDev {
  const int64_t* n;        // count
  const int64_t* offp;     // element offset of matrix i in the padded FP32 / 16-bit copies (ld = n rounded to 8)
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
  int* err;                // device status word of bounded waits
  RefineDev rf;            // the FP64 refinement, run by the same CTA right after a matrix's FP32 phase
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

// ---- A streamed through shared memory: a ring of BE_NS stages filled by bulk asynchronous copies ----
// The FP32 and 16-bit copies of every matrix are stored column-major with the leading dimension rounded up
// to 8 elements (zero rows below n) at 16-byte aligned offsets, so kc consecutive columns are one
// contiguous, aligned block: one cp.async.bulk per stage, completing on the stage's `full` mbarrier.
// Every warp arrives on the stage's `empty` mbarrier once it has read the stage; thread 0 refills a stage
// after its `empty` phase completes.  The chunk counter runs on across products, so the barrier parities
// follow from it.  Every wait is bounded (about 2 s); a wait that runs out records a status word and the
// CTA leaves the kernel after the copies it issued have landed (again bounded).
constexpr int BE_NS = 4;           // stages
constexpr int BE_STAGE = 16384;    // bytes per stage

struct BeRing {
  unsigned char* buf;  // BE_NS x BE_STAGE (shared)
  uint64_t* full;      // BE_NS (shared)
  uint64_t* empty;     // BE_NS (shared)
  uint32_t count;      // chunks consumed so far (uniform across the CTA)
  int* err;            // device status word
};

__device__ __forceinline__ void be_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void be_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

// Row layout of a product for n rows: G thread groups split the columns of A (round-robin within a chunk),
// each group of Tg threads (a multiple of 32) covers the rows with R rows per thread.  Chosen to keep
// the most threads busy: maximise G / R subject to Tg R >= n.
__device__ __forceinline__ void be_layout(int n, int* G, int* R) {
  int bg = 1, br = 4;
  for (int r = 1; r <= 4; ++r)
    for (int g = 1; g <= 16; ++g) {
      const int tg = ((BE_T / g) / 32) * 32;
      if (tg * r >= n && g * br > bg * r) {
        bg = g;
        br = r;
      }
    }
  *G = bg;
  *R = br;
}

// W (n x b, row-major, shared) = A (n x n, column-major with leading dimension ld, global, type TA)
// V (n x b, row-major, shared), FP32 accumulation.  Partial sums of the G groups are added in group order
// (results do not depend on timing).  Returns false (uniformly) when a bounded wait ran out.
template <class TA, int R>
__device__ bool be_matmul_r(int n, int ld, const TA* __restrict__ A, const float* V, float* W, BeRing& rg, int G) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int Tg = ((BE_T / G) / 32) * 32;
  const int g = tid / Tg, t = tid % Tg;
  const bool active = g < G;
  const int kc = min(n, BE_STAGE / (ld * (int)sizeof(TA)));
  const int nck = (n + kc - 1) / kc;
  const uint32_t base = rg.count;
  auto issue = [&](int c) {
    const uint32_t gc = base + (uint32_t)c;
    const int st = (int)(gc % BE_NS);
    const int k0 = c * kc, cols = min(kc, n - k0);
    const uint32_t bytes = (uint32_t)(cols * ld * (int)sizeof(TA));
    tc::mbar_expect_tx(&rg.full[st], bytes);
    be_bulk_g2s(rg.buf + (size_t)st * BE_STAGE, A + (int64_t)k0 * ld, bytes, &rg.full[st]);
  };
  // refills wait for the stage's previous use to be released (that use belongs to an earlier chunk, or
  // to the previous product)
  bool bad = false;
  if (tid == 0) {
    for (int c = 0; c < min(nck, BE_NS); ++c) {
      const uint32_t gc = base + (uint32_t)c;
      if (gc >= BE_NS && !tc::mbar_wait(&rg.empty[gc % BE_NS], ((gc / BE_NS) + 1) & 1, rg.err, 21)) {
        bad = true;
        break;
      }
      issue(c);
    }
  }
  float acc[R][BE_B];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < BE_B; ++c) acc[r][c] = 0.f;
  int c = 0;
  for (; c < nck && !bad; ++c) {
    const uint32_t gc = base + (uint32_t)c;
    const int st = (int)(gc % BE_NS);
    if (!tc::mbar_wait(&rg.full[st], (gc / BE_NS) & 1, rg.err, 22)) {
      bad = true;
      break;
    }
    const TA* sA = reinterpret_cast<const TA*>(rg.buf + (size_t)st * BE_STAGE);
    const int k0 = c * kc, cols = min(kc, n - k0);
    if (active) {
      for (int kk = g; kk < cols; kk += G) {
        const float4* vk = reinterpret_cast<const float4*>(V + (k0 + kk) * BE_B);
        const int sw = (k0 + kk) & 3;
        float v[BE_B];
#pragma unroll
        for (int q = 0; q < BE_B / 4; ++q) {
          const float4 x = vk[q ^ sw];
          v[4 * q] = x.x;
          v[4 * q + 1] = x.y;
          v[4 * q + 2] = x.z;
          v[4 * q + 3] = x.w;
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int i = t + r * Tg;
          const float a = (i < n) ? be_ld(sA + kk * ld + i) : 0.f;
#pragma unroll
          for (int q = 0; q < BE_B; ++q) acc[r][q] = fmaf(a, v[q], acc[r][q]);
        }
      }
    }
    __syncwarp();
    if (lane == 0) be_arrive(&rg.empty[st]);
    if (tid == 0 && c + BE_NS < nck) {
      const uint32_t gn = base + (uint32_t)(c + BE_NS);
      if (!tc::mbar_wait(&rg.empty[st], ((gn / BE_NS) + 1) & 1, rg.err, 23)) {
        bad = true;
        break;
      }
      issue(c + BE_NS);
    }
  }
  if (__syncthreads_or(bad)) {
    // leave only after every copy this CTA issued has landed (bounded)
    if (tid == 0)
      for (int j = 0; j < nck && j < c + BE_NS; ++j) {
        const uint32_t gc = base + (uint32_t)j;
        if (j >= c) tc::mbar_wait(&rg.full[gc % BE_NS], (gc / BE_NS) & 1, rg.err, 24);
      }
    __syncthreads();
    return false;
  }
  rg.count = base + (uint32_t)nck;
  for (int gg = 0; gg < G; ++gg) {
    if (g == gg) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = t + r * Tg;
        if (i < n) {
          float4* w = reinterpret_cast<float4*>(W + i * BE_B);
          const int sw = i & 3;
#pragma unroll
          for (int q = 0; q < BE_B / 4; ++q) {
            float4 x = make_float4(acc[r][4 * q], acc[r][4 * q + 1], acc[r][4 * q + 2], acc[r][4 * q + 3]);
            if (gg > 0) {
              const float4 y = w[q ^ sw];
              x.x += y.x;
              x.y += y.y;
              x.z += y.z;
              x.w += y.w;
            }
            w[q ^ sw] = x;
          }
        }
      }
    }
    __syncthreads();
  }
  return true;
}

template <class TA>
__device__ bool be_matmul(int n, int ld, const TA* A, const float* V, float* W, BeRing& rg) {
  int G, R;
  be_layout(n, &G, &R);
  switch (R) {
    case 1: return be_matmul_r<TA, 1>(n, ld, A, V, W, rg, G);
    case 2: return be_matmul_r<TA, 2>(n, ld, A, V, W, rg, G);
    case 3: return be_matmul_r<TA, 3>(n, ld, A, V, W, rg, G);
    default: return be_matmul_r<TA, 4>(n, ld, A, V, W, rg, G);
  }
}

// per column of X (n x b, row-major): the signed value of largest magnitude (first row on ties), all
// columns in one pass; redv / redi: (BE_T / 32) x BE_B scratch
__device__ void be_colmax(int n, int b, const float* X, float* out, float* redv, int* redi) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  float best[BE_B];
  int bi[BE_B];
#pragma unroll
  for (int c = 0; c < BE_B; ++c) {
    best[c] = -1.f;
    bi[c] = 0x7fffffff;
  }
  for (int i = tid; i < n; i += BE_T) {
#pragma unroll
    for (int c = 0; c < BE_B; ++c) {
      const float a = fabsf(X[be_at(i, c)]);
      if (a > best[c]) {
        best[c] = a;
        bi[c] = i;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < BE_B; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best[c], o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi[c], o);
      if (ob > best[c] || (ob == best[c] && oi < bi[c])) {
        best[c] = ob;
        bi[c] = oi;
      }
    }
  }
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < BE_B; ++c) {
      redv[wid * BE_B + c] = best[c];
      redi[wid * BE_B + c] = bi[c];
    }
  __syncthreads();
  if (tid < b) {
    float bb = -1.f;
    int ii = 0x7fffffff;
    for (int w = 0; w < BE_T / 32; ++w) {
      const float v = redv[w * BE_B + tid];
      const int vi = redi[w * BE_B + tid];
      if (v > bb || (v == bb && vi < ii)) {
        bb = v;
        ii = vi;
      }
    }
    out[tid] = (ii < n) ? X[be_at(ii, tid)] : 0.f;
  }
  __syncthreads();
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
    // FP32 rotations leave ~b eps^2 of dn off the diagonal: 1e-13 is reachable (off-diagonal ~3e-7)
    if (off <= 1e-13f * dn || off == 0.f) break;
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


constexpr int BR_K2 = 2 * BE_B;  // width of [X, R]

// Y (n x k, ld n, global FP64) = A (n x n, column-major, FP64) X (n x k, ld n, global).  X is first copied
// into shared memory row-major (Xs: n x BE_B doubles) so that its values are broadcast reads; A is read
// once per column pass with coalesced loads.  GB300's FP64 pipe (about 1.7 FMA per clock per SM), not
// HBM, bounds this product, so the layout keeps every thread busy: G groups split the columns of A,
// each thread covers R <= 2 rows and 16 / R columns of X per pass; the groups' partial sums are added in
// group order (results do not depend on timing).
__device__ void br_matmul(int n, int k, const double* __restrict__ A, const double* X, double* Y, double* Xs) {
  const int tid = threadIdx.x;
  for (int e = tid; e < n * BE_B; e += BE_T) {
    const int i = e / BE_B, c = e % BE_B;
    Xs[e] = (c < k) ? X[i + (int64_t)c * n] : 0.0;
  }
  int G = 1, R = 2;
  for (int r = 1; r <= 2; ++r)
    for (int g = 1; g <= 16; ++g) {
      const int tg = ((BE_T / g) / 32) * 32;
      if (tg * r >= n && g * R > G * r) {
        G = g;
        R = r;
      }
    }
  __syncthreads();
  const int Tg = ((BE_T / G) / 32) * 32;
  const int g = tid / Tg, t = tid % Tg;
  const int CW = BE_B / R;
  for (int c0 = 0; c0 < k; c0 += CW) {
    double acc[2][BE_B];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int c = 0; c < BE_B; ++c) acc[r][c] = 0.0;
    if (g < G) {
      const int i0 = t, i1 = t + Tg;
      const bool v0 = i0 < n, v1 = (R == 2) && i1 < n;
      if (R == 1) {
        for (int kk = g; kk < n; kk += G) {
          const double a0 = v0 ? __ldg(A + i0 + (int64_t)kk * n) : 0.0;
          const double* xr = Xs + kk * BE_B;
#pragma unroll
          for (int c = 0; c < BE_B; ++c) acc[0][c] = fma(a0, xr[c], acc[0][c]);
        }
      } else {
        for (int kk = g; kk < n; kk += G) {
          const double a0 = v0 ? __ldg(A + i0 + (int64_t)kk * n) : 0.0;
          const double a1 = v1 ? __ldg(A + i1 + (int64_t)kk * n) : 0.0;
          const double* xr = Xs + kk * BE_B + c0;
#pragma unroll
          for (int c = 0; c < BE_B / 2; ++c) {
            acc[0][c] = fma(a0, xr[c], acc[0][c]);
            acc[1][c] = fma(a1, xr[c], acc[1][c]);
          }
        }
      }
    }
    for (int gg = 0; gg < G; ++gg) {
      if (g == gg) {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const int i = t + r * Tg;
          if (r >= R || i >= n) continue;
#pragma unroll
          for (int c = 0; c < BE_B; ++c) {
            if (c >= CW || c0 + c >= k) continue;
            double* y = Y + i + (int64_t)(c0 + c) * n;
            *y = (gg == 0) ? acc[r][c] : *y + acc[r][c];
          }
        }
      }
      __syncthreads();
    }
  }
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

// Rayleigh-Ritz of the symmetric pencil (G, M) of k2 <= 32 unit columns on one warp in FP64 (lane l owns
// row / column l): M + tiny I = L L' with columns whose part outside the span of the earlier ones is
// below 1e-4 of their norm dropped (their row and column of the pencil removed), C = L^-1 sym(G) L^-T,
// a parallel cyclic Jacobi method (round-robin pairs, every round rotating k2 / 2 disjoint pairs), and
// the kb largest eigenvalues' vectors Z = L^-T U (k2 x kb, row-major, into Zout).  All arrays k2 x k2
// row-major in shared memory; G becomes U, M becomes C.
__device__ void br_rayleigh_ritz_warp(int k2, int kb, double* G, double* M, double* L, double* T, double* Zout,
                                      double* cs, int* pq, int* s_idx) {
  const int lane = threadIdx.x & 31;
  __shared__ int s_drop[BR_K2];
  double mx = 0.0;
  for (int i = 0; i < k2; ++i) mx = fmax(mx, M[i * k2 + i]);
  for (int e = lane; e < k2 * k2; e += 32) L[e] = 0.0;
  __syncwarp();
  for (int j = 0; j < k2; ++j) {
    // row j of L left of the diagonal is final
    double dj = M[j * k2 + j] + 1e-14 * mx;
    for (int q = 0; q < j; ++q) dj -= L[j * k2 + q] * L[j * k2 + q];
    const bool drop = !(dj > 1e-8 * M[j * k2 + j]);
    if (lane == 0) s_drop[j] = drop ? 1 : 0;
    if (drop) {
      __syncwarp();
      for (int q = lane; q < k2; q += 32) {
        L[j * k2 + q] = (q == j) ? 1.0 : 0.0;
        G[j * k2 + q] = 0.0;
        G[q * k2 + j] = 0.0;
      }
      __syncwarp();
      continue;
    }
    dj = sqrt(dj);
    const int i = lane;
    double lij = 0.0;
    if (i > j && i < k2) {
      double v = M[i * k2 + j];
      for (int q = 0; q < j; ++q) v -= L[i * k2 + q] * L[j * k2 + q];
      lij = v / dj;
    }
    __syncwarp();
    if (i > j && i < k2) L[i * k2 + j] = lij;
    if (lane == 0) L[j * k2 + j] = dj;
    __syncwarp();
  }
  // T = L^-1 sym(G): lane c solves column c
  for (int c = lane; c < k2; c += 32)
    for (int i = 0; i < k2; ++i) {
      double v = 0.5 * (G[i * k2 + c] + G[c * k2 + i]);
      for (int q = 0; q < i; ++q) v -= L[i * k2 + q] * T[q * k2 + c];
      T[i * k2 + c] = v / L[i * k2 + i];
    }
  __syncwarp();
  // C = T L^-T: lane r solves row r (into M)
  for (int r = lane; r < k2; r += 32)
    for (int i = 0; i < k2; ++i) {
      double v = T[r * k2 + i];
      for (int q = 0; q < i; ++q) v -= L[i * k2 + q] * M[r * k2 + q];
      M[r * k2 + i] = v / L[i * k2 + i];
    }
  __syncwarp();
  double* Cm = M;
  double* U = G;
  for (int e = lane; e < k2 * k2; e += 32) {
    const int i = e / k2, j = e % k2;
    U[e] = (i == j) ? 1.0 : 0.0;
    if (i < j) {
      const double a = 0.5 * (Cm[i * k2 + j] + Cm[j * k2 + i]);
      Cm[i * k2 + j] = a;
      Cm[j * k2 + i] = a;
    }
  }
  __syncwarp();
  const int np = k2 / 2;
  for (int sweep = 0; sweep < 20; ++sweep) {
    double off = 0.0, dn = 0.0;
    for (int e = lane; e < k2 * k2; e += 32) {
      const double v = Cm[e] * Cm[e];
      if (e / k2 != e % k2) off += v;
      else dn += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dn += __shfl_xor_sync(0xffffffffu, dn, o);
    }
    if (off <= 1e-28 * dn) break;
    for (int round = 0; round < k2 - 1; ++round) {
      if (lane < np) {  // round-robin pairs: position 0 fixed, the others rotate
        const int a = (lane == 0) ? 0 : 1 + (lane - 1 + round) % (k2 - 1);
        const int b = 1 + (k2 - 2 - lane + round) % (k2 - 1);
        const int p = min(a, b), q = max(a, b);
        const double apq = Cm[p * k2 + q];
        double c = 1.0, sn = 0.0;
        if (fabs(apq) > 1e-300) {
          const double theta = (Cm[q * k2 + q] - Cm[p * k2 + p]) / (2.0 * apq);
          const double tt = copysign(1.0, theta) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
          c = 1.0 / sqrt(fma(tt, tt, 1.0));
          sn = tt * c;
        }
        cs[2 * lane] = c;
        cs[2 * lane + 1] = sn;
        pq[2 * lane] = p;
        pq[2 * lane + 1] = q;
      }
      __syncwarp();
      if (lane < k2) {  // columns: C = C J, U = U J (row `lane`)
        for (int m = 0; m < np; ++m) {
          const int p = pq[2 * m], q = pq[2 * m + 1];
          const double c = cs[2 * m], sn = cs[2 * m + 1];
          const double sp = Cm[lane * k2 + p], sq = Cm[lane * k2 + q];
          Cm[lane * k2 + p] = c * sp - sn * sq;
          Cm[lane * k2 + q] = sn * sp + c * sq;
          const double up = U[lane * k2 + p], uq = U[lane * k2 + q];
          U[lane * k2 + p] = c * up - sn * uq;
          U[lane * k2 + q] = sn * up + c * uq;
        }
      }
      __syncwarp();
      if (lane < k2) {  // rows: C = J' C (column `lane`)
        for (int m = 0; m < np; ++m) {
          const int p = pq[2 * m], q = pq[2 * m + 1];
          const double c = cs[2 * m], sn = cs[2 * m + 1];
          const double sp = Cm[p * k2 + lane], sq = Cm[q * k2 + lane];
          Cm[p * k2 + lane] = c * sp - sn * sq;
          Cm[q * k2 + lane] = sn * sp + c * sq;
        }
      }
      __syncwarp();
    }
  }
  // the kb largest eigenvalues among the kept directions (a dropped index keeps U = e_j, C_jj = 0)
  if (lane == 0) {
    int nk = 0;
    for (int i = 0; i < k2; ++i)
      if (!s_drop[i]) s_idx[nk++] = i;
    for (int i = 1; i < nk; ++i) {
      const int v = s_idx[i];
      int j = i - 1;
      while (j >= 0 && Cm[s_idx[j] * k2 + s_idx[j]] < Cm[v * k2 + v]) {
        s_idx[j + 1] = s_idx[j];
        --j;
      }
      s_idx[j + 1] = v;
    }
    for (int i = nk; i < k2; ++i) s_idx[i] = s_idx[nk > 0 ? nk - 1 : 0];
  }
  __syncwarp();
  // Z = L^-T U(:, idx): lane c solves column c (into T, then Zout)
  for (int c = lane; c < kb; c += 32) {
    const int src = s_idx[c];
    for (int i = k2 - 1; i >= 0; --i) {
      double v = U[i * k2 + src];
      for (int q = i + 1; q < k2; ++q) v -= L[q * k2 + i] * T[q * k2 + c];
      T[i * k2 + c] = v / L[i * k2 + i];
    }
  }
  __syncwarp();
  for (int e = lane; e < k2 * kb; e += 32) Zout[e] = T[(e / kb) * k2 + (e % kb)];
  __syncwarp();
}

// The whole FP32 block (b columns, the nev wanted plus guard vectors) is refined: block steps of
// Rayleigh-Ritz on [X, A X - X diag(l)] with FP64 products from the FP64 input, until the FP64 residuals of
// the nev leading pairs meet tol (or `steps` steps).  The guard columns keep the nearby part of the
// spectrum inside the search space, so each step removes the error along it instead of only damping it.
// One matrix (index mi, order n) from its FP32 block in d.X32.  Xs: BE_NMAX x BE_B doubles of shared memory
// (the right-hand block of a product); arena: 4 BR_K2^2 + BR_K2 BE_B doubles of shared memory (the pencil).
__device__ void be_refine_one(const RefineDev& d, int mi, int n, double* Xs, double* arena) {
  __shared__ double s_red[BE_T / 32];
  __shared__ double s_lam[2 * BE_B];
  __shared__ double s_cs[BR_K2];
  __shared__ int s_pq[BR_K2], s_idx[BR_K2];
  double* s_G = arena;
  double* s_M = s_G + BR_K2 * BR_K2;
  double* s_L = s_M + BR_K2 * BR_K2;
  double* s_T = s_L + BR_K2 * BR_K2;
  double* s_Z = s_T + BR_K2 * BR_K2;
  double* br_sm = Xs;
  const int tid = threadIdx.x;
  const int kb = d.b, k2 = 2 * d.b, nev = d.nev;
  double* Sx = d.scratch + (size_t)blockIdx.x * 3 * BE_NMAX * BR_K2;  // [X | R] (n x 2 kb)
  double* Sa = Sx + (size_t)BE_NMAX * BR_K2;                          // A [X | R]
  double* Sy = Sa + (size_t)BE_NMAX * BR_K2;                          // new X, A X
  {
    const double* A = d.A64 + d.off[mi];
    const float* X32 = d.X32 + d.xoff[mi];
    for (int e = tid; e < n * kb; e += BE_T) Sx[e] = (double)X32[e];
    __syncthreads();
    br_matmul(n, kb, A, Sx, Sa, br_sm);
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
      br_matmul(n, kb, A, Sx + (size_t)kb * n, Sa + (size_t)kb * n, br_sm);
      {
        // G = S' A S and M = S' S (both symmetric: the upper triangles, mirrored), one warp per entry
        const int lane = tid & 31, wid = tid >> 5;
        const int ntri = k2 * (k2 + 1) / 2;
        for (int e = wid; e < 2 * ntri; e += BE_T / 32) {
          const int which = e / ntri;
          int pr = e % ntri, r = 0;
          while (pr >= k2 - r) {
            pr -= k2 - r;
            ++r;
          }
          const int c = r + pr;
          const double* Bc = which ? Sx : Sa;
          double acc = 0.0;
          for (int i = lane; i < n; i += 32) acc = fma(Sx[i + r * n], Bc[i + c * n], acc);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) {
            double* D = which ? s_M : s_G;
            D[r * k2 + c] = acc;
            D[c * k2 + r] = acc;
          }
        }
      }
      __syncthreads();
      if (tid < 32) br_rayleigh_ritz_warp(k2, kb, s_G, s_M, s_L, s_T, s_Z, s_cs, s_pq, s_idx);
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


template <class T16>
__global__ void __launch_bounds__(BE_T, 1) k_batch_si(BatchDev d) {
  extern __shared__ __align__(128) float be_sm[];
  float* V = be_sm;                  // BE_NMAX x BE_B
  float* W = V + BE_NMAX * BE_B;     // BE_NMAX x BE_B
  unsigned char* ring = reinterpret_cast<unsigned char*>(W + BE_NMAX * BE_B);  // BE_NS x BE_STAGE
  __shared__ uint64_t s_full[BE_NS], s_empty[BE_NS];
  __shared__ float s_red[BE_T / 32 * BE_B];
  __shared__ int s_redi[BE_T / 32 * BE_B];
  __shared__ float s_c[BE_B];
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
  if (tid == 0) {
    for (int st = 0; st < BE_NS; ++st) {
      tc::mbar_init(&s_full[st], 1);
      tc::mbar_init(&s_empty[st], BE_T / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  BeRing rg{ring, s_full, s_empty, 0u, d.err};
  while (true) {
    if (tid == 0) s_job = (int)atomicAdd(d.queue, 1u);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= d.count) return;
    const int mi = d.order[job];
    if (tid == 0) d.tstart[mi] = tc_globaltimer();
    const int n = (int)d.n[mi];
    const int ld = (n + 7) & ~7;
    const int64_t off = d.offp[mi];
    const T16* A16 = reinterpret_cast<const T16*>(d.A16) + off;
    const float* A32 = d.A32 + off;
    // start block: Gaussian-like draws (sum of uniforms) from the matrix's key, scaled to unit maximum
    for (int e = tid; e < n * BE_B; e += BE_T) {
      const int i = e / BE_B, c = be_col(e);
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
        if (!(phase == 0 ? be_matmul<T16>(n, ld, A16, V, W, rg) : be_matmul<float>(n, ld, A32, V, W, rg))) return;
        be_colmax(n, b, W, s_piv, s_red, s_redi);
        for (int e = tid; e < n * BE_B; e += BE_T) {
          const int c = be_col(e);
          const float pv = s_piv[c];
          V[e] = (c < b && pv != 0.f) ? W[e] / pv : 0.f;
        }
        __syncthreads();
      }
      // ---- Hessenberg basis of V (in place): MGS order, pivot on the first largest entry.  The
      //      coefficients of column j come from a forward substitution on the pivot rows (thread 0, the
      //      same fused multiply-adds in the same order as the column-by-column eliminations), then one
      //      pass updates the column and finds its pivot ----
      for (int j = 0; j < b; ++j) {
        if (tid == 0) {
          for (int l = 0; l < j; ++l) {
            float cl = 0.f;
            if (s_sel[l]) {
              const int pr = s_perm[l];
              cl = V[be_at(pr, j)];
              for (int l2 = 0; l2 < l; ++l2) cl = fmaf(-s_c[l2], V[be_at(pr, l2)], cl);
            }
            s_c[l] = cl;
          }
        }
        __syncthreads();
        float bv = -1.f;
        int bi = 0x7fffffff;
        for (int i = tid; i < n; i += BE_T) {
          float v = V[be_at(i, j)];
          for (int l = 0; l < j; ++l) v = fmaf(-s_c[l], V[be_at(i, l)], v);
          V[be_at(i, j)] = v;
          const float a = fabsf(v);
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
          s_piv[j] = keep ? V[be_at(ii, j)] : 0.f;
        }
        __syncthreads();
        const float pv = s_piv[j];
        for (int i = tid; i < n; i += BE_T) V[be_at(i, j)] = (pv != 0.f) ? V[be_at(i, j)] / pv : 0.f;
        __syncthreads();
      }
      // ---- Rayleigh-Ritz: W = A Q, G = Q' W, M = Q' Q (64-row FP32 chunks summed in FP64) ----
      if (!(phase == 0 ? be_matmul<T16>(n, ld, A16, V, W, rg) : be_matmul<float>(n, ld, A32, V, W, rg))) return;
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
              for (int i = ch * 64; i < i1; ++i) s = fmaf(V[be_at(i, r)], which ? V[be_at(i, c)] : W[be_at(i, c)], s);
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
        {
          // Cholesky of M + tau I, row-major lower factor in s_L; lane i computes L(i, j) of column j
          double mx = 0.0;
          for (int i = 0; i < b; ++i) mx = fmax(mx, s_M[i * BE_B + i]);
          const double tau = 1e-12 * mx + 1e-300;
          for (int e = lane; e < BE_B * BE_B; e += 32) s_L[e] = 0.0;
          __syncwarp();
          for (int j = 0; j < b; ++j) {
            double dj = s_M[j * BE_B + j] + tau;
            for (int k = 0; k < j; ++k) dj -= s_L[j * BE_B + k] * s_L[j * BE_B + k];
            dj = sqrt(fmax(dj, 1e-300));
            double lij = 0.0;
            if (lane > j && lane < b) {
              double v = s_M[lane * BE_B + j];
              for (int k = 0; k < j; ++k) v -= s_L[lane * BE_B + k] * s_L[j * BE_B + k];
              lij = v / dj;
            }
            __syncwarp();
            if (lane > j && lane < b) s_L[lane * BE_B + j] = lij;
            if (lane == 0) s_L[j * BE_B + j] = dj;
            __syncwarp();
          }
        }
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
          q[c] = V[be_at(i, c)];
          a[c] = W[be_at(i, c)];
        }
#pragma unroll 1
        for (int c = 0; c < BE_B; ++c) {
          float x = 0.f, ax = 0.f;
#pragma unroll
          for (int r = 0; r < BE_B; ++r) {
            x = fmaf(q[r], s_Z[r * BE_B + c], x);
            ax = fmaf(a[r], s_Z[r * BE_B + c], ax);
          }
          V[be_at(i, c)] = (c < b) ? x : 0.f;
          W[be_at(i, c)] = (c < b) ? ax : 0.f;
        }
      }
      __syncthreads();
      float maxres = 0.f;
      const float lmax = fmaxf(fabsf(s_lam[0]), 1e-30f);
      {
        // residual and vector norms of the nev leading columns in one pass (sums in a fixed order)
        float rr[BE_NEV], xx[BE_NEV];
#pragma unroll
        for (int c = 0; c < BE_NEV; ++c) rr[c] = xx[c] = 0.f;
        for (int i = tid; i < n; i += BE_T) {
#pragma unroll
          for (int c = 0; c < BE_NEV; ++c) {
            const float x = V[be_at(i, c)];
            const float r = W[be_at(i, c)] - s_lam[c] * x;
            rr[c] = fmaf(r, r, rr[c]);
            xx[c] = fmaf(x, x, xx[c]);
          }
        }
#pragma unroll
        for (int c = 0; c < BE_NEV; ++c)
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            rr[c] += __shfl_xor_sync(0xffffffffu, rr[c], o);
            xx[c] += __shfl_xor_sync(0xffffffffu, xx[c], o);
          }
        if ((tid & 31) == 0)
#pragma unroll
          for (int c = 0; c < BE_NEV; ++c) {
            s_red[(tid >> 5) * BE_B + c] = rr[c];
            s_red[(tid >> 5) * BE_B + BE_NEV + c] = xx[c];
          }
        __syncthreads();
        for (int c = 0; c < d.nev; ++c) {
          float r2 = 0.f, x2 = 0.f;
          for (int w = 0; w < BE_T / 32; ++w) {
            r2 += s_red[w * BE_B + c];
            x2 += s_red[w * BE_B + BE_NEV + c];
          }
          maxres = fmaxf(maxres, (x2 > 0.f) ? sqrtf(r2 / x2) / lmax : INFINITY);
        }
        __syncthreads();
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
        const int i = e / BE_B, c = be_col(e);
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
      const int i = e / BE_B, c = be_col(e);
      X[i + (int64_t)c * n] = V[e];
    }
    if (tid < BE_B) d.lam[(int64_t)mi * BE_B + tid] = (tid < b) ? s_lam[tid] : 0.f;
    if (tid == 0) {
      d.iters[mi] = it;
      d.phase2[mi] = p2;
    }
    __syncthreads();
    // ---- FP64 refinement of this matrix by the same CTA: the product block in the V / W area, the
    //      pencil in the ring (no copy is in flight between products) ----
    be_refine_one(d.rf, mi, n, reinterpret_cast<double*>(be_sm), reinterpret_cast<double*>(ring));
    // the ring was written through the generic proxy: order that before the next bulk copies into it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
}

// The FP32 and 16-bit working copies of every matrix, one CTA per matrix: column-major with the leading
// dimension rounded up to 8 (zero rows below n) at the padded offsets, each value rounded once from FP64.
template <class T16>
__global__ void k_be_pack(const int64_t* __restrict__ n, const int64_t* __restrict__ off,
                          const int64_t* __restrict__ offp, const double* __restrict__ A, float* __restrict__ A32,
                          T16* __restrict__ A16) {
  const int mi = blockIdx.x;
  const int nn = (int)n[mi], ld = (nn + 7) & ~7;
  const double* src = A + off[mi];
  float* d32 = A32 + offp[mi];
  T16* d16 = A16 + offp[mi];
  const int64_t total = (int64_t)nn * ld;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
    const int j = (int)(e / ld), i = (int)(e % ld);
    const double v = (i < nn) ? src[(int64_t)j * nn + i] : 0.0;
    d32[e] = (float)v;
    d16[e] = from_c<T16, double>(v);
  }
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
  std::vector<int64_t> offp(count);
  for (int i = 0; i < count; ++i) {
    if (n_host[i] < b || n_host[i] > BE_NMAX || offset_host[i] < 0) return OFRR_ERR_BLAS_INVALID_SIZE;
    offp[i] = total;
    total += n_host[i] * ((n_host[i] + 7) & ~7);  // padded copies: ld = n rounded up to 8
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
  int64_t* doffp = ws_get<int64_t>(ctx, (size_t)count, &st);
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
  if (!A32 || !A16 || !X32 || !lam32 || !dn || !doff || !doffp || !dxo || !dxo64 || !dorder || !dit || !dlam || !dres ||
      !queues || !scratch || !times)
    return st;
  OFRR_CUDA(cudaMemcpyAsync(dn, n_host, sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(doff, offset_host, sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(doffp, offp.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(dxo, xo32.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(dxo64, xo64.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(dorder, order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_CUDA(cudaMemsetAsync(queues, 0, 2 * sizeof(unsigned int), ctx->stream));
  // the FP32 and 16-bit copies of every matrix (one pass over the FP64 input)
  if (t16 == OFRR_F16) k_be_pack<__half><<<count, 256, 0, ctx->stream>>>(dn, doff, doffp, A, A32, (__half*)A16);
  else k_be_pack<__nv_bfloat16><<<count, 256, 0, ctx->stream>>>(dn, doff, doffp, A, A32, (__nv_bfloat16*)A16);
  OFRR_LAUNCHED(ctx, "k_be_pack");
  BatchDev d{};
  d.n = dn;
  d.offp = doffp;
  d.err = ctx->dev_flags + kFlagTcWait;
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
  r.count = count;
  r.nev = nev;
  r.b = b;
  r.steps = 12;
  r.tol = opt->tol > 0 ? opt->tol : 1e-7;
  d.rf = r;
  const size_t smem = (size_t)2 * BE_NMAX * BE_B * sizeof(float) + (size_t)BE_NS * BE_STAGE;
  if (t16 == OFRR_F16) {
    OFRR_TRY(allow_smem(k_batch_si<__half>));
    k_batch_si<__half><<<grid, BE_T, smem, ctx->stream>>>(d);
  } else {
    OFRR_TRY(allow_smem(k_batch_si<__nv_bfloat16>));
    k_batch_si<__nv_bfloat16><<<grid, BE_T, smem, ctx->stream>>>(d);
  }
  OFRR_LAUNCHED(ctx, "k_batch_si");
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
