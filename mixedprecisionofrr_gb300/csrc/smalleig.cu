// Small dense FP64 (generalized) symmetric eigenproblems on the device, one CTA per pencil.
//
// Replaces the host LAPACKE dsyev/dsygv wrappers of the reference (CPP/linalg/blas/mvops.cu:1601-1664)
// and MATLAB eig(VAV, VV + tau I) inside eig_rr.m:50-54 / svd_rr.m:58-77.
// Algorithm: Cholesky M = L L' (right-looking), C = L^-1 G L^-T (two forward substitutions, one
// thread per right-hand side), cyclic Jacobi on C with round-robin parallel ordering (n/2 disjoint
// rotations per round, Golub & Van Loan sym.Schur2 rotation), eigenvalue sort, U = L^-T W.
// Everything stays in shared memory when 3 n^2 doubles fit, otherwise in a global workspace.
// The eigenvectors are M-orthonormal (U' M U = I), the LAPACK sygv / MATLAB 'chol' normalisation.
#include "ofrr_internal.cuh"

namespace ofrr {

struct GeigParams {
  int n;
  const double* G;
  int ldg;
  const double* M;  // may be null (standard problem)
  int ldm;
  int symmetrize;
  int descending;
  double* w;   // out, n
  double* U;   // out, n x n (ldu)
  int ldu;
  double* gws;  // global workspace (3 n^2) when shared memory is too small
  int* flag;    // out: 1 if the Cholesky factor needed a clamp (near-singular M)
  int max_sweeps;
};

__device__ __forceinline__ int rr_index(int i, int r, int N) { return i == 0 ? 0 : ((i - 1 + r) % (N - 1)) + 1; }

__global__ void __launch_bounds__(512) k_geig_sym(GeigParams P) {
  extern __shared__ double sm[];
  const int n = P.n, tid = threadIdx.x, nt = blockDim.x;
  const bool in_smem = (P.gws == nullptr);
  double* C = in_smem ? sm : P.gws;
  double* W = C + (size_t)n * n;
  double* L = W + (size_t)n * n;
  __shared__ double s_c[160], s_s[160];
  __shared__ int s_p[160], s_q[160];
  __shared__ double s_red[32];
  __shared__ int s_stop;
  __shared__ double s_maxdiag;

  // ---- Cholesky of M (lower) ------------------------------------------------------
  const bool gen = (P.M != nullptr);
  if (gen) {
    for (int e = tid; e < n * n; e += nt) {
      int i = e % n, j = e / n;
      L[e] = (i >= j) ? P.M[i + (size_t)j * P.ldm] : 0.0;
    }
    __syncthreads();
    if (tid == 0) {
      double md = 0.0;
      for (int k = 0; k < n; ++k) md = fmax(md, fabs(L[k + (size_t)k * n]));
      s_maxdiag = md;
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
      if (tid == 0) {
        double d = L[k + (size_t)k * n];
        const double floor_d = s_maxdiag * 1e-15 + 1e-300;
        if (!(d > floor_d)) {
          d = floor_d;
          if (P.flag) *P.flag = 1;
        }
        L[k + (size_t)k * n] = sqrt(d);
      }
      __syncthreads();
      const double dk = L[k + (size_t)k * n];
      for (int i = k + 1 + tid; i < n; i += nt) L[i + (size_t)k * n] /= dk;
      __syncthreads();
      const int rem = n - k - 1;
      for (int e = tid; e < rem * rem; e += nt) {
        int i = k + 1 + e % rem, j = k + 1 + e / rem;
        if (i >= j) L[i + (size_t)j * n] -= L[i + (size_t)k * n] * L[j + (size_t)k * n];
      }
      __syncthreads();
    }
  }

  // ---- C = G (symmetrised), reduced by L when generalized -------------------------
  for (int e = tid; e < n * n; e += nt) {
    int i = e % n, j = e / n;
    double g = P.G[i + (size_t)j * P.ldg];
    if (P.symmetrize) g = 0.5 * (g + P.G[j + (size_t)i * P.ldg]);
    C[e] = g;
  }
  __syncthreads();
  if (gen) {
    // W <- L^-1 C   (column j solved by one thread)
    for (int j = tid; j < n; j += nt) {
      for (int i = 0; i < n; ++i) {
        double s = C[i + (size_t)j * n];
        for (int k = 0; k < i; ++k) s -= L[i + (size_t)k * n] * W[k + (size_t)j * n];
        W[i + (size_t)j * n] = s / L[i + (size_t)i * n];
      }
    }
    __syncthreads();
    // C <- L^-1 W'   (right-hand side j is row j of W)
    for (int j = tid; j < n; j += nt) {
      for (int i = 0; i < n; ++i) {
        double s = W[j + (size_t)i * n];
        for (int k = 0; k < i; ++k) s -= L[i + (size_t)k * n] * C[k + (size_t)j * n];
        C[i + (size_t)j * n] = s / L[i + (size_t)i * n];
      }
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {
      int i = e % n, j = e / n;
      if (i < j) {
        double a = 0.5 * (C[i + (size_t)j * n] + C[j + (size_t)i * n]);
        C[i + (size_t)j * n] = a;
        C[j + (size_t)i * n] = a;
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nt) W[e] = ((e % n) == (e / n)) ? 1.0 : 0.0;
  __syncthreads();

  // ---- cyclic Jacobi, round-robin ordering ------------------------------------------
  const int N = n + (n & 1);
  const int npair = N / 2;
  for (int sweep = 0; sweep < P.max_sweeps && n > 1; ++sweep) {
    // convergence test: off(C)^2 <= eps^2 * ||C||_F^2
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < n * n; e += nt) {
      double v = C[e] * C[e];
      tot += v;
      if ((e % n) != (e / n)) off += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_down_sync(0xffffffffu, off, o);
      tot += __shfl_down_sync(0xffffffffu, tot, o);
    }
    if ((tid & 31) == 0) s_red[tid >> 5] = off;
    __syncthreads();
    if (tid == 0) {
      double a = 0.0;
      for (int w = 0; w < (nt >> 5); ++w) a += s_red[w];
      s_red[0] = a;
    }
    __syncthreads();
    off = s_red[0];
    __syncthreads();
    if ((tid & 31) == 0) s_red[tid >> 5] = tot;
    __syncthreads();
    if (tid == 0) {
      double a = 0.0;
      for (int w = 0; w < (nt >> 5); ++w) a += s_red[w];
      s_stop = (off <= 1.0e-32 * a) ? 1 : 0;
    }
    __syncthreads();
    if (s_stop) break;
    for (int r = 0; r < N - 1; ++r) {
      for (int k = tid; k < npair; k += nt) {
        int p = rr_index(k, r, N), q = rr_index(N - 1 - k, r, N);
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = C[p + (size_t)q * n];
          if (apq != 0.0) {
            const double app = C[p + (size_t)p * n], aqq = C[q + (size_t)q * n];
            const double tau = (aqq - app) / (2.0 * apq);
            const double t = (tau >= 0.0) ? 1.0 / (tau + sqrt(1.0 + tau * tau)) : -1.0 / (-tau + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        s_p[k] = p;
        s_q[k] = (q < n) ? q : -1;
        s_c[k] = c;
        s_s[k] = s;
      }
      __syncthreads();
      // rows: C <- J' C
      for (int e = tid; e < npair * n; e += nt) {
        const int k = e / n, j = e % n;
        const int q = s_q[k];
        if (q < 0 || s_s[k] == 0.0) continue;
        const int p = s_p[k];
        const double c = s_c[k], s = s_s[k];
        const double ap = C[p + (size_t)j * n], aq = C[q + (size_t)j * n];
        C[p + (size_t)j * n] = c * ap - s * aq;
        C[q + (size_t)j * n] = s * ap + c * aq;
      }
      __syncthreads();
      // columns: C <- C J, W <- W J
      for (int e = tid; e < npair * n; e += nt) {
        const int k = e / n, i = e % n;
        const int q = s_q[k];
        if (q < 0 || s_s[k] == 0.0) continue;
        const int p = s_p[k];
        const double c = s_c[k], s = s_s[k];
        double ap = C[i + (size_t)p * n], aq = C[i + (size_t)q * n];
        C[i + (size_t)p * n] = c * ap - s * aq;
        C[i + (size_t)q * n] = s * ap + c * aq;
        ap = W[i + (size_t)p * n];
        aq = W[i + (size_t)q * n];
        W[i + (size_t)p * n] = c * ap - s * aq;
        W[i + (size_t)q * n] = s * ap + c * aq;
      }
      __syncthreads();
      for (int k = tid; k < npair; k += nt) {
        const int q = s_q[k];
        if (q >= 0 && s_s[k] != 0.0) {
          const int p = s_p[k];
          C[p + (size_t)q * n] = 0.0;
          C[q + (size_t)p * n] = 0.0;
        }
      }
      __syncthreads();
    }
  }

  // ---- sort and back-transform --------------------------------------------------------
  // rank of each eigenvalue (stable): descending or ascending
  for (int i = tid; i < n; i += nt) {
    const double di = C[i + (size_t)i * n];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double dj = C[j + (size_t)j * n];
      const bool before = P.descending ? (dj > di || (dj == di && j < i)) : (dj < di || (dj == di && j < i));
      rank += before ? 1 : 0;
    }
    P.w[rank] = di;
    // U(:, rank) = L^-T W(:, i)  (back substitution) or W(:, i)
    if (gen) {
      for (int r = n - 1; r >= 0; --r) {
        double s = W[r + (size_t)i * n];
        for (int k = r + 1; k < n; ++k) s -= L[k + (size_t)r * n] * P.U[k + (size_t)rank * P.ldu];
        P.U[r + (size_t)rank * P.ldu] = s / L[r + (size_t)r * n];
      }
    } else {
      for (int r = 0; r < n; ++r) P.U[r + (size_t)rank * P.ldu] = W[r + (size_t)i * n];
    }
  }
}

static int geig_launch(ofrr_ctx* ctx, GeigParams P) {
  const size_t need = (size_t)3 * P.n * P.n * sizeof(double);
  int st = OFRR_SUCCESS;
  size_t smem = 0;
  if (need <= 200 * 1024) {
    smem = need;
    P.gws = nullptr;
    OFRR_TRY(allow_smem(k_geig_sym));
  } else {
    P.gws = ws_get<double>(ctx, (size_t)3 * P.n * P.n, &st);
    if (!P.gws) return st;
  }
  k_geig_sym<<<1, 512, smem, ctx->stream>>>(P);
  OFRR_LAUNCHED(ctx, "k_geig_sym");
  return OFRR_SUCCESS;
}

int geig_dev(ofrr_ctx* ctx, int n, const double* G, int ldg, const double* M, int ldm, int symmetric, double* w,
             double* U, int ldu) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 300) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (!symmetric) return OFRR_ERR_NOT_IMPLEMENTED;
  WsScope scope(ctx);
  GeigParams P{};
  P.n = n;
  P.G = G;
  P.ldg = ldg;
  P.M = M;
  P.ldm = ldm;
  P.symmetrize = 1;
  P.descending = 1;
  P.w = w;
  P.U = U;
  P.ldu = ldu;
  P.flag = ctx->dev_flags + 1;
  P.max_sweeps = 30;
  return geig_launch(ctx, P);
}

int syev_dev(ofrr_ctx* ctx, int n, double* A, int lda, double* w) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 300) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double* U = ws_get<double>(ctx, (size_t)n * n, &st);
  if (!U) return st;
  GeigParams P{};
  P.n = n;
  P.G = A;
  P.ldg = lda;
  P.M = nullptr;
  P.symmetrize = 1;
  P.descending = 0;
  P.w = w;
  P.U = U;
  P.ldu = n;
  P.flag = ctx->dev_flags + 1;
  P.max_sweeps = 30;
  OFRR_TRY(geig_launch(ctx, P));
  OFRR_CUDA(cudaMemcpy2DAsync(A, lda * sizeof(double), U, n * sizeof(double), n * sizeof(double), n,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  return OFRR_SUCCESS;
}

int sygv_dev(ofrr_ctx* ctx, int n, double* A, int lda, double* B, int ldb, double* w) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > 300) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  double* U = ws_get<double>(ctx, (size_t)n * n, &st);
  if (!U) return st;
  GeigParams P{};
  P.n = n;
  P.G = A;
  P.ldg = lda;
  P.M = B;
  P.ldm = ldb;
  P.symmetrize = 1;
  P.descending = 0;
  P.w = w;
  P.U = U;
  P.ldu = n;
  P.flag = ctx->dev_flags + 1;
  P.max_sweeps = 30;
  OFRR_TRY(geig_launch(ctx, P));
  OFRR_CUDA(cudaMemcpy2DAsync(A, lda * sizeof(double), U, n * sizeof(double), n * sizeof(double), n,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  return OFRR_SUCCESS;
}

}  // namespace ofrr

using namespace ofrr;

extern "C" int ofrr_syev(ofrr_ctx* ctx, int n, double* A, int lda, double* w) {
  if (!ctx || n < 0 || (n > 0 && (!A || !w || lda < n))) return OFRR_ERR_INVALID_ARGUMENT;
  return syev_dev(ctx, n, A, lda, w);
}

extern "C" int ofrr_sygv(ofrr_ctx* ctx, int n, double* A, int lda, double* B, int ldb, double* w) {
  if (!ctx || n < 0 || (n > 0 && (!A || !B || !w || lda < n || ldb < n))) return OFRR_ERR_INVALID_ARGUMENT;
  return sygv_dev(ctx, n, A, lda, B, ldb, w);
}
