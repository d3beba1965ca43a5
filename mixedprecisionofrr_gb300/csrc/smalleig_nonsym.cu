// Small nonsymmetric projected eigenproblems: eig(G, M + tau I) for the Krylov Rayleigh-Ritz step of
// arnoldi_hess_eig.m:93-95 (eig_rr.m:52-55 with a nonsymmetric operator) and for the upper
// Hessenberg matrix of the orthogonal Arnoldi comparison path (arnoldi_mgs_eig.m:95-100).
//
// The pencil is reduced to a standard problem with the FP64 Cholesky factor of M + tau I
// (C = L^-1 G L^-T, smalleig_fast.cu's kernels); C is then solved in FP32 on one warp by the
// classical dense algorithm: Householder reduction to upper Hessenberg form with the
// transformations accumulated, Francis double-shift QR iteration to real Schur form (with the
// EISPACK/JAMA exceptional shifts at 10 and 30 iterations), and back substitution on the
// quasi-triangular factor for the eigenvectors (complex pairs in real arithmetic).  Scalar
// decisions are computed redundantly by every lane from shared memory, so the whole warp follows
// one control flow; the O(n) row and column updates are spread over the lanes.  The eigenvectors
// of the quasi-triangular factor are found one per lane (each lane owns one eigenvalue).
//
// Outputs follow the oracle's convention for real arithmetic: eigenvalues are the real parts, an
// eigenvector of a complex pair is the real part of the complex eigenvector, every vector has unit
// 2-norm, and pairs are sorted by descending real part (stable).  Accuracy is FP32 relative to
// ||C||; the callers are the 16-bit/32-bit Krylov bases of the mixed schedule.
#include "ofrr_internal.cuh"

namespace ofrr {

constexpr int NS_MAX = 128;

template <class T>
__device__ __forceinline__ void cdivf(T xr, T xi, T yr, T yi, T& cr, T& ci) {
  T r, d;
  if (fabs(yr) > fabs(yi)) {
    r = yi / yr;
    d = yr + r * yi;
    cr = (xr + r * xi) / d;
    ci = (xi - r * xr) / d;
  } else {
    r = yr / yi;
    d = yi + r * yr;
    cr = (r * xr + xi) / d;
    ci = (r * xi - xr) / d;
  }
}

// One warp.  C: n x n (FP64, ld ldc).  Outputs: wr, wi (n), X (n x n, FP64, ld n): eigenvectors of C
// (real parts, unit norm), unsorted; *flag = 1 when the QR iteration did not converge.
// VEC = false: eigenvalues only (EISPACK hqr instead of hqr2): no transformations accumulated, the QR
// sweeps restricted to the active block, no eigenvectors (X is not written)
template <class T, bool VEC = true>
__global__ void __launch_bounds__(32) k_nonsym_eig(int nn, const double* __restrict__ C, int ldc,
                                                       double* __restrict__ wr, double* __restrict__ wi,
                                                       double* __restrict__ X, int* __restrict__ flag,
                                                       int pair_imag) {
  extern __shared__ unsigned char sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  const int ld = nn + 1;
  T* H = sm;             // n x n (row i, column j at i + j * ld)
  T* V = H + nn * ld;    // Schur vectors
  T* Y = V + nn * ld;    // eigenvectors of the quasi-triangular factor
  T* ort = Y + nn * ld;  // n
  T* d = ort + nn;       // n
  T* e = d + nn;         // n
  const int lane = threadIdx.x;
#define HH(i, j) H[(i) + (j) * ld]
#define VV(i, j) V[(i) + (j) * ld]
#define YY(i, j) Y[(i) + (j) * ld]
  for (int idx = lane; idx < nn * nn; idx += 32) {
    const int i = idx % nn, j = idx / nn;
    HH(i, j) = (T)C[i + (size_t)j * ldc];
    VV(i, j) = (i == j) ? T(1.) : T(0.);
    YY(i, j) = T(0.);
  }
  __syncwarp();
  const int low = 0, high = nn - 1;
  // ---- Householder reduction to upper Hessenberg form ----
  for (int m = low + 1; m <= high - 1; ++m) {
    T scale = T(0.);
    for (int i = m + lane; i <= high; i += 32) scale += fabs(HH(i, m - 1));
    for (int o = 16; o > 0; o >>= 1) scale += __shfl_xor_sync(0xffffffffu, scale, o);
    if (scale == T(0.)) continue;
    T h = T(0.);
    for (int i = m + lane; i <= high; i += 32) {
      ort[i] = HH(i, m - 1) / scale;
      h += ort[i] * ort[i];
    }
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    __syncwarp();
    T g = sqrt(h);
    if (ort[m] > T(0.)) g = -g;
    h = h - ort[m] * g;
    __syncwarp();
    if (lane == 0) ort[m] = ort[m] - g;
    __syncwarp();
    // H = (I - u u'/h) H (I - u u'/h)
    for (int j = m + lane; j < nn; j += 32) {
      T f = T(0.);
      for (int i = high; i >= m; --i) f += ort[i] * HH(i, j);
      f /= h;
      for (int i = m; i <= high; ++i) HH(i, j) -= f * ort[i];
    }
    __syncwarp();
    for (int i = lane; i <= high; i += 32) {
      T f = T(0.);
      for (int j = high; j >= m; --j) f += ort[j] * HH(i, j);
      f /= h;
      for (int j = m; j <= high; ++j) HH(i, j) -= f * ort[j];
    }
    __syncwarp();
    if (lane == 0) {
      ort[m] = scale * ort[m];
      HH(m, m - 1) = scale * g;
    }
    __syncwarp();
  }
  // accumulate the transformations (the reflectors below the subdiagonal and in ort)
  for (int m = high - 1; VEC && m >= low + 1; --m) {
    if (HH(m, m - 1) == T(0.)) continue;
    for (int i = m + 1 + lane; i <= high; i += 32) ort[i] = HH(i, m - 1);
    __syncwarp();
    for (int j = m + lane; j <= high; j += 32) {
      T g = T(0.);
      for (int i = m; i <= high; ++i) g += ort[i] * VV(i, j);
      g = (g / ort[m]) / HH(m, m - 1);  // double division avoids underflow
      for (int i = m; i <= high; ++i) VV(i, j) += g * ort[i];
    }
    __syncwarp();
  }
  for (int idx = lane; idx < nn * nn; idx += 32) {  // clear the reflector storage below the subdiagonal
    const int i = idx % nn, j = idx / nn;
    if (i > j + 1) HH(i, j) = T(0.);
  }
  __syncwarp();

  // ---- Francis double-shift QR to real Schur form (EISPACK hqr2) ----
  const T eps = (sizeof(T) == 8) ? T(2.220446049250313e-16) : T(1.1920929e-07);
  int n = nn - 1;
  T exshift = T(0.), p = T(0.), q = T(0.), r = T(0.), s = T(0.), z = T(0.), t, w, x, y;
  T norm = T(0.);
  for (int i = 0; i < nn; ++i)
    for (int j = (i > 0 ? i - 1 : 0); j < nn; ++j) norm += fabs(HH(i, j));
  int iter = 0, total_iter = 0;
  const int max_total = 40 * nn;
  bool failed = false;
  while (n >= low) {
    int l = n;
    while (l > low) {
      s = fabs(HH(l - 1, l - 1)) + fabs(HH(l, l));
      if (s == T(0.)) s = norm;
      if (fabs(HH(l, l - 1)) < eps * s) break;
      --l;
    }
    if (l == n) {  // one root
      const T hn = HH(n, n) + exshift;
      __syncwarp();
      if (lane == 0) {
        HH(n, n) = hn;
        d[n] = hn;
        e[n] = T(0.);
      }
      __syncwarp();
      --n;
      iter = 0;
    } else if (l == n - 1) {  // two roots
      w = HH(n, n - 1) * HH(n - 1, n);
      p = (HH(n - 1, n - 1) - HH(n, n)) / T(2.);
      q = p * p + w;
      z = sqrt(fabs(q));
      const T hnn = HH(n, n) + exshift, hmm = HH(n - 1, n - 1) + exshift;
      __syncwarp();
      if (lane == 0) {
        HH(n, n) = hnn;
        HH(n - 1, n - 1) = hmm;
      }
      __syncwarp();
      x = hnn;
      if (q >= T(0.)) {  // real pair
        z = (p >= T(0.)) ? p + z : p - z;
        const T dn1 = x + z;
        const T dn = (z != T(0.)) ? x - w / z : dn1;
        x = HH(n, n - 1);
        s = fabs(x) + fabs(z);
        p = x / s;
        q = z / s;
        r = sqrt(p * p + q * q);
        p /= r;
        q /= r;
        __syncwarp();
        if (lane == 0) {
          d[n - 1] = dn1;
          d[n] = dn;
          e[n - 1] = T(0.);
          e[n] = T(0.);
        }
        for (int j = n - 1 + lane; VEC && j < nn; j += 32) {  // row modification
          const T zz = HH(n - 1, j);
          HH(n - 1, j) = q * zz + p * HH(n, j);
          HH(n, j) = q * HH(n, j) - p * zz;
        }
        __syncwarp();
        for (int i = lane; VEC && i <= n; i += 32) {  // column modification
          const T zz = HH(i, n - 1);
          HH(i, n - 1) = q * zz + p * HH(i, n);
          HH(i, n) = q * HH(i, n) - p * zz;
        }
        for (int i = low + lane; VEC && i <= high; i += 32) {  // accumulate
          const T zz = VV(i, n - 1);
          VV(i, n - 1) = q * zz + p * VV(i, n);
          VV(i, n) = q * VV(i, n) - p * zz;
        }
        __syncwarp();
      } else {  // complex pair
        __syncwarp();
        if (lane == 0) {
          d[n - 1] = x + p;
          d[n] = x + p;
          e[n - 1] = z;
          e[n] = -z;
        }
        __syncwarp();
      }
      n -= 2;
      iter = 0;
    } else {  // no convergence yet: one double-shift step
      if (++total_iter > max_total) {
        failed = true;
        break;
      }
      x = HH(n, n);
      y = T(0.);
      w = T(0.);
      if (l < n) {
        y = HH(n - 1, n - 1);
        w = HH(n, n - 1) * HH(n - 1, n);
      }
      if (iter == 10) {  // Wilkinson's ad hoc shift
        exshift += x;
        __syncwarp();
        for (int i = low + lane; i <= n; i += 32) HH(i, i) -= x;
        __syncwarp();
        s = fabs(HH(n, n - 1)) + fabs(HH(n - 1, n - 2));
        x = y = T(0.75) * s;
        w = -T(0.4375) * s * s;
      }
      if (iter == 30) {  // the second ad hoc shift
        s = (y - x) / T(2.);
        s = s * s + w;
        if (s > T(0.)) {
          s = sqrt(s);
          if (y < x) s = -s;
          s = x - w / ((y - x) / T(2.) + s);
          __syncwarp();
          for (int i = low + lane; i <= n; i += 32) HH(i, i) -= s;
          __syncwarp();
          exshift += s;
          x = y = w = T(0.964);
        }
      }
      ++iter;
      // two consecutive small subdiagonal elements
      int m = n - 2;
      while (m >= l) {
        z = HH(m, m);
        r = x - z;
        s = y - z;
        p = (r * s - w) / HH(m + 1, m) + HH(m, m + 1);
        q = HH(m + 1, m + 1) - z - r - s;
        r = HH(m + 2, m + 1);
        s = fabs(p) + fabs(q) + fabs(r);
        p /= s;
        q /= s;
        r /= s;
        if (m == l) break;
        if (fabs(HH(m, m - 1)) * (fabs(q) + fabs(r)) <
            eps * (fabs(p) * (fabs(HH(m - 1, m - 1)) + fabs(z) + fabs(HH(m + 1, m + 1)))))
          break;
        --m;
      }
      __syncwarp();
      for (int i = m + 2 + lane; i <= n; i += 32) {
        HH(i, i - 2) = T(0.);
        if (i > m + 2) HH(i, i - 3) = T(0.);
      }
      __syncwarp();
      // double QR step on rows l..n and columns m..n
      for (int k = m; k <= n - 1; ++k) {
        const bool notlast = (k != n - 1);
        if (k != m) {
          p = HH(k, k - 1);
          q = HH(k + 1, k - 1);
          r = notlast ? HH(k + 2, k - 1) : T(0.);
          x = fabs(p) + fabs(q) + fabs(r);
          if (x == T(0.)) continue;
          p /= x;
          q /= x;
          r /= x;
        }
        s = sqrt(p * p + q * q + r * r);
        if (p < T(0.)) s = -s;
        if (s == T(0.)) continue;
        const T hk = (k != m) ? -s * x : ((l != m) ? -HH(k, k - 1) : T(0.));
        const bool set_hk = (k != m) || (l != m);
        p = p + s;
        x = p / s;
        y = q / s;
        z = r / s;
        q = q / p;
        r = r / p;
        __syncwarp();
        if (lane == 0 && set_hk) HH(k, k - 1) = hk;
        const int jmax = VEC ? nn - 1 : n;  // values only: the active block's columns
        for (int j = k + lane; j <= jmax; j += 32) {  // row modification
          T pp = HH(k, j) + q * HH(k + 1, j);
          if (notlast) {
            pp += r * HH(k + 2, j);
            HH(k + 2, j) -= pp * z;
          }
          HH(k, j) -= pp * x;
          HH(k + 1, j) -= pp * y;
        }
        __syncwarp();
        const int imax = (n < k + 3) ? n : k + 3;
        for (int i = (VEC ? 0 : l) + lane; i <= imax; i += 32) {  // column modification
          T pp = x * HH(i, k) + y * HH(i, k + 1);
          if (notlast) {
            pp += z * HH(i, k + 2);
            HH(i, k + 2) -= pp * r;
          }
          HH(i, k) -= pp;
          HH(i, k + 1) -= pp * q;
        }
        for (int i = low + lane; VEC && i <= high; i += 32) {  // accumulate
          T pp = x * VV(i, k) + y * VV(i, k + 1);
          if (notlast) {
            pp += z * VV(i, k + 2);
            VV(i, k + 2) -= pp * r;
          }
          VV(i, k) -= pp;
          VV(i, k + 1) -= pp * q;
        }
        __syncwarp();
      }
    }
  }
  if (failed) {
    if (lane == 0 && flag) *flag = 1;
    for (int i = lane; i < nn; i += 32) {
      wr[i] = 0.0;
      wi[i] = 0.0;
    }
    for (int idx = lane; VEC && idx < nn * nn; idx += 32) X[idx] = 0.0;
    return;
  }
  __syncwarp();
  if (!VEC) {
    for (int j = lane; j < nn; j += 32) {
      wr[j] = (double)d[j];
      wi[j] = (double)e[j];
    }
    return;
  }
  // ---- eigenvectors of the quasi-triangular factor: one lane per eigenvalue ----
  if (norm != T(0.)) {
    for (int nv = nn - 1 - lane; nv >= 0; nv -= 32) {
      const T pr = d[nv], qi = e[nv];
      if (qi == T(0.)) {  // real vector
        int l = nv;
        YY(nv, nv) = T(1.);
        T zs = T(0.), ss = T(0.);
        for (int i = nv - 1; i >= 0; --i) {
          const T ww = HH(i, i) - pr;
          T rr = T(0.);
          for (int j = l; j <= nv; ++j) rr += HH(i, j) * YY(j, nv);
          if (e[i] < T(0.)) {
            zs = ww;
            ss = rr;
          } else {
            l = i;
            if (e[i] == T(0.)) {
              YY(i, nv) = (ww != T(0.)) ? -rr / ww : -rr / (eps * norm);
            } else {  // real 2x2 block
              const T xx = HH(i, i + 1), yy = HH(i + 1, i);
              const T qq = (d[i] - pr) * (d[i] - pr) + e[i] * e[i];
              const T tt = (xx * ss - zs * rr) / qq;
              YY(i, nv) = tt;
              YY(i + 1, nv) = (fabs(xx) > fabs(zs)) ? (-rr - ww * tt) / xx : (-ss - yy * tt) / zs;
            }
            const T tt = fabs(YY(i, nv));
            if ((eps * tt) * tt > T(1.))
              for (int j = i; j <= nv; ++j) YY(j, nv) /= tt;
          }
        }
      } else if (qi < T(0.)) {  // complex vector: columns nv-1 (real part) and nv (imaginary part)
        int l = nv - 1;
        if (fabs(HH(nv, nv - 1)) > fabs(HH(nv - 1, nv))) {
          YY(nv - 1, nv - 1) = qi / HH(nv, nv - 1);
          YY(nv - 1, nv) = -(HH(nv, nv) - pr) / HH(nv, nv - 1);
        } else {
          T cr, ci;
          cdivf(T(0.), -HH(nv - 1, nv), HH(nv - 1, nv - 1) - pr, qi, cr, ci);
          YY(nv - 1, nv - 1) = cr;
          YY(nv - 1, nv) = ci;
        }
        YY(nv, nv - 1) = T(0.);
        YY(nv, nv) = T(1.);
        T zs = T(0.), rs = T(0.), ss = T(0.);
        for (int i = nv - 2; i >= 0; --i) {
          T ra = T(0.), sa = T(0.);
          for (int j = l; j <= nv; ++j) {
            ra += HH(i, j) * YY(j, nv - 1);
            sa += HH(i, j) * YY(j, nv);
          }
          const T ww = HH(i, i) - pr;
          if (e[i] < T(0.)) {
            zs = ww;
            rs = ra;
            ss = sa;
          } else {
            l = i;
            T cr, ci;
            if (e[i] == T(0.)) {
              cdivf(-ra, -sa, ww, qi, cr, ci);
              YY(i, nv - 1) = cr;
              YY(i, nv) = ci;
            } else {
              const T xx = HH(i, i + 1), yy = HH(i + 1, i);
              T vr = (d[i] - pr) * (d[i] - pr) + e[i] * e[i] - qi * qi;
              const T vi = (d[i] - pr) * T(2.) * qi;
              if (vr == T(0.) && vi == T(0.))
                vr = eps * norm * (fabs(ww) + fabs(qi) + fabs(xx) + fabs(yy) + fabs(zs));
              cdivf(xx * rs - zs * ra + qi * sa, xx * ss - zs * sa - qi * ra, vr, vi, cr, ci);
              YY(i, nv - 1) = cr;
              YY(i, nv) = ci;
              if (fabs(xx) > fabs(zs) + fabs(qi)) {
                YY(i + 1, nv - 1) = (-ra - ww * YY(i, nv - 1) + qi * YY(i, nv)) / xx;
                YY(i + 1, nv) = (-sa - ww * YY(i, nv) - qi * YY(i, nv - 1)) / xx;
              } else {
                cdivf(-rs - yy * YY(i, nv - 1), -ss - yy * YY(i, nv), zs, qi, cr, ci);
                YY(i + 1, nv - 1) = cr;
                YY(i + 1, nv) = ci;
              }
            }
            const T tt = fmaxf(fabs(YY(i, nv - 1)), fabs(YY(i, nv)));
            if ((eps * tt) * tt > T(1.))
              for (int j = i; j <= nv; ++j) {
                YY(j, nv - 1) /= tt;
                YY(j, nv) /= tt;
              }
          }
        }
      }
    }
  }
  __syncwarp();
  // ---- back transformation X = V Y (upper part of Y), real parts, unit norm ----
  for (int j = lane; j < nn; j += 32) {
    // the vector for eigenvalue j: column j, or for the second member of a complex pair the real part
    // (column j - 1) of the pair's vector
    // (pair_imag: the imaginary part, column j, instead -- with the real part in column j - 1 the pair
    // then spans the real invariant subspace of the two eigenvalues)
    const int src = (e[j] < T(0.) && !pair_imag) ? j - 1 : j;
    const int top = (e[j] != T(0.)) ? ((e[j] > T(0.)) ? j + 1 : j) : j;  // last nonzero row of column src
    T nrm = T(0.);
    for (int i = 0; i < nn; ++i) {
      T zz = T(0.);
      for (int k = 0; k <= top; ++k) zz += VV(i, k) * YY(k, src);
      nrm += zz * zz;
      X[i + (size_t)j * nn] = (double)zz;
    }
    const double inv = (nrm > T(0.)) ? 1.0 / sqrt((double)nrm) : 0.0;
    for (int i = 0; i < nn; ++i) X[i + (size_t)j * nn] *= inv;
    wr[j] = (double)d[j];
    wi[j] = (double)e[j];
  }
#undef HH
#undef VV
#undef YY
}

// FP64 Newton refinement of the real eigenpairs from the FP32 solve, one CTA per pair.  With x
// normalised so that x_k = 1 at its largest entry k, Newton's method on (C - l I) x = 0, e_k' x = 1
// solves the bordered system [[C - l I, -x], [e_k', 0]] [dx; dl] = [-(C x - l x); 0] (Gaussian
// elimination with partial pivoting, FP64) and converges quadratically.  A step is kept only when it
// moves l by less than 1e-3 ||C||_F (the FP32 start is that close to its own eigenvalue, so a larger
// move means a jump to a neighbour) and reduces the residual.  Complex pairs keep the FP32 result.
constexpr int NR_T = 128;
__global__ void __launch_bounds__(NR_T) k_nonsym_refine_f64(int n, const double* __restrict__ C, double cnorm,
                                                            double* __restrict__ wr, const double* __restrict__ wi,
                                                            double* __restrict__ X, int steps) {
  extern __shared__ double smd[];
  const int N = n + 1, ld = N + 1;
  double* J = smd;             // N x N (+ padding), column-major
  double* rhs = J + N * ld;    // N
  double* x = rhs + N;         // n
  double* r = x + n;           // n (residual)
  double* xp = r + n;          // n (the last accepted vector)
  __shared__ ArgMaxK red[NR_T / 32];
  __shared__ double s_red[NR_T / 32];
  __shared__ int s_ok;
  const int j = blockIdx.x, tid = threadIdx.x;
  if (wi[j] != 0.0) return;
  double lam = wr[j];
  for (int i = tid; i < n; i += NR_T) x[i] = X[i + (size_t)j * n];
  __syncthreads();
  double res_prev = INFINITY, lam_prev = lam;
  for (int it = 0; it <= steps; ++it) {  // the last pass only checks the last step
    // normalise x_k = 1 at the largest entry
    ArgMaxK a{-1, 0x7fffffffffffffffLL};
    for (int i = tid; i < n; i += NR_T) {
      const long long key = amax_key(x[i]);
      if (key > a.key) a = ArgMaxK{key, i};
    }
    const ArgMaxK am = block_argmaxk(a, red);
    const int k = (am.key < 0) ? 0 : (int)am.i;
    const double xk = x[k];
    __syncthreads();
    if (xk == 0.0) break;
    for (int i = tid; i < n; i += NR_T) x[i] /= xk;
    __syncthreads();
    // residual r = C x - l x and its norm
    double rr = 0.0;
    for (int i = tid; i < n; i += NR_T) {
      double s = -lam * x[i];
      for (int l = 0; l < n; ++l) s = fma(C[i + (size_t)l * n], x[l], s);
      r[i] = s;
      rr = fma(s, s, rr);
    }
    for (int o = 16; o > 0; o >>= 1) rr += __shfl_xor_sync(0xffffffffu, rr, o);
    if ((tid & 31) == 0) s_red[tid >> 5] = rr;
    __syncthreads();
    double res = 0.0;
    for (int w = 0; w < NR_T / 32; ++w) res += s_red[w];
    res = sqrt(res);
    __syncthreads();
    if (!(res < res_prev)) {  // the last step did not help (or reached the FP64 floor): undo it
      if (it > 0) {
        for (int i = tid; i < n; i += NR_T) x[i] = xp[i];
        lam = lam_prev;
      }
      __syncthreads();
      break;
    }
    res_prev = res;
    lam_prev = lam;
    for (int i = tid; i < n; i += NR_T) xp[i] = x[i];
    if (it == steps) break;
    // bordered system
    for (int e = tid; e < N * N; e += NR_T) {
      const int i = e % N, l = e / N;
      double v;
      if (i < n && l < n) v = C[i + (size_t)l * n] - (i == l ? lam : 0.0);
      else if (i < n) v = -x[i];             // l == n
      else v = (l == k) ? 1.0 : 0.0;         // i == n
      J[i + l * ld] = v;
    }
    for (int i = tid; i < N; i += NR_T) rhs[i] = (i < n) ? -r[i] : 0.0;
    __syncthreads();
    // Gaussian elimination with partial pivoting
    if (tid == 0) s_ok = 1;
    for (int c = 0; c < N; ++c) {
      ArgMaxK b{-1, 0x7fffffffffffffffLL};
      for (int i = c + tid; i < N; i += NR_T) {
        const long long key = amax_key(J[i + c * ld]);
        if (key > b.key) b = ArgMaxK{key, i};
      }
      const ArgMaxK pv = block_argmaxk(b, red);
      const int p = (pv.key < 0) ? c : (int)pv.i;
      if (p != c) {
        for (int l = c + tid; l < N; l += NR_T) {
          const double t = J[c + l * ld];
          J[c + l * ld] = J[p + l * ld];
          J[p + l * ld] = t;
        }
        if (tid == 0) {
          const double t = rhs[c];
          rhs[c] = rhs[p];
          rhs[p] = t;
        }
      }
      __syncthreads();
      const double piv = J[c + c * ld];
      if (piv == 0.0) {
        if (tid == 0) s_ok = 0;
        break;
      }
      const double ip = 1.0 / piv;
      for (int i = c + 1 + tid; i < N; i += NR_T) {
        const double m = J[i + c * ld] * ip;
        for (int l = c + 1; l < N; ++l) J[i + l * ld] = fma(-m, J[c + l * ld], J[i + l * ld]);
        rhs[i] = fma(-m, rhs[c], rhs[i]);
      }
      __syncthreads();
    }
    __syncthreads();
    if (!s_ok) break;
    // back substitution (column-oriented): solution into rhs
    for (int c = N - 1; c >= 0; --c) {
      if (tid == 0) rhs[c] /= J[c + c * ld];
      __syncthreads();
      const double xc = rhs[c];
      for (int i = tid; i < c; i += NR_T) rhs[i] = fma(-J[i + c * ld], xc, rhs[i]);
      __syncthreads();
    }
    const double dl = rhs[n];
    if (!(fabs(dl) < 1e-3 * cnorm)) break;  // a jump to another eigenvalue: keep the previous pair
    for (int i = tid; i < n; i += NR_T) x[i] += rhs[i];
    lam += dl;
    __syncthreads();
  }
  // unit 2-norm and write back
  double ss = 0.0;
  for (int i = tid; i < n; i += NR_T) ss = fma(x[i], x[i], ss);
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  __syncthreads();
  if ((tid & 31) == 0) s_red[tid >> 5] = ss;
  __syncthreads();
  double nrm = 0.0;
  for (int w = 0; w < NR_T / 32; ++w) nrm += s_red[w];
  const double inv = (nrm > 0.0) ? 1.0 / sqrt(nrm) : 0.0;
  for (int i = tid; i < n; i += NR_T) X[i + (size_t)j * n] = x[i] * inv;
  if (tid == 0) wr[j] = lam;
}

__global__ void k_frob(int n, const double* __restrict__ C, double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) s = fma(C[e], C[e], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    *out = sqrt(t);
  }
}

// eig(C) for a nonsymmetric n x n C (FP64, ld n): wr/wi (n), X (n x n, ld n), unsorted.  refine: FP64
// Newton steps on the real pairs (FP64 bases); without it the pairs are FP32-accurate.
int nonsym_eig_dev(ofrr_ctx* ctx, int n, const double* C, double* wr, double* wi, double* X, bool refine,
                   bool pair_imag, bool values_only) {
  if (n <= 0) return OFRR_SUCCESS;
  if (n > NS_MAX) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (values_only) {  // FP32 eigenvalues (no vectors, no refinement)
    const size_t smem = ((size_t)3 * n * (n + 1) + 3 * (size_t)n) * sizeof(float);
    OFRR_TRY(allow_smem(k_nonsym_eig<float, false>));
    k_nonsym_eig<float, false><<<1, 32, smem, ctx->stream>>>(n, C, n, wr, wi, X, ctx->dev_flags + 3, 0);
    OFRR_LAUNCHED(ctx, "k_nonsym_eig_values_f32");
    return OFRR_SUCCESS;
  }
  // refine: the whole Hessenberg-QR in FP64 when it fits in shared memory (backward stable to FP64; the
  // Newton refinement below cannot separate clustered eigenvalues from an FP32 start), else FP32 + Newton
  const size_t smem64 = ((size_t)3 * n * (n + 1) + 3 * (size_t)n) * sizeof(double);
  if (refine && smem64 <= 227 * 1024) {
    OFRR_TRY(allow_smem(k_nonsym_eig<double>));
    k_nonsym_eig<double><<<1, 32, smem64, ctx->stream>>>(n, C, n, wr, wi, X, ctx->dev_flags + 3, pair_imag ? 1 : 0);
    OFRR_LAUNCHED(ctx, "k_nonsym_eig_f64");
    return OFRR_SUCCESS;
  }
  const size_t smem = ((size_t)3 * n * (n + 1) + 3 * (size_t)n) * sizeof(float);
  OFRR_TRY(allow_smem(k_nonsym_eig<float>));
  k_nonsym_eig<float><<<1, 32, smem, ctx->stream>>>(n, C, n, wr, wi, X, ctx->dev_flags + 3, pair_imag ? 1 : 0);
  OFRR_LAUNCHED(ctx, "k_nonsym_eig_f32");
  if (!refine) return OFRR_SUCCESS;
  // ||C||_F on the host side of the acceptance test: one small reduction, read back
  int st = OFRR_SUCCESS;
  WsScope scope(ctx);
  double* fro = ws_get<double>(ctx, 1, &st);
  if (!fro) return st;
  k_frob<<<1, 256, 0, ctx->stream>>>(n, C, fro);
  OFRR_LAUNCHED(ctx, "k_frob");
  double cn = 0.0;
  OFRR_CUDA(cudaMemcpyAsync(&cn, fro, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  const size_t smem2 = ((size_t)(n + 1) * (n + 2) + (n + 1) + 3 * (size_t)n) * sizeof(double);
  OFRR_TRY(allow_smem(k_nonsym_refine_f64));
  k_nonsym_refine_f64<<<n, NR_T, smem2, ctx->stream>>>(n, C, cn, wr, wi, X, 3);
  OFRR_LAUNCHED(ctx, "k_nonsym_refine_f64");
  return OFRR_SUCCESS;
}

}  // namespace ofrr
