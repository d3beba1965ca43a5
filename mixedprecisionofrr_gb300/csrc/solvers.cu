// Host orchestration of the projection solvers (all device work on ctx->stream).
//
// Behavioural definitions (the reference's C++ solver bodies are stubs):
//   si_eig       MATLAB/+src/+subspace/subspace_iter_eig.m:50-68 (+ test2 wrappers, +tests/+test2/test.m:358-397)
//   rr_eig       MATLAB/+src/+rr/eig_rr.m:46-57
//   si_svd       MATLAB/+src/+subspace/subspace_iter_svd.m:53-77
//   rr_svd       MATLAB/+src/+rr/svd_rr.m:50-91
//   arnoldi_eig  MATLAB/+src/+krylov/arnoldi_hess_eig.m:51-107 (Hessenberg process)
// Convergence control (tol, nev) is new: the reference runs a fixed maxiter.
#include "ofrr_internal.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

namespace ofrr {

int hess_krylov_first(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int ncolmax, void* V, int64_t ldv,
                      double select_tol, int* select, int* perm, void* pivrows, void* pvals, double* R, int* stop);
size_t mgs_scratch_bytes();
int mgs_step(ofrr_ctx* ctx, ofrr_dtype po, ofrr_dtype pc, int64_t n, int i, void* V, int64_t ldv, bool reorth,
             double stol, int* stop, void* scratch);
int hess_krylov_step(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int ncolmax, int i, void* V,
                     int64_t ldv, double select_tol, int* select, int* perm, void* pivrows, void* pvals, double* R,
                     int* stop);
int hess_scale_col(ofrr_ctx* ctx, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int i, void* V, int64_t ldv,
                   const int* select, const void* pvals, const int* stop);

namespace {

// operator wrapper: dense copies per storage type are made once per solve
struct Op {
  const ofrr_operator* A;
  const void* dense[4] = {nullptr, nullptr, nullptr, nullptr};
  int64_t ld[4] = {0, 0, 0, 0};
  int64_t m() const { return A->nrows; }
  int64_t n() const { return A->ncols; }

  int dense_as(ofrr_ctx* ctx, ofrr_dtype t, const void** p, int64_t* l) {
    if (!dense[t]) {
      if (A->dtype == t) {
        dense[t] = A->data;
        ld[t] = A->ld;
      } else {
        // 16-bit copies with the leading dimension rounded up to 8 elements: 16-byte aligned columns, as
        // the tensor-core product's TMA needs, whatever the row count
        int st = OFRR_SUCCESS;
        const int64_t ldp = (dtype_size(t) == 2) ? ((m() + 7) & ~int64_t(7)) : m();
        void* w = ws_alloc(ctx, (size_t)ldp * n() * dtype_size(t), &st);
        if (!w) return st;
        OFRR_TRY(cast_impl(ctx, A->dtype, t, m(), n(), A->data, A->ld, w, ldp));
        dense[t] = w;
        ld[t] = ldp;
      }
    }
    *p = dense[t];
    *l = ld[t];
    return OFRR_SUCCESS;
  }

  // Y = op(A) X: dense A taken in storage type ta (the MATLAB code casts A to the output precision
  // once, subspace_iter_eig.m:56-58), computed in tc, stored as ty.
  int apply(ofrr_ctx* ctx, int trans, ofrr_dtype ta, ofrr_dtype tx, const void* X, int64_t ldx, int64_t nrhs,
            ofrr_dtype tc, ofrr_dtype ty, void* Y, int64_t ldy) {
    if (A->kind == OFRR_OP_CSR) {
      if (trans && have_csrT) return csrmm_impl(ctx, &csrT, 0, tx, tc, ty, nrhs, X, ldx, Y, ldy);
      return csrmm_impl(ctx, &A->csr, trans, tx, tc, ty, nrhs, X, ldx, Y, ldy);
    }
    const void* Ad = nullptr;
    int64_t lda = 0;
    const int64_t M = trans ? n() : m(), K = trans ? m() : n();
    if (ctx->emulate_f64 && ta == OFRR_F64 && tx == OFRR_F64 && tc == OFRR_F64 && ty == OFRR_F64 &&
        (trans ? have_sA : have_sAt)) {
      // FP64-accurate A V / A' U from the cached digit stacks of A (exact BF16 slices, tcgen05)
      return sliced_gemm_tn(ctx, trans ? sA : sAt, nrhs, (const double*)X, ldx, (double*)Y, ldy);
    }
    if (!trans && tc == OFRR_F32 && ta == tx && (ta == OFRR_F16 || ta == OFRR_BF16)) {
      // A V as (A')' V on the K-contiguous copy of A: the tensor-core TN kernel
      OFRR_TRY(dense_t_as(ctx, ta, &Ad, &lda));
      return gemm_impl(ctx, 1, 0, ta, tx, tc, ty, M, nrhs, K, 1.0, Ad, lda, X, ldx, 0.0, Y, ldy);
    }
    OFRR_TRY(dense_as(ctx, ta, &Ad, &lda));
    return gemm_impl(ctx, trans, 0, ta, tx, tc, ty, M, nrhs, K, 1.0, Ad, lda, X, ldx, 0.0, Y, ldy);
  }

  // Y = op(A) X, then scalecols(Y) (storage t, compute tc): one power step.  16-bit dense products with
  // FP32 accumulation combine their split-K partial sums inside the scaling kernel (same results).
  // E4M3 copies of A for the FP8 variant of the 16-bit power steps: f8[0] = A' (K = n, for A V), f8[1] = A
  // (K = m, for A' U), each column (one output row) with its power-of-two scale; made once per solve in the
  // solve's outermost workspace scope
  void* f8[2] = {nullptr, nullptr};
  float* f8s[2] = {nullptr, nullptr};
  int64_t f8ld[2] = {0, 0};
  int prepare_f8(ofrr_ctx* ctx, ofrr_dtype t16) {
    if (A->kind != OFRR_OP_DENSE) return OFRR_SUCCESS;
    int st = OFRR_SUCCESS;
    for (int trans = 0; trans < 2; ++trans) {
      const int64_t M = trans ? n() : m(), K = trans ? m() : n();
      const void* Ap = nullptr;
      int64_t lda = 0;
      if (trans) OFRR_TRY(dense_as(ctx, t16, &Ap, &lda));
      else OFRR_TRY(dense_t_as(ctx, t16, &Ap, &lda));
      f8ld[trans] = (K + 127) / 128 * 128;
      if (!(f8[trans] = ws_alloc(ctx, (size_t)f8ld[trans] * M, &st))) return st;
      if (!(f8s[trans] = ws_get<float>(ctx, (size_t)M, &st))) return st;
      OFRR_TRY(quant_e4m3(ctx, t16, K, M, Ap, lda, f8[trans], f8ld[trans], f8s[trans]));
    }
    return OFRR_SUCCESS;
  }

  int apply_scale(ofrr_ctx* ctx, int trans, ofrr_dtype t, ofrr_dtype tc, const void* X, int64_t ldx, int64_t nrhs,
                  void* Y, int64_t ldy, bool fast) {
    const int64_t M = trans ? n() : m(), K = trans ? m() : n();
    if (ctx->power_f8 && f8[trans] && (t == OFRR_F16 || t == OFRR_BF16)) {
      // the FP8 variant: the basis block quantized per column, the E4M3 product on the tensor cores, the
      // FP32 result rounded to the 16-bit basis and scaled (scalecols)
      WsScope tmp(ctx);
      int st = OFRR_SUCCESS;
      const int64_t ld8 = f8ld[trans];
      void* X8 = ws_alloc(ctx, (size_t)ld8 * nrhs, &st);
      float* sx = ws_get<float>(ctx, (size_t)nrhs, &st);
      float* C = ws_get<float>(ctx, (size_t)M * nrhs, &st);
      if (!X8 || !sx || !C) return st;
      OFRR_TRY(quant_e4m3(ctx, t, K, nrhs, X, ldx, X8, ld8, sx));
      OFRR_TRY(gemm_e4m3_tn(ctx, M, nrhs, ld8, f8[trans], ld8, f8s[trans], X8, ld8, sx, C, M));
      OFRR_TRY(cast_impl(ctx, OFRR_F32, t, M, nrhs, C, M, Y, ldy));
      return scalecols_impl(ctx, t, tc, M, nrhs, Y, ldy, nullptr, fast);
    }
    if (A->kind == OFRR_OP_DENSE && tc == OFRR_F32 && (t == OFRR_F16 || t == OFRR_BF16)) {
      const void* Ad = nullptr;
      int64_t lda = 0;
      if (trans) OFRR_TRY(dense_as(ctx, t, &Ad, &lda));
      else OFRR_TRY(dense_t_as(ctx, t, &Ad, &lda));
      bool handled = false;
      OFRR_TRY(gemm_tc_scalecols(ctx, t, M, nrhs, K, Ad, lda, X, ldx, Y, ldy, fast, &handled));
      if (handled) return OFRR_SUCCESS;
    }
    OFRR_TRY(apply(ctx, trans, t, t, X, ldx, nrhs, tc, t, Y, ldy));
    return scalecols_impl(ctx, t, tc, M, nrhs, Y, ldy, nullptr, fast);
  }

  // Y = op(A) X for X already split into digits (scalecols_sliced); dense operators in the emulated mode
  bool can_apply_pre(const ofrr_ctx* ctx) const {
    return ctx->emulate_f64 && A->kind == OFRR_OP_DENSE && have_sA && have_sAt;
  }
  int apply_pre(ofrr_ctx* ctx, int trans, const SlicedOperand& Xs, double* Y, int64_t ldy) {
    return sliced_gemm_tn_pre(ctx, trans ? sA : sAt, Xs, Y, ldy);
  }
  // apply_pre, then scalecols and the digit split of Y (into Ys); write_y = false may leave Y unwritten
  int apply_pre_scale(ofrr_ctx* ctx, int trans, const SlicedOperand& Xs, double* Y, int64_t ldy, bool write_y,
                      __nv_bfloat16* stack, int* expo, SlicedOperand* Ys) {
    return sliced_gemm_scalecols_pre(ctx, trans ? sA : sAt, Xs, Y, ldy, write_y, stack, expo, Ys);
  }

  // digit stacks of A for the FP64 emulation: sAt for A V (operand A', K = n), sA for A' U (K = m).
  // Must be called in the solve's outermost workspace scope (the stacks live as long as the solve).
  SlicedOperand sA, sAt;
  bool have_sA = false, have_sAt = false;
  // |A| in a 16-bit type in both K-contiguous orientations (absA[0] = |A'| for A X, absA[1] = |A| for
  // A' X), for the bounds on the emulation error; made once per solve by prepare_abs
  void* absA[2] = {nullptr, nullptr};
  ofrr_dtype abs_t = OFRR_F16;
  int prepare_abs(ofrr_ctx* ctx, ofrr_dtype t16);
  int prepare_sliced(ofrr_ctx* ctx) {
    if (A->kind != OFRR_OP_DENSE) return OFRR_SUCCESS;
    const double* A64;
    int64_t lda64 = 0;
    {
      const void* p = nullptr;
      OFRR_TRY(dense_as(ctx, OFRR_F64, &p, &lda64));
      A64 = (const double*)p;
    }
    OFRR_TRY(sliced_prepare(ctx, m(), n(), A64, lda64, &sA));
    have_sA = true;
    // A' (n x m) in FP64 is only needed while slicing: allocated after the stacks, released at once
    sAt.K = n();
    sAt.Kp = (n() + 63) / 64 * 64;
    sAt.M = m();
    int st = OFRR_SUCCESS;
    sAt.stack = ws_get<__nv_bfloat16>(ctx, (size_t)m() * kSliceDigits * sAt.Kp, &st);
    if (!sAt.stack) return st;
    sAt.expo = ws_get<int>(ctx, (size_t)m(), &st);
    if (!sAt.expo) return st;
    WsScope tmp(ctx);
    double* At = ws_get<double>(ctx, (size_t)m() * n(), &st);
    if (!At) return st;
    OFRR_TRY(cast_transpose_impl(ctx, A->dtype, OFRR_F64, m(), n(), A->data, A->ld, At, n()));
    SlicedOperand t;
    OFRR_TRY(sliced_prepare_into(ctx, n(), m(), At, n(), sAt.stack, sAt.expo, &t));
    have_sAt = true;
    return OFRR_SUCCESS;
  }

  // the transpose of a CSR operator, built once per solve for the A' U products (deterministic); must be
  // called in the solve's outermost workspace scope
  ofrr_csr csrT{};
  bool have_csrT = false;
  int prepare_csr_t(ofrr_ctx* ctx) {
    if (A->kind != OFRR_OP_CSR || have_csrT) return OFRR_SUCCESS;
    OFRR_TRY(csr_transpose_impl(ctx, &A->csr, &csrT));
    have_csrT = true;
    return OFRR_SUCCESS;
  }

  // A' stored column-major (n x m) in type t, made once per solve
  const void* dense_t[4] = {nullptr, nullptr, nullptr, nullptr};
  int64_t ldt[4] = {0, 0, 0, 0};
  int dense_t_as(ofrr_ctx* ctx, ofrr_dtype t, const void** p, int64_t* l) {
    if (!dense_t[t]) {
      int st = OFRR_SUCCESS;
      const int64_t ldp = (dtype_size(t) == 2) ? ((n() + 7) & ~int64_t(7)) : n();
      void* w = ws_alloc(ctx, (size_t)ldp * m() * dtype_size(t), &st);
      if (!w) return st;
      OFRR_TRY(cast_transpose_impl(ctx, A->dtype, t, m(), n(), A->data, A->ld, w, ldp));
      dense_t[t] = w;
      ldt[t] = ldp;
    }
    *p = dense_t[t];
    *l = ldt[t];
    return OFRR_SUCCESS;
  }
};

template <class T>
int dmalloc(ofrr_ctx* ctx, T** p, size_t count) {
  int st = OFRR_SUCCESS;
  *p = ws_get<T>(ctx, count, &st);
  return *p ? OFRR_SUCCESS : st;
}

__global__ void k_add_diag(int n, double* M, int ldm, double tau) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) M[i + (int64_t)i * ldm] += tau;
}

// gather selected columns of Q (keep order) into the first w columns
int compact_columns(ofrr_ctx* ctx, ofrr_dtype t, int64_t m, void* Q, int64_t ldq, const std::vector<int>& sel,
                    int* width) {
  int w = 0;
  const size_t es = dtype_size(t);
  for (size_t j = 0; j < sel.size(); ++j) {
    if (!sel[j]) continue;
    if ((int)j != w)
      OFRR_CUDA(cudaMemcpyAsync((char*)Q + (size_t)w * ldq * es, (char*)Q + j * ldq * es, (size_t)m * es,
                                cudaMemcpyDeviceToDevice, ctx->stream));
    ++w;
  }
  *width = w;
  return OFRR_SUCCESS;
}

struct Precisions {
  ofrr_dtype pc, po, phc, pho, prc, pro;
  bool fast = false;  // production modes: FP32 Jacobi + FP64 refinement small solver, FMA/reciprocal FP64
                      // Hessenberg and column scaling
  int refine = 2;     // FP64 refinement steps of the small solver (0 for 16-bit bases)
};

Precisions precisions_of(const ofrr_options* o) {
  Precisions p;
  if (o->mode == OFRR_MODE_FP64) {
    p.pc = p.po = p.phc = p.pho = p.prc = p.pro = OFRR_F64;
    p.fast = true;
  } else {
    p.pc = o->p_compute;
    p.po = o->p_output;
    p.phc = o->p_hess_compute;
    p.pho = o->p_hess_output;
    p.prc = o->p_rr_compute;
    p.pro = o->p_rr_output;
  }
  return p;
}

// The basis of a block (the `function_orth` of subspace_iter_eig.m:65 / subspace_iter_svd.m): the
// Hessenberg process (the orthogonalization-free default of this library), or a Gram-Schmidt QR --
// mgs.m, the reference's own default (subspace_iter_eig.m:114-115), or cgs.m -- as the orthogonal
// comparison, or the column-pivoted LU basis of lu.m.  All leave Q at the input's column positions
// with select flags.
int basis_impl(ofrr_ctx* ctx, int orth, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tc, int64_t m, int64_t n,
               const void* A, int64_t lda, void* Q, int64_t ldq, double select_tol, double* R, int* sel, int* perm,
               bool fast) {
  if (orth == OFRR_ORTH_LU) return lu_basis_impl(ctx, tin, tout, tc, m, n, A, lda, Q, ldq, select_tol, R, sel);
  if (orth == OFRR_ORTH_MGS || orth == OFRR_ORTH_CGS)
    return gs_basis_impl(ctx, orth == OFRR_ORTH_CGS, tin, tout, tc, m, n, A, lda, Q, ldq, select_tol, R, sel);
  return hessenberg_impl(ctx, tin, tout, tc, m, n, A, lda, Q, ldq, select_tol, R, sel, perm, fast);
}

int validate_options(const ofrr_options* o) {
  if (!o) return OFRR_ERR_INVALID_ARGUMENT;
  if (o->mode < 0 || o->mode > 2) return OFRR_ERR_INVALID_ARGUMENT;
  if (o->maxiter < 0 || o->step_size < 1 || o->step_size_f64 < 0 || o->block < 1 || o->nev < 0 ||
      o->restart_keep < 0)
    return OFRR_ERR_INVALID_ARGUMENT;
  if (o->orth != OFRR_ORTH_HESSENBERG && o->orth != OFRR_ORTH_MGS && o->orth != OFRR_ORTH_CGS &&
      o->orth != OFRR_ORTH_LU)
    return OFRR_ERR_INVALID_ARGUMENT;
  const int ps[6] = {o->p_compute, o->p_output, o->p_hess_compute, o->p_hess_output, o->p_rr_compute,
                     o->p_rr_output};
  for (int p : ps)
    if (!dtype_valid(p)) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (o->mode != OFRR_MODE_FP64) {
    if (o->p_compute != OFRR_F64 && o->p_compute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
    if (o->p_hess_compute != OFRR_F64 && o->p_hess_compute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
    if (o->p_rr_compute != OFRR_F64 && o->p_rr_compute != OFRR_F32) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  }
  return OFRR_SUCCESS;
}

int validate_op(const ofrr_operator* A) {
  if (!A || A->nrows < 0 || A->ncols < 0) return OFRR_ERR_INVALID_ARGUMENT;
  if (A->kind == OFRR_OP_DENSE) {
    if (!dtype_valid(A->dtype)) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
    if (A->nrows > 0 && A->ncols > 0 && (!A->data || A->ld < A->nrows)) return OFRR_ERR_INVALID_ARGUMENT;
  } else if (A->kind == OFRR_OP_CSR) {
    if (A->csr.nrows != A->nrows || A->csr.ncols != A->ncols || !A->csr.indptr) return OFRR_ERR_INVALID_ARGUMENT;
    if (A->csr.nnz > 0 && !A->csr.indices) return OFRR_ERR_INVALID_ARGUMENT;
    if (!A->csr.a_double && !A->csr.a_single) return OFRR_ERR_INVALID_ARGUMENT;
  } else {
    return OFRR_ERR_INVALID_ARGUMENT;
  }
  return OFRR_SUCCESS;
}

// ---------------------------------------------------------------------------------------
// Rayleigh-Ritz on a basis Q (n x b, type tq): eig_rr.m:46-57.
// Outputs: Ritz vectors into Vout (n x b, type tq), Ritz values d (device, b, descending).
// ---------------------------------------------------------------------------------------
// Ritz back-transform of a 16-bit basis with FP32 arithmetic: Out = tq(Q (m x b) * f32(Cf) (b x b)),
// one thread per row and 32 output columns, the coefficient block in shared memory (FP32), the FP32
// result rounded once to the basis type.  Replaces widening Q to FP32, a library SGEMM and a cast.
template <class TQ>
__global__ void __launch_bounds__(128) k_backtransform16(int64_t m, int b, const TQ* __restrict__ Q, int64_t ldq,
                                                         const double* __restrict__ Cf, int ldc, TQ* __restrict__ Out,
                                                         int64_t ldo) {
  __shared__ float Zs[128][33];
  const int j0 = blockIdx.y * 32;
  const int nj = min(32, b - j0);
  for (int e = threadIdx.x; e < b * 32; e += blockDim.x) {
    const int k = e >> 5, jj = e & 31;
    Zs[k][jj] = (jj < nj) ? __double2float_rn(Cf[k + (size_t)(j0 + jj) * ldc]) : 0.f;
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float acc[32];
#pragma unroll
  for (int jj = 0; jj < 32; ++jj) acc[jj] = 0.f;
  for (int k0 = 0; k0 < b; k0 += 64) {  // the row's basis entries loaded 64 at a time (one latency)
    float u[64];
#pragma unroll
    for (int t = 0; t < 64; ++t) u[t] = (k0 + t < b) ? to_c<float, TQ>(Q[i + (int64_t)(k0 + t) * ldq]) : 0.f;
#pragma unroll
    for (int t = 0; t < 64; ++t) {
      if (k0 + t < b) {
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) acc[jj] = fmaf(u[t], Zs[k0 + t][jj], acc[jj]);
      }
    }
  }
#pragma unroll
  for (int jj = 0; jj < 32; ++jj)
    if (jj < nj) Out[i + (int64_t)(j0 + jj) * ldo] = from_c<TQ, float>(acc[jj]);
}

// Out (type tq) = tq(gemm(Q, Cf, pmc) rounded to pmo): the fused kernel for 16-bit bases with FP32
// compute and output, the general product and cast otherwise
int back_transform(ofrr_ctx* ctx, ofrr_dtype tq, ofrr_dtype pmc, ofrr_dtype pmo, int64_t m, int b, const void* Q,
                   int64_t ldq, const double* Cf, void* Out, int64_t ldo) {
  if ((tq == OFRR_F16 || tq == OFRR_BF16) && pmc == OFRR_F32 && pmo == OFRR_F32 && b <= 128 && Out != Q) {
    const dim3 grid((unsigned)((m + 127) / 128), (unsigned)((b + 31) / 32));
    if (tq == OFRR_F16)
      k_backtransform16<__half><<<grid, 128, 0, ctx->stream>>>(m, b, (const __half*)Q, ldq, Cf, b, (__half*)Out, ldo);
    else
      k_backtransform16<__nv_bfloat16><<<grid, 128, 0, ctx->stream>>>(m, b, (const __nv_bfloat16*)Q, ldq, Cf, b,
                                                                     (__nv_bfloat16*)Out, ldo);
    OFRR_LAUNCHED(ctx, "k_backtransform16");
    return OFRR_SUCCESS;
  }
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  void* Vn = Out;
  int64_t ldvn = ldo;
  if (pmo != tq || Out == Q) {
    Vn = ws_alloc(ctx, (size_t)m * b * dtype_size(pmo), &st);
    if (!Vn) return st;
    ldvn = m;
  }
  OFRR_TRY(gemm_impl(ctx, 0, 0, tq, OFRR_F64, pmc, pmo, m, b, b, 1.0, Q, ldq, Cf, b, 0.0, Vn, ldvn));
  if (Vn != Out) OFRR_TRY(cast_impl(ctx, pmo, tq, m, b, Vn, ldvn, Out, ldo));
  return OFRR_SUCCESS;
}

// A V with a dense 16-bit A and a basis of the same 16-bit type, accumulated in FP32: the basis
// values are exact in FP32, so widening it first changes nothing but the route (a library SGEMM on a
// widened A instead of the tensor cores)
bool tc16_direct(const Op& op, ofrr_dtype ta, ofrr_dtype tq, ofrr_dtype pAmc) {
  return op.A->kind == OFRR_OP_DENSE && (ta == OFRR_F16 || ta == OFRR_BF16) && tq == ta && pAmc == OFRR_F32;
}

int rr_eig_dev(ofrr_ctx* ctx, Op& op, ofrr_dtype ta, const void* Q, ofrr_dtype tq, int64_t ldq, int b,
               ofrr_dtype pmc, ofrr_dtype pmo, ofrr_dtype pAmc, ofrr_dtype pAmo, bool use_gen, double gtol,
               bool symmetric, void* Vout, int64_t ldvo, double* d, bool fast = false, int refine = 2) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t n = op.m();
  // AV = pmc(matvec(A, 'N', pAmc(Q), pAmc, pAmo)) -- kept in pAmo storage, widened by the Gram gemm
  const void* Qa = Q;
  int64_t ldqa = ldq;
  ofrr_dtype tqa = pAmc;
  if (tc16_direct(op, ta, tq, pAmc)) {
    tqa = tq;  // 16-bit A and basis, FP32 accumulation: the tensor-core product reads the basis as is
  } else if (tq != pAmc) {
    void* w = ws_alloc(ctx, (size_t)n * b * dtype_size(pAmc), &st);
    if (!w) return st;
    OFRR_TRY(cast_impl(ctx, tq, pAmc, n, b, Q, ldq, w, n));
    Qa = w;
    ldqa = n;
  }
  void* AV = ws_alloc(ctx, (size_t)n * b * dtype_size(pAmo), &st);
  if (!AV) return st;
  OFRR_TRY(op.apply(ctx, 0, ta, tqa, Qa, ldqa, b, pAmc, pAmo, AV, n));
  ofrr_dtype tav = pAmo;
  if (pAmo != pmc) {  // the MATLAB code rounds to pAmo then converts to pmc: identical values
    // no storage change needed: gemm widens pAmo to pmc exactly
  }
  double *G, *M = nullptr, *U;
  OFRR_TRY(dmalloc(ctx, &G, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &U, (size_t)b * b));
  void* tmp = ws_alloc(ctx, (size_t)b * b * dtype_size(pmo), &st);
  if (!tmp) return st;
  // VAV = peig(gemm(V, 'T', AV, pmc, pmo))
  OFRR_TRY(gemm_impl(ctx, 1, 0, tq, tav, pmc, pmo, b, b, n, 1.0, Q, ldq, AV, n, 0.0, tmp, b));
  OFRR_TRY(cast_impl(ctx, pmo, OFRR_F64, b, b, tmp, b, G, b));
  if (use_gen) {
    OFRR_TRY(dmalloc(ctx, &M, (size_t)b * b));
    OFRR_TRY(gemm_impl(ctx, 1, 0, tq, tq, pmc, pmo, b, b, n, 1.0, Q, ldq, Q, ldq, 0.0, tmp, b));
    OFRR_TRY(cast_impl(ctx, pmo, OFRR_F64, b, b, tmp, b, M, b));
    if (gtol != 0.0 && !(fast && symmetric && b <= 128)) {
      k_add_diag<<<(b + 255) / 256, 256, 0, ctx->stream>>>(b, M, b, gtol);
      OFRR_LAUNCHED(ctx, "k_add_diag");
    }
  }
  if (fast && symmetric && b <= 128) {
    OFRR_TRY(geig_fast(ctx, b, G, M, use_gen ? gtol : 0.0, d, U, refine));
  } else if (!symmetric && b <= 128) {
    // M already holds VV + gtol I; FP64 refinement unless the basis is 16-bit
    OFRR_TRY(geig_nonsym(ctx, b, G, M, d, U, tq == OFRR_F64 || tq == OFRR_F32));
  } else {
    OFRR_TRY(geig_dev(ctx, b, G, b, M, b, symmetric ? 1 : 0, d, U, b));
  }
  // V = gemm(V, 'N', U, pmc, pmo) then back to V's precision
  return back_transform(ctx, tq, pmc, pmo, n, b, Q, ldq, U, Vout, ldvo);
}

// at most 4 CTAs per column: each thread handles several rows of one column
inline dim3 grid_cols(int64_t m, int64_t n) {
  return dim3(std::min(grid_2d(m, n, 256).x, 4u), (unsigned)std::min<int64_t>(n, 65535));
}

__global__ void k_normalize_cols(int64_t m, int64_t n, double* X, const double* nrm);

// |X| rounded to T (16-bit), column-major
template <class TI, class T>
__global__ void k_abs_cast(int64_t m, int64_t n, const TI* __restrict__ X, int64_t ldx, T* __restrict__ Y,
                           int64_t ldy) {
  OFRR_FOR_2D(i, j, m, n) Y[i + j * ldy] = from_c<T, float>(fabsf(to_c<float, TI>(X[i + j * ldx])));
}
__global__ void k_abs_cast_f64(int64_t m, int64_t n, const double* __restrict__ X, int64_t ldx, __half* Yh,
                               __nv_bfloat16* Yb, int64_t ldy) {
  OFRR_FOR_2D(i, j, m, n) {
    const double a = fabs(X[i + j * ldx]);
    if (Yh) Yh[i + j * ldy] = __double2half(a);
    else Yb[i + j * ldy] = __double2bfloat16(a);
  }
}

// Bound on the exact-slice emulation error of Y = op(A) X for unit columns X (FP64, ld ldx):
// |Y_emul - Y| <= 2^-33 |op(A)| |X| element-wise (the tested bound of the emulated product), and
// ||(|op(A)| |x_j|)||_2 is computed from the 16-bit copies of A (abs, exact) and |x_j| rounded to
// 16 bits with FP32 accumulation of non-negative terms; the factor 1.01 covers those roundings
// (2^-8 relative for the 16-bit values, K 2^-24 for the sums).  out[j] = the bound for column j.
int emulation_bounds(ofrr_ctx* ctx, Op& op, int trans, ofrr_dtype t16, const double* X, int64_t ldx, int k,
                     double* out_dev) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t m = op.m(), n = op.n();
  const int64_t M = trans ? n : m, K = trans ? m : n;
  // |op(A)| as the K-contiguous operand of the TN kernel: A' (K = n) for A X, A itself (K = m) for A' X
  const void* Ap = nullptr;
  int64_t lda = 0;
  if (trans) OFRR_TRY(op.dense_as(ctx, t16, &Ap, &lda));
  else OFRR_TRY(op.dense_t_as(ctx, t16, &Ap, &lda));
  const bool cached = op.absA[trans] != nullptr && op.abs_t == t16;
  const int64_t ldK = (K + 7) & ~int64_t(7);  // 16-byte aligned columns for the tensor-core product
  void* absA = cached ? op.absA[trans] : ws_alloc(ctx, (size_t)ldK * M * 2, &st);
  void* absX = ws_alloc(ctx, (size_t)ldK * k * 2, &st);
  float* Bnd = ws_get<float>(ctx, (size_t)M * k, &st);
  if (!absA || !absX || !Bnd) return st;
  if (t16 == OFRR_F16) {
    if (!cached) {
      k_abs_cast<__half, __half><<<grid_2d(K, M, 256), 256, 0, ctx->stream>>>(K, M, (const __half*)Ap, lda,
                                                                               (__half*)absA, ldK);
      OFRR_LAUNCHED(ctx, "k_abs_cast");
    }
    k_abs_cast_f64<<<grid_2d(K, k, 256), 256, 0, ctx->stream>>>(K, k, X, ldx, (__half*)absX, nullptr, ldK);
  } else {
    if (!cached) {
      k_abs_cast<__nv_bfloat16, __nv_bfloat16><<<grid_2d(K, M, 256), 256, 0, ctx->stream>>>(
          K, M, (const __nv_bfloat16*)Ap, lda, (__nv_bfloat16*)absA, ldK);
      OFRR_LAUNCHED(ctx, "k_abs_cast");
    }
    k_abs_cast_f64<<<grid_2d(K, k, 256), 256, 0, ctx->stream>>>(K, k, X, ldx, nullptr, (__nv_bfloat16*)absX, ldK);
  }
  OFRR_LAUNCHED(ctx, "k_abs_cast_f64");
  OFRR_TRY(gemm_impl(ctx, 1, 0, t16, t16, OFRR_F32, OFRR_F32, M, k, K, 1.0, absA, ldK, absX, ldK, 0.0, Bnd, M));
  OFRR_TRY(column_norms(ctx, OFRR_F32, M, k, Bnd, M, out_dev));
  return OFRR_SUCCESS;
}
constexpr double kEmulBound = 1.01 * 1.16415321826934814453125e-10;  // 1.01 * 2^-33

// |A| in t16 in both orientations, in the caller's (solve-lifetime) workspace scope
int Op::prepare_abs(ofrr_ctx* ctx, ofrr_dtype t16) {
  if (A->kind != OFRR_OP_DENSE || (t16 != OFRR_F16 && t16 != OFRR_BF16)) return OFRR_SUCCESS;
  int st = OFRR_SUCCESS;
  for (int trans = 0; trans < 2; ++trans) {
    const int64_t M = trans ? n() : m(), K = trans ? m() : n();
    const void* Ap = nullptr;
    int64_t lda = 0;
    if (trans) OFRR_TRY(dense_as(ctx, t16, &Ap, &lda));
    else OFRR_TRY(dense_t_as(ctx, t16, &Ap, &lda));
    const int64_t ldK = (K + 7) & ~int64_t(7);
    void* w = ws_alloc(ctx, (size_t)ldK * M * 2, &st);
    if (!w) return st;
    if (t16 == OFRR_F16)
      k_abs_cast<__half, __half><<<grid_2d(K, M, 256), 256, 0, ctx->stream>>>(K, M, (const __half*)Ap, lda,
                                                                               (__half*)w, ldK);
    else
      k_abs_cast<__nv_bfloat16, __nv_bfloat16><<<grid_2d(K, M, 256), 256, 0, ctx->stream>>>(
          K, M, (const __nv_bfloat16*)Ap, lda, (__nv_bfloat16*)w, ldK);
    OFRR_LAUNCHED(ctx, "k_abs_cast");
    absA[trans] = w;
  }
  abs_t = t16;
  return OFRR_SUCCESS;
}

// FP64 residuals of Ritz pairs (X in type tx), normalised by normA and ||x||
// certify16 >= 0: emulated products; the bound on their error is added, computed only when every
// emulated residual is at most bounds_below
int residuals_dev(ofrr_ctx* ctx, Op& op, ofrr_dtype tx, const void* X, int64_t ldx, int k, const double* lam_host,
                  double normA, double* out_host, int certify16 = -1, double* emul_host = nullptr,
                  double bounds_below = INFINITY) {
  if (k <= 0) return OFRR_SUCCESS;
  WsScope scope(ctx);
  const int64_t n = op.m();
  double *X64, *AX, *lam, *res, *nrm;
  OFRR_TRY(dmalloc(ctx, &X64, (size_t)n * k));
  OFRR_TRY(dmalloc(ctx, &AX, (size_t)n * k));
  OFRR_TRY(dmalloc(ctx, &lam, (size_t)k));
  OFRR_TRY(dmalloc(ctx, &res, (size_t)2 * k));
  nrm = res + k;
  OFRR_TRY(cast_impl(ctx, tx, OFRR_F64, n, k, X, ldx, X64, n));
  OFRR_TRY(op.apply(ctx, 0, OFRR_F64, OFRR_F64, X64, n, k, OFRR_F64, OFRR_F64, AX, n));
  OFRR_CUDA(cudaMemcpyAsync(lam, lam_host, sizeof(double) * k, cudaMemcpyHostToDevice, ctx->stream));
  OFRR_TRY(residual_columns(ctx, n, k, AX, n, X64, n, lam, res));
  OFRR_TRY(column_norms(ctx, OFRR_F64, n, k, X64, n, nrm));
  std::vector<double> h(3 * k, 0.0);
  OFRR_CUDA(cudaMemcpyAsync(h.data(), res, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  if (normA <= 0) {
    normA = 0;
    for (int j = 0; j < k; ++j) normA = std::max(normA, std::fabs(lam_host[j]));
    if (normA == 0) normA = 1;
  }
  double emax = 0;
  for (int j = 0; j < k; ++j) emax = std::max(emax, (h[k + j] > 0) ? h[j] / (normA * h[k + j]) : INFINITY);
  if (certify16 >= 0 && emax <= bounds_below) {  // emulated A X: the bound on its error (unit columns)
    double* bnd = nullptr;
    OFRR_TRY(dmalloc(ctx, &bnd, (size_t)k));
    k_normalize_cols<<<grid_cols(n, k), 256, 0, ctx->stream>>>(n, k, X64, nrm);
    OFRR_LAUNCHED(ctx, "k_normalize_cols");
    OFRR_TRY(emulation_bounds(ctx, op, 0, (ofrr_dtype)certify16, X64, n, k, bnd));
    OFRR_CUDA(cudaMemcpyAsync(h.data() + 2 * k, bnd, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
  }
  for (int j = 0; j < k; ++j) {
    out_host[j] = (h[k + j] > 0) ? h[j] / (normA * h[k + j]) + kEmulBound * h[2 * k + j] / normA : INFINITY;
    if (emul_host) emul_host[j] = (h[k + j] > 0) ? h[j] / (normA * h[k + j]) : INFINITY;
  }
  return OFRR_SUCCESS;
}

}  // namespace
}  // namespace ofrr

using namespace ofrr;

extern "C" void ofrr_options_default(ofrr_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->mode = OFRR_MODE_REFERENCE;
  o->maxiter = 5;  // subspace_iter_eig.m:108-110
  o->step_size = 1;
  o->block = 8;
  o->nev = 8;
  o->kdim = 0;  // 0 -> maxiter (arnoldi_hess_eig.m:165-167)
  o->tol = 0.0;
  o->use_generalized = 1;
  o->generalized_tol = 0.0;
  o->select_tol = -1.0;
  o->seed = 42;
  o->use_start_block = 0;
  o->orth = OFRR_ORTH_HESSENBERG;
  o->reorth = 1;
  o->p_compute = o->p_output = OFRR_F64;
  o->p_hess_compute = o->p_hess_output = OFRR_F64;
  o->p_rr_compute = o->p_rr_output = OFRR_F64;
  o->check_every = 1;
}

extern "C" int ofrr_rr_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, int64_t ncols, void* V,
                           int64_t ldv, double* evals) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  OFRR_TRY(validate_options(opt));
  if (A->nrows != A->ncols) return OFRR_ERR_BLAS_INVALID_SIZE;
  const int64_t n = A->nrows;
  if (ncols <= 0 || n == 0) return OFRR_SUCCESS;
  if (!V || ldv < n || !evals || ncols > 1024) return OFRR_ERR_INVALID_ARGUMENT;
  const Precisions P = precisions_of(opt);
  WsScope scope(ctx);
  Op op{A};
  OFRR_TRY(op.prepare_csr_t(ctx));
  double* d;
  OFRR_TRY(dmalloc(ctx, &d, (size_t)ncols));
  // eig_rr on V (type p_output): pmc = p_rr_compute, pmo = p_rr_output, A-matvec in (p_compute, p_output)
  OFRR_TRY(rr_eig_dev(ctx, op, P.po, V, P.po, ldv, (int)ncols, P.prc, P.pro, P.pc, P.po, opt->use_generalized != 0,
                      opt->generalized_tol, A->symmetric != 0, V, ldv, d));
  OFRR_CUDA(cudaMemcpyAsync(evals, d, sizeof(double) * ncols, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

extern "C" int ofrr_ofrr_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_operator* B, const ofrr_options* opt,
                             int64_t ncols, void* V, int64_t ldv, double* evals) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  OFRR_TRY(validate_op(B));
  OFRR_TRY(validate_options(opt));
  const int64_t n = A->nrows;
  if (A->ncols != n || B->nrows != n || B->ncols != n) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (ncols <= 0 || n == 0) return OFRR_SUCCESS;
  if (!V || ldv < n || !evals || ncols > 1024) return OFRR_ERR_INVALID_ARGUMENT;
  const Precisions P = precisions_of(opt);
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  Op opA{A}, opB{B};
  const int b = (int)ncols;
  void *AV, *BV, *tmp, *Vn;
  double *G, *M, *U, *d;
  if (!(AV = ws_alloc(ctx, (size_t)n * b * dtype_size(P.pc), &st))) return st;
  if (!(BV = ws_alloc(ctx, (size_t)n * b * dtype_size(P.pc), &st))) return st;
  if (!(tmp = ws_alloc(ctx, (size_t)b * b * dtype_size(P.pro), &st))) return st;
  if (!(Vn = ws_alloc(ctx, (size_t)n * b * dtype_size(P.pro), &st))) return st;
  OFRR_TRY(dmalloc(ctx, &G, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &M, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &U, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &d, (size_t)b));
  OFRR_TRY(opA.apply(ctx, 0, P.po, P.po, V, ldv, b, P.pc, P.pc, AV, n));
  OFRR_TRY(opB.apply(ctx, 0, P.po, P.po, V, ldv, b, P.pc, P.pc, BV, n));
  OFRR_TRY(gemm_impl(ctx, 1, 0, P.po, P.pc, P.prc, P.pro, b, b, n, 1.0, V, ldv, AV, n, 0.0, tmp, b));
  OFRR_TRY(cast_impl(ctx, P.pro, OFRR_F64, b, b, tmp, b, G, b));
  OFRR_TRY(gemm_impl(ctx, 1, 0, P.po, P.pc, P.prc, P.pro, b, b, n, 1.0, V, ldv, BV, n, 0.0, tmp, b));
  OFRR_TRY(cast_impl(ctx, P.pro, OFRR_F64, b, b, tmp, b, M, b));
  if (opt->generalized_tol != 0.0) {
    k_add_diag<<<(b + 255) / 256, 256, 0, ctx->stream>>>(b, M, b, opt->generalized_tol);
    OFRR_LAUNCHED(ctx, "k_add_diag");
  }
  OFRR_TRY(geig_dev(ctx, b, G, b, M, b, 1, d, U, b));
  OFRR_TRY(gemm_impl(ctx, 0, 0, P.po, OFRR_F64, P.prc, P.pro, n, b, b, 1.0, V, ldv, U, b, 0.0, Vn, n));
  OFRR_TRY(cast_impl(ctx, P.pro, P.po, n, b, Vn, n, V, ldv));
  OFRR_CUDA(cudaMemcpyAsync(evals, d, sizeof(double) * b, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

extern "C" int ofrr_residual_norms(ofrr_ctx* ctx, const ofrr_operator* A, ofrr_dtype tx, int64_t ncols, const void* X,
                                   int64_t ldx, const double* evals, double normA, double* resid) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  if (!dtype_valid(tx)) return OFRR_ERR_BLAS_UNSUPPORTED_TYPE;
  if (ncols <= 0) return OFRR_SUCCESS;
  if (!X || !evals || !resid || ldx < A->nrows || A->nrows != A->ncols) return OFRR_ERR_INVALID_ARGUMENT;
  WsScope scope(ctx);
  Op op{A};
  return residuals_dev(ctx, op, tx, X, ldx, (int)ncols, evals, normA, resid);
}

// ======================================================================================
// subspace iteration SVD and RR-SVD
// ======================================================================================
namespace ofrr {
namespace {

__global__ void k_scale_f64(int64_t m, int64_t n, double* X, int64_t ldx, double s) {
  OFRR_FOR_2D(i, j, m, n) X[i + j * ldx] *= s;
}

// Z = Lu^-T Y, W = Lv^-T X from the SVD of C = Lu^-1 B Lv^-T is the same pencil as
// eig([[0,B],[B',0]], blkdiag(UU,VV)+tau I) (svd_rr.m:58-77).  We form the symmetric
// 2b x 2b pencil explicitly and hand it to the FP64 generalized solver, which keeps the
// reference's normalisation (M-orthonormal eigenvectors, hence the sqrt(2) of svd_rr.m:87-91).
__global__ void k_build_aug(int b, const double* B, const double* UU, const double* VV, double* Aext, double* Mext,
                            double tau) {
  const int nn = 2 * b;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nn * nn; e += gridDim.x * blockDim.x) {
    const int i = e % nn, j = e / nn;
    double a = 0.0, m = 0.0;
    if (i < b && j >= b) a = B[i + (j - b) * b];
    if (i >= b && j < b) a = B[j + (i - b) * b];
    if (i < b && j < b) m = UU[i + j * b];
    if (i >= b && j >= b) m = VV[(i - b) + (j - b) * b];
    if (i == j) m += tau;
    Aext[e] = a;
    Mext[e] = m;
  }
}

int rr_svd_dev(ofrr_ctx* ctx, Op& op, ofrr_dtype ta, const void* U, const void* V, ofrr_dtype tq, int64_t ldu,
               int64_t ldv, int b, ofrr_dtype pmc, ofrr_dtype pmo, ofrr_dtype pAmc, ofrr_dtype pAmo, bool use_gen,
               double gtol, void* Uout, int64_t lduo, void* Vout, int64_t ldvo, double* s_dev, bool fast = false,
               int refine = 2) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t m = op.m(), n = op.n();
  if (!use_gen) return OFRR_ERR_NOT_IMPLEMENTED;  // svd(UAV) path: the oblique bases need the pencil
  const void* Va = V;
  int64_t ldva = ldv;
  ofrr_dtype tva = pAmc;
  if (tc16_direct(op, ta, tq, pAmc)) {
    tva = tq;  // 16-bit A and basis, FP32 accumulation: the tensor-core product reads the basis as is
  } else if (tq != pAmc) {
    void* w = ws_alloc(ctx, (size_t)n * b * dtype_size(pAmc), &st);
    if (!w) return st;
    OFRR_TRY(cast_impl(ctx, tq, pAmc, n, b, V, ldv, w, n));
    Va = w;
    ldva = n;
  }
  void* AV = ws_alloc(ctx, (size_t)m * b * dtype_size(pAmo), &st);
  if (!AV) return st;
  double *B, *UU, *VV, *Aext, *Mext, *X, *d;
  OFRR_TRY(dmalloc(ctx, &B, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &UU, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &VV, (size_t)b * b));
  OFRR_TRY(dmalloc(ctx, &Aext, (size_t)4 * b * b));
  OFRR_TRY(dmalloc(ctx, &Mext, (size_t)4 * b * b));
  OFRR_TRY(dmalloc(ctx, &X, (size_t)4 * b * b));
  OFRR_TRY(dmalloc(ctx, &d, (size_t)2 * b));
  void* tmp = ws_alloc(ctx, (size_t)b * b * dtype_size(pmo), &st);
  void* tmpu = ws_alloc(ctx, (size_t)b * b * dtype_size(pmo), &st);
  void* tmpv = ws_alloc(ctx, (size_t)b * b * dtype_size(pmo), &st);
  if (!tmp || !tmpu || !tmpv) return st;
  // the Gram matrices U'U and V'V do not depend on A V: auxiliary stream
  ofrr_ctx* aux = nullptr;
  OFRR_TRY(aux_begin(ctx, &aux));
  OFRR_TRY(gemm_impl(aux, 1, 0, tq, tq, pmc, pmo, b, b, m, 1.0, U, ldu, U, ldu, 0.0, tmpu, b));
  OFRR_TRY(cast_impl(aux, pmo, OFRR_F64, b, b, tmpu, b, UU, b));
  OFRR_TRY(gemm_impl(aux, 1, 0, tq, tq, pmc, pmo, b, b, n, 1.0, V, ldv, V, ldv, 0.0, tmpv, b));
  OFRR_TRY(cast_impl(aux, pmo, OFRR_F64, b, b, tmpv, b, VV, b));
  OFRR_TRY(op.apply(ctx, 0, ta, tva, Va, ldva, b, pAmc, pAmo, AV, m));
  OFRR_TRY(gemm_impl(ctx, 1, 0, tq, pAmo, pmc, pmo, b, b, m, 1.0, U, ldu, AV, m, 0.0, tmp, b));
  OFRR_TRY(cast_impl(ctx, pmo, OFRR_F64, b, b, tmp, b, B, b));
  OFRR_TRY(aux_end(ctx));
  if (fast && b <= 128) {
    // the same pencil through two Cholesky factors: sigma, Zf = Lu^-T Y, Wf = Lv^-T X;
    // U Zf and V Wf are the unit singular-vector estimates (svd_rr.m's sqrt(2) U Z and sqrt(2) V W)
    double *Zf, *Wf;
    OFRR_TRY(dmalloc(ctx, &Zf, (size_t)b * b));
    OFRR_TRY(dmalloc(ctx, &Wf, (size_t)b * b));
    OFRR_TRY(gsvd_fast(ctx, b, B, UU, VV, gtol, s_dev, Zf, Wf, refine));
    // the two back-transforms are independent: V's on the auxiliary stream
    OFRR_TRY(aux_begin(ctx, &aux));
    OFRR_TRY(back_transform(aux, tq, pmc, pmo, n, b, V, ldv, Wf, Vout, ldvo));
    OFRR_TRY(back_transform(ctx, tq, pmc, pmo, m, b, U, ldu, Zf, Uout, lduo));
    OFRR_TRY(aux_end(ctx));
    return OFRR_SUCCESS;
  }
  k_build_aug<<<grid_for(4 * b * b, 256), 256, 0, ctx->stream>>>(b, B, UU, VV, Aext, Mext, gtol);
  OFRR_LAUNCHED(ctx, "k_build_aug");
  OFRR_TRY(geig_dev(ctx, 2 * b, Aext, 2 * b, Mext, 2 * b, 1, d, X, 2 * b));
  OFRR_CUDA(cudaMemcpyAsync(s_dev, d, sizeof(double) * b, cudaMemcpyDeviceToDevice, ctx->stream));
  // Z = X(1:b, 1:b), W = X(b+1:2b, 1:b), both rounded to pmo (svd_rr.m:81-82); U = sqrt2 * U Z
  void* Zp = ws_alloc(ctx, (size_t)b * b * dtype_size(pmo), &st);
  void* Wp = ws_alloc(ctx, (size_t)b * b * dtype_size(pmo), &st);
  if (!Zp || !Wp) return st;
  OFRR_TRY(cast_impl(ctx, OFRR_F64, pmo, b, b, X, 2 * b, Zp, b));
  OFRR_TRY(cast_impl(ctx, OFRR_F64, pmo, b, b, X + b, 2 * b, Wp, b));
  double* Un64;
  double* Vn64;
  OFRR_TRY(dmalloc(ctx, &Un64, (size_t)m * b));
  OFRR_TRY(dmalloc(ctx, &Vn64, (size_t)n * b));
  // gemm in pmc with pmo output, then scaled by pmo(sqrt 2) in pmo: emulate by rounding through pmo
  void* Uo = ws_alloc(ctx, (size_t)m * b * dtype_size(pmo), &st);
  void* Vo = ws_alloc(ctx, (size_t)n * b * dtype_size(pmo), &st);
  if (!Uo || !Vo) return st;
  OFRR_TRY(gemm_impl(ctx, 0, 0, tq, pmo, pmc, pmo, m, b, b, 1.0, U, ldu, Zp, b, 0.0, Uo, m));
  OFRR_TRY(gemm_impl(ctx, 0, 0, tq, pmo, pmc, pmo, n, b, b, 1.0, V, ldv, Wp, b, 0.0, Vo, n));
  OFRR_TRY(cast_impl(ctx, pmo, OFRR_F64, m, b, Uo, m, Un64, m));
  OFRR_TRY(cast_impl(ctx, pmo, OFRR_F64, n, b, Vo, n, Vn64, n));
  const double r2 = 1.4142135623730951;
  k_scale_f64<<<grid_2d(m, b, 256), 256, 0, ctx->stream>>>(m, b, Un64, m, r2);
  OFRR_LAUNCHED(ctx, "k_scale_f64");
  k_scale_f64<<<grid_2d(n, b, 256), 256, 0, ctx->stream>>>(n, b, Vn64, n, r2);
  OFRR_LAUNCHED(ctx, "k_scale_f64");
  OFRR_TRY(cast_impl(ctx, OFRR_F64, tq, m, b, Un64, m, Uout, lduo));
  OFRR_TRY(cast_impl(ctx, OFRR_F64, tq, n, b, Vn64, n, Vout, ldvo));
  return OFRR_SUCCESS;
}

__global__ void k_rescol2(int64_t m, int64_t n, const double* AV, const double* U, const double* s, double* out) {
  // ||A v_j - s_j u_j|| with unit u, v (computed after normalisation): FP64
  __shared__ double red[32];
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      double r = AV[i + j * m] - s[j] * U[i + j * m];
      acc = fma(r, r, acc);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
      out[j] = sqrt(t);
    }
    __syncthreads();
  }
}

// X(:, j) *= 1 / nrm[j] (columns of zero norm untouched); one reciprocal per thread and column, the
// FP64 pipe being 1/64 rate.  The unit columns feed residual estimates only.
__global__ void k_normalize_cols(int64_t m, int64_t n, double* X, const double* nrm) {
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    const double s = nrm[j];
    if (!(s > 0)) continue;
    const double r = 1.0 / s;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
      X[i + j * m] *= r;
  }
}

// certify16 >= 0: emulated products; the bounds on their errors are added to the residuals, computed
// only when every emulated residual is at most bounds_below (they decide nothing otherwise)
int svd_residuals_dev(ofrr_ctx* ctx, Op& op, ofrr_dtype tx, const void* U, int64_t ldu, const void* V, int64_t ldv,
                      int k, const double* s_host, double normA, double* out_host, int certify16 = -1,
                      double* emul_host = nullptr, double bounds_below = INFINITY) {
  if (k <= 0) return OFRR_SUCCESS;
  WsScope scope(ctx);
  const int64_t m = op.m(), n = op.n();
  double *U64, *V64, *AV, *ATU, *sd, *nr;
  OFRR_TRY(dmalloc(ctx, &U64, (size_t)m * k));
  OFRR_TRY(dmalloc(ctx, &V64, (size_t)n * k));
  OFRR_TRY(dmalloc(ctx, &AV, (size_t)m * k));
  OFRR_TRY(dmalloc(ctx, &ATU, (size_t)n * k));
  OFRR_TRY(dmalloc(ctx, &sd, (size_t)k));
  OFRR_TRY(dmalloc(ctx, &nr, (size_t)4 * k));
  OFRR_TRY(cast_impl(ctx, tx, OFRR_F64, m, k, U, ldu, U64, m));
  OFRR_TRY(cast_impl(ctx, tx, OFRR_F64, n, k, V, ldv, V64, n));
  OFRR_TRY(column_norms(ctx, OFRR_F64, m, k, U64, m, nr));
  OFRR_TRY(column_norms(ctx, OFRR_F64, n, k, V64, n, nr + k));
  k_normalize_cols<<<grid_cols(m, k), 256, 0, ctx->stream>>>(m, k, U64, nr);
  OFRR_LAUNCHED(ctx, "k_normalize_cols");
  k_normalize_cols<<<grid_cols(n, k), 256, 0, ctx->stream>>>(n, k, V64, nr + k);
  OFRR_LAUNCHED(ctx, "k_normalize_cols");
  OFRR_TRY(op.apply(ctx, 0, OFRR_F64, OFRR_F64, V64, n, k, OFRR_F64, OFRR_F64, AV, m));
  OFRR_TRY(op.apply(ctx, 1, OFRR_F64, OFRR_F64, U64, m, k, OFRR_F64, OFRR_F64, ATU, n));
  OFRR_CUDA(cudaMemcpyAsync(sd, s_host, sizeof(double) * k, cudaMemcpyHostToDevice, ctx->stream));
  if (k <= 1024) {
    OFRR_TRY(residual_columns2(ctx, m, k, AV, U64, sd, nr + 2 * k));
    OFRR_TRY(residual_columns2(ctx, n, k, ATU, V64, sd, nr + 3 * k));
  } else {
    k_rescol2<<<k, 256, 0, ctx->stream>>>(m, k, AV, U64, sd, nr + 2 * k);
    OFRR_LAUNCHED(ctx, "k_rescol2");
    k_rescol2<<<k, 256, 0, ctx->stream>>>(n, k, ATU, V64, sd, nr + 3 * k);
    OFRR_LAUNCHED(ctx, "k_rescol2");
  }
  std::vector<double> h(4 * k, 0.0);
  OFRR_CUDA(cudaMemcpyAsync(h.data(), nr + 2 * k, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  if (normA <= 0) {
    normA = 0;
    for (int j = 0; j < k; ++j) normA = std::max(normA, std::fabs(s_host[j]));
    if (normA == 0) normA = 1;
  }
  double emax = 0;
  for (int j = 0; j < k; ++j) emax = std::max(emax, std::max(h[j], h[k + j]) / normA);
  if (certify16 >= 0 && emax <= bounds_below) {  // emulated A v and A' u: the bounds on their errors
    double* bnd;
    OFRR_TRY(dmalloc(ctx, &bnd, (size_t)2 * k));
    OFRR_TRY(emulation_bounds(ctx, op, 0, (ofrr_dtype)certify16, V64, n, k, bnd));
    OFRR_TRY(emulation_bounds(ctx, op, 1, (ofrr_dtype)certify16, U64, m, k, bnd + k));
    OFRR_CUDA(cudaMemcpyAsync(h.data() + 2 * k, bnd, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
  }
  for (int j = 0; j < k; ++j) {
    out_host[j] = std::max(h[j] + kEmulBound * h[2 * k + j], h[k + j] + kEmulBound * h[3 * k + j]) / normA;
    if (emul_host) emul_host[j] = std::max(h[j], h[k + j]) / normA;
  }
  return OFRR_SUCCESS;
}

// The certification's fallback for the columns J only: those columns are gathered into contiguous
// buffers and their residuals recomputed with true FP64 products (normA is the full set's, so the
// values are the ones the full recomputation gives).  Usually one or two columns miss the
// certified bound by a hair; the others keep their certified values.
double norm_of_values(const double* v, int k) {
  double a = 0;
  for (int j = 0; j < k; ++j) a = std::max(a, std::fabs(v[j]));
  return a > 0 ? a : 1.0;
}

int svd_residuals_subset(ofrr_ctx* ctx, Op& op, const double* U, int64_t ldu, const double* V, int64_t ldv,
                         const std::vector<int>& J, const double* s_host, double normA, double* out_host) {
  if (J.empty()) return OFRR_SUCCESS;
  WsScope scope(ctx);
  const int64_t m = op.m(), n = op.n();
  const int q = (int)J.size();
  double *Ug, *Vg;
  OFRR_TRY(dmalloc(ctx, &Ug, (size_t)m * q));
  OFRR_TRY(dmalloc(ctx, &Vg, (size_t)n * q));
  std::vector<double> sq(q), rq(q);
  for (int t = 0; t < q; ++t) {
    OFRR_CUDA(cudaMemcpyAsync(Ug + (size_t)t * m, U + (size_t)J[t] * ldu, sizeof(double) * m,
                              cudaMemcpyDeviceToDevice, ctx->stream));
    OFRR_CUDA(cudaMemcpyAsync(Vg + (size_t)t * n, V + (size_t)J[t] * ldv, sizeof(double) * n,
                              cudaMemcpyDeviceToDevice, ctx->stream));
    sq[t] = s_host[J[t]];
  }
  OFRR_TRY(svd_residuals_dev(ctx, op, OFRR_F64, Ug, m, Vg, n, q, sq.data(), normA, rq.data()));
  for (int t = 0; t < q; ++t) out_host[J[t]] = rq[t];
  return OFRR_SUCCESS;
}

int residuals_subset(ofrr_ctx* ctx, Op& op, const double* X, int64_t ldx, const std::vector<int>& J,
                     const double* lam_host, double normA, double* out_host) {
  if (J.empty()) return OFRR_SUCCESS;
  WsScope scope(ctx);
  const int64_t n = op.m();
  const int q = (int)J.size();
  double* Xg;
  OFRR_TRY(dmalloc(ctx, &Xg, (size_t)n * q));
  std::vector<double> lq(q), rq(q);
  for (int t = 0; t < q; ++t) {
    OFRR_CUDA(cudaMemcpyAsync(Xg + (size_t)t * n, X + (size_t)J[t] * ldx, sizeof(double) * n,
                              cudaMemcpyDeviceToDevice, ctx->stream));
    lq[t] = lam_host[J[t]];
  }
  OFRR_TRY(residuals_dev(ctx, op, OFRR_F64, Xg, n, q, lq.data(), normA, rq.data()));
  for (int t = 0; t < q; ++t) out_host[J[t]] = rq[t];
  return OFRR_SUCCESS;
}


}  // namespace
}  // namespace ofrr

extern "C" int ofrr_rr_svd(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, int64_t ncols, void* U,
                           int64_t ldu, double* s, void* V, int64_t ldv) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  OFRR_TRY(validate_options(opt));
  const int64_t m = A->nrows, n = A->ncols;
  if (ncols <= 0 || m == 0 || n == 0) return OFRR_SUCCESS;
  if (!U || !V || !s || ldu < m || ldv < n || ncols > 512) return OFRR_ERR_INVALID_ARGUMENT;
  const Precisions P = precisions_of(opt);
  WsScope scope(ctx);
  Op op{A};
  OFRR_TRY(op.prepare_csr_t(ctx));
  double* d;
  OFRR_TRY(dmalloc(ctx, &d, (size_t)ncols));
  const int b = (int)ncols;
  int st = OFRR_SUCCESS;
  void* Ut = ws_alloc(ctx, (size_t)m * b * dtype_size(P.po), &st);
  void* Vt = ws_alloc(ctx, (size_t)n * b * dtype_size(P.po), &st);
  if (!Ut || !Vt) return st;
  OFRR_TRY(rr_svd_dev(ctx, op, P.po, U, V, P.po, ldu, ldv, b, P.prc, P.pro, P.pc, P.po, opt->use_generalized != 0,
                      opt->generalized_tol, Ut, m, Vt, n, d));
  OFRR_CUDA(cudaMemcpy2DAsync(U, ldu * dtype_size(P.po), Ut, m * dtype_size(P.po), m * dtype_size(P.po), b,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpy2DAsync(V, ldv * dtype_size(P.po), Vt, n * dtype_size(P.po), n * dtype_size(P.po), b,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(s, d, sizeof(double) * b, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_and_check(ctx);
}

// ======================================================================================
// Krylov eigensolver, production modes: thick-restart Hessenberg process (new behaviour)
// ======================================================================================
// arnoldi_hess_eig.m:99-106 restarts from the leading Ritz vector alone; on 20 clustered eigenvalues
// (the 3D convection-diffusion operator) that never reaches a tolerance.  The production modes keep a
// block Y spanning the invariant subspace of the leading Ritz values at each restart -- the Ritz vectors
// for a symmetric operator, the range of the matrix-sign projector otherwise (close Ritz values of a
// non-normal projection can have nearly parallel Ritz vectors, whose span is lost to rounding and then
// stalls the restarts) -- plus the Galerkin residual direction f = A v_last - V M^-1 V' A v_last.  The
// residuals of the Ritz vectors of a Galerkin projection onto a Krylov space are all parallel to f, so
// span{Y, f, A f, ...} is again a Krylov space (the thick restart of Wu and Simon, and of Stathopoulos,
// Saad and Wu; Stewart's Krylov-Schur for the nonsymmetric case), here built on the oblique Hessenberg
// basis: the block [Y, f] gets a Hessenberg basis, the Krylov steps continue from f (krylov_tr.cu), and
// Rayleigh-Ritz is the generalized one of arnoldi_hess_eig.m:89-95 (eig(V'AV, V'V + tau I)).
// Mixed mode: a 16-bit phase (16-bit basis, FP32 matvec on the FP32 value copy, FP32 arithmetic) until
// its residuals stop improving, then an FP64 phase restarted from the sum of the unit Ritz vectors (the
// 16-bit rounding leaves the kept block's residuals no longer parallel, and a kept block then stalls).
// Ritz vectors kept at a thick restart when the caller leaves restart_keep at 0 (the cut then sits at the
// widest gap among the next few Ritz values).  Nonsymmetric operators: the nev wanted ones, so that each
// cycle adds kdim - nev new directions -- on the 128^3 convection-diffusion operator (nev 20, kdim 64)
// keep 20 converged in 70 cycles (2.63 s), 24 in 74 (2.89 s), 28 in 81, 32 in 92, 36 in 110.  Symmetric
// operators: max(nev + 4, 1.2 nev) -- on ten of the serving stream's clustered Laplacians keeping only
// nev converged 2 instead of 4.
static int default_keep(int nev, int kdim, bool symmetric) {
  return std::min(symmetric ? std::max(nev + 4, (nev * 6 + 4) / 5) : nev, kdim - 2);
}

static int arnoldi_thick_body(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, const void* v0,
                              void* X, int64_t ldx, double* evals, double* resid, ofrr_info* info) {
  const int64_t n = A->nrows;
  const int kdim = opt->kdim > 0 ? opt->kdim : opt->maxiter;
  const int nb = kdim + 1;
  const int nev = (int)std::min<int64_t>(opt->nev, n);
  // nb <= 128: the projected pencil's solvers hold at most 128 columns
  if (nb > std::min(kKryMaxNb, 128) || nb > n || kdim < 4) return OFRR_ERR_BLAS_INVALID_SIZE;
  int keep = opt->restart_keep > 0 ? opt->restart_keep : default_keep(nev, kdim, A->symmetric != 0);
  keep = std::min(std::max(keep, nev), kdim - 2);
  if (nev > keep) return OFRR_ERR_INVALID_ARGUMENT;  // nev > kdim - 2
  const bool symmetric = A->symmetric != 0;
  const bool mixed = opt->mode == OFRR_MODE_MIXED;
  const ofrr_dtype t16 = (opt->p_output == OFRR_BF16) ? OFRR_BF16 : OFRR_F16;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  Op op{A};
  const int64_t ld = kry_ld(n);
  const int wcols = nev + keep + 6;
  double* AVb = ws_get<double>(ctx, (size_t)ld * nb, &st);
  double* Wb = ws_get<double>(ctx, (size_t)ld * wcols, &st);
  double* svec = ws_get<double>(ctx, (size_t)ld, &st);
  if (!AVb || !Wb || !svec) return st;
  double *G, *M, *U, *d, *xg, *Cf, *R, *nrm;
  int *sel, *perm;
  OFRR_TRY(dmalloc(ctx, &G, (size_t)nb * nb));
  OFRR_TRY(dmalloc(ctx, &M, (size_t)nb * nb));
  OFRR_TRY(dmalloc(ctx, &U, (size_t)nb * nb));
  OFRR_TRY(dmalloc(ctx, &Cf, (size_t)nb * (wcols + keep + 6)));
  OFRR_TRY(dmalloc(ctx, &R, (size_t)(keep + 6) * (keep + 6)));
  OFRR_TRY(dmalloc(ctx, &d, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &xg, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &nrm, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &sel, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &perm, (size_t)nb));
  // the start vector (FP64) as the first block
  if (opt->use_start_block) {
    OFRR_CUDA(cudaMemcpyAsync(Wb, v0, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    OFRR_TRY(ofrr_randn(ctx, opt->seed, n, 1, OFRR_F64, Wb, ld));
  }
  ofrr_dtype tw = OFRR_F64;  // type of the block in Wb
  void* blk = Wb;            // the next block: q0 columns at blk (leading dimension ld)
  int q0 = 1;
  int phase = 0;
  KryState S;
  const double stol = opt->select_tol < 0 ? 0.0 : opt->select_tol;
  OFRR_TRY(kry_state_init(ctx, &S, &A->csr, mixed ? t16 : OFRR_F64, nb, stol));
  std::vector<double> hd(nb), hres(nb, INFINITY);
  std::vector<int> hsel(nb), hperm(nb), cperm(nb);
  int cycles = 0, steps = 0, nmv = 0, escalations = 0, ncols = 0, in_phase = 0, k = std::min(nev, nb);
  double best_in_phase = INFINITY, last_maxres = INFINITY, best64 = INFINITY;
  int stall64 = 0;
  std::array<double, 16> hist64{};  // the FP64 phase's last 16 residuals
  bool converged = false, exact_rr = false;
  const bool kry_debug = getenv("OFRR_KRYLOV_DEBUG") != nullptr;  // per-cycle progress on stderr
  while (true) {
    TraceScope ts(ctx, "krylov.block");
    const ofrr_dtype t = S.t, ta = kry_arith_type(t);
    // (1) Hessenberg basis of the block [Y, f] (columns scaled to a unit maximum first, so that the
    //     selection threshold is relative): columns 0 .. q-1 of the new basis
    int q = 0;
    {
      WsScope inner(ctx);
      OFRR_TRY(scalecols_impl(ctx, tw, tw, n, q0, blk, ld, nullptr, tw == OFRR_F64));
      const double stol_blk = (t == OFRR_F64) ? 1e-12 : 4.0 * dtype_eps(t);
      OFRR_TRY(hessenberg_impl(ctx, tw, t, ta, n, q0, blk, ld, S.V, S.ldv, stol_blk, R, sel, perm, true));
      OFRR_CUDA(cudaMemcpyAsync(hsel.data(), sel, sizeof(int) * q0, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_CUDA(cudaMemcpyAsync(hperm.data(), perm, sizeof(int) * q0, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
      std::vector<int> s0(hsel.begin(), hsel.begin() + q0);
      for (int j = 0; j < q0; ++j)
        if (s0[j]) cperm[q++] = hperm[j];
      int w = 0;
      OFRR_TRY(compact_columns(ctx, t, n, S.V, S.ldv, s0, &w));
    }
    if (q == 0) return OFRR_ERR_SOLVER_DIVERGENCE;  // the start vector is zero
    OFRR_CUDA(cudaMemcpyAsync(S.perm, cperm.data(), sizeof(int) * q, cudaMemcpyHostToDevice, ctx->stream));
    // (2) Krylov steps q .. nb-1
    ts.next("krylov.steps");
    OFRR_TRY(kry_cycle_steps(ctx, S, q));
    int hstop = -1;
    OFRR_CUDA(cudaMemcpyAsync(&hstop, S.stop, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
    ncols = (hstop >= 0) ? hstop : nb;
    steps += ncols - q;
    // (3) generalized Rayleigh-Ritz on the ncols columns, the Ritz vectors, the kept block and the
    //     residual direction
    ts.next("rr");
    const ofrr_dtype tav = ta;
    int pp = 0;
    bool sign_ok = false;
    {
      WsScope inner(ctx);
      TraceScope tsr(ctx, "rr.spmm");
      OFRR_TRY(csrmm_impl(ctx, &A->csr, 0, t, ta, tav, ncols, S.V, S.ldv, AVb, ld));
      nmv += ncols;
      tsr.next(t == OFRR_F64 ? "rr.gram.f64" : "rr.gram.16bit");
      ctx->emulate_f64 = mixed && t == OFRR_F64;
      int rst = OFRR_SUCCESS;
      if (exact_rr && t == OFRR_F64) {  // FP64 arithmetic for the Grams once the emulated phase stalls
        rst = gram_f64(ctx, ncols, ncols, n, (const double*)S.V, S.ldv, (const double*)S.V, S.ldv, M, ncols);
        if (rst == OFRR_SUCCESS)
          rst = gram_f64(ctx, ncols, ncols, n, (const double*)S.V, S.ldv, (const double*)AVb, ld, G, ncols);
      } else {
        rst = gemm_impl(ctx, 1, 0, t, t, ta, OFRR_F64, ncols, ncols, n, 1.0, S.V, S.ldv, S.V, S.ldv, 0.0, M, ncols);
      }
      if (rst == OFRR_SUCCESS && !(exact_rr && t == OFRR_F64)) {
        if ((t == OFRR_F16 || t == OFRR_BF16) && tav == OFRR_F32)
          rst = kry_gram16(ctx, t, n, ncols, S.V, S.ldv, (const float*)AVb, ld, G);
        else
          rst = gemm_impl(ctx, 1, 0, t, tav, ta, OFRR_F64, ncols, ncols, n, 1.0, S.V, S.ldv, AVb, ld, 0.0, G, ncols);
      }
      ctx->emulate_f64 = false;
      OFRR_TRY(rst);
      if (opt->generalized_tol != 0.0) {
        k_add_diag<<<(ncols + 255) / 256, 256, 0, ctx->stream>>>(ncols, M, ncols, opt->generalized_tol);
        OFRR_LAUNCHED(ctx, "k_add_diag");
      }
      tsr.next(t == OFRR_F64 ? "rr.eig.f64" : "rr.eig.16bit");
      // FP64 phase, nonsymmetric: the whole pencil in FP32 only to place the restart cut; the k leading
      // pairs come in FP64 from the invariant subspace below (restricted pencil)
      const bool restricted = !symmetric && t == OFRR_F64 && ncols <= 96;
      if (symmetric) OFRR_TRY(geig_fast(ctx, ncols, G, M, 0.0, d, U, t == OFRR_F64 ? 2 : 1));
      else OFRR_TRY(geig_nonsym(ctx, ncols, G, M, d, U, t == OFRR_F64 && !restricted, true, restricted));
      OFRR_CUDA(cudaMemcpyAsync(hd.data(), d, sizeof(double) * ncols, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
      k = std::min(nev, ncols);
      // the kept block ends at the widest gap of the real parts near `keep` (never inside a complex pair)
      pp = std::min(keep, ncols - 1);
      {
        double best_gap = -1.0;
        const int lo = std::max(nev, keep - 3), hi = std::min(keep + 4, ncols - 2);
        for (int c = lo; c <= hi; ++c) {
          const double gap = hd[c - 1] - hd[c];
          if (gap > best_gap) {
            best_gap = gap;
            pp = c;
          }
        }
        if (best_gap <= 0.0) pp = std::min(keep, ncols - 1);
      }
      OFRR_TRY(kry_spd_solve(ctx, ncols, M, G + (size_t)(ncols - 1) * ncols, xg));
      const double* Yc = U;
      double* Ys = Cf + (size_t)ncols * (k + pp + 1);
      tsr.next("rr.sign");
      if (!symmetric && ncols <= 96 && pp < ncols) {
        const double sigma = 0.5 * (hd[pp - 1] + hd[pp]);
        const int ist = invariant_subspace_nonsym(ctx, ncols, G, M, sigma, pp, Ys);
        if (ist == OFRR_SUCCESS) Yc = Ys;
        else if (ist != OFRR_ERR_SINGULAR_MATRIX) return ist;
        sign_ok = (ist == OFRR_SUCCESS);
      }
      if (restricted) {
        tsr.next("rr.ritz.f64");
        if (sign_ok) {
          OFRR_TRY(ritz_from_invariant(ctx, ncols, G, M, Ys, pp, k, d, U));
          OFRR_CUDA(cudaMemcpyAsync(hd.data(), d, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
        } else {  // no invariant subspace (sigma met an eigenvalue): the whole pencil in FP64
          OFRR_TRY(geig_nonsym(ctx, ncols, G, M, d, U, true, true));
          OFRR_CUDA(cudaMemcpyAsync(hd.data(), d, sizeof(double) * ncols, cudaMemcpyDeviceToHost, ctx->stream));
        }
        OFRR_TRY(sync_and_check(ctx));
      }
      // Wb = V [U(:, :k), Yc, -M^-1 G(:, last)] (+ A v_last in the last column): the k Ritz vectors, then
      // the next block
      tsr.next("rr.update");
      OFRR_TRY(kry_coef_matrix(ctx, ncols, k, U, pp, Yc, xg, Cf));
      tw = (t == OFRR_F64) ? OFRR_F64 : OFRR_F32;
      ctx->emulate_f64 = mixed && t == OFRR_F64;
      // the emulated back-transform's error is relative to |V||C| (the Krylov basis is not orthogonal), which
      // floors the Ritz residuals near 1e-8 of ||A|| (higher for ill-conditioned bases of clustered
      // spectra): targets below 1e-9, and a stalled FP64 phase, finish with FP64 arithmetic
      const bool exact_bt = mixed && t == OFRR_F64 &&
                            (exact_rr || (opt->tol > 0 && opt->tol < 1e-9 && last_maxres <= 1e3 * opt->tol));
      rst = kry_backtransform(ctx, t, n, ncols, S.V, S.ldv, Cf, k + pp + 1, tw, Wb, ld, exact_bt);
      ctx->emulate_f64 = false;
      OFRR_TRY(rst);
      OFRR_TRY(kry_add_col(ctx, tw, n, (char*)Wb + (size_t)(k + pp) * ld * dtype_size(tw), tav,
                           (const char*)AVb + (size_t)(ncols - 1) * ld * dtype_size(tav)));
    }
    cycles++;
    in_phase++;
    // (4) true FP64 residuals of the k leading Ritz vectors
    ts.next("check");
    OFRR_TRY(residuals_dev(ctx, op, tw, Wb, ld, k, hd.data(), -1.0, hres.data()));
    double maxres = 0;
    for (int j = 0; j < k; ++j) maxres = std::max(maxres, hres[j]);
    last_maxres = maxres;
    if (kry_debug)
      fprintf(stderr, "[ofrr krylov] cycle %d phase %d exact %d type %d q %d ncols %d pp %d sign %d maxres %.3e d0 %.10e\n",
              cycles, phase, exact_rr ? 1 : 0, (int)t, q, ncols, pp, sign_ok ? 1 : 0, maxres, hd[0]);
    if (opt->tol > 0 && maxres <= opt->tol) {
      converged = true;
      break;
    }
    if (hstop >= 0 || steps >= opt->maxiter) break;  // invariant subspace found, or the step budget spent
    // (5) next block: the kept block and the residual direction, or (phase change) the sum of the unit
    //     Ritz vectors alone
    const double switch_at = (t == OFRR_BF16) ? 1e-2 : 1e-3;
    const bool stalled = in_phase >= 3 && maxres > 0.7 * best_in_phase;
    best_in_phase = std::min(best_in_phase, maxres);
    // FP64 phase: a floor of the emulated products -- FP64 products from here on.  A floor is flat: the
    // last 16 residuals within 2x of each other (a clustered spectrum's slow convergence swings by 10x
    // from cycle to cycle and is not a floor), and no gain over them -- 10 % for symmetric operators
    // (clustered spectra give ill-conditioned Hessenberg bases, whose emulated products then stall the
    // solve well above tol; below 1e-4), 2x for nonsymmetric ones (they gain slowly but steadily, and
    // FP64 Grams cost ~50 ms per cycle at two million rows; below 1e-6)
    const double gain = symmetric ? 0.9 : 0.5;
    if (maxres < gain * best64) {
      best64 = maxres;
      stall64 = 0;
    } else {
      ++stall64;
    }
    hist64[in_phase % 16] = maxres;
    double wmin = INFINITY, wmax = 0.0;
    for (double v : hist64) {
      wmin = std::min(wmin, v);
      wmax = std::max(wmax, v);
    }
    const bool to_exact = mixed && phase == 1 && !exact_rr && stall64 >= 16 && in_phase >= 16 &&
                          wmax <= 2.0 * wmin && maxres < (symmetric ? 1e-4 : 1e-6);
    // a floor of the FP64 products themselves (the basis's conditioning): no gain over 32 cycles and the
    // last 16 residuals within 10 % of each other (a plateau of a clustered spectrum's convergence moves
    // more) -- the step budget cannot lower it, so the solve ends here (not converged, best pairs returned)
    if (exact_rr && stall64 >= 32 && in_phase >= 32 && wmax <= 1.1 * wmin) break;
    const bool to_f64 = mixed && phase == 0 && (maxres <= switch_at || stalled);
    if (to_f64 || to_exact) {
      // a restart from one vector, the sum of the unit Ritz vectors: a thick restart carries the error
      // of the Krylov relation A [Yc] = [Yc, f] H of the cycle before (the 16-bit basis's rounding, or
      // the emulated products' floor) into every later cycle, so the residuals could not fall below it;
      // one vector starts an exact Krylov relation in the new arithmetic
      OFRR_TRY(column_norms(ctx, tw, n, k, Wb, ld, nrm));
      OFRR_TRY(kry_sum_unit_cols(ctx, tw, n, k, Wb, ld, nrm, svec));
      OFRR_CUDA(cudaMemcpyAsync(Wb, svec, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
      tw = OFRR_F64;
      blk = Wb;
      q0 = 1;
      if (to_exact) exact_rr = true;
      phase = 1;
      in_phase = 0;
      best_in_phase = INFINITY;
      best64 = INFINITY;
      stall64 = 0;
      escalations++;
      if (to_f64) OFRR_TRY(kry_state_init(ctx, &S, &A->csr, OFRR_F64, nb, stol));
    } else {
      blk = (char*)Wb + (size_t)k * ld * dtype_size(tw);
      q0 = pp + 1;
    }
  }
  // Ritz vectors (FP64) and values out
  OFRR_TRY(cast_impl(ctx, tw, OFRR_F64, n, k, Wb, ld, X, ldx));
  OFRR_TRY(sync_and_check(ctx));
  int conv = 0;
  double maxr = 0;
  for (int j = 0; j < nev; ++j) {
    evals[j] = (j < k) ? hd[j] : NAN;
    if (resid) resid[j] = (j < k) ? hres[j] : NAN;
  }
  for (int j = 0; j < k; ++j) {
    conv += (opt->tol > 0 && hres[j] <= opt->tol) ? 1 : 0;
    maxr = std::max(maxr, hres[j]);
  }
  if (info) {
    info->iterations = cycles;
    info->matvecs = steps + nmv;
    info->converged = conv;
    info->basis_width = ncols;
    info->max_residual = maxr;
    info->escalations = escalations;
    info->status_detail = 0;
  }
  if (opt->tol > 0 && !converged) return OFRR_ERR_SOLVER_MAX_ITERATIONS;
  return OFRR_SUCCESS;
}

// ======================================================================================
// Krylov eigensolver: Hessenberg process with restarts (arnoldi_hess_eig.m:51-107)
// ======================================================================================
static int arnoldi_eig_body(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, const void* v0,
                            void* X, int64_t ldx, double* evals, double* resid, ofrr_info* info) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  OFRR_TRY(validate_options(opt));
  if (A->nrows != A->ncols) return OFRR_ERR_BLAS_INVALID_SIZE;
  if (opt->orth != OFRR_ORTH_HESSENBERG && opt->orth != OFRR_ORTH_MGS) return OFRR_ERR_INVALID_ARGUMENT;
  const bool mgs = opt->orth == OFRR_ORTH_MGS;
  if (!mgs && opt->mode != OFRR_MODE_REFERENCE && A->kind == OFRR_OP_CSR && opt->restart_keep != 1) {
    if (A->nrows == 0 || opt->nev <= 0) return OFRR_SUCCESS;
    if (!X || ldx < A->nrows || !evals || (opt->use_start_block && !v0)) return OFRR_ERR_INVALID_ARGUMENT;
    return arnoldi_thick_body(ctx, A, opt, v0, X, ldx, evals, resid, info);
  }
  const int64_t n = A->nrows;
  const int kdim = opt->kdim > 0 ? opt->kdim : opt->maxiter;
  const int nev = (int)std::min<int64_t>(opt->nev, n);
  if (n == 0 || nev <= 0) return OFRR_SUCCESS;
  if (!X || ldx < n || !evals || kdim < 1 || kdim + 1 > 1024 || (opt->use_start_block && !v0))
    return OFRR_ERR_INVALID_ARGUMENT;
  const Precisions P = precisions_of(opt);
  const ofrr_dtype po = P.po, pc = P.pc;
  const bool symmetric = A->symmetric != 0;
  const int nb = kdim + 1;
  const double stol = opt->select_tol < 0 ? dtype_eps(po) : opt->select_tol;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  Op op{A};
  void *V, *pivrows, *pvals, *Vr;
  double *R, *d;
  int *sel, *perm, *stop;
  if (!(V = ws_alloc(ctx, (size_t)n * nb * dtype_size(po), &st))) return st;
  if (!(Vr = ws_alloc(ctx, (size_t)n * nb * dtype_size(po), &st))) return st;
  if (!(pivrows = ws_alloc(ctx, (size_t)nb * nb * dtype_size(po), &st))) return st;
  if (!(pvals = ws_alloc(ctx, (size_t)nb * dtype_size(po), &st))) return st;
  OFRR_TRY(dmalloc(ctx, &R, (size_t)nb * nb));
  OFRR_TRY(dmalloc(ctx, &d, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &sel, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &perm, (size_t)nb));
  OFRR_TRY(dmalloc(ctx, &stop, (size_t)4));
  void* mscratch = nullptr;
  if (mgs) {
    if (!(mscratch = ws_alloc(ctx, mgs_scratch_bytes(), &st))) return st;
    OFRR_TRY(fill_zero(ctx, mscratch, mgs_scratch_bytes()));
  }
  OFRR_TRY(fill_zero(ctx, V, (size_t)n * nb * dtype_size(po)));
  if (opt->use_start_block) {
    OFRR_CUDA(cudaMemcpyAsync(V, v0, (size_t)n * dtype_size(po), cudaMemcpyDeviceToDevice, ctx->stream));
  } else {
    OFRR_TRY(ofrr_randn(ctx, opt->seed, n, 1, po, V, n));
  }
  int tits = 1, cycles = 0, nmv = 0;
  std::vector<double> hd(nb), hres(nb, INFINITY);
  int hstop[2];
  int ncols_final = 0;
  bool have_result = false;
  while (tits < opt->maxiter) {
    TraceScope ts(ctx, "krylov");
    // column 0: pivot + scale (Hessenberg, arnoldi_hess_eig.m:64-71) or normalise (MGS,
    // arnoldi_mgs_eig.m:60-65); break if the pivot / norm is below select_tol
    if (mgs) {
      OFRR_CUDA(cudaMemsetAsync(stop, 0xFF, 2 * sizeof(int), ctx->stream));
      OFRR_TRY(mgs_step(ctx, po, pc, n, 0, V, n, opt->reorth != 0, stol, stop, mscratch));
    } else {
      OFRR_TRY(hess_krylov_first(ctx, po, pc, n, nb, V, n, stol, sel, perm, pivrows, pvals, R, stop));
    }
    OFRR_CUDA(cudaMemcpyAsync(hstop, stop, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
    if (hstop[0] >= 0) break;  // start vector below select_tol
    int ncols = nb;
    for (int i = 1; i <= kdim; ++i) {
      // V(:,i) = po(matvec(A, pc(V(:,i-1)), pc, pc)); column i-1 was scaled by the previous step
      OFRR_TRY(op.apply(ctx, 0, po, po, (char*)V + (size_t)(i - 1) * n * dtype_size(po), n, 1, pc, po,
                        (char*)V + (size_t)i * n * dtype_size(po), n));
      if (mgs) {
        OFRR_TRY(mgs_step(ctx, po, pc, n, i, V, n, opt->reorth != 0, stol, stop, mscratch));
      } else {
        OFRR_TRY(hess_krylov_step(ctx, po, pc, n, nb, i, V, n, stol, sel, perm, pivrows, pvals, R, stop));
        OFRR_TRY(hess_scale_col(ctx, po, pc, n, i, V, n, sel, pvals, stop));
      }
    }
    OFRR_CUDA(cudaMemcpyAsync(hstop, stop, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
    int steps = kdim;
    if (hstop[0] >= 0) {  // breakdown at step hstop[0]: invariant subspace found
      steps = hstop[0] - 1;
      ncols = hstop[0];
      tits = opt->maxiter;
    } else {
      tits += kdim;
    }
    nmv += steps;
    cycles++;
    ts.next("rr");
    // RR on the ncols columns: generalized for the oblique Hessenberg basis (arnoldi_hess_eig.m:93),
    // as the options say for the orthonormal MGS basis (arnoldi_mgs_eig.m:95-100)
    OFRR_TRY(rr_eig_dev(ctx, op, po, V, po, n, ncols, pc, po, pc, pc, mgs ? opt->use_generalized != 0 : true,
                        opt->generalized_tol, symmetric, Vr, n, d));
    nmv += ncols;
    ncols_final = ncols;
    have_result = true;
    ts.next("check");
    if (tits < opt->maxiter) {
      OFRR_CUDA(cudaMemcpyAsync(V, Vr, (size_t)n * dtype_size(po), cudaMemcpyDeviceToDevice, ctx->stream));
      if (opt->tol > 0) {  // convergence check on the current Ritz pairs (new behaviour)
        OFRR_CUDA(cudaMemcpyAsync(hd.data(), d, sizeof(double) * ncols, cudaMemcpyDeviceToHost, ctx->stream));
        OFRR_TRY(sync_and_check(ctx));
        const int k = std::min(nev, ncols);
        OFRR_TRY(residuals_dev(ctx, op, po, Vr, n, k, hd.data(), -1.0, hres.data()));
        bool ok = true;
        for (int j = 0; j < k; ++j) ok = ok && (hres[j] <= opt->tol);
        if (ok) break;
      }
    }
  }
  if (!have_result) return OFRR_ERR_SOLVER_DIVERGENCE;
  const int k = std::min(nev, ncols_final);
  OFRR_CUDA(cudaMemcpy2DAsync(X, ldx * dtype_size(po), Vr, n * dtype_size(po), n * dtype_size(po), k,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  OFRR_CUDA(cudaMemcpyAsync(hd.data(), d, sizeof(double) * ncols_final, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  for (int j = 0; j < nev; ++j) evals[j] = (j < k) ? hd[j] : NAN;
  OFRR_TRY(residuals_dev(ctx, op, po, X, ldx, k, hd.data(), -1.0, hres.data()));
  if (resid)
    for (int j = 0; j < nev; ++j) resid[j] = (j < k) ? hres[j] : NAN;
  int conv = 0;
  double maxr = 0;
  for (int j = 0; j < k; ++j) {
    conv += (opt->tol > 0 && hres[j] <= opt->tol) ? 1 : 0;
    maxr = std::max(maxr, hres[j]);
  }
  if (info) {
    info->iterations = cycles;
    info->matvecs = nmv;
    info->converged = conv;
    info->basis_width = ncols_final;
    info->max_residual = maxr;
    info->escalations = 0;
    info->status_detail = 0;
  }
  if (opt->tol > 0 && conv < k) return OFRR_ERR_SOLVER_MAX_ITERATIONS;
  return OFRR_SUCCESS;
}

extern "C" int ofrr_arnoldi_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, const void* v0,
                                void* X, int64_t ldx, double* evals, double* resid, ofrr_info* info) {
  if (!ctx || !ctx->tracer) return arnoldi_eig_body(ctx, A, opt, v0, X, ldx, evals, resid, info);
  ofrr_info local{};
  ofrr_info* inf = info ? info : &local;
  const unsigned long long l0 = ofrr_ctx_launch_count(ctx);
  trace_begin_solve(ctx);
  const int st = arnoldi_eig_body(ctx, A, opt, v0, X, ldx, evals, resid, inf);
  trace_end_solve(ctx, "arnoldi_eig", A ? A->nrows : 0, A ? A->ncols : 0, opt, st, inf,
                  ofrr_ctx_launch_count(ctx) - l0);
  return st;
}

// ======================================================================================
// subspace iteration: one precision phase, shared by the reference, FP64 and mixed modes
// ======================================================================================
namespace ofrr {
namespace {

struct PhaseState {
  int b = 0;           // current basis width
  int it = 0;          // outer iterations done (all phases)
  int nmv = 0;         // operator applications (columns)
  int converged = 0;   // pairs at tol after the last check
  bool done = false;   // all nev pairs at tol
  std::vector<double> d, res, dprev;
  double delta = INFINITY, delta_prev = INFINITY;
  // emulated FP64 phase: best certified residual, checks without a 10 % gain, and the floor flag
  double best_emul = INFINITY;
  int stall_emul = 0;
  bool emul_floor = false;
};

// The emulated products' accuracy floor: a certified check that has not improved the residual by 10 %
// for 4 checks ends the emulated phase (the caller continues with FP64 products).
bool emulation_floor(PhaseState& S, int kk) {
  double mr = 0;
  for (int j = 0; j < kk; ++j) mr = std::max(mr, S.res[j]);
  if (mr < 0.9 * S.best_emul) {
    S.best_emul = mr;
    S.stall_emul = 0;
  } else {
    ++S.stall_emul;
  }
  S.emul_floor = S.stall_emul >= 4;
  return S.emul_floor;
}

// Ritz-value stagnation test of the low-precision phase: relative change of the top nev values
bool stagnated(PhaseState& S, int nev, double stag_tol, int iters_in_phase) {
  double scale = 0;
  for (int j = 0; j < nev; ++j) scale = std::max(scale, std::fabs(S.d[j]));
  if (scale == 0) scale = 1;
  double delta = 0;
  for (int j = 0; j < nev; ++j) delta = std::max(delta, std::fabs(S.d[j] - S.dprev[j]) / scale);
  S.delta_prev = S.delta;
  S.delta = delta;
  S.dprev = S.d;
  if (iters_in_phase < 2) return false;
  return delta <= stag_tol || (iters_in_phase >= 4 && delta > 0.7 * S.delta_prev);
}

// One phase of subspace_iter_eig.m:60-68 on the iterate V (n x b, type P.po, in the caller's buffer).
// Exits after maxit iterations, when the nev residuals reach tol (checked every check_every) or,
// if stag_tol > 0, when the Ritz values stop improving.
int eig_phase(ofrr_ctx* ctx, Op& op, const Precisions& P, const ofrr_options* opt, void* V, int64_t ldv, int maxit,
              double tol, int nev, double stag_tol, PhaseState& S, double* d_dev, int certify16 = -1) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t n = op.m();
  const int b0 = S.b;
  const bool symmetric = op.A->symmetric != 0;
  void *W, *Q;
  double* R;
  int *sel, *perm;
  if (!(W = ws_alloc(ctx, (size_t)n * b0 * dtype_size(P.po), &st))) return st;
  if (!(Q = ws_alloc(ctx, (size_t)n * b0 * dtype_size(P.pho), &st))) return st;
  OFRR_TRY(dmalloc(ctx, &R, (size_t)b0 * b0));
  OFRR_TRY(dmalloc(ctx, &sel, (size_t)b0));
  OFRR_TRY(dmalloc(ctx, &perm, (size_t)b0));
  std::vector<int> hsel(b0);
  const int check_every = std::max(1, opt->check_every);
  void* cur = V;
  int64_t ldcur = ldv;
  const size_t es = dtype_size(P.po);
  const bool f64 = P.po == OFRR_F64;
  for (int k = 0; k < maxit && !S.done; ++k) {
    int b = S.b;
    TraceScope ts(ctx, f64 ? "power.f64" : "power.16bit");
    for (int s = 0; s < opt->step_size; ++s) {
      void* dst = (cur == V) ? W : V;
      int64_t lddst = (cur == V) ? n : ldv;
      OFRR_TRY(op.apply_scale(ctx, 0, P.po, P.pc, cur, ldcur, b, dst, lddst, P.fast));
      S.nmv += b;
      cur = dst;
      ldcur = lddst;
    }
    ts.next(f64 ? "basis.f64" : "basis.16bit");
    // [Q,~] = hessenberg(V): the economic form drops deselected columns
    OFRR_TRY(basis_impl(ctx, opt->orth, P.po, P.pho, P.phc, n, b, cur, ldcur, Q, n, opt->select_tol, R, sel, perm,
                        P.fast));
    OFRR_CUDA(cudaMemcpyAsync(hsel.data(), sel, sizeof(int) * b, cudaMemcpyDeviceToHost, ctx->stream));
    OFRR_TRY(sync_and_check(ctx));
    int w = b;
    OFRR_TRY(compact_columns(ctx, P.pho, n, Q, n, std::vector<int>(hsel.begin(), hsel.begin() + b), &w));
    if (w == 0) return OFRR_ERR_SOLVER_DIVERGENCE;
    S.b = b = w;
    ts.next(f64 ? "rr.f64" : "rr.16bit");
    // [V,D] = eig_rr(A, Q), V = po(V)
    void* dst = (cur == V) ? V : W;
    int64_t lddst = (cur == V) ? ldv : n;
    if (P.pho == P.po) {
      OFRR_TRY(rr_eig_dev(ctx, op, P.po, Q, P.pho, n, b, P.prc, P.pro, P.pc, P.po, opt->use_generalized != 0,
                          opt->generalized_tol, symmetric, dst, lddst, d_dev, P.fast, P.refine));
    } else {
      void* tmpv = ws_alloc(ctx, (size_t)n * b * dtype_size(P.pho), &st);
      if (!tmpv) return st;
      OFRR_TRY(rr_eig_dev(ctx, op, P.po, Q, P.pho, n, b, P.prc, P.pro, P.pc, P.po, opt->use_generalized != 0,
                          opt->generalized_tol, symmetric, tmpv, n, d_dev, P.fast, P.refine));
      OFRR_TRY(cast_impl(ctx, P.pho, P.po, n, b, tmpv, n, dst, lddst));
    }
    S.nmv += b;
    S.it++;
    cur = dst;
    ldcur = lddst;
    ts.next(f64 ? "check.f64" : "check.16bit");
    const int kk = std::min(nev, b);
    const bool last = (k + 1 == maxit);
    const bool check = tol > 0 && ((S.it % check_every) == 0 || last);
    if (check || stag_tol > 0) {
      OFRR_CUDA(cudaMemcpyAsync(S.d.data(), d_dev, sizeof(double) * b, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
    }
    if (check && certify16 >= 0) {
      // certified check (emulated products), as in svd_phase
      std::vector<double> emul(kk);
      OFRR_TRY(residuals_dev(ctx, op, P.po, cur, ldcur, kk, S.d.data(), -1.0, S.res.data(), certify16, emul.data(),
                             tol));
      std::vector<int> J;
      bool hopeless = false;
      for (int j = 0; j < kk; ++j)
        if (!(S.res[j] <= tol)) {
          if (emul[j] <= tol) J.push_back(j);
          else hopeless = true;
        }
      if (!hopeless && !J.empty()) {
        TraceScope tsc(ctx, "certify.fp64");
        const bool em = ctx->emulate_f64;
        ctx->emulate_f64 = false;
        const int st2 = residuals_subset(ctx, op, (const double*)cur, ldcur, J, S.d.data(),
                                         norm_of_values(S.d.data(), kk), S.res.data());
        ctx->emulate_f64 = em;
        OFRR_TRY(st2);
      }
      S.converged = 0;
      for (int j = 0; j < kk; ++j) S.converged += (S.res[j] <= tol) ? 1 : 0;
      if (S.converged >= kk) S.done = true;
      if (!S.done && emulation_floor(S, kk)) break;
    } else if (check) {
      OFRR_TRY(residuals_dev(ctx, op, P.po, cur, ldcur, kk, S.d.data(), -1.0, S.res.data()));
      S.converged = 0;
      for (int j = 0; j < kk; ++j) S.converged += (S.res[j] <= tol) ? 1 : 0;
      if (S.converged >= kk) S.done = true;
    }
    if (!S.done && stag_tol > 0 && stagnated(S, kk, stag_tol, k + 1)) break;
  }
  if (cur != V)
    OFRR_CUDA(cudaMemcpy2DAsync(V, ldv * es, cur, ldcur * es, n * es, S.b, cudaMemcpyDeviceToDevice, ctx->stream));
  return OFRR_SUCCESS;
}

// One phase of subspace_iter_svd.m:60-75 on U (m x b) and V (n x b), type P.po.
int svd_phase(ofrr_ctx* ctx, Op& op, const Precisions& P, const ofrr_options* opt, void* U, int64_t ldu, void* V,
              int64_t ldv, int maxit, double tol, int nev, double stag_tol, PhaseState& S, double* d_dev,
              int certify16 = -1) {
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  const int64_t m = op.m(), n = op.n();
  const int b0 = S.b;
  void *P1, *Q1, *Ut, *Vt;
  double *R, *R2;
  int *sel, *perm, *perm2;
  if (!(P1 = ws_alloc(ctx, (size_t)m * b0 * dtype_size(P.pho), &st))) return st;
  if (!(Q1 = ws_alloc(ctx, (size_t)n * b0 * dtype_size(P.pho), &st))) return st;
  if (!(Ut = ws_alloc(ctx, (size_t)m * b0 * dtype_size(P.pho), &st))) return st;
  if (!(Vt = ws_alloc(ctx, (size_t)n * b0 * dtype_size(P.pho), &st))) return st;
  OFRR_TRY(dmalloc(ctx, &R, (size_t)b0 * b0));
  OFRR_TRY(dmalloc(ctx, &R2, (size_t)b0 * b0));
  OFRR_TRY(dmalloc(ctx, &sel, (size_t)2 * b0));
  OFRR_TRY(dmalloc(ctx, &perm, (size_t)b0));
  OFRR_TRY(dmalloc(ctx, &perm2, (size_t)b0));
  std::vector<int> hsel(2 * b0);
  const int check_every = std::max(1, opt->check_every);
  const bool f64 = P.po == OFRR_F64;
  // fused scaling + digit split for the emulated FP64 products (columns of at most 8192 rows)
  const bool fused = f64 && P.fast && op.can_apply_pre(ctx) && m <= 8192 && n <= 8192;
  __nv_bfloat16 *dig_u = nullptr, *dig_v = nullptr;
  int *exp_u = nullptr, *exp_v = nullptr;
  if (fused) {
    dig_u = ws_get<__nv_bfloat16>(ctx, (size_t)b0 * kSliceDigits * ((m + 63) / 64 * 64), &st);
    dig_v = ws_get<__nv_bfloat16>(ctx, (size_t)b0 * kSliceDigits * ((n + 63) / 64 * 64), &st);
    exp_u = ws_get<int>(ctx, (size_t)b0, &st);
    exp_v = ws_get<int>(ctx, (size_t)b0, &st);
    if (!dig_u || !dig_v || !exp_u || !exp_v) return st;
  }
  for (int k = 0; k < maxit && !S.done; ++k) {
    int b = S.b;
    {
      TraceScope ts(ctx, f64 ? "power.f64" : "power.16bit");
      if (fused) {
        // emulated FP64 products: each scalecols also writes the digits of the scaled block, the
        // operand of the next product (bit-identical to scaling, then splitting); inside the loop
        // the scaling kernel also combines the product's partial sums, and the FP64 blocks are
        // stored only where the steps after the loop read them
        SlicedOperand Us, Vs;
        for (int j = 0; j < opt->step_size; ++j) {
          const bool last = j + 1 == opt->step_size;
          if (j == 0) {
            OFRR_TRY(op.apply(ctx, 0, P.po, P.po, V, ldv, b, P.pc, P.po, U, ldu));
            OFRR_TRY(scalecols_sliced(ctx, m, b, (double*)U, ldu, dig_u, exp_u, &Us));
          } else {
            OFRR_TRY(op.apply_pre_scale(ctx, 0, Vs, (double*)U, ldu, last, dig_u, exp_u, &Us));
          }
          if (!last) {
            OFRR_TRY(op.apply_pre_scale(ctx, 1, Us, (double*)V, ldv, false, dig_v, exp_v, &Vs));
          } else {
            OFRR_TRY(op.apply_pre(ctx, 1, Us, (double*)V, ldv));
            OFRR_TRY(scalecols_impl(ctx, P.po, P.pc, n, b, V, ldv, nullptr, P.fast));
          }
          S.nmv += 2 * b;
        }
      } else {
        for (int j = 0; j < opt->step_size; ++j) {
          OFRR_TRY(op.apply_scale(ctx, 0, P.po, P.pc, V, ldv, b, U, ldu, P.fast));
          OFRR_TRY(op.apply_scale(ctx, 1, P.po, P.pc, U, ldu, b, V, ldv, P.fast));
          S.nmv += 2 * b;
        }
      }
    }
    {
      // the two bases are independent: V's is built on the auxiliary stream beside U's
      TraceScope ts(ctx, f64 ? "basis.f64" : "basis.16bit");
      ofrr_ctx* aux = nullptr;
      OFRR_TRY(aux_begin(ctx, &aux));
      OFRR_TRY(basis_impl(aux, opt->orth, P.po, P.pho, P.phc, n, b, V, ldv, Q1, n, opt->select_tol, R2, sel + b0,
                          perm2, P.fast));
      OFRR_TRY(basis_impl(ctx, opt->orth, P.po, P.pho, P.phc, m, b, U, ldu, P1, m, opt->select_tol, R, sel, perm,
                          P.fast));
      OFRR_TRY(aux_end(ctx));
      OFRR_CUDA(cudaMemcpyAsync(hsel.data(), sel, sizeof(int) * 2 * b0, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
    }
    {
      TraceScope ts(ctx, f64 ? "rr.f64" : "rr.16bit");
      int wu = b, wv = b;
      OFRR_TRY(compact_columns(ctx, P.pho, m, P1, m, std::vector<int>(hsel.begin(), hsel.begin() + b), &wu));
      OFRR_TRY(
          compact_columns(ctx, P.pho, n, Q1, n, std::vector<int>(hsel.begin() + b0, hsel.begin() + b0 + b), &wv));
      const int w = std::min(wu, wv);  // svd_rr.m:61 keeps k = min(ku, kv)
      if (w == 0) return OFRR_ERR_SOLVER_DIVERGENCE;
      S.b = b = w;
      if (P.pho == P.po) {  // the Ritz vectors go straight into U and V (the bases live in P1, Q1)
        OFRR_TRY(rr_svd_dev(ctx, op, P.po, P1, Q1, P.pho, m, n, b, P.prc, P.pro, P.pc, P.po,
                            opt->use_generalized != 0, opt->generalized_tol, U, ldu, V, ldv, d_dev, P.fast, P.refine));
      } else {
        OFRR_TRY(rr_svd_dev(ctx, op, P.po, P1, Q1, P.pho, m, n, b, P.prc, P.pro, P.pc, P.po,
                            opt->use_generalized != 0, opt->generalized_tol, Ut, m, Vt, n, d_dev, P.fast, P.refine));
        OFRR_TRY(cast_impl(ctx, P.pho, P.po, m, b, Ut, m, U, ldu));
        OFRR_TRY(cast_impl(ctx, P.pho, P.po, n, b, Vt, n, V, ldv));
      }
    }
    S.nmv += b;
    S.it++;
    const int kk = std::min(nev, b);
    const bool last = (k + 1 == maxit);
    const bool check = tol > 0 && ((S.it % check_every) == 0 || last);
    TraceScope ts(ctx, f64 ? "check.f64" : "check.16bit");
    if (check || stag_tol > 0) {
      OFRR_CUDA(cudaMemcpyAsync(S.d.data(), d_dev, sizeof(double) * b, cudaMemcpyDeviceToHost, ctx->stream));
      OFRR_TRY(sync_and_check(ctx));
    }
    if (check && certify16 >= 0) {
      // certified check (emulated products): the emulated residuals plus the bounds on the emulation
      // errors must meet tol; columns that miss only by the bound get a true FP64 residual instead
      std::vector<double> emul(kk);
      OFRR_TRY(svd_residuals_dev(ctx, op, P.po, U, ldu, V, ldv, kk, S.d.data(), -1.0, S.res.data(), certify16,
                                 emul.data(), tol));
      std::vector<int> J;
      bool hopeless = false;
      for (int j = 0; j < kk; ++j)
        if (!(S.res[j] <= tol)) {
          if (emul[j] <= tol) J.push_back(j);
          else hopeless = true;
        }
      if (!hopeless && !J.empty()) {
        TraceScope tsc(ctx, "certify.fp64");
        const bool em = ctx->emulate_f64;
        ctx->emulate_f64 = false;
        const int st2 = svd_residuals_subset(ctx, op, (const double*)U, ldu, (const double*)V, ldv, J, S.d.data(),
                                             norm_of_values(S.d.data(), kk), S.res.data());
        ctx->emulate_f64 = em;
        OFRR_TRY(st2);
      }
      S.converged = 0;
      for (int j = 0; j < kk; ++j) S.converged += (S.res[j] <= tol) ? 1 : 0;
      if (S.converged >= kk) S.done = true;
      if (!S.done && emulation_floor(S, kk)) break;
    } else if (check) {
      OFRR_TRY(svd_residuals_dev(ctx, op, P.po, U, ldu, V, ldv, kk, S.d.data(), -1.0, S.res.data()));
      S.converged = 0;
      for (int j = 0; j < kk; ++j) S.converged += (S.res[j] <= tol) ? 1 : 0;
      if (S.converged >= kk) S.done = true;
    }
    if (!S.done && stag_tol > 0 && stagnated(S, kk, stag_tol, k + 1)) break;
  }
  return OFRR_SUCCESS;
}

// low-precision phase settings of the mixed mode
Precisions mixed_low(const ofrr_options* o) {
  Precisions p;
  p.po = (o->p_output == OFRR_BF16) ? OFRR_BF16 : OFRR_F16;  // 16-bit basis storage
  p.pho = p.po;
  p.pc = p.phc = p.prc = OFRR_F32;  // FP32 accumulation
  p.pro = OFRR_F32;                 // Gram matrices kept in FP32 (not rounded to 16 bits), then FP64
  p.fast = true;
  // one FP64 refinement step: the FP32 Jacobi vectors' errors (~3e-5 / relative gap) would otherwise
  // leave ~1e-5 noise in the Ritz values that drive the stagnation test
  p.refine = 1;
  return p;
}
Precisions all_f64() {
  Precisions p;
  p.pc = p.po = p.phc = p.pho = p.prc = p.pro = OFRR_F64;
  p.fast = true;
  return p;
}

void fill_info(ofrr_info* info, const PhaseState& S, int nev, int escalations) {
  if (!info) return;
  double maxr = 0;
  for (int j = 0; j < std::min(nev, S.b); ++j) maxr = std::max(maxr, S.res[j]);
  info->iterations = S.it;
  info->matvecs = S.nmv;
  info->converged = S.converged;
  info->basis_width = S.b;
  info->max_residual = maxr;
  info->escalations = escalations;
  info->status_detail = 0;
}

}  // namespace
}  // namespace ofrr

// ======================================================================================
// subspace iteration eigensolver (si_eig)
// ======================================================================================
static int si_eig_body(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, void* V, int64_t ldv,
                       double* evals, double* resid, ofrr_info* info) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  OFRR_TRY(validate_options(opt));
  if (A->nrows != A->ncols) return OFRR_ERR_BLAS_INVALID_SIZE;
  const int64_t n = A->nrows;
  const int b0 = (int)std::min<int64_t>(opt->block, n);
  if (n == 0 || b0 == 0) return OFRR_SUCCESS;
  if (!V || ldv < n || !evals) return OFRR_ERR_INVALID_ARGUMENT;
  if (b0 > 1024) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  Op op{A};
  OFRR_TRY(op.prepare_csr_t(ctx));
  const int nev = std::min(opt->nev > 0 ? opt->nev : b0, b0);
  PhaseState S;
  S.b = b0;
  S.d.assign(b0, 0.0);
  S.dprev.assign(b0, 0.0);
  S.res.assign(b0, INFINITY);
  double* d;
  OFRR_TRY(dmalloc(ctx, &d, (size_t)b0));
  int escalations = 0;
  // the caller's V holds p_output (reference mode) or FP64 (FP64 and mixed modes)
  const ofrr_dtype tV = (opt->mode == OFRR_MODE_REFERENCE) ? opt->p_output : OFRR_F64;
  if (opt->mode == OFRR_MODE_MIXED) {
    const Precisions L = mixed_low(opt);
    void* V16 = ws_alloc(ctx, (size_t)n * b0 * dtype_size(L.po), &st);
    if (!V16) return st;
    if (opt->use_start_block) OFRR_TRY(cast_impl(ctx, OFRR_F64, L.po, n, b0, V, ldv, V16, n));
    else OFRR_TRY(ofrr_randn(ctx, opt->seed, n, b0, L.po, V16, n));
    OFRR_TRY(scalecols_impl(ctx, L.po, L.pc, n, b0, V16, n, nullptr));
    const double stag = (L.po == OFRR_BF16) ? 1e-4 : 1e-5;
    if (op.A->kind == OFRR_OP_DENSE) {  // operator copies live for the whole solve
      const void* p = nullptr;
      int64_t l = 0;
      OFRR_TRY(op.dense_as(ctx, L.po, &p, &l));
      OFRR_TRY(op.dense_t_as(ctx, L.po, &p, &l));
    }
    // the 16-bit phase cannot reach tolerances below ~1e-4: skip its FP64 residual checks then
    const double low_tol = opt->tol >= 1e-4 ? opt->tol : 0.0;
    OFRR_TRY(eig_phase(ctx, op, L, opt, V16, n, opt->maxiter, low_tol, nev, stag, S, d));
    OFRR_TRY(cast_impl(ctx, L.po, OFRR_F64, n, S.b, V16, n, V, ldv));
    escalations = 1;
    if (!S.done && S.it < opt->maxiter) {
      // refinement: FP64-accurate products from exact BF16 slices on the tensor cores
      const bool dense = op.A->kind == OFRR_OP_DENSE;
      {
        TraceScope ts(ctx, "prepare.f64");
        OFRR_TRY(op.prepare_sliced(ctx));
        if (dense) OFRR_TRY(op.prepare_abs(ctx, L.po));
      }
      // certified checks in the FP64 phase (see si_svd); its own power steps per iteration
      ofrr_options o64 = *opt;
      if (opt->step_size_f64 > 0) o64.step_size = opt->step_size_f64;
      ctx->emulate_f64 = dense;
      st = eig_phase(ctx, op, all_f64(), &o64, V, ldv, opt->maxiter - S.it, opt->tol, nev, 0.0, S, d,
                     dense ? (int)L.po : -1);
      ctx->emulate_f64 = false;
      OFRR_TRY(st);
      if (!S.done && S.emul_floor && S.it < opt->maxiter) {
        // the emulated products' floor is above tol: the last iterations with FP64 products
        TraceScope ts(ctx, "fp64.exact");
        escalations = 2;
        OFRR_TRY(eig_phase(ctx, op, all_f64(), &o64, V, ldv, opt->maxiter - S.it, opt->tol, nev, 0.0, S, d));
      }
    }
  } else {
    const Precisions P = precisions_of(opt);
    if (!opt->use_start_block) OFRR_TRY(ofrr_randn(ctx, opt->seed, n, b0, P.po, V, ldv));
    OFRR_TRY(scalecols_impl(ctx, P.po, P.pc, n, b0, V, ldv, nullptr));
    OFRR_TRY(eig_phase(ctx, op, P, opt, V, ldv, opt->maxiter, opt->tol, nev, 0.0, S, d));
  }
  OFRR_CUDA(cudaMemcpyAsync(S.d.data(), d, sizeof(double) * S.b, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  for (int j = 0; j < b0; ++j) evals[j] = (j < S.b) ? S.d[j] : NAN;
  if (resid) {
    if (opt->tol <= 0) OFRR_TRY(residuals_dev(ctx, op, tV, V, ldv, S.b, S.d.data(), -1.0, S.res.data()));
    for (int j = 0; j < b0; ++j) resid[j] = (j < S.b) ? S.res[j] : NAN;
  }
  fill_info(info, S, nev, escalations);
  if (opt->tol > 0 && !S.done) return OFRR_ERR_SOLVER_MAX_ITERATIONS;
  return OFRR_SUCCESS;
}

extern "C" int ofrr_si_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, void* V, int64_t ldv,
                           double* evals, double* resid, ofrr_info* info) {
  if (!ctx || !ctx->tracer) return si_eig_body(ctx, A, opt, V, ldv, evals, resid, info);
  ofrr_info local{};
  ofrr_info* inf = info ? info : &local;
  const unsigned long long l0 = ofrr_ctx_launch_count(ctx);
  trace_begin_solve(ctx);
  const int st = si_eig_body(ctx, A, opt, V, ldv, evals, resid, inf);
  trace_end_solve(ctx, "si_eig", A ? A->nrows : 0, A ? A->ncols : 0, opt, st, inf, ofrr_ctx_launch_count(ctx) - l0);
  return st;
}

// ======================================================================================
// subspace iteration SVD (si_svd)
// ======================================================================================
static int si_svd_body(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, void* U, int64_t ldu, double* s,
                       void* V, int64_t ldv, double* resid, ofrr_info* info) {
  if (!ctx) return OFRR_ERR_INVALID_ARGUMENT;
  OFRR_TRY(validate_op(A));
  OFRR_TRY(validate_options(opt));
  const int64_t m = A->nrows, n = A->ncols;
  const int b0 = (int)std::min<int64_t>(opt->block, n);
  if (m == 0 || n == 0 || b0 == 0) return OFRR_SUCCESS;
  if (!U || !V || ldu < m || ldv < n || !s) return OFRR_ERR_INVALID_ARGUMENT;
  if (b0 > 512 || b0 > m) return OFRR_ERR_BLAS_INVALID_SIZE;
  WsScope scope(ctx);
  int st = OFRR_SUCCESS;
  Op op{A};
  OFRR_TRY(op.prepare_csr_t(ctx));
  const int nev = std::min(opt->nev > 0 ? opt->nev : b0, b0);
  PhaseState S;
  S.b = b0;
  S.d.assign(b0, 0.0);
  S.dprev.assign(b0, 0.0);
  S.res.assign(b0, INFINITY);
  double* d;
  OFRR_TRY(dmalloc(ctx, &d, (size_t)b0));
  int escalations = 0;
  const ofrr_dtype tV = (opt->mode == OFRR_MODE_REFERENCE) ? opt->p_output : OFRR_F64;
  if (opt->mode == OFRR_MODE_MIXED) {
    const Precisions L = mixed_low(opt);
    void* U16 = ws_alloc(ctx, (size_t)m * b0 * dtype_size(L.po), &st);
    void* V16 = ws_alloc(ctx, (size_t)n * b0 * dtype_size(L.po), &st);
    if (!U16 || !V16) return st;
    if (opt->use_start_block) OFRR_TRY(cast_impl(ctx, OFRR_F64, L.po, n, b0, V, ldv, V16, n));
    else OFRR_TRY(ofrr_randn(ctx, opt->seed, n, b0, L.po, V16, n));
    OFRR_TRY(scalecols_impl(ctx, L.po, L.pc, n, b0, V16, n, nullptr));
    // the 16-bit phase ends when the leading singular values change by less than 1e-4 (relative) per
    // iteration: later 16-bit iterations gain less than a few more FP64-phase power steps cost (measured
    // on the dense 8192 x 2048 benchmark: 1e-5 took one more 16-bit iteration and 0.3 ms more per solve)
    const double stag = 1e-4;
    if (op.A->kind == OFRR_OP_DENSE) {  // operator copies live for the whole solve
      const void* p = nullptr;
      int64_t l = 0;
      OFRR_TRY(op.dense_as(ctx, L.po, &p, &l));
      OFRR_TRY(op.dense_t_as(ctx, L.po, &p, &l));
      if (opt->power_fp8) OFRR_TRY(op.prepare_f8(ctx, L.po));
    }
    // the 16-bit phase cannot reach tolerances below ~1e-4: skip its FP64 residual checks then
    const double low_tol = opt->tol >= 1e-4 ? opt->tol : 0.0;
    ctx->power_f8 = opt->power_fp8 != 0;
    const int lst = svd_phase(ctx, op, L, opt, U16, m, V16, n, opt->maxiter, low_tol, nev,
                              opt->power_fp8 ? 1e-3 : stag, S, d);
    ctx->power_f8 = false;
    OFRR_TRY(lst);
    OFRR_TRY(cast_impl(ctx, L.po, OFRR_F64, m, S.b, U16, m, U, ldu));
    OFRR_TRY(cast_impl(ctx, L.po, OFRR_F64, n, S.b, V16, n, V, ldv));
    escalations = 1;
    if (!S.done && S.it < opt->maxiter) {
      // refinement: FP64-accurate products from exact BF16 slices on the tensor cores
      const bool dense = op.A->kind == OFRR_OP_DENSE;
      {
        TraceScope ts(ctx, "prepare.f64");
        OFRR_TRY(op.prepare_sliced(ctx));
        if (dense) OFRR_TRY(op.prepare_abs(ctx, L.po));
      }
      // the FP64 phase's checks are certified (emulated residuals plus the bounds on the emulation
      // errors, true FP64 residuals for the columns that miss only by the bound); the phase has its own
      // power steps per iteration (step_size_f64)
      ofrr_options o64 = *opt;
      if (opt->step_size_f64 > 0) o64.step_size = opt->step_size_f64;
      ctx->emulate_f64 = dense;
      st = svd_phase(ctx, op, all_f64(), &o64, U, ldu, V, ldv, opt->maxiter - S.it, opt->tol, nev, 0.0, S, d,
                     dense ? (int)L.po : -1);
      ctx->emulate_f64 = false;
      OFRR_TRY(st);
      if (!S.done && S.emul_floor && S.it < opt->maxiter) {
        // the emulated products' floor is above tol: the last iterations with FP64 products
        TraceScope ts(ctx, "fp64.exact");
        escalations = 2;
        OFRR_TRY(svd_phase(ctx, op, all_f64(), &o64, U, ldu, V, ldv, opt->maxiter - S.it, opt->tol, nev, 0.0, S, d));
      }
    }
  } else {
    const Precisions P = precisions_of(opt);
    if (!opt->use_start_block) OFRR_TRY(ofrr_randn(ctx, opt->seed, n, b0, P.po, V, ldv));
    OFRR_TRY(scalecols_impl(ctx, P.po, P.pc, n, b0, V, ldv, nullptr));
    OFRR_TRY(svd_phase(ctx, op, P, opt, U, ldu, V, ldv, opt->maxiter, opt->tol, nev, 0.0, S, d));
  }
  OFRR_CUDA(cudaMemcpyAsync(S.d.data(), d, sizeof(double) * S.b, cudaMemcpyDeviceToHost, ctx->stream));
  OFRR_TRY(sync_and_check(ctx));
  for (int j = 0; j < b0; ++j) s[j] = (j < S.b) ? S.d[j] : NAN;
  if (resid) {
    if (opt->tol <= 0) OFRR_TRY(svd_residuals_dev(ctx, op, tV, U, ldu, V, ldv, S.b, S.d.data(), -1.0, S.res.data()));
    for (int j = 0; j < b0; ++j) resid[j] = (j < S.b) ? S.res[j] : NAN;
  }
  fill_info(info, S, nev, escalations);
  if (opt->tol > 0 && !S.done) return OFRR_ERR_SOLVER_MAX_ITERATIONS;
  return OFRR_SUCCESS;
}

extern "C" int ofrr_si_svd(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, void* U, int64_t ldu,
                           double* s, void* V, int64_t ldv, double* resid, ofrr_info* info) {
  if (!ctx || !ctx->tracer) return si_svd_body(ctx, A, opt, U, ldu, s, V, ldv, resid, info);
  ofrr_info local{};
  ofrr_info* inf = info ? info : &local;
  const unsigned long long l0 = ofrr_ctx_launch_count(ctx);
  trace_begin_solve(ctx);
  const int st = si_svd_body(ctx, A, opt, U, ldu, s, V, ldv, resid, inf);
  trace_end_solve(ctx, "si_svd", A ? A->nrows : 0, A ? A->ncols : 0, opt, st, inf, ofrr_ctx_launch_count(ctx) - l0);
  return st;
}
