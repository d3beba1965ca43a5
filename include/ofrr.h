/*
 * ofrr.h -- C ABI of libofrr_gb300.so, the GB300 (sm_103a) implementation of the
 * orthogonalization-free projection eigen/SVD path of MixedPrecisionOFRR.
 *
 * Plain pointers and sizes only.  All matrices are column-major with an explicit
 * leading dimension.  Device pointers are marked (dev), host pointers (host).
 * Every entry point returns an int status whose values equal msvd::MSVDStatus
 * (reference CPP/core/utils/error_handling.hpp:24-62); no entry point throws.
 *
 * Each declaration names the reference interface it replaces.  The reference's
 * C++ solver bodies are stubs; their behaviour is defined by the MATLAB code under
 * MATLAB/+src, cited beside the solver entry points.
 */
#ifndef OFRR_GB300_H
#define OFRR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: same numeric values as msvd::MSVDStatus ------------------------- */
enum {
  OFRR_SUCCESS = 0,
  OFRR_ERR_INVALID_ARGUMENT = 1000,
  OFRR_ERR_INVALID_OPERATION = 1001,
  OFRR_ERR_OUT_OF_MEMORY = 1002,
  OFRR_ERR_NOT_IMPLEMENTED = 1003,
  OFRR_ERR_INTERNAL = 1004,
  OFRR_ERR_NAN = 1005,
  OFRR_ERR_INF = 1006,
  OFRR_ERR_BLAS_INVALID_LOCATION = 2000,
  OFRR_ERR_BLAS_UNSUPPORTED_TYPE = 2003,
  OFRR_ERR_BLAS_CUBLAS = 2004,
  OFRR_ERR_BLAS_INVALID_SIZE = 2005,
  OFRR_ERR_FACTORIZATION_FAILED = 3000,
  OFRR_ERR_SINGULAR_MATRIX = 3001,
  OFRR_ERR_SOLVER_DIVERGENCE = 4000,
  OFRR_ERR_SOLVER_MAX_ITERATIONS = 4001,
  OFRR_ERR_FILE_NOT_FOUND = 5000,
  OFRR_ERR_INVALID_FORMAT = 5001,
  OFRR_ERR_CUDA_GENERAL = 6000,
  OFRR_ERR_CUDA_MEMORY = 6001,
  OFRR_ERR_CUDA_LAUNCH = 6002,
  OFRR_ERR_CUDA_SYNC = 6003,
  /* new: a bounded device-side wait ran out; the context stays usable */
  OFRR_ERR_DEVICE_TIMEOUT = 6004
};

/* element types (reference: T in {double, float, __half}; bf16 is new) */
typedef enum { OFRR_F64 = 0, OFRR_F32 = 1, OFRR_F16 = 2, OFRR_BF16 = 3 } ofrr_dtype;

/* ---- context ---------------------------------------------------------------------- *
 * Replaces the process-global CUDAHandler singleton (CPP/core/utils/cuda_handler.hpp:15-81):
 * one context per host thread, an explicit stream, a cached device workspace and the
 * library handles.  stream == NULL means a new non-blocking stream owned by the context. */
typedef struct ofrr_ctx ofrr_ctx;
int ofrr_ctx_create(ofrr_ctx** ctx, int device, void* cuda_stream);
int ofrr_ctx_destroy(ofrr_ctx* ctx);
int ofrr_ctx_set_stream(ofrr_ctx* ctx, void* cuda_stream);
void* ofrr_ctx_get_stream(ofrr_ctx* ctx);
int ofrr_ctx_synchronize(ofrr_ctx* ctx);
/* number of kernels this library has launched on ctx since creation (or the last reset) */
uint64_t ofrr_ctx_launch_count(ofrr_ctx* ctx);
void ofrr_ctx_reset_launch_count(ofrr_ctx* ctx);
/* bytes of device workspace currently cached by ctx (allocated on first need) */
size_t ofrr_ctx_workspace_bytes(ofrr_ctx* ctx);
const char* ofrr_status_string(int status);
const char* ofrr_version(void);

/* ---- project RNG ------------------------------------------------------------------ *
 * Counter-based N(0,1) block (splitmix64 hashes + Box-Muller, element counter i+n*j).
 * Stands in for MATLAB rng(seed); randn(n,k) (MATLAB/+src/+subspace/subspace_iter_eig.m:53-54)
 * and replaces Vector::fill_random (CPP/containers/vector.cu:188-225). */
int ofrr_randn(ofrr_ctx* ctx, uint64_t seed, int64_t n, int64_t k, ofrr_dtype dt,
               void* out /*dev*/, int64_t ld);
void ofrr_randn_host(uint64_t seed, int64_t n, int64_t k, double* out /*host, n*k*/);

/* ---- level-1/2 building blocks ---------------------------------------------------- */
/* iamax: 1-based index of the first max |x| and the signed value there.
 * Replaces msvd::iamax (CPP/linalg/blas/mvops.hpp:98-99, mvops.cu:799-876). */
int ofrr_iamax(ofrr_ctx* ctx, ofrr_dtype dt, int64_t n, const void* x /*dev*/,
               int* idx1 /*host*/, double* val /*host*/);
/* per-column 0-based argmax |A(:,j)|, lowest row on ties.
 * Replaces msvd::matrix_iamax (mvops.hpp:113-114, mvops.cu:955-1199). */
int ofrr_matrix_iamax(ofrr_ctx* ctx, ofrr_dtype dt, int64_t m, int64_t n, const void* A /*dev*/,
                      int64_t lda, int* idx /*dev, n*/);
/* scalecols: U(:,j) = po(pc(U(:,j)) / pc(U(k_j,j))), k_j = argmax|U(:,j)|, skipped if 0.
 * MATLAB/+src/+mvops/scalecols.m:21-34.  piv (dev, optional) receives k_j (0-based). */
int ofrr_scalecols(ofrr_ctx* ctx, ofrr_dtype po, ofrr_dtype pc, int64_t m, int64_t n,
                   void* U /*dev*/, int64_t ldu, int* piv /*dev or NULL*/);
/* element cast between storage types (replaces Vector::cast, CPP/containers/vector.cu:248-290) */
int ofrr_cast(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, int64_t m, int64_t n,
              const void* in /*dev*/, int64_t ldin, void* out /*dev*/, int64_t ldout);
/* NaN/Inf scan: returns OFRR_SUCCESS, OFRR_ERR_NAN or OFRR_ERR_INF.
 * Replaces msvd::check_special_values (mvops.hpp:159-174). */
int ofrr_check_special_values(ofrr_ctx* ctx, ofrr_dtype dt, int64_t m, int64_t n,
                              const void* A /*dev*/, int64_t lda);

/* ---- oblique basis: Hessenberg process -------------------------------------------- *
 * Q (m x n, type tout) with |Q| <= 1 and unit entries at the pivot rows, R (n x n) with
 * A = Q R over the selected columns, skip[j] = 1 for deselected (near-dependent) columns.
 * Arithmetic follows MATLAB/+src/+qr/hessenberg.m:45-85 element by element (MGS order,
 * one rounding to tout per elimination), so the result is bit-identical to the MATLAB
 * restatement in the same precisions.  Replaces msvd::hessenberg / hessenberg_v2 /
 * hessenberg_v3 (CPP/linalg/factorization/hessenberg.hpp:22-78, hessenberg.cu:197-748).
 * select_tol < 0 selects the default eps(tout) (MATLAB/+src/+utils/eps.m).
 * R_host (n*n col-major), skip_host (n) and perm_host (n, 0-based or -1) may be NULL. */
int ofrr_hessenberg(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute,
                    int64_t m, int64_t n, const void* A /*dev*/, int64_t lda,
                    void* Q /*dev*/, int64_t ldq, double select_tol,
                    double* R_host, int* skip_host, int* perm_host);

/* ---- dense contractions ----------------------------------------------------------- *
 * C = alpha op(A) op(B) + beta C with MATLAB gemm.m semantics (MATLAB/+src/+mvops/gemm.m:27-59):
 * inputs converted to tcompute, product accumulated in tcompute (FP32 accumulation for
 * 16-bit inputs), result stored as tout.  Replaces msvd::gemm (mvops.hpp:79-90,
 * mvops.cu:466-568).  F16/BF16 operands with F32 compute run on the tcgen05 kernel. */
int ofrr_gemm(ofrr_ctx* ctx, int transA, int transB, ofrr_dtype ta, ofrr_dtype tb,
              ofrr_dtype tcompute, ofrr_dtype tout, int64_t M, int64_t N, int64_t K,
              double alpha, const void* A /*dev*/, int64_t lda, const void* B /*dev*/,
              int64_t ldb, double beta, void* C /*dev*/, int64_t ldc);

/* C (M x N, FP32) = A' B for FP32 A (K x M, K >= 32) and B (K x N): both quantized per column to E4M3
 * with power-of-two scales, multiplied on the tcgen05 tensor cores (kind::f8f6f4, FP32 accumulation) and
 * scaled back (no reference counterpart; the product of the FP8 variant of the power steps). */
int ofrr_gemm_e4m3(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const float* A /*dev*/, int64_t lda,
                   const float* B /*dev*/, int64_t ldb, float* C /*dev*/, int64_t ldc);

/* Tile autotuner of the 16-bit tcgen05 product (no reference counterpart): times every tile width
 * BN in {32, 64, 128} and K split in {1, 2, ..., 64} of C (M x N, FP32) = A' B (A: K x M, B: K x N, type t16)
 * over reps launches on seeded operands and keeps the fastest plan for that exact shape and type
 * (process-wide); later 16-bit products of the shape use it.  ofrr_gemm16_plan reports the plan a
 * product of a shape would use (tuned = 1 when it came from the autotuner). */
int ofrr_autotune_gemm16(ofrr_ctx* ctx, int t16, int64_t M, int64_t N, int64_t K, int reps, int* best_bn,
                         int* best_splits, double* best_us);
int ofrr_gemm16_plan(int t16, int64_t M, int64_t N, int64_t K, int* bn, int* splits, int* tuned);

/* C (M x N) = A' B for FP64 A (K x M) and B (K x N), computed on the tcgen05 tensor cores from
 * exact BF16 digit slices of both operands (five 7-bit digits per column after a power-of-two
 * column scaling; digit products summed exactly in FP32, combined in FP64).  Element error is
 * about 2^-35 |A'| |B|.  The FP64 TN case of msvd::gemm (mvops.hpp:79-90) at tensor-core speed;
 * the mixed solver's refinement phase uses it for A V, A' U and the Gram products. */
int ofrr_gemm_f64_emulated(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                           const double* B, int64_t ldb, double* C, int64_t ldc);

/* Profiling form of ofrr_gemm_f64_emulated (no reference counterpart): slices A and B once, then
 * runs the fused product kernel reps (>= 2) times and returns its mean time per launch (CUDA events
 * on the context's stream, synchronous) and the kernel's algorithmic bytes per launch (digit stacks
 * read once, partial results written once).  C holds A' B afterwards. */
int ofrr_profile_gemm_f64_emulated(ofrr_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                                   const double* B, int64_t ldb, double* C, int64_t ldc, int reps,
                                   double* us_per_launch, double* bytes_per_launch);

/* ---- sparse operator: CSR with value copies per precision ------------------------- *
 * Mirrors MATLAB/+src/+csr/sparse2csr.m:21-50 (0-based int32 here).  Any of the value
 * arrays may be NULL if that precision is never requested. */
typedef struct {
  int64_t nrows, ncols, nnz;
  const int32_t* indptr;   /* dev, nrows+1 */
  const int32_t* indices;  /* dev, nnz */
  const double* a_double;  /* dev, nnz */
  const float* a_single;   /* dev, nnz */
  const void* a_half;      /* dev, nnz (__half) */
} ofrr_csr;

/* Y = op(A) X for nrhs columns, MATLAB/+src/+csr/csrmv.m:27-78 (compute in tcompute using
 * the value copy of that precision, store as ty). */
int ofrr_csrmm(ofrr_ctx* ctx, const ofrr_csr* A, int trans, ofrr_dtype tx, ofrr_dtype tcompute,
               ofrr_dtype ty, int64_t nrhs, const void* X /*dev*/, int64_t ldx,
               void* Y /*dev*/, int64_t ldy);

/* Gram-Schmidt basis of A (m x n, m >= n): MATLAB/+src/+qr/mgs.m (classical = 0) or cgs.m
 * (classical = 1), element arithmetic as those files (one rounding to tout per projection term, dots
 * and norms in tcompute then rounded to tout; summation order of the dots is the GPU's), adaptive
 * re-orthogonalisation while the norm stays at least orth_tol and drops below reorth_tol times the
 * previous one (reorth_tol < 0: none), columns with a norm below select_tol dropped.  Defaults of the
 * reference (qr.hpp:21-29): select_tol < 0 -> eps(tout); orth_tol NaN -> eps(tout); reorth_tol NaN
 * -> 1/sqrt(2); all are rounded to tout.  Q (m x n) keeps the column positions, dropped columns zero;
 * R_host (n*n, col-major) and skip_host (n) may be NULL.  Replaces msvd::mgs / mgs_v2 / cgs2
 * (CPP/linalg/factorization/qr.hpp:21-132) for the comparison runs. */
int ofrr_gs_basis(ofrr_ctx* ctx, int classical, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute, int64_t m,
                  int64_t n, const void* A /*dev*/, int64_t lda, void* Q /*dev*/, int64_t ldq, double select_tol,
                  double orth_tol, double reorth_tol, double* R_host, int* skip_host);

/* ---- test-problem generators (CPP/testproblems/gaussian_kernel.hpp, MATLAB/+src/+kernel) ---- *
 * ofrr_rand_points: n points (X: n x d, FP64, device) of generate_pts.m's types 20 (square), 30 (cube),
 * 21 (disk), 22 (circle), 23 (grid, n a square), 31 (ball), 32 (sphere), or type 0: the uniform box
 * [0, n^(1/d))^d of generate_gaussian_kernel for any d.  Uniform draws from the library's counter-based
 * generator (splitmix64 of the seed-keyed element counter; the reference's std / MATLAB generators
 * cannot be reproduced).  ofrr_gaussian_kernel: K (m x n, tout, device) in FP64 then rounded once;
 * form 0 = generate_gaussian_kernel (gaussian_kernel.hpp:14-77; X == Y, m == n; diagonal
 * f^2 (1 + s^2), off-diagonal f^2 exp(-|x_i - x_j|^2 / (2 l^2)), 0 below exp(-700)); form 1 =
 * gaussian.m:21-27 (K(X, Y) = f^2 exp(-D2 / (2 l^2)) + s^2 eye, D2 = -2 X Y' + |x|^2 + |y|^2).
 * l <= 0, s < 0, non-positive sizes: OFRR_ERR_INVALID_ARGUMENT (the reference throws). */
int ofrr_rand_points(ofrr_ctx* ctx, uint64_t seed, int64_t n, int d, int type, double* X /*dev*/, int64_t ldx);
/* Dense test matrices with a prescribed spectrum (no reference counterpart; the inputs of the batched and
 * serving workloads): symmetric = 0: A (m x n, m >= n) = H_1 .. H_r [diag(s); 0] G_1 .. G_r, singular values
 * exactly s; symmetric = 1: A (n x n) = H_1 .. H_r diag(s) H_r .. H_1, eigenvalues exactly s.  H, G are
 * Householder reflectors (r = reflectors <= 16 per side) with Gaussian vectors from the library's
 * generator keyed by seed.  s: host array of n values; A: device, FP64, column-major. */
int ofrr_test_matrix_spectrum(ofrr_ctx* ctx, int symmetric, uint64_t seed, int64_t m, int64_t n, int reflectors,
                              const double* s /*host*/, double* A /*dev*/, int64_t lda);
int ofrr_gaussian_kernel(ofrr_ctx* ctx, int form, int64_t m, int64_t n, int d, const double* X /*dev*/, int64_t ldx,
                         const double* Y /*dev*/, int64_t ldy, double l, double f, double s, ofrr_dtype tout,
                         void* K /*dev*/, int64_t ldk);

/* Column-pivoted LU basis of A (m x n, m >= n), MATLAB/+src/+qr/lu.m:47-94: right-looking with the
 * rows swapped in place (pivot = first maximum of |A_work(j:m, j)| in the current row order), a
 * column whose maximum is below select_tol dropped (its row consumed; select_tol < 0: eps(tout)),
 * arithmetic in tcompute rounded to tout per operation as lu.m does.  Q (m x n) = the un-permuted L
 * (lu.m's two-output form before the column selection), dropped columns zero; U_host (n*n) and
 * skip_host (n) may be NULL. */
int ofrr_lu_basis(ofrr_ctx* ctx, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute, int64_t m, int64_t n,
                  const void* A /*dev*/, int64_t lda, void* Q /*dev*/, int64_t ldq, double select_tol, double* U_host,
                  int* skip_host);

/* ---- on-disk CSR matrices (CPP/io/matrix_reader.cpp:8-50) -------------------------- *
 * <prefix>_row_ptr.bin (int32, nrows+1), <prefix>_col_ind.bin (int32, 0-based, nnz) and
 * <prefix>_values.bin (float64, nnz); element counts from the file sizes, ncols = largest column
 * index + 1.  Missing file: OFRR_ERR_FILE_NOT_FOUND; empty file, partial element, col_ind/values
 * length mismatch or a malformed structure (row_ptr[0] != 0, decreasing row_ptr,
 * row_ptr[nrows] != nnz, negative column index): OFRR_ERR_INVALID_FORMAT.
 * ofrr_csr_file_read fills caller buffers of the sizes ofrr_csr_file_sizes reported: host buffers
 * (on_device = 0, ctx may be NULL) or device buffers (on_device = 1: streamed through pinned staging
 * buffers on the context's stream and validated on the GPU; synchronous). */
int ofrr_csr_file_sizes(const char* prefix, int64_t* nrows, int64_t* nnz);
int ofrr_csr_file_read(ofrr_ctx* ctx, const char* prefix, int64_t nrows, int64_t nnz, int32_t* indptr,
                       int32_t* indices, double* values, int64_t* ncols, int on_device);
/* <prefix>_singular_values.bin (float64, matrix_reader.cpp:47-50).  values == NULL: *count = the
 * number of values; otherwise *count is the capacity of values (host) on entry and the number read
 * on return. */
int ofrr_read_singular_values(const char* prefix, int64_t* count, double* values);

/* ---- small dense FP64 eigenproblems on the device --------------------------------- *
 * Replace the host LAPACKE wrappers msvd::syev / msvd::sygv (mvops.hpp:184-197,
 * mvops.cu:1601-1664).  Ascending eigenvalues; A is overwritten by the eigenvectors
 * (orthonormal for syev, B-orthonormal for sygv).  n <= 256. */
int ofrr_syev(ofrr_ctx* ctx, int n, double* A /*dev*/, int lda, double* w /*dev*/);
int ofrr_sygv(ofrr_ctx* ctx, int n, double* A /*dev*/, int lda, double* B /*dev*/, int ldb,
              double* w /*dev*/);

/* ---- operators and solver options ------------------------------------------------- */
typedef enum { OFRR_OP_DENSE = 0, OFRR_OP_CSR = 1 } ofrr_op_kind;

typedef struct {
  int kind;               /* ofrr_op_kind */
  int64_t nrows, ncols;
  int symmetric;          /* 1: A = A' (symmetric Rayleigh-Ritz), 0: general */
  /* dense (kind == OFRR_OP_DENSE): column-major device matrix */
  ofrr_dtype dtype;
  const void* data;
  int64_t ld;
  /* sparse (kind == OFRR_OP_CSR) */
  ofrr_csr csr;
} ofrr_operator;

/* Solver modes.
 * OFRR_MODE_REFERENCE: the reference's semantics -- exactly maxiter outer iterations, every
 *   cast of the MATLAB code at the same place, precisions from the p_* fields.
 * OFRR_MODE_MIXED: production mixed precision -- 16-bit basis storage (p_output), FP32
 *   accumulation on tensor cores, split-precision Gram matrices, FP64 small pencil,
 *   precision escalation and FP64 residual checks; stops when nev pairs reach tol.
 * OFRR_MODE_FP64: the same loop with every operand in FP64 (the comparison path).
 * In OFRR_MODE_MIXED and OFRR_MODE_FP64 the caller's basis buffers (V, U, X) hold FP64: the start
 * block on entry and the final Ritz vectors on exit; p_output then only selects the 16-bit working
 * precision of the mixed mode (OFRR_F16 or OFRR_BF16). */
typedef enum { OFRR_MODE_REFERENCE = 0, OFRR_MODE_MIXED = 1, OFRR_MODE_FP64 = 2 } ofrr_mode;
/* Basis of a block: the Hessenberg process (orthogonalization-free, the default here); Gram-Schmidt
 * QR as the orthogonal comparison -- modified (MATLAB/+src/+qr/mgs.m, the reference's default
 * function_orth of subspace_iter_eig.m:114-115) or classical (cgs.m), both with the adaptive
 * re-orthogonalisation of those files; or the column-pivoted LU basis (MATLAB/+src/+qr/lu.m, the
 * un-permuted L).  si_eig / si_svd accept all four; arnoldi_eig the first two
 * (OFRR_ORTH_MGS there is the MGS Arnoldi of arnoldi_mgs_eig.m). */
typedef enum { OFRR_ORTH_HESSENBERG = 0, OFRR_ORTH_MGS = 1, OFRR_ORTH_CGS = 2, OFRR_ORTH_LU = 3 } ofrr_orth;

typedef struct {
  int mode;                /* ofrr_mode */
  int maxiter;             /* outer iterations (subspace) or matvec budget (Krylov) */
  int step_size;           /* power steps per outer iteration (subspace_iter_eig.m:61) */
  int block;               /* basis width b (subspace) */
  int nev;                 /* wanted pairs k */
  int kdim;                /* Krylov dimension (arnoldi_hess_eig.m:24-25) */
  double tol;              /* residual target ||Ax - lx|| / ||A||; 0 = run maxiter */
  int use_generalized;     /* generalized Rayleigh-Ritz on the oblique basis */
  double generalized_tol;  /* tau in eig(V'AV, V'V + tau I) (eig_rr.m:52) */
  double select_tol;       /* Hessenberg column selection; < 0 = eps(p_hess_output) */
  uint64_t seed;           /* start block seed when use_start_block == 0 */
  int use_start_block;     /* 1: V (or v0) holds the start block on entry */
  int orth;                /* ofrr_orth */
  int reorth;              /* MGS Arnoldi re-orthogonalisation (arnoldi_mgs_eig.m:80) */
  ofrr_dtype p_compute, p_output;            /* subspace / Krylov precisions */
  ofrr_dtype p_hess_compute, p_hess_output;  /* basis build */
  ofrr_dtype p_rr_compute, p_rr_output;      /* Rayleigh-Ritz Gram / update */
  int check_every;         /* residual check period in outer iterations (>= 1) */
  /* Krylov restarts: Ritz vectors kept at a restart.  1 = arnoldi_hess_eig.m:99-106 (the leading Ritz
   * vector alone; the reference mode always does this); 0 = the production default of OFRR_MODE_MIXED
   * and OFRR_MODE_FP64 with a CSR operator: a thick restart keeping the invariant subspace of about nev
   * (nonsymmetric operators) or max(nev + 4, 1.2 nev) (symmetric) leading Ritz values (cut at the widest
   * gap nearby; at most kdim - 2) and the Galerkin residual direction (new behaviour); k > 1 keeps about
   * k. */
  int restart_keep;
  /* OFRR_MODE_MIXED si_svd with a dense operator: 1 = the FP8 variant of the 16-bit phase, whose power
   * steps multiply E4M3 copies of A (per-row power-of-two scales, made once per solve) and of the basis
   * block (per column) on the tensor cores (kind::f8f6f4, FP32 accumulation); 0 = 16-bit products. */
  int power_fp8;
  /* OFRR_MODE_MIXED si_svd / si_eig: power steps per outer iteration of the FP64 phase; 0 = step_size.
   * The FP64 phase starts from 16-bit-accurate vectors, and each of its outer iterations carries a
   * Hessenberg basis, a Rayleigh-Ritz and a certified check: more steps per iteration there means fewer
   * of them for the same number of power steps (new behaviour; the reference has one step_size). */
  int step_size_f64;
} ofrr_options;

typedef struct {
  int iterations;          /* outer iterations (subspace) or restart cycles (Krylov) */
  int matvecs;             /* operator applications (columns) */
  int converged;           /* pairs with residual <= tol */
  int basis_width;         /* final basis width after column selection */
  double max_residual;     /* max over the nev returned pairs */
  int escalations;         /* precision escalations taken (mixed mode) */
  int status_detail;       /* first device-side error code seen, 0 if none */
} ofrr_info;

void ofrr_options_default(ofrr_options* opt);

/* ---- solvers ------------------------------------------------------------------------ */
/* Subspace iteration eigensolver.  MATLAB/+src/+subspace/subspace_iter_eig.m:50-68 with the
 * Hessenberg orth and eig_rr wrappers of MATLAB/+tests/+test2/test.m:358-397.
 * Replaces msvd::si_eig (CPP/linalg/solvers/eig/si_eig.hpp:24-27, si_eig.cu:10-18).
 * V: n x block (dev, type p_output) -- start block in (if use_start_block), Ritz vectors out,
 * sorted by descending real part of the Ritz values.  evals/resid: host, block entries. */
int ofrr_si_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt,
                void* V /*dev*/, int64_t ldv, double* evals /*host*/, double* resid /*host|NULL*/,
                ofrr_info* info /*host|NULL*/);

/* Rayleigh-Ritz on a given (non-orthogonal) basis.  MATLAB/+src/+rr/eig_rr.m:46-57.
 * Replaces msvd::rr_eig (CPP/linalg/solvers/eig/rr_eig.hpp:21-22, rr_eig.cu:9-13). */
int ofrr_rr_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, int64_t ncols,
                void* V /*dev, n x ncols, type p_output*/, int64_t ldv, double* evals /*host*/);

/* Projection with an explicit B (reference msvd::ofrr_eig, rr_eig.hpp:34-35): eigenpairs of
 * the pencil (V'AV, V'BV + tau I) for dense symmetric A, B. */
int ofrr_ofrr_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_operator* B,
                  const ofrr_options* opt, int64_t ncols, void* V /*dev*/, int64_t ldv,
                  double* evals /*host*/);

/* Subspace iteration SVD.  MATLAB/+src/+subspace/subspace_iter_svd.m:53-77 + svd_rr.m:50-91.
 * Replaces msvd::si_svd (CPP/linalg/solvers/svd/si_svd.hpp:25-28, si_svd.cu:10-18).
 * U: m x block, V: n x block (dev, type p_output); V holds the start block if
 * use_start_block.  s/resid: host, block entries, descending. */
int ofrr_si_svd(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt,
                void* U /*dev*/, int64_t ldu, double* s /*host*/, void* V /*dev*/, int64_t ldv,
                double* resid /*host|NULL*/, ofrr_info* info /*host|NULL*/);

/* Rayleigh-Ritz SVD on given bases U (m x ncols), V (n x ncols).  MATLAB/+src/+rr/svd_rr.m.
 * Replaces msvd::rr_svd (CPP/linalg/solvers/svd/rr_svd.hpp:22-24, rr_svd.cu:10-15). */
int ofrr_rr_svd(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt, int64_t ncols,
                void* U /*dev*/, int64_t ldu, double* s /*host*/, void* V /*dev*/, int64_t ldv);

/* Krylov eigensolver with restarts: Hessenberg process (orth = OFRR_ORTH_HESSENBERG,
 * MATLAB/+src/+krylov/arnoldi_hess_eig.m:51-107) or MGS Arnoldi (OFRR_ORTH_MGS,
 * MATLAB/+src/+krylov/arnoldi_mgs_eig.m:54-113).  Replaces msvd::arnoldi_eig
 * (CPP/linalg/solvers/eig/arnoldi_eig.hpp:25-28, arnoldi_eig.cu:10-18).
 * v0: n (dev, type p_output; FP64 in OFRR_MODE_MIXED / OFRR_MODE_FP64) start vector when
 * use_start_block; X: n x nev Ritz vectors out (FP64 in those modes).  With a CSR operator the
 * production modes use the thick restart of ofrr_options.restart_keep (kdim + 1 <= 128, nonsymmetric
 * operators kdim + 1 <= 96 for the invariant-subspace restart); maxiter is the budget of Krylov steps.
 * OFRR_MODE_MIXED: a 16-bit basis (p_output F16 or BF16) with the FP32 value copy of A and FP32
 * arithmetic until the residuals stop improving, then an FP64 phase (FP64 values; Gram and Ritz products
 * on the tensor cores through the exact-slice emulation). */
int ofrr_arnoldi_eig(ofrr_ctx* ctx, const ofrr_operator* A, const ofrr_options* opt,
                     const void* v0 /*dev|NULL*/, void* X /*dev*/, int64_t ldx,
                     double* evals /*host, nev*/, double* resid /*host|NULL*/,
                     ofrr_info* info /*host|NULL*/);

/* Profiling form of one step of the thick-restart Krylov path (no reference counterpart; the step of
 * arnoldi_hess_eig.m:73-87): builds a synthetic basis of i + 1 columns of type t (OFRR_F16 / OFRR_BF16 /
 * OFRR_F32 with A's FP32 values and FP32 arithmetic, OFRR_F64 with FP64) on the square CSR operator A,
 * runs the fused step kernel reps (>= 2) times and returns its mean time per launch (CUDA events on the
 * context's stream, synchronous) and the step's algorithmic HBM bytes (CSR once, staging vector read and
 * written, the new column written, i - 1 earlier columns read, pivot marks). */
int ofrr_profile_krylov_step(ofrr_ctx* ctx, const ofrr_csr* A, ofrr_dtype t, int i, int reps, double* us_per_launch,
                             double* bytes_per_launch);

/* Residual norms ||A x_j - l_j x_j||_2 / (normA ||x_j||_2) in FP64 for ncols pairs
 * (MATLAB/+tests/+test4/test.m:340-350 with unit-norm scaling).  normA <= 0 uses max|l|. */
int ofrr_residual_norms(ofrr_ctx* ctx, const ofrr_operator* A, ofrr_dtype tx, int64_t ncols,
                        const void* X /*dev*/, int64_t ldx, const double* evals /*host*/,
                        double normA, double* resid /*host*/);

/* ---- Hessenberg basis without allocation ----------------------------------------------- *
 * No counterpart in the reference.  For callers that cannot allocate GPU memory (their pool owns
 * all of HBM, or they must not pay cudaMalloc's implicit device synchronisation): the same
 * arithmetic and results as ofrr_hessenberg, with no context, no workspace and no allocation.
 * Its scratch (pivot rows and values, argmax partials, a ticket counter) is one fixed 1 MiB
 * __device__ array that every GPU loading the library keeps until process exit, so the basis
 * width is limited: n * n * sizeof(tout) + n * sizeof(tout) + about 5 KB must fit in 1 MiB
 * (n <= 360 for FP64 output, <= 510 for FP32, <= 721 for 16-bit, and never above 1024); larger
 * n returns OFRR_ERR_BLAS_INVALID_SIZE with a message on stderr.  All calls share the array:
 * calls whose work overlaps on the GPU (different streams, or several threads) race and must be
 * serialised by the caller.  Every call looks up the array's device address (cudaGetSymbolAddress).
 * With CUDA's default lazy module loading the module holding the array and the kernels is loaded by
 * the first call on a device, and that load itself reserves device memory: make one call (any small
 * size), or run with CUDA_MODULE_LOADING=EAGER, before the caller's pool takes all of HBM, and before
 * any stream capture.  A, Q with A == Q must share the element type and leading dimension.
 * Outputs are device arrays: R (n x n, FP64, column-major), select (n ints, 1 = kept) and
 * perm (n ints, pivot rows, -1 for dropped columns).  ofrr_hessenberg_noalloc_scratch_bytes()
 * returns the scratch size. */
int ofrr_hessenberg_noalloc(void* cuda_stream, ofrr_dtype tin, ofrr_dtype tout, ofrr_dtype tcompute, int64_t m,
                            int64_t n, const void* A /*dev*/, int64_t lda, void* Q /*dev*/, int64_t ldq,
                            double select_tol, double* R /*dev*/, int* select /*dev*/, int* perm /*dev*/);
size_t ofrr_hessenberg_noalloc_scratch_bytes(void);

/* ---- solve engine: batched solves and a serving queue ------------------------------- *
 * No counterpart in the reference (its C++ solvers are stubs and it has no batch or serving
 * layer).  An engine owns `workers` host threads, each with its own ofrr_ctx (stream, cuBLAS
 * handle, cached workspace), so independent solves overlap on one GPU.  Requests run in FIFO
 * order; each is charged an estimate of its device workspace against hbm_budget_bytes (0 = half
 * of the free memory) and starts when the charge fits (a request larger than the budget runs
 * alone).  The caller owns every buffer a request points to (operator data, outputs; host arrays
 * for values/resid/info) and keeps them valid until the request has completed.  A ticket is
 * released by ofrr_serve_wait.  Results do not depend on the other requests in flight. */
typedef struct ofrr_serve ofrr_serve;
typedef enum { OFRR_REQ_SI_EIG = 0, OFRR_REQ_SI_SVD = 1, OFRR_REQ_ARNOLDI_EIG = 2 } ofrr_request_kind;
typedef struct {
  int kind;               /* ofrr_request_kind */
  ofrr_operator A;
  ofrr_options opt;
  void* V;                /* dev: si_eig V (in/out), si_svd V (out), arnoldi X (out) */
  int64_t ldv;
  void* U;                /* dev: si_svd U (out) */
  int64_t ldu;
  const void* v0;         /* dev: arnoldi start vector (opt.use_start_block) */
  double* values;         /* host: eigen/singular values (block, or nev for arnoldi) */
  double* resid;          /* host|NULL */
  ofrr_info* info;        /* host|NULL */
} ofrr_request;
typedef struct {
  uint64_t completed, failed, queued;
  size_t charged_bytes, budget_bytes;
  double wall_ms;         /* first submit to last completion */
  double busy_ms;         /* summed solve time over workers */
  double p50_ms, p99_ms;  /* submit-to-completion latency */
} ofrr_serve_report;
int ofrr_serve_create(ofrr_serve** engine, int device, int workers, size_t hbm_budget_bytes);
int ofrr_serve_destroy(ofrr_serve* engine); /* finishes queued requests first */
int ofrr_serve_submit(ofrr_serve* engine, const ofrr_request* request, uint64_t* ticket);
int ofrr_serve_poll(ofrr_serve* engine, uint64_t ticket, int* done, int* status);
int ofrr_serve_wait(ofrr_serve* engine, uint64_t ticket, int* status, double* latency_ms);
int ofrr_serve_stats(ofrr_serve* engine, ofrr_serve_report* stats);
/* count independent si_eig solves with shared options through the engine (submit all, wait all);
 * per-problem status in statuses[i]; returns the first submission error, if any. */
int ofrr_batch_si_eig(ofrr_serve* engine, int count, const ofrr_operator* ops, const ofrr_options* opt,
                      void* const* V /*dev*/, const int64_t* ldv, double* const* evals /*host*/,
                      double* const* resid /*host|NULL*/, ofrr_info* infos /*host|NULL*/, int* statuses);
/* Batched dense symmetric eigensolves in one persistent launch (no reference counterpart; the per-matrix
 * algorithm is subspace_iter_eig.m:50-68 with the Hessenberg basis and eig_rr.m).  count matrices A_i
 * (n_i x n_i, b <= n_i <= 1024, FP64, column-major, packed in one device buffer at element offsets
 * offset[i]); opt: block (<= 16), nev (<= 8), step_size, maxiter (outer iterations), tol (residual
 * ||A x - l x|| / max|l| target, >= 1e-7 in the FP32 phase, certified in FP64), p_output (OFRR_BF16 or
 * OFRR_F16: the storage type of A in the first phase), seed.  Phases per matrix: 16-bit A with FP32
 * accumulation, then FP32 A, on the CUDA cores of one SM per matrix (a persistent grid pulling matrices
 * largest first); then a second persistent pass takes the nev leading Ritz pairs to FP64 accuracy (block
 * Rayleigh-Ritz on [X, A X - X L] with FP64 products) and computes their FP64 residuals.  Outputs: X
 * (device, n_i x nev unit-norm FP64 Ritz vectors at element offsets xoffset[i]), evals (host, count x nev,
 * descending), resid (host, count x nev, or NULL), iterations (host, count, or NULL: outer iterations of
 * the first pass), statuses (host, count: OFRR_SUCCESS or OFRR_ERR_SOLVER_MAX_ITERATIONS). */
int ofrr_batch_sym_eig(ofrr_ctx* ctx, int count, const int64_t* n /*host*/, const int64_t* offset /*host*/,
                       const double* A /*dev*/, const ofrr_options* opt, double* X /*dev*/,
                       const int64_t* xoffset /*host*/, double* evals /*host*/, double* resid /*host|NULL*/,
                       int* iterations /*host|NULL*/, int* statuses /*host*/);
/* ofrr_batch_sym_eig with each matrix's time from leaving the queue to its certified result (host, count,
 * milliseconds, from the GPU's global timer); no reference counterpart. */
int ofrr_batch_sym_eig_timed(ofrr_ctx* ctx, int count, const int64_t* n, const int64_t* offset, const double* A,
                             const ofrr_options* opt, double* X, const int64_t* xoffset, double* evals, double* resid,
                             int* iterations, int* statuses, double* latency_ms /*host*/);

/* releases a context's cached workspace (no allocation of it may be live: call between solves) */
int ofrr_ctx_trim(ofrr_ctx* ctx);

/* Failure-detection self-test: queues one kernel that waits on an mbarrier nothing arrives on, with the
 * same bounded wait the library's pipelines use (timeout_ns, clamped to [1 us, 1 s]); when the wait gives
 * up the kernel records a timeout in the context's status words and returns.  The next
 * ofrr_ctx_synchronize then returns OFRR_ERR_DEVICE_TIMEOUT and clears the words; the context stays
 * usable.  No fault, trap or unbounded wait is involved. */
int ofrr_debug_bounded_wait(ofrr_ctx* ctx, int64_t timeout_ns);

/* Self-test of the fused scale-and-split kernels of the emulated FP64 power iteration (no reference
 * counterpart; the power loop of subspace_iter_svd.m:63-69, scalecols.m after each product).
 * mode 0: X (M x N, M <= 8192) is scaled in place as ofrr_scalecols does (FP64, reciprocal multiply);
 * mode 1: X = A' B (A: K x M, B: K x N, FP64) by the exact-slice product, its partial sums combined
 * inside the scaling kernel, then scaled likewise; mode 2: X is left as it is.  Every mode writes the
 * digit stack of the resulting X (N columns of 5 x roundup(M, 64) BF16 digits, device) and the N
 * column exponents (device ints). */
int ofrr_debug_scale_slice(ofrr_ctx* ctx, int mode, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                           const double* B, int64_t ldb, double* X, int64_t ldx, void* digits, int* expo);

/* Self-test of the 16-bit power step (no reference counterpart; subspace_iter_svd.m:63-69 in the
 * low-precision phase): C = A' B for 16-bit A (K x M, M <= 8192) and B (K x N) of type t16 (OFRR_F16 or
 * OFRR_BF16), FP32 accumulation, C stored as t16, then scalecols of C computed in FP32 (fast != 0: the
 * production form).  The split-K partial sums are combined inside the scaling kernel.  Returns
 * OFRR_ERR_INVALID_ARGUMENT when the shape or layout (16-byte aligned operands) does not take that path. */
int ofrr_debug_gemm16_scalecols(ofrr_ctx* ctx, int t16, int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                                const void* B, int64_t ldb, void* C, int64_t ldc, int fast);

/* Self-test of the thick-restart Krylov path's restart block (no reference counterpart): Y (n x p) spanning
 * the invariant subspace of the pencil (G, M) (M SPD) for its eigenvalues with real part above sigma,
 * from the matrix sign function; G, M, Y device FP64 column-major with ld n, n <= 96.
 * OFRR_ERR_SINGULAR_MATRIX when sigma is an eigenvalue. */
int ofrr_debug_invariant_subspace(ofrr_ctx* ctx, int n, const double* G, const double* M, double sigma, int p,
                                  double* Y);

/* Per-solve tracing: with a path set, every si_eig / si_svd / arnoldi_eig solve on this context appends
 * one JSON line to that file (solver, sizes, status, iterations, residual, kernel launches, total and
 * per-phase device time from CUDA events on the context's stream).  NULL or "" turns it off.  A context
 * created while the environment variable OFRR_TRACE_FILE is set starts with that path.  NVTX ranges
 * name the same phases for external profilers whether or not a path is set. */
int ofrr_ctx_set_trace(ofrr_ctx* ctx, const char* path);

#ifdef __cplusplus
}
#endif
#endif /* OFRR_GB300_H */
