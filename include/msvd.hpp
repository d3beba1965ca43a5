// msvd.hpp -- header-only C++ drop-in for the reference's solver entry points and containers,
// implemented over the C ABI of libofrr_gb300.so (include/ofrr.h).
//
// Same namespace, class and function names, template parameters and defaults as the reference:
//   containers   Vector<T>, Matrix<T>  (CPP/containers/vector.hpp:20-214, matrix.hpp:14-189), Location
//   status       MSVDStatus            (CPP/core/utils/error_handling.hpp:24-62)
//   handles      CUDAHandler::init / finalize (CPP/core/utils/cuda_handler.hpp:15-81)
//   blocks       hessenberg, hessenberg_v2, hessenberg_v3 (CPP/linalg/factorization/hessenberg.hpp:22-78),
//                iamax, matrix_iamax, gemm, check_special_values, syev, sygv (CPP/linalg/blas/mvops.hpp)
//   solvers      si_eig, rr_eig, ofrr_eig, arnoldi_eig, si_svd, rr_svd, arnoldi_svd
//                (CPP/linalg/solvers/eig/*.hpp, CPP/linalg/solvers/svd/*.hpp)
// plus CsrMatrix<T> (new: the reference has no sparse operator in its C++ API) and overloads of the
// eigensolvers that take it.  Programmer errors (wrong location or shape) throw std::runtime_error
// like the reference; numerical outcomes are returned as MSVDStatus.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "ofrr.h"

namespace msvd {

enum class Location { kHOST = 0, kDEVICE };

enum class MSVDStatus {
  kSuccess = 0,
  kErrorInvalidArgument = 1000,
  kErrorInvalidOperation = 1001,
  kErrorOutOfMemory = 1002,
  kErrorNotImplemented = 1003,
  kErrorInternalError = 1004,
  kErrorNaN = 1005,
  kErrorInf = 1006,
  kErrorBLASInvalidLocation = 2000,
  kErrorBLASMixedPrecisionCPU = 2001,
  kErrorBLASHalfPrecisionCPU = 2002,
  kErrorBLASUnsupportedType = 2003,
  kErrorBLASCuBLASFailure = 2004,
  kErrorBLASInvalidSize = 2005,
  kErrorFactorizationFailed = 3000,
  kErrorSingularMatrix = 3001,
  kErrorSolverDivergence = 4000,
  kErrorSolverMaxIterations = 4001,
  kErrorFileNotFound = 5000,
  kErrorInvalidFormat = 5001,
  kErrorCUDAGeneral = 6000,
  kErrorCUDAMemory = 6001,
  kErrorCUDALaunch = 6002,
  kErrorCUDASync = 6003,
  kErrorDeviceTimeout = 6004
};

inline std::string GetStatusString(MSVDStatus s) { return ofrr_status_string((int)s); }

namespace detail {
inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
template <class T> struct dtype_of;
template <> struct dtype_of<double> { static constexpr ofrr_dtype value = OFRR_F64; };
template <> struct dtype_of<float> { static constexpr ofrr_dtype value = OFRR_F32; };
template <> struct dtype_of<__half> { static constexpr ofrr_dtype value = OFRR_F16; };
template <> struct dtype_of<__nv_bfloat16> { static constexpr ofrr_dtype value = OFRR_BF16; };
template <class T> constexpr ofrr_dtype dt() { return dtype_of<T>::value; }
}  // namespace detail

// ---- library handle (replaces the CUDAHandler singleton with one ofrr context) -------------
class CUDAHandler {
 public:
  static void init(int device = 0) {
    if (ctx_()) return;
    ofrr_ctx* c = nullptr;
    int st = ofrr_ctx_create(&c, device, nullptr);
    if (st != OFRR_SUCCESS) throw std::runtime_error(std::string("ofrr_ctx_create: ") + ofrr_status_string(st));
    ctx_() = c;
  }
  static void finalize() {
    if (ctx_()) ofrr_ctx_destroy(ctx_());
    ctx_() = nullptr;
  }
  static ofrr_ctx* ctx() {
    if (!ctx_()) init();
    return ctx_();
  }
  static cudaStream_t stream() { return (cudaStream_t)ofrr_ctx_get_stream(ctx()); }

 private:
  static ofrr_ctx*& ctx_() {
    static ofrr_ctx* c = nullptr;
    return c;
  }
};

// ---- Vector<T> ------------------------------------------------------------------------------
template <typename T>
class Matrix;

template <typename T>
class Vector {
 public:
  Vector(size_t size, Location loc = Location::kDEVICE) : _length(size), _location(loc), _owns(true) {
    if (loc == Location::kHOST) _ptr = new T[size > 0 ? size : 1];
    else detail::cuda_check(cudaMalloc(&_ptr, (size > 0 ? size : 1) * sizeof(T)), "cudaMalloc");
  }
  Vector(T* external_data, size_t size, Location loc) : _ptr(external_data), _length(size), _location(loc), _owns(false) {}
  Vector(const Vector& o) : Vector(o._length, o._location) { copy_from(o); }
  Vector(Vector&& o) noexcept : _ptr(o._ptr), _length(o._length), _location(o._location), _owns(o._owns) {
    o._ptr = nullptr;
    o._owns = false;
  }
  Vector& operator=(const Vector& o) {
    if (this != &o) {
      Free();
      _length = o._length;
      _location = o._location;
      _owns = true;
      if (_location == Location::kHOST) _ptr = new T[_length > 0 ? _length : 1];
      else detail::cuda_check(cudaMalloc(&_ptr, (_length > 0 ? _length : 1) * sizeof(T)), "cudaMalloc");
      copy_from(o);
    }
    return *this;
  }
  Vector& operator=(Vector&& o) noexcept {
    if (this != &o) {
      Free();
      _ptr = o._ptr;
      _length = o._length;
      _location = o._location;
      _owns = o._owns;
      o._ptr = nullptr;
      o._owns = false;
    }
    return *this;
  }
  ~Vector() { Free(); }

  void to_device() { move_to(Location::kDEVICE); }
  void to_host() { move_to(Location::kHOST); }
  void fill(T val) {
    if (_location == Location::kHOST) {
      for (size_t i = 0; i < _length; ++i) _ptr[i] = val;
    } else {
      std::vector<T> h(_length, val);
      detail::cuda_check(cudaMemcpy(_ptr, h.data(), _length * sizeof(T), cudaMemcpyHostToDevice), "fill");
    }
  }
  // N(0,1) entries from the library's counter-based generator (the reference used cuRAND U[-1,1])
  void fill_random(unsigned long long seed = 815) {
    if (_location == Location::kDEVICE) {
      ofrr_randn(CUDAHandler::ctx(), seed, (int64_t)_length, 1, detail::dt<T>(), _ptr, (int64_t)_length);
      ofrr_ctx_synchronize(CUDAHandler::ctx());
    } else {
      std::vector<double> h(_length);
      ofrr_randn_host(seed, (int64_t)_length, 1, h.data());
      for (size_t i = 0; i < _length; ++i) _ptr[i] = (T)h[i];
    }
  }
  void scale(T alpha) {
    bool dev = _location == Location::kDEVICE;
    if (dev) to_host();
    for (size_t i = 0; i < _length; ++i) _ptr[i] = (T)((double)_ptr[i] * (double)alpha);
    if (dev) to_device();
  }
  template <typename U>
  Vector<U> cast() const {
    Vector<U> out(_length, _location);
    if (_location == Location::kDEVICE) {
      ofrr_cast(CUDAHandler::ctx(), detail::dt<T>(), detail::dt<U>(), (int64_t)_length, 1, _ptr, (int64_t)_length,
                out.data(), (int64_t)_length);
      ofrr_ctx_synchronize(CUDAHandler::ctx());
    } else {
      for (size_t i = 0; i < _length; ++i) out.data()[i] = (U)(double)_ptr[i];
    }
    return out;
  }
  void Free() {
    if (_ptr && _owns) {
      if (_location == Location::kHOST) delete[] _ptr;
      else cudaFree(_ptr);
    }
    _ptr = nullptr;
  }
  T* data() const { return _ptr; }
  T& operator[](size_t i) { return _ptr[i]; }
  const T& operator[](size_t i) const { return _ptr[i]; }
  Location location() const { return _location; }
  size_t length() const { return _length; }
  bool owns_data() const { return _owns; }

 private:
  void copy_from(const Vector& o) {
    cudaMemcpyKind k = (o._location == Location::kHOST)
                           ? (_location == Location::kHOST ? cudaMemcpyHostToHost : cudaMemcpyHostToDevice)
                           : (_location == Location::kHOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
    if (_length) detail::cuda_check(cudaMemcpy(_ptr, o._ptr, _length * sizeof(T), k), "copy");
  }
  void move_to(Location to) {
    if (_location == to) return;
    T* p = nullptr;
    if (to == Location::kDEVICE) {
      detail::cuda_check(cudaMalloc(&p, (_length > 0 ? _length : 1) * sizeof(T)), "cudaMalloc");
      if (_length) detail::cuda_check(cudaMemcpy(p, _ptr, _length * sizeof(T), cudaMemcpyHostToDevice), "to_device");
      if (_owns) delete[] _ptr;
    } else {
      p = new T[_length > 0 ? _length : 1];
      if (_length) detail::cuda_check(cudaMemcpy(p, _ptr, _length * sizeof(T), cudaMemcpyDeviceToHost), "to_host");
      if (_owns) cudaFree(_ptr);
    }
    _ptr = p;
    _owns = true;  // a view that moves takes ownership of its copy (vector.cu:116-121)
    _location = to;
  }
  T* _ptr = nullptr;
  size_t _length = 0;
  Location _location = Location::kDEVICE;
  bool _owns = true;
  template <typename U>
  friend class Matrix;
};

// ---- Matrix<T>: column-major with leading dimension ------------------------------------------
template <typename T>
class Matrix {
 public:
  Matrix(size_t rows, size_t cols, Location loc = Location::kDEVICE)
      : _data(rows * cols, loc), _rows(rows), _cols(cols), _ld(rows > 0 ? rows : 1) {}
  Matrix(T* external_data, size_t rows, size_t cols, size_t ld, Location loc)
      : _data(external_data, ld * cols, loc), _rows(rows), _cols(cols), _ld(ld) {}
  T& operator()(size_t i, size_t j) { return _data.data()[i + j * _ld]; }
  const T& operator()(size_t i, size_t j) const { return _data.data()[i + j * _ld]; }
  Matrix<T> submatrix(size_t r0, size_t c0, size_t nr, size_t nc) {
    return Matrix<T>(_data.data() + r0 + c0 * _ld, nr, nc, _ld, _data.location());
  }
  void to_host() { _data.to_host(); }
  void to_device() { _data.to_device(); }
  void fill(T v) { _data.fill(v); }
  void fill_random(unsigned long long seed = 815) {
    if (_data.location() == Location::kDEVICE) {
      ofrr_randn(CUDAHandler::ctx(), seed, (int64_t)_rows, (int64_t)_cols, detail::dt<T>(), _data.data(), (int64_t)_ld);
      ofrr_ctx_synchronize(CUDAHandler::ctx());
    } else {
      std::vector<double> h(_rows * _cols);
      ofrr_randn_host(seed, (int64_t)_rows, (int64_t)_cols, h.data());
      for (size_t j = 0; j < _cols; ++j)
        for (size_t i = 0; i < _rows; ++i) (*this)(i, j) = (T)h[i + j * _rows];
    }
  }
  void scale(T a) { _data.scale(a); }
  template <typename U>
  Matrix<U> cast() const {
    Matrix<U> out(_rows, _cols, _data.location());
    if (_data.location() == Location::kDEVICE) {
      ofrr_cast(CUDAHandler::ctx(), detail::dt<T>(), detail::dt<U>(), (int64_t)_rows, (int64_t)_cols, _data.data(),
                (int64_t)_ld, out.data(), (int64_t)out.ld());
      ofrr_ctx_synchronize(CUDAHandler::ctx());
    } else {
      for (size_t j = 0; j < _cols; ++j)
        for (size_t i = 0; i < _rows; ++i) out(i, j) = (U)(double)(*this)(i, j);
    }
    return out;
  }
  T* data() { return _data.data(); }
  const T* data() const { return _data.data(); }
  size_t rows() const { return _rows; }
  size_t cols() const { return _cols; }
  size_t ld() const { return _ld; }
  Location location() const { return _data.location(); }

 private:
  Vector<T> _data;
  size_t _rows, _cols, _ld;
};

// ---- CsrMatrix<T>: 0-based int32 CSR on the device with FP64/FP32/FP16 value copies -------------
template <typename T>
class CsrMatrix {
 public:
  // from host arrays (row_ptr: nrows+1, col_ind/values: nnz)
  CsrMatrix(size_t nrows, size_t ncols, const std::vector<int32_t>& row_ptr, const std::vector<int32_t>& col_ind,
            const std::vector<double>& values, bool symmetric)
      : _ip(nrows + 1, Location::kHOST), _ix(col_ind.size() > 0 ? col_ind.size() : 1, Location::kHOST),
        _ad(values.size() > 0 ? values.size() : 1, Location::kHOST),
        _as(values.size() > 0 ? values.size() : 1, Location::kHOST),
        _ah(values.size() > 0 ? values.size() : 1, Location::kHOST), _nrows(nrows), _ncols(ncols),
        _nnz(values.size()), _sym(symmetric) {
    std::memcpy(_ip.data(), row_ptr.data(), (nrows + 1) * sizeof(int32_t));
    for (size_t k = 0; k < _nnz; ++k) {
      _ix[k] = col_ind[k];
      _ad[k] = values[k];
      _as[k] = (float)values[k];
      _ah[k] = __double2half(values[k]);
    }
    _ip.to_device();
    _ix.to_device();
    _ad.to_device();
    _as.to_device();
    _ah.to_device();
  }
  size_t rows() const { return _nrows; }
  size_t cols() const { return _ncols; }
  size_t nnz() const { return _nnz; }
  bool symmetric() const { return _sym; }
  ofrr_operator op() const {
    ofrr_operator o{};
    o.kind = OFRR_OP_CSR;
    o.nrows = (int64_t)_nrows;
    o.ncols = (int64_t)_ncols;
    o.symmetric = _sym ? 1 : 0;
    o.dtype = detail::dt<T>();
    o.csr.nrows = (int64_t)_nrows;
    o.csr.ncols = (int64_t)_ncols;
    o.csr.nnz = (int64_t)_nnz;
    o.csr.indptr = _ip.data();
    o.csr.indices = _ix.data();
    o.csr.a_double = _ad.data();
    o.csr.a_single = _as.data();
    o.csr.a_half = _ah.data();
    return o;
  }

 private:
  Vector<int32_t> _ip, _ix;
  Vector<double> _ad;
  Vector<float> _as;
  Vector<__half> _ah;
  size_t _nrows, _ncols, _nnz;
  bool _sym;
};

namespace detail {
template <class T>
inline void need(const Matrix<T>& M, Location loc, const char* what) {
  if (M.location() != loc)
    throw std::runtime_error(std::string(what) + (loc == Location::kDEVICE ? " must be on device" : " must be on host"));
}
template <class T>
inline ofrr_operator dense_op(const Matrix<T>& A, bool symmetric) {
  ofrr_operator o{};
  o.kind = OFRR_OP_DENSE;
  o.nrows = (int64_t)A.rows();
  o.ncols = (int64_t)A.cols();
  o.symmetric = symmetric ? 1 : 0;
  o.dtype = dt<T>();
  o.data = A.data();
  o.ld = (int64_t)A.ld();
  return o;
}
template <class T_O, class T_C>
inline ofrr_options ref_options(int max_iter, double tol, bool use_generalized, double select_tol, int block) {
  ofrr_options o;
  ofrr_options_default(&o);
  o.mode = OFRR_MODE_REFERENCE;
  o.maxiter = max_iter;
  o.tol = tol;
  o.use_generalized = use_generalized ? 1 : 0;
  o.select_tol = select_tol;
  o.block = block;
  o.nev = block;
  o.use_start_block = 1;  // V carries the initial block (si_eig.hpp:16)
  o.p_output = o.p_hess_output = o.p_rr_output = dt<T_O>();
  const ofrr_dtype pc = std::is_same<T_C, double>::value ? OFRR_F64 : OFRR_F32;
  o.p_compute = o.p_hess_compute = o.p_rr_compute = pc;
  return o;
}
// write eigenvalues on the diagonal of D (D's own location)
template <class T>
inline void write_diag(Matrix<T>& D, const std::vector<double>& w) {
  const size_t k = std::min(std::min(D.rows(), D.cols()), w.size());
  std::vector<T> h(D.ld() * D.cols(), (T)0.0);
  for (size_t i = 0; i < k; ++i) h[i + i * D.ld()] = (T)w[i];
  if (D.location() == Location::kHOST) std::memcpy(D.data(), h.data(), h.size() * sizeof(T));
  else cuda_check(cudaMemcpy(D.data(), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "D");
}
inline MSVDStatus st(int s) { return (MSVDStatus)s; }
}  // namespace detail

// ---- building blocks ------------------------------------------------------------------------------
template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> hessenberg(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, T_O select_tol = T_O(-1.0),
                            T_O orth_tol = T_O(0.0), T_O reorth_tol = T_O(0.0)) {
  (void)orth_tol;
  (void)reorth_tol;
  detail::need(A, Location::kDEVICE, "Input matrix A");
  detail::need(Q, Location::kDEVICE, "Output matrix Q");
  detail::need(R, Location::kHOST, "Output matrix R");
  const size_t m = A.rows(), n = A.cols();
  if (Q.rows() != m || Q.cols() != n) throw std::runtime_error("Output matrix Q has incorrect dimensions");
  if (R.rows() != n || R.cols() != n) throw std::runtime_error("Output matrix R has incorrect dimensions");
  std::vector<double> Rh(n * n);
  std::vector<int> skip(n), perm(n);
  const ofrr_dtype tc = std::is_same<T_COMPUTE, double>::value ? OFRR_F64 : OFRR_F32;
  int s = ofrr_hessenberg(CUDAHandler::ctx(), detail::dt<T_I>(), detail::dt<T_O>(), tc, (int64_t)m, (int64_t)n,
                          A.data(), (int64_t)A.ld(), Q.data(), (int64_t)Q.ld(), (double)select_tol, Rh.data(),
                          skip.data(), perm.data());
  if (s != OFRR_SUCCESS) throw std::runtime_error(std::string("hessenberg: ") + ofrr_status_string(s));
  for (size_t j = 0; j < n; ++j)
    for (size_t i = 0; i < n; ++i) R(i, j) = (T_O)Rh[i + j * n];
  return skip;
}
// the three GPU variants of the reference collapse onto one kernel
template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> hessenberg_v2(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, T_O select_tol = T_O(-1.0),
                               T_O orth_tol = T_O(0.0), T_O reorth_tol = T_O(0.0)) {
  return hessenberg<T_I, T_O, T_COMPUTE>(A, Q, R, select_tol, orth_tol, reorth_tol);
}
template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> hessenberg_v3(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, T_O select_tol = T_O(-1.0),
                               T_O orth_tol = T_O(0.0), T_O reorth_tol = T_O(0.0)) {
  return hessenberg<T_I, T_O, T_COMPUTE>(A, Q, R, select_tol, orth_tol, reorth_tol);
}

// ---- orthogonal comparison bases (CPP/linalg/factorization/qr.hpp:21-132) -------------------------
// mgs: MATLAB/+src/+qr/mgs.m with adaptive re-orthogonalisation; mgs_v2: one MGS pass (its
// orth_tol / reorth_tol are placeholders in the reference, qr.hpp:33-41); cgs2: classical
// Gram-Schmidt with the same re-orthogonalisation (cgs.m).  Defaults eps(T_O), eps(T_O), 1/sqrt(2);
// a negative select_tol also selects eps(T_O).  Q on the device, R on the host, skip flags returned.
namespace detail {
template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> gs(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, int classical, double select_tol,
                    double orth_tol, double reorth_tol, const char* what) {
  need(A, Location::kDEVICE, "Input matrix A");
  need(Q, Location::kDEVICE, "Output matrix Q");
  need(R, Location::kHOST, "Output matrix R");
  const size_t m = A.rows(), n = A.cols();
  if (Q.rows() != m || Q.cols() != n) throw std::runtime_error("Output matrix Q has incorrect dimensions");
  if (R.rows() != n || R.cols() != n) throw std::runtime_error("Output matrix R has incorrect dimensions");
  std::vector<double> Rh(n * n);
  std::vector<int> skip(n);
  const ofrr_dtype tc = std::is_same<T_COMPUTE, double>::value ? OFRR_F64 : OFRR_F32;
  int s = ofrr_gs_basis(CUDAHandler::ctx(), classical, dt<T_I>(), dt<T_O>(), tc, (int64_t)m, (int64_t)n, A.data(),
                        (int64_t)A.ld(), Q.data(), (int64_t)Q.ld(), select_tol, orth_tol, reorth_tol, Rh.data(),
                        skip.data());
  if (s != OFRR_SUCCESS) throw std::runtime_error(std::string(what) + ": " + ofrr_status_string(s));
  for (size_t j = 0; j < n; ++j)
    for (size_t i = 0; i < n; ++i) R(i, j) = (T_O)Rh[i + j * n];
  return skip;
}
}  // namespace detail

template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> mgs(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, T_O select_tol = T_O(-1.0),
                     T_O orth_tol = T_O(-1.0), T_O reorth_tol = T_O(0.70710678118654752)) {
  const double ot = (double)orth_tol < 0 ? NAN : (double)orth_tol;
  return detail::gs<T_I, T_O, T_COMPUTE>(A, Q, R, 0, (double)select_tol, ot, (double)reorth_tol, "mgs");
}
template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> mgs_v2(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, T_O select_tol = T_O(-1.0),
                        T_O orth_tol = T_O(-1.0), T_O reorth_tol = T_O(-1.0)) {
  (void)orth_tol, (void)reorth_tol;
  return detail::gs<T_I, T_O, T_COMPUTE>(A, Q, R, 0, (double)select_tol, NAN, -1.0, "mgs_v2");
}
template <typename T_I, typename T_O, typename T_COMPUTE>
std::vector<int> cgs2(const Matrix<T_I>& A, Matrix<T_O>& Q, Matrix<T_O>& R, T_O select_tol = T_O(-1.0),
                      T_O orth_tol = T_O(-1.0), T_O reorth_tol = T_O(0.70710678118654752)) {
  const double ot = (double)orth_tol < 0 ? NAN : (double)orth_tol;
  return detail::gs<T_I, T_O, T_COMPUTE>(A, Q, R, 1, (double)select_tol, ot, (double)reorth_tol, "cgs2");
}

template <typename T, typename T_O = T>
MSVDStatus iamax(const Vector<T>& x, int& result, T_O& result_val, Location location = Location::kHOST) {
  (void)location;
  if (x.location() != Location::kDEVICE) throw std::runtime_error("iamax: x must be on device");
  double v = 0;
  int s = ofrr_iamax(CUDAHandler::ctx(), detail::dt<T>(), (int64_t)x.length(), x.data(), &result, &v);
  result_val = (T_O)v;
  return detail::st(s);
}

template <typename T>
MSVDStatus matrix_iamax(const Matrix<T>& A, int* results, Location location = Location::kHOST) {
  detail::need(A, Location::kDEVICE, "matrix_iamax: A");
  Vector<int> d(A.cols(), Location::kDEVICE);
  int s = ofrr_matrix_iamax(CUDAHandler::ctx(), detail::dt<T>(), (int64_t)A.rows(), (int64_t)A.cols(), A.data(),
                            (int64_t)A.ld(), d.data());
  if (s != OFRR_SUCCESS) return detail::st(s);
  cudaMemcpyKind k = (location == Location::kHOST) ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  ofrr_ctx_synchronize(CUDAHandler::ctx());
  detail::cuda_check(cudaMemcpy(results, d.data(), A.cols() * sizeof(int), k), "matrix_iamax");
  return MSVDStatus::kSuccess;
}

template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus gemm(bool transA, bool transB, const T_COMPUTE& alpha, const Matrix<T_I>& A, const Matrix<T_I>& B,
                const T_COMPUTE& beta, Matrix<T_O>& C) {
  detail::need(A, Location::kDEVICE, "gemm: A");
  detail::need(B, Location::kDEVICE, "gemm: B");
  detail::need(C, Location::kDEVICE, "gemm: C");
  const int64_t M = (int64_t)(transA ? A.cols() : A.rows()), K = (int64_t)(transA ? A.rows() : A.cols());
  const int64_t N = (int64_t)(transB ? B.rows() : B.cols());
  const ofrr_dtype tc = std::is_same<T_COMPUTE, double>::value ? OFRR_F64 : OFRR_F32;
  int s = ofrr_gemm(CUDAHandler::ctx(), transA, transB, detail::dt<T_I>(), detail::dt<T_I>(), tc, detail::dt<T_O>(), M,
                    N, K, (double)alpha, A.data(), (int64_t)A.ld(), B.data(), (int64_t)B.ld(), (double)beta, C.data(),
                    (int64_t)C.ld());
  ofrr_ctx_synchronize(CUDAHandler::ctx());
  return detail::st(s);
}

template <typename T>
MSVDStatus check_special_values(const Matrix<T>& A) {
  if (A.location() == Location::kHOST) {
    for (size_t j = 0; j < A.cols(); ++j)
      for (size_t i = 0; i < A.rows(); ++i) {
        double v = (double)A(i, j);
        if (v != v) return MSVDStatus::kErrorNaN;
        if (v - v != 0) return MSVDStatus::kErrorInf;
      }
    return MSVDStatus::kSuccess;
  }
  return detail::st(ofrr_check_special_values(CUDAHandler::ctx(), detail::dt<T>(), (int64_t)A.rows(),
                                              (int64_t)A.cols(), A.data(), (int64_t)A.ld()));
}

// small symmetric (generalized) eigenproblems, FP64 on the device (mvops.hpp:184-197); A may live on
// either side, the result comes back to A's location; work/lwork are accepted for API parity
template <typename T>
MSVDStatus syev(Matrix<T>& A, Vector<T>& W, T* work = nullptr, int lwork = -1) {
  static_assert(std::is_same<T, double>::value, "syev: FP64 only");
  if (lwork == -1 && work) {
    *work = 1;
    return MSVDStatus::kSuccess;
  }
  const bool host = A.location() == Location::kHOST;
  if (host) A.to_device();
  Vector<double> w(A.rows(), Location::kDEVICE);
  int s = ofrr_syev(CUDAHandler::ctx(), (int)A.rows(), A.data(), (int)A.ld(), w.data());
  ofrr_ctx_synchronize(CUDAHandler::ctx());
  if (host) A.to_host();
  w.to_host();
  for (size_t i = 0; i < A.rows(); ++i) W[i] = w[i];
  return detail::st(s);
}
template <typename T>
MSVDStatus sygv(Matrix<T>& A, Matrix<T>& B, Vector<T>& W, T* work = nullptr, int lwork = -1) {
  static_assert(std::is_same<T, double>::value, "sygv: FP64 only");
  if (lwork == -1 && work) {
    *work = 1;
    return MSVDStatus::kSuccess;
  }
  const bool host = A.location() == Location::kHOST;
  if (host) {
    A.to_device();
    B.to_device();
  }
  Vector<double> w(A.rows(), Location::kDEVICE);
  int s = ofrr_sygv(CUDAHandler::ctx(), (int)A.rows(), A.data(), (int)A.ld(), B.data(), (int)B.ld(), w.data());
  ofrr_ctx_synchronize(CUDAHandler::ctx());
  if (host) {
    A.to_host();
    B.to_host();
  }
  w.to_host();
  for (size_t i = 0; i < A.rows(); ++i) W[i] = w[i];
  return detail::st(s);
}

// ---- solvers ------------------------------------------------------------------------------------
template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus si_eig(const Matrix<T_I>& A, Matrix<T_O>& V, Matrix<T_O>& D, int max_iter = 100, T_COMPUTE tol = 1e-10,
                  bool use_generalized = false, T_COMPUTE select_tol = 1e-10) {
  detail::need(A, Location::kDEVICE, "si_eig: A");
  detail::need(V, Location::kDEVICE, "si_eig: V");
  ofrr_operator op = detail::dense_op(A, true);
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(max_iter, (double)tol, use_generalized, (double)select_tol,
                                                       (int)V.cols());
  std::vector<double> w(V.cols());
  int s = ofrr_si_eig(CUDAHandler::ctx(), &op, &o, V.data(), (int64_t)V.ld(), w.data(), nullptr, nullptr);
  detail::write_diag(D, w);
  return detail::st(s);
}
template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus si_eig(const CsrMatrix<T_I>& A, Matrix<T_O>& V, Matrix<T_O>& D, int max_iter = 100, T_COMPUTE tol = 1e-10,
                  bool use_generalized = false, T_COMPUTE select_tol = 1e-10) {
  detail::need(V, Location::kDEVICE, "si_eig: V");
  ofrr_operator op = A.op();
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(max_iter, (double)tol, use_generalized, (double)select_tol,
                                                       (int)V.cols());
  std::vector<double> w(V.cols());
  int s = ofrr_si_eig(CUDAHandler::ctx(), &op, &o, V.data(), (int64_t)V.ld(), w.data(), nullptr, nullptr);
  detail::write_diag(D, w);
  return detail::st(s);
}

template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus rr_eig(const Matrix<T_I>& A, Matrix<T_O>& V, Matrix<T_O>& D, bool use_generalized = false,
                  T_COMPUTE select_tol = 1e-10) {
  detail::need(A, Location::kDEVICE, "rr_eig: A");
  detail::need(V, Location::kDEVICE, "rr_eig: V");
  ofrr_operator op = detail::dense_op(A, true);
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(1, 0.0, use_generalized, (double)select_tol, (int)V.cols());
  o.generalized_tol = std::is_same<T_COMPUTE, double>::value ? 1e-10 : 1e-5;  // eig_rr.m:105-113
  std::vector<double> w(V.cols());
  int s = ofrr_rr_eig(CUDAHandler::ctx(), &op, &o, (int64_t)V.cols(), V.data(), (int64_t)V.ld(), w.data());
  detail::write_diag(D, w);
  return detail::st(s);
}

template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus ofrr_eig(const Matrix<T_I>& A, const Matrix<T_I>& B, Matrix<T_O>& V, Matrix<T_O>& D,
                    T_COMPUTE select_tol = 1e-10) {
  detail::need(A, Location::kDEVICE, "ofrr_eig: A");
  detail::need(B, Location::kDEVICE, "ofrr_eig: B");
  detail::need(V, Location::kDEVICE, "ofrr_eig: V");
  ofrr_operator oa = detail::dense_op(A, true), ob = detail::dense_op(B, true);
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(1, 0.0, true, 0.0, (int)V.cols());
  o.generalized_tol = (double)select_tol;  // rr_eig.hpp:33: tolerance for the stability of the pencil
  std::vector<double> w(V.cols());
  int s = ::ofrr_ofrr_eig(CUDAHandler::ctx(), &oa, &ob, &o, (int64_t)V.cols(), V.data(), (int64_t)V.ld(), w.data());
  detail::write_diag(D, w);
  return detail::st(s);
}

template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus arnoldi_eig(const Matrix<T_I>& A, Matrix<T_O>& V, Matrix<T_O>& D, int max_iter = 100,
                       T_COMPUTE tol = 1e-10, bool use_generalized = false, T_COMPUTE select_tol = 1e-10) {
  (void)use_generalized;  // the Hessenberg-process Krylov path always projects on the pencil
  detail::need(A, Location::kDEVICE, "arnoldi_eig: A");
  detail::need(V, Location::kDEVICE, "arnoldi_eig: V");
  ofrr_operator op = detail::dense_op(A, false);
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(max_iter, (double)tol, true, (double)select_tol, 1);
  o.kdim = max_iter;  // arnoldi_eig.hpp:18: max_iter is the maximum Krylov dimension
  o.maxiter = max_iter + 1;
  o.nev = (int)V.cols();
  o.generalized_tol = 0.0;
  std::vector<double> w(V.cols());
  int s = ofrr_arnoldi_eig(CUDAHandler::ctx(), &op, &o, V.data(), V.data(), (int64_t)V.ld(), w.data(), nullptr, nullptr);
  detail::write_diag(D, w);
  return detail::st(s);
}

template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus si_svd(const Matrix<T_I>& A, Matrix<T_O>& U, Matrix<T_O>& S, Matrix<T_O>& V, int max_iter = 100,
                  T_COMPUTE tol = 1e-10, bool use_generalized = false, T_COMPUTE select_tol = 1e-10) {
  detail::need(A, Location::kDEVICE, "si_svd: A");
  detail::need(U, Location::kDEVICE, "si_svd: U");
  detail::need(V, Location::kDEVICE, "si_svd: V");
  ofrr_operator op = detail::dense_op(A, false);
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(max_iter, (double)tol, true, (double)select_tol,
                                                       (int)V.cols());
  (void)use_generalized;  // the oblique bases need the generalized pencil (svd_rr.m:58-77)
  std::vector<double> s(V.cols());
  int st = ofrr_si_svd(CUDAHandler::ctx(), &op, &o, U.data(), (int64_t)U.ld(), s.data(), V.data(), (int64_t)V.ld(),
                       nullptr, nullptr);
  detail::write_diag(S, s);
  return detail::st(st);
}

template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus rr_svd(const Matrix<T_I>& A, Matrix<T_O>& U, Matrix<T_O>& S, Matrix<T_O>& V, bool use_generalized = false,
                  T_COMPUTE select_tol = 1e-10) {
  detail::need(A, Location::kDEVICE, "rr_svd: A");
  ofrr_operator op = detail::dense_op(A, false);
  ofrr_options o = detail::ref_options<T_O, T_COMPUTE>(1, 0.0, true, (double)select_tol, (int)V.cols());
  (void)use_generalized;
  o.generalized_tol = std::is_same<T_COMPUTE, double>::value ? 1e-10 : 1e-5;
  std::vector<double> s(V.cols());
  int st = ofrr_rr_svd(CUDAHandler::ctx(), &op, &o, (int64_t)V.cols(), U.data(), (int64_t)U.ld(), s.data(), V.data(),
                       (int64_t)V.ld());
  detail::write_diag(S, s);
  return detail::st(st);
}

// Krylov SVD: not defined by the reference beyond its signature (arnoldi_svd.cu:10-18 is a stub);
// reported as not implemented rather than silently succeeding.
template <typename T_I, typename T_O, typename T_COMPUTE>
MSVDStatus arnoldi_svd(const Matrix<T_I>& A, Matrix<T_O>& U, Matrix<T_O>& S, Matrix<T_O>& V, int max_iter = 100,
                       T_COMPUTE tol = 1e-10, bool use_generalized = false, T_COMPUTE select_tol = 1e-10) {
  (void)A, (void)U, (void)S, (void)V, (void)max_iter, (void)tol, (void)use_generalized, (void)select_tol;
  return MSVDStatus::kErrorNotImplemented;
}

// ---- on-disk CSR (CPP/io/matrix_reader.hpp:7-44): host arrays, as the reference returns them ---------
class CSRMatrix {
 public:
  std::vector<int> row_ptr;
  std::vector<int> col_ind;
  std::vector<double> values;
  int rows;
  int cols;
  CSRMatrix() : rows(0), cols(0) {}
};

class MatrixReader {
 public:
  // <prefix>_row_ptr.bin, _col_ind.bin, _values.bin; throws std::runtime_error when a file is missing,
  // empty or malformed (matrix_reader.cpp:8-45)
  static CSRMatrix read_csr_matrix(const std::string& prefix) {
    int64_t nrows = 0, nnz = 0, ncols = 0;
    int st = ofrr_csr_file_sizes(prefix.c_str(), &nrows, &nnz);
    if (st != OFRR_SUCCESS) throw std::runtime_error("read_csr_matrix(" + prefix + "): " + ofrr_status_string(st));
    CSRMatrix m;
    m.row_ptr.resize((size_t)nrows + 1);
    m.col_ind.resize((size_t)nnz);
    m.values.resize((size_t)nnz);
    st = ofrr_csr_file_read(nullptr, prefix.c_str(), nrows, nnz, m.row_ptr.data(), m.col_ind.data(), m.values.data(),
                            &ncols, 0);
    if (st != OFRR_SUCCESS) throw std::runtime_error("read_csr_matrix(" + prefix + "): " + ofrr_status_string(st));
    m.rows = (int)nrows;
    m.cols = (int)ncols;
    return m;
  }
  // <prefix>_singular_values.bin; empty when the file cannot be read (matrix_reader.cpp:47-50)
  static std::vector<double> read_singular_values(const std::string& prefix) {
    int64_t n = 0;
    if (ofrr_read_singular_values(prefix.c_str(), &n, nullptr) != OFRR_SUCCESS) return {};
    std::vector<double> v((size_t)n);
    if (ofrr_read_singular_values(prefix.c_str(), &n, v.data()) != OFRR_SUCCESS) return {};
    return v;
  }
};

// device operator from a file-read CSRMatrix
template <typename T>
CsrMatrix<T> to_device(const CSRMatrix& m, bool symmetric) {
  return CsrMatrix<T>((size_t)m.rows, (size_t)m.cols, m.row_ptr, m.col_ind, m.values, symmetric);
}

// ---- test problems (CPP/testproblems/gaussian_kernel.hpp:14-77) -------------------------------------
// Gaussian kernel of n points uniform in [0, n^(1/d))^d, computed on the GPU in FP64 and rounded to T;
// returned on the host as the reference does.  The points come from the library's seeded counter-based
// generator (the reference's host generator cannot be reproduced), so the same seed gives the same
// matrix as api.generate_gaussian_kernel, not as the reference.
template <typename T>
Matrix<T> generate_gaussian_kernel(double f, double l, double s, unsigned long long seed, int n, int d) {
  if (l <= 0.0) throw std::invalid_argument("Length scale l must be positive");
  if (s < 0.0) throw std::invalid_argument("Noise scale s must be non-negative");
  if (n <= 0 || d <= 0) throw std::invalid_argument("Data dimensions must be positive");
  Matrix<double> X((size_t)n, (size_t)d, Location::kDEVICE);
  Matrix<T> K((size_t)n, (size_t)n, Location::kDEVICE);
  ofrr_ctx* ctx = CUDAHandler::ctx();
  int st = ofrr_rand_points(ctx, (uint64_t)seed, n, d, 0, X.data(), (int64_t)X.ld());
  if (st == OFRR_SUCCESS)
    st = ofrr_gaussian_kernel(ctx, 0, n, n, d, X.data(), (int64_t)X.ld(), X.data(), (int64_t)X.ld(), l, f, s,
                              detail::dt<T>(), K.data(), (int64_t)K.ld());
  if (st == OFRR_SUCCESS) st = ofrr_ctx_synchronize(ctx);
  if (st != OFRR_SUCCESS) throw std::runtime_error(std::string("generate_gaussian_kernel: ") + ofrr_status_string(st));
  K.to_host();
  return K;
}

}  // namespace msvd
