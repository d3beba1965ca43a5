// Drop-in check: code written against the reference's C++ API (msvd::Matrix, hessenberg, syev,
// sygv, si_eig, si_svd, MatrixReader) compiles against include/msvd.hpp and runs on libofrr_gb300.so.
// Prints one line per check; exits non-zero on the first failure.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "msvd.hpp"

using namespace msvd;

static int fail(const char* what) {
  std::printf("FAIL %s\n", what);
  return 1;
}

int main(int argc, char** argv) {
  CUDAHandler::init();
  // hessenberg_test.cpp:30-92 shape: A = QR and the duplicated-column skip pattern
  {
    const size_t m = 2000, n = 200;
    Matrix<double> A(m, n, Location::kDEVICE), Q(m, n, Location::kDEVICE), R(n, n, Location::kHOST);
    A.fill_random(815);
    std::vector<int> skip = hessenberg<double, double, double>(A, Q, R);
    for (int s : skip)
      if (s) return fail("hessenberg skip");
    A.to_host();
    Q.to_host();
    double md = 0;
    for (size_t i = 0; i < m; i += 7)
      for (size_t j = 0; j < n; ++j) {
        double acc = 0;
        for (size_t k = 0; k <= j; ++k) acc += Q(i, k) * R(k, j);
        md = std::fmax(md, std::fabs(acc - A(i, j)));
      }
    if (!(md < 1e-10)) return fail("A = QR");
    std::printf("hessenberg ok max|A-QR| = %.3e\n", md);
    for (size_t i = 0; i < m; ++i)
      for (size_t j = 3; j < 6; ++j) A(i, j) = A(i, j - 3);
    A.to_device();
    Q.to_device();
    skip = hessenberg<double, double, double>(A, Q, R, 1e-12);
    for (size_t j = 0; j < n; ++j)
      if (skip[j] != (j >= 3 && j <= 5 ? 1 : 0)) return fail("skip pattern");
    std::printf("skip pattern ok\n");
  }
  // mvops_test.cpp SYEV / SYGV known answers
  {
    const int n = 10;
    Matrix<double> A(n, n, Location::kHOST), B(n, n, Location::kHOST);
    A.fill(0.0);
    B.fill(0.0);
    for (int i = 0; i < n; ++i) {
      A(i, i) = 2.0;
      if (i < n - 1) A(i, i + 1) = A(i + 1, i) = -1.0;
      B(i, i) = i + 1;
    }
    Matrix<double> V(A);
    Vector<double> W(n, Location::kHOST);
    if (syev(V, W) != MSVDStatus::kSuccess) return fail("syev status");
    if (std::fabs(W[0] - 0.0810140527710052) > 1e-10 || std::fabs(W[9] - 3.91898594722899) > 1e-10)
      return fail("syev values");
    Matrix<double> V2(A);
    if (sygv(V2, B, W) != MSVDStatus::kSuccess) return fail("sygv status");
    if (std::fabs(W[0] - 0.0141309446511971) > 1e-10 || std::fabs(W[9] - 2.38801544566837) > 1e-10)
      return fail("sygv values");
    std::printf("syev/sygv ok\n");
  }
  // si_eig on a dense symmetric matrix with a known spectrum 0.7^i
  {
    const size_t n = 300, b = 12;
    Matrix<double> A(n, n, Location::kHOST);
    A.fill(0.0);
    for (size_t i = 0; i < n; ++i) A(i, i) = std::pow(0.7, (double)i);
    A.to_device();
    Matrix<double> V(n, b, Location::kDEVICE), D(b, b, Location::kHOST);
    V.fill_random(42);
    MSVDStatus s = si_eig<double, double, double>(A, V, D, 200, 1e-10, true, 1e-10);
    if (s != MSVDStatus::kSuccess) {
      std::printf("si_eig status %d\n", (int)s);
      return fail("si_eig status");
    }
    for (size_t i = 0; i < 4; ++i)
      if (std::fabs(D(i, i) - std::pow(0.7, (double)i)) > 1e-9) return fail("si_eig values");
    std::printf("si_eig ok D(0,0)=%.12f\n", D(0, 0));
  }
  // si_svd on a diagonal 400 x 100 matrix with s_i = 0.8^i
  {
    const size_t m = 400, n = 100, b = 16;
    Matrix<double> A(m, n, Location::kHOST);
    A.fill(0.0);
    for (size_t i = 0; i < n; ++i) A(i, i) = std::pow(0.8, (double)i);
    A.to_device();
    Matrix<double> U(m, b, Location::kDEVICE), V(n, b, Location::kDEVICE), S(b, b, Location::kHOST);
    V.fill_random(7);
    MSVDStatus s = si_svd<double, double, double>(A, U, S, V, 200, 1e-10, true, 1e-10);
    if (s != MSVDStatus::kSuccess) return fail("si_svd status");
    for (size_t i = 0; i < 4; ++i)
      if (std::fabs(S(i, i) - std::pow(0.8, (double)i)) > 1e-9) return fail("si_svd values");
    std::printf("si_svd ok S(1,1)=%.12f\n", S(1, 1));
  }
  // mgs / cgs2 (qr.hpp:21-132): columns 3..5 duplicate 0..2 and are skipped; A = QR
  {
    const size_t m = 300, n = 20;
    Matrix<double> A(m, n, Location::kHOST);
    for (size_t j = 0; j < n; ++j)
      for (size_t i = 0; i < m; ++i) A(i, j) = std::sin(0.37 * (double)(i + 1) * (double)(j % 17 + 1) + 0.1 * j);
    for (size_t j = 3; j < 6; ++j)
      for (size_t i = 0; i < m; ++i) A(i, j) = A(i, j - 3);
    A.to_device();
    for (int variant = 0; variant < 2; ++variant) {
      Matrix<double> Q(m, n, Location::kDEVICE), R(n, n, Location::kHOST);
      std::vector<int> skip = variant == 0 ? mgs<double, double, double>(A, Q, R, 1e-12)
                                           : cgs2<double, double, double>(A, Q, R, 1e-12);
      for (size_t j = 0; j < n; ++j)
        if (skip[j] != (j >= 3 && j <= 5 ? 1 : 0)) return fail("gram-schmidt skip pattern");
    }
    std::printf("mgs/cgs2 ok\n");
  }
  // generate_gaussian_kernel (gaussian_kernel.hpp:14-77): symmetric, diagonal f^2 (1 + s^2), entries in
  // [0, f^2]; invalid parameters throw std::invalid_argument
  {
    const double f = 1.5, l = 2.0, s = 0.1;
    Matrix<double> K = generate_gaussian_kernel<double>(f, l, s, 42, 10, 3);
    if (K.rows() != 10 || K.cols() != 10 || K.location() != Location::kHOST) return fail("kernel shape");
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j) {
        if (K(i, j) != K(j, i)) return fail("kernel symmetry");
        if (i == j && K(i, i) != f * f * (1.0 + s * s)) return fail("kernel diagonal");
        if (i != j && !(K(i, j) >= 0.0 && K(i, j) <= f * f)) return fail("kernel range");
      }
    bool threw = false;
    try {
      generate_gaussian_kernel<double>(1.0, 0.0, 0.1, 42, 10, 3);
    } catch (const std::invalid_argument&) {
      threw = true;
    }
    if (!threw) return fail("kernel invalid length scale");
    Matrix<float> Kf = generate_gaussian_kernel<float>(1.0, 1.0, 0.05, 123, 5, 2);
    if (Kf(0, 0) != (float)(1.0 * 1.0 * (1.0 + 0.05 * 0.05))) return fail("float kernel diagonal");
    std::printf("generate_gaussian_kernel ok K(0,1)=%.12f\n", K(0, 1));
  }
  // MatrixReader (matrix_reader.hpp:21-44): a diagonal CSR written to <argv[1]>_*.bin, read back,
  // solved through the CSR overload of si_eig; the _singular_values file holds the spectrum
  if (argc > 1) {
    const std::string prefix = argv[1];
    const int n = 120;
    std::vector<int> ip(n + 1), ix(n);
    std::vector<double> va(n), sv(n);
    for (int i = 0; i < n; ++i) {
      ip[i] = i;
      ix[i] = i;
      va[i] = sv[i] = std::pow(0.7, (double)i);
    }
    ip[n] = n;
    auto put = [&](const char* suffix, const void* p, size_t bytes) {
      FILE* f = std::fopen((prefix + suffix).c_str(), "wb");
      if (!f) return false;
      const bool ok = std::fwrite(p, 1, bytes, f) == bytes;
      std::fclose(f);
      return ok;
    };
    if (!put("_row_ptr.bin", ip.data(), ip.size() * 4) || !put("_col_ind.bin", ix.data(), ix.size() * 4) ||
        !put("_values.bin", va.data(), va.size() * 8) || !put("_singular_values.bin", sv.data(), sv.size() * 8))
      return fail("write csr files");
    CSRMatrix m = MatrixReader::read_csr_matrix(prefix);
    if (m.rows != n || m.cols != n || m.values != va || m.row_ptr != ip) return fail("read_csr_matrix");
    std::vector<double> s = MatrixReader::read_singular_values(prefix);
    if (s != sv) return fail("read_singular_values");
    if (!MatrixReader::read_singular_values(prefix + "_missing").empty()) return fail("missing singular values");
    bool threw = false;
    try {
      MatrixReader::read_csr_matrix(prefix + "_missing");
    } catch (const std::runtime_error&) {
      threw = true;
    }
    if (!threw) return fail("read_csr_matrix on a missing file");
    CsrMatrix<double> A = to_device<double>(m, true);
    Matrix<double> V(n, 12, Location::kDEVICE), D(12, 12, Location::kHOST);
    V.fill_random(42);
    MSVDStatus st = si_eig<double, double, double>(A, V, D, 200, 1e-10, true, 1e-10);
    if (st != MSVDStatus::kSuccess) return fail("si_eig on the file operator");
    for (int i = 0; i < 4; ++i)
      if (std::fabs(D(i, i) - s[i]) > 1e-9) return fail("si_eig values on the file operator");
    std::printf("MatrixReader ok rows=%d nnz=%zu D(0,0)=%.12f\n", m.rows, m.values.size(), D(0, 0));
  }
  CUDAHandler::finalize();
  std::printf("ALL OK\n");
  return 0;
}
