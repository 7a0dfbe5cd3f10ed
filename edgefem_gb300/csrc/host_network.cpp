// Network-parameter post-processing of S matrices and the Touchstone writer:
// the host-side consumers of a sweep's output (include/edgefem/coupling.hpp,
// include/edgefem/io/touchstone.hpp).  Matrices are at most 99 x 99, so
// everything here is plain host code: a cyclic Jacobi eigensolver for the
// singular values, Gaussian elimination with complete pivoting for the
// rank test and the inverses.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>

#include "edgefem.hpp"

namespace edgefem {

namespace {

constexpr double kPi = 3.14159265358979323846;

std::size_t square_size(const MatC &S) {
  const std::size_t n = S.size();
  for (const auto &row : S)
    if (row.size() != n) throw std::runtime_error("S-matrix must be square");
  return n;
}

MatC identity(std::size_t n) {
  MatC I(n, VecC(n, 0.0));
  for (std::size_t i = 0; i < n; ++i) I[i][i] = 1.0;
  return I;
}

MatC matmul(const MatC &A, const MatC &B) {
  const std::size_t n = A.size(), m = B.empty() ? 0 : B[0].size(), k = B.size();
  MatC C(n, VecC(m, 0.0));
  for (std::size_t i = 0; i < n; ++i)
    for (std::size_t l = 0; l < k; ++l)
      for (std::size_t j = 0; j < m; ++j) C[i][j] += A[i][l] * B[l][j];
  return C;
}

double frobenius(const MatC &A) {
  double s = 0;
  for (const auto &row : A)
    for (const auto &v : row) s += std::norm(v);
  return std::sqrt(s);
}

// ||A - B||_F <= tol * min(||A||_F, ||B||_F): the relative comparison of
// Eigen's isApprox, which is_lossless and is_reciprocal use
// (src/coupling.cpp:116-136).
bool approx_equal(const MatC &A, const MatC &B, double tol) {
  MatC D = A;
  for (std::size_t i = 0; i < D.size(); ++i)
    for (std::size_t j = 0; j < D[i].size(); ++j) D[i][j] -= B[i][j];
  return frobenius(D) <= tol * std::min(frobenius(A), frobenius(B));
}

// Gauss-Jordan inversion with complete pivoting.  Returns the numerical rank
// (pivots above n * eps * the largest pivot); `inv` is valid only at full rank.
std::size_t invert(MatC A, MatC &inv) {
  const std::size_t n = A.size();
  inv = identity(n);
  std::vector<std::size_t> colperm(n);
  for (std::size_t i = 0; i < n; ++i) colperm[i] = i;
  double first = 0;
  std::size_t rank = 0;
  for (std::size_t k = 0; k < n; ++k) {
    std::size_t pr = k, pc = k;
    double best = -1;
    for (std::size_t i = k; i < n; ++i)
      for (std::size_t j = k; j < n; ++j)
        if (std::abs(A[i][j]) > best) best = std::abs(A[i][j]), pr = i, pc = j;
    if (k == 0) first = best;
    if (!(best > first * std::numeric_limits<double>::epsilon() * static_cast<double>(n)) || best == 0) break;
    ++rank;
    std::swap(A[k], A[pr]);
    std::swap(inv[k], inv[pr]);
    if (pc != k) {
      for (std::size_t i = 0; i < n; ++i) std::swap(A[i][k], A[i][pc]);
      std::swap(colperm[k], colperm[pc]);
    }
    const cplx d = 1.0 / A[k][k];
    for (std::size_t j = 0; j < n; ++j) A[k][j] *= d, inv[k][j] *= d;
    for (std::size_t i = 0; i < n; ++i) {
      if (i == k || A[i][k] == cplx(0.0)) continue;
      const cplx f = A[i][k];
      for (std::size_t j = 0; j < n; ++j) A[i][j] -= f * A[k][j], inv[i][j] -= f * inv[k][j];
    }
  }
  if (rank == n) {
    // A P = I' after elimination: the rows of inv belong to permuted columns.
    MatC out(n, VecC(n));
    for (std::size_t k = 0; k < n; ++k) out[colperm[k]] = inv[k];
    inv = out;
  }
  return rank;
}

MatC inverse_or_regularised(const MatC &A) {
  MatC inv;
  if (invert(A, inv) == A.size()) return inv;
  // Singular: (A + 1e-12 I)^-1, as src/coupling.cpp:30-35 does.
  MatC R = A;
  for (std::size_t i = 0; i < R.size(); ++i) R[i][i] += 1e-12;
  if (invert(R, inv) != R.size()) throw std::runtime_error("matrix is singular after regularisation");
  return inv;
}

// Eigenvalues of a Hermitian matrix by cyclic Jacobi rotations (two-sided,
// complex Givens rotations that zero one off-diagonal pair at a time).
std::vector<double> hermitian_eigenvalues(MatC H) {
  const std::size_t n = H.size();
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, diag = 0;
    for (std::size_t i = 0; i < n; ++i)
      for (std::size_t j = 0; j < n; ++j) (i == j ? diag : off) += std::norm(H[i][j]);
    if (off <= 1e-30 * diag || off == 0) break;
    for (std::size_t p = 0; p + 1 < n; ++p)
      for (std::size_t q = p + 1; q < n; ++q) {
        const double a = std::abs(H[p][q]);
        if (a == 0) continue;
        const cplx ph = H[p][q] / a;  // H[p][q] = a e^{j phi}
        const double app = H[p][p].real(), aqq = H[q][q].real();
        const double theta = 0.5 * std::atan2(2 * a, aqq - app);
        const double c = std::cos(theta), s = std::sin(theta);
        // columns: p' = c p - s conj(ph) q, q' = s ph p + c q (unitary J)
        for (std::size_t k = 0; k < n; ++k) {
          const cplx hp = H[k][p], hq = H[k][q];
          H[k][p] = c * hp - s * std::conj(ph) * hq;
          H[k][q] = s * ph * hp + c * hq;
        }
        for (std::size_t k = 0; k < n; ++k) {
          const cplx hp = H[p][k], hq = H[q][k];
          H[p][k] = c * hp - s * ph * hq;
          H[q][k] = s * std::conj(ph) * hp + c * hq;
        }
        H[p][q] = H[q][p] = 0.0;
      }
  }
  std::vector<double> ev(n);
  for (std::size_t i = 0; i < n; ++i) ev[i] = H[i][i].real();
  std::sort(ev.begin(), ev.end(), [](double x, double y) { return x > y; });
  return ev;
}

void write_value(std::ostream &os, cplx v, TouchstoneFormat fmt) {
  // src/io/touchstone.cpp:26-44
  switch (fmt) {
    case TouchstoneFormat::RI:
      os << v.real() << ' ' << v.imag();
      break;
    case TouchstoneFormat::MA:
      os << std::abs(v) << ' ' << std::arg(v) * 180.0 / kPi;
      break;
    case TouchstoneFormat::DB:
      os << 20.0 * std::log10(std::max(std::abs(v), 1e-20)) << ' ' << std::arg(v) * 180.0 / kPi;
      break;
  }
}

const char *format_name(TouchstoneFormat fmt) {
  switch (fmt) {
    case TouchstoneFormat::MA: return "MA";
    case TouchstoneFormat::DB: return "DB";
    default: return "RI";
  }
}

}  // namespace

std::vector<double> singular_values(const MatC &S) {
  const std::size_t n = square_size(S);
  MatC H(n, VecC(n, 0.0));  // S^H S
  for (std::size_t i = 0; i < n; ++i)
    for (std::size_t j = 0; j < n; ++j)
      for (std::size_t k = 0; k < n; ++k) H[i][j] += std::conj(S[k][i]) * S[k][j];
  std::vector<double> ev = hermitian_eigenvalues(H);
  for (auto &v : ev) v = std::sqrt(std::max(v, 0.0));
  return ev;
}

CouplingMatrix compute_coupling(const MatC &S, double freq, double z0) {
  // src/coupling.cpp:9-50: Z = z0 (I + S)(I - S)^-1, Y = (I - S)(I + S)^-1 / z0.
  const std::size_t n = square_size(S);
  CouplingMatrix cm;
  cm.S = S;
  cm.frequency = freq;
  cm.z0 = z0;
  cm.num_ports = static_cast<int>(n);
  MatC Ip = identity(n), Im = identity(n);
  for (std::size_t i = 0; i < n; ++i)
    for (std::size_t j = 0; j < n; ++j) Ip[i][j] += S[i][j], Im[i][j] -= S[i][j];
  cm.Z = matmul(Ip, inverse_or_regularised(Im));
  for (auto &row : cm.Z)
    for (auto &v : row) v *= z0;
  cm.Y = matmul(Im, inverse_or_regularised(Ip));
  for (auto &row : cm.Y)
    for (auto &v : row) v /= z0;
  return cm;
}

std::vector<std::vector<double>> mutual_coupling_db(const CouplingMatrix &cm) {
  // src/coupling.cpp:52-65
  const std::size_t n = static_cast<std::size_t>(cm.num_ports);
  std::vector<std::vector<double>> out(n, std::vector<double>(n));
  for (std::size_t i = 0; i < n; ++i)
    for (std::size_t j = 0; j < n; ++j) out[i][j] = 20.0 * std::log10(std::max(std::abs(cm.S[i][j]), 1e-20));
  return out;
}

VecC active_reflection(const MatC &S, const VecC &excitation) {
  // src/coupling.cpp:67-94: (S a)_i / a_i, 0 where port i is not excited.
  const std::size_t n = square_size(S);
  if (excitation.size() != n) throw std::runtime_error("Excitation vector size must match S-matrix dimension");
  VecC g(n, 0.0);
  for (std::size_t i = 0; i < n; ++i) {
    cplx acc = 0.0;
    for (std::size_t j = 0; j < n; ++j) acc += S[i][j] * excitation[j];
    g[i] = std::abs(excitation[i]) < 1e-20 ? cplx(0.0) : acc / excitation[i];
  }
  return g;
}

bool is_passive(const MatC &S, double tol) {
  // src/coupling.cpp:96-112
  for (const auto &row : S)
    if (row.size() != S.size()) return false;
  if (S.empty()) return true;
  return singular_values(S)[0] <= 1.0 + tol;
}

bool is_lossless(const MatC &S, double tol) {
  // src/coupling.cpp:114-126: S^H S approximately I.
  for (const auto &row : S)
    if (row.size() != S.size()) return false;
  const std::size_t n = S.size();
  MatC H(n, VecC(n, 0.0));
  for (std::size_t i = 0; i < n; ++i)
    for (std::size_t j = 0; j < n; ++j)
      for (std::size_t k = 0; k < n; ++k) H[i][j] += std::conj(S[k][i]) * S[k][j];
  return approx_equal(H, identity(n), tol);
}

bool is_reciprocal(const MatC &S, double tol) {
  // src/coupling.cpp:128-136: S approximately S^T.
  for (const auto &row : S)
    if (row.size() != S.size()) return false;
  MatC T = S;
  for (std::size_t i = 0; i < S.size(); ++i)
    for (std::size_t j = 0; j < S.size(); ++j) T[i][j] = S[j][i];
  return approx_equal(S, T, tol);
}

bool check_passivity(const MatC &S, double tol) {
  // pyedgefem.cpp:701-730: is_passive plus a warning with the largest
  // singular value (and the two column power sums of a 2-port).
  if (is_passive(S, tol)) return true;
  std::ostringstream oss;
  const double smax = S.size() == square_size(S) && !S.empty() ? singular_values(S)[0] : 0.0;
  oss << "WARNING: S-parameters violate passivity! Max singular value = " << smax << " (should be <= "
      << (1.0 + tol) << ")\n";
  if (S.size() == 2) {
    const double s11 = std::abs(S[0][0]), s21 = std::abs(S[1][0]), s12 = std::abs(S[0][1]),
                 s22 = std::abs(S[1][1]);
    oss << "  |S11|=" << s11 << ", |S21|=" << s21 << ", |S11|^2+|S21|^2=" << s11 * s11 + s21 * s21 << "\n";
    oss << "  |S12|=" << s12 << ", |S22|=" << s22 << ", |S12|^2+|S22|^2=" << s12 * s12 + s22 * s22 << "\n";
  }
  std::cerr << oss.str();
  return false;
}

void write_touchstone(const std::string &path, const std::vector<double> &freq, const std::vector<SParams2> &data) {
  // src/io/touchstone.cpp:48-60 (2-port legacy form, always RI, 50 ohm)
  if (data.size() < freq.size()) throw std::runtime_error("Frequency and S-parameter count mismatch");
  std::ofstream ofs(path);
  if (!ofs) throw std::runtime_error("Cannot open file for writing: " + path);
  ofs << "# Hz S RI R 50\n" << std::setprecision(12);
  for (std::size_t i = 0; i < freq.size(); ++i) {
    const SParams2 &s = data[i];
    ofs << freq[i];
    for (cplx v : {s.s11, s.s21, s.s12, s.s22}) ofs << ' ' << v.real() << ' ' << v.imag();
    ofs << '\n';
  }
}

void write_touchstone_nport(const std::string &path, const std::vector<double> &freq,
                            const std::vector<MatC> &S_matrices, const TouchstoneOptions &opts) {
  // src/io/touchstone.cpp:64-139: two comment lines, the option line, then
  // per frequency the matrix row by row; above 2 ports a line holds at most
  // 4 complex values, continuation lines carry no frequency.
  if (freq.empty() || S_matrices.empty()) throw std::runtime_error("Empty frequency or S-parameter data");
  const std::size_t np = S_matrices[0].size();
  if (np < 1 || np > 99) throw std::runtime_error("Invalid number of ports: " + std::to_string(np));
  for (std::size_t f = 0; f < S_matrices.size(); ++f) {
    bool ok = S_matrices[f].size() == np;
    for (const auto &row : S_matrices[f]) ok = ok && row.size() == np;
    if (!ok) throw std::runtime_error("S-matrix dimension mismatch at frequency " + std::to_string(f));
  }
  if (freq.size() != S_matrices.size()) throw std::runtime_error("Frequency and S-matrix count mismatch");
  std::ofstream ofs(path);
  if (!ofs) throw std::runtime_error("Cannot open file for writing: " + path);
  ofs << std::setprecision(12);
  ofs << "! Touchstone file generated by EdgeFEM\n! Number of ports: " << np << "\n";
  ofs << "# Hz S " << format_name(opts.format) << " R " << opts.z0 << "\n";
  for (std::size_t f = 0; f < freq.size(); ++f) {
    ofs << freq[f];
    std::size_t count = 0;
    for (std::size_t i = 0; i < np; ++i)
      for (std::size_t j = 0; j < np; ++j) {
        if (np > 2 && count > 0 && count % 4 == 0) ofs << '\n';
        ofs << ' ';
        write_value(ofs, S_matrices[f][i][j], opts.format);
        ++count;
      }
    ofs << '\n';
  }
}

std::string touchstone_extension(int num_ports) {
  // src/io/touchstone.cpp:141-149
  if (num_ports < 1 || num_ports > 99) throw std::runtime_error("Invalid number of ports: " + std::to_string(num_ports));
  return ".s" + std::to_string(num_ports) + "p";
}

}  // namespace edgefem
