// ref_driver.cc -- thin extern "C" shim (test infrastructure only) around the
// reference's own header-only CPU code, compiled from the reference sources by
// oracle/build_ref.sh into oracle/_ref/.  Used to pin the oracle:
//   BK5::Serial::SumFactorization  CEED_BK/include/kernels/BK5/serial_kernels.hpp:9-85
//   BK1::Serial::SumFactorization  CEED_BK/include/kernels/BK1/serial_kernels.hpp:8-130
//   BK3::Serial::SumFactorization  CEED_BK/include/kernels/BK3/serial_kernels.hpp:9-197
//   LagrangeBasis<T>               sum_factorization/include/math/lagrange_basis.hpp:9-70
#include <cmath>
#include <vector>
#include <kernels/BK1/serial_kernels.hpp>
#include <kernels/BK3/serial_kernels.hpp>
#include <kernels/BK5/serial_kernels.hpp>
#include <math/lagrange_basis.hpp>

extern "C" {

// Reference serial BK5 on caller arrays; returns sum(out^2) as the reference does.
double ref_bk5_serial(unsigned nq, unsigned nelmt, const double* dbasis, const double* G,
                      const double* in, double* out) {
  return BK5::Serial::SumFactorization<double>(nq, nq, nq, nelmt, dbasis, dbasis, dbasis, G, in, out);
}

// The reference serial verification run (CEED_BK/src/BK5/serial_verification.cc:8-47):
// G = 2, in = 3, dbasis[i*nq+a] = cos(i*nq+a); returns the printed norm.
double ref_bk5_serial_verification_norm(unsigned p, unsigned nelmt) {
  const unsigned nq = p + 1, nt = nq * nq * nq;
  std::vector<double> dbasis(nq * nq), G((size_t)nelmt * nt * 6, 2.0), in((size_t)nelmt * nt, 3.0),
      out((size_t)nelmt * nt, 0.0);
  for (unsigned i = 0; i < nq; ++i)
    for (unsigned a = 0; a < nq; ++a) dbasis[i * nq + a] = std::cos((double)(i * nq + a));
  double s = BK5::Serial::SumFactorization<double>(nq, nq, nq, nelmt, dbasis.data(), dbasis.data(),
                                                   dbasis.data(), G.data(), in.data(), out.data());
  return std::sqrt(s);
}

double ref_lagrange_value(unsigned n, const double* nodes, unsigned j, double x) {
  LagrangeBasis<double> b(std::vector<double>(nodes, nodes + n));
  return b(j, x);
}

double ref_lagrange_derivative(unsigned n, const double* nodes, unsigned j, double x) {
  LagrangeBasis<double> b(std::vector<double>(nodes, nodes + n));
  return b.derivative(j, x);
}

// Reference serial BK1 (mass) on caller arrays: nq points, nm = nq - 1 modes,
// basis[q*nm + i], JxW[e][nq^3], in/out [e][nm^3]; returns sum(out^2).
double ref_bk1_serial(unsigned nq, unsigned nelmt, const double* basis, const double* JxW,
                      const double* in, double* out) {
  const unsigned nm = nq - 1;
  std::vector<double> u(in, in + (size_t)nelmt * nm * nm * nm);
  return BK1::Serial::SumFactorization<double>(nq, nq, nq, nelmt, basis, basis, basis, JxW,
                                               u.data(), out);
}

// CEED_BK/src/BK1/serial_verification.cc:6-60: JxW = 1, in = 3,
// basis[q*nm + i] = cos(q*nm + i), nq = p + 2; returns the printed norm.
double ref_bk1_serial_verification_norm(unsigned p, unsigned nelmt) {
  const unsigned nq = p + 2, nm = nq - 1;
  std::vector<double> basis(nq * nm), JxW((size_t)nelmt * nq * nq * nq, 1.0),
      in((size_t)nelmt * nm * nm * nm, 3.0), out((size_t)nelmt * nm * nm * nm, 0.0);
  for (unsigned q = 0; q < nq; ++q)
    for (unsigned i = 0; i < nm; ++i) basis[q * nm + i] = std::cos((double)(q * nm + i));
  return std::sqrt(BK1::Serial::SumFactorization<double>(nq, nq, nq, nelmt, basis.data(),
                                                         basis.data(), basis.data(), JxW.data(),
                                                         in.data(), out.data()));
}

// Reference serial BK3 (Laplacian with interpolation): basis[q*nm + i],
// dbasis[q*nq + n], G[e][p][q][6][r] (the serial kernel's layout); returns sum(out^2).
double ref_bk3_serial(unsigned nq, unsigned nelmt, const double* basis, const double* dbasis,
                      const double* G, const double* in, double* out) {
  const unsigned nm = nq - 1;
  std::vector<double> u(in, in + (size_t)nelmt * nm * nm * nm);
  return BK3::Serial::SumFactorization<double>(nq, nq, nq, nelmt, basis, basis, basis, dbasis,
                                               dbasis, dbasis, G, u.data(), out);
}

// CEED_BK/src/BK3/serial_verification.cc:6-80: G = 2, in = 3, basis = cos(q*nm + i),
// dbasis[i*nq + p] = cos(i*nq + p), nq = p + 2; returns the printed norm.
double ref_bk3_serial_verification_norm(unsigned p, unsigned nelmt) {
  const unsigned nq = p + 2, nm = nq - 1;
  std::vector<double> basis(nq * nm), dbasis(nq * nq), G((size_t)nelmt * nq * nq * nq * 6, 2.0),
      in((size_t)nelmt * nm * nm * nm, 3.0), out((size_t)nelmt * nm * nm * nm, 0.0);
  for (unsigned q = 0; q < nq; ++q)
    for (unsigned i = 0; i < nm; ++i) basis[q * nm + i] = std::cos((double)(q * nm + i));
  for (unsigned i = 0; i < nq; ++i)
    for (unsigned a = 0; a < nq; ++a) dbasis[i * nq + a] = std::cos((double)(i * nq + a));
  return std::sqrt(BK3::Serial::SumFactorization<double>(
      nq, nq, nq, nelmt, basis.data(), basis.data(), basis.data(), dbasis.data(), dbasis.data(),
      dbasis.data(), G.data(), in.data(), out.data()));
}
}
