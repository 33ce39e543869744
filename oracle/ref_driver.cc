// ref_driver.cc -- thin extern "C" shim (test infrastructure only) around the
// reference's own header-only CPU code, compiled from the reference sources by
// oracle/build_ref.sh into oracle/_ref/.  Used to pin the oracle:
//   BK5::Serial::SumFactorization  CEED_BK/include/kernels/BK5/serial_kernels.hpp:9-85
//   LagrangeBasis<T>               sum_factorization/include/math/lagrange_basis.hpp:9-70
#include <cmath>
#include <vector>
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
}
