// host_quadrature.hh -- quadrature rules of the engine (host, long double).
//
//   * Gauss-Legendre on [0,1]: gl_rule01 of gbint/gl_rule.hh (header-only, shared with the host
//     loop integrals), the rule the reference takes from GSL's fixed Legendre type
//     (DiFfRG/src/DiFfRG/common/quadrature/quadrature.cu:12-60).
//   * Gauss rules from a Jacobi matrix (DiFfRG/include/DiFfRG/common/quadrature/quadrature.hh:28-45):
//     eigenvalues by Sturm-sequence bisection, weights from the Christoffel function
//     w_i = mu0 / sum_k p_k(x_i)^2 of the orthonormal recurrence polynomials.
//   * Monien's bosonic Matsubara rule (DiFfRG/src/DiFfRG/common/quadrature/matsubara.cu:12-161),
//     including the size prediction and the T=0 / E >> T vacuum fallback.
#pragma once

#include <vector>

#include "gbint/gl_rule.hh"

namespace gbint
{
  // a: diagonal (n), b: squared off-diagonals (b[i] couples i and i+1; n entries, last unused)
  void jacobi_gauss(const std::vector<long double> &a, const std::vector<long double> &b, long double mu0,
                    std::vector<long double> &x, std::vector<long double> &w);

  struct MatsRule {
    double T_rule = 0;  // 0 for the vacuum (T = 0) rule
    std::vector<double> x, w;
  };
  // MatsubaraQuadrature(T, E, step, min_size, max_size, vacuum_quad_size, precision_factor)
  MatsRule matsubara_rule(double T, double E, int step, int min_size, int max_size, int vacuum_quad_size,
                          int precision_factor);
} // namespace gbint
