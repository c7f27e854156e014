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
  // The rules of the reference's QuadratureType (common/quadrature/quadrature.hh:47), as its
  // Quadrature<NT>::reinit takes them from GSL's fixed types with a = 0, b = 1, alpha = beta = 0
  // (quadrature.cu:12-60): Legendre on [0,1]; Chebyshev (first kind) on [0,1], weight
  // 1/sqrt(x (1-x)); Laguerre on [0,inf), weight exp(-x); Hermite on the real line, weight
  // exp(-x^2); Jacobi(0,0) on [0,1] (the Legendre rule).  Nodes ascending.
  enum RuleType : int { RULE_LEGENDRE = 0, RULE_CHEBYSHEV = 1, RULE_LAGUERRE = 2, RULE_HERMITE = 3, RULE_JACOBI = 4 };
  void fixed_rule(int type, int n, std::vector<double> &x, std::vector<double> &w);

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
