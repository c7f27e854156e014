// gl_rule.hh -- the n-point Gauss-Legendre rule on [0,1] (nodes ascending, weights summing to 1),
// header-only host code shared by libgbint's quadrature pool and by the host loop integrals of
// gbint/loop_integrals.hh.
//
// The reference takes this rule from GSL's fixed Legendre type
// (DiFfRG/src/DiFfRG/common/quadrature/quadrature.cu:12-60) and, for its CPU loop integrals,
// from deal.II's QGauss<1> (DiFfRG/include/DiFfRG/physics/loop_integrals.hh:35-39); both are
// the same rule to the rounding of their last step.  Here: Newton's method on P_n in long
// double with the Bonnet three-term recurrence, started from the asymptotic root estimate
// cos(pi (4i+3) / (4n+2)); weight 1 / ((1 - z^2) P_n'(z)^2), halved for [0,1].
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <thread>
#include <vector>

namespace gbint
{
  namespace gl_detail
  {
    constexpr long double kPiL = 3.141592653589793238462643383279502884L;

    // P_n(z) and P_{n-1}(z) by the Bonnet recurrence
    inline void legendre_pair(int n, long double z, long double &pn, long double &pn1)
    {
      long double p0 = 1, p1 = z;
      if (n == 0) {
        pn = 1;
        pn1 = 0;
        return;
      }
      for (int j = 2; j <= n; ++j) {
        const long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      pn = p1;
      pn1 = p0;
    }

    // the i-th largest root of P_n and its weight on [0,1], into both mirrored slots
    inline void gl_root(int n, int i, double *x, double *w)
    {
      // initial guess from the asymptotic formula
      long double z = std::cos(kPiL * (4 * i + 3) / (4 * n + 2));
      long double pn = 0, pn1 = 0;
      for (int it = 0; it < 64; ++it) {
        legendre_pair(n, z, pn, pn1);
        const long double dp = n * (pn1 - z * pn) / (1 - z * z);
        const long double step = pn / dp;
        z -= step;
        if (std::fabs(step) <= 4 * std::numeric_limits<long double>::epsilon()) break;
      }
      legendre_pair(n, z, pn, pn1);
      const long double dp = n * (pn1 - z * pn) / (1 - z * z);
      const long double wt = 1 / ((1 - z * z) * dp * dp);  // weight on [0,1] = half of [-1,1]'s
      x[n - 1 - i] = (double)((1 + z) / 2);
      x[i] = (double)((1 - z) / 2);
      w[n - 1 - i] = (double)wt;
      w[i] = (double)wt;
    }
  } // namespace gl_detail

  // Each root costs O(n) per Newton step, a rule O(n^2): rules of 512 points and more spread
  // their roots over the host's threads (every root is computed alone, so the result does not
  // depend on the split).
  inline void gl_rule01(int n, std::vector<double> &x, std::vector<double> &w)
  {
    if (n <= 0) throw std::invalid_argument("Gauss-Legendre order must be positive");
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const int half = (n + 1) / 2;
    const unsigned hw = std::thread::hardware_concurrency();
    const int T = n >= 512 ? (int)std::min<unsigned>(hw ? hw : 1u, (unsigned)(half / 64)) : 1;
    if (T <= 1) {
      for (int i = 0; i < half; ++i) gl_detail::gl_root(n, i, x.data(), w.data());
    } else {
      std::vector<std::thread> pool;
      pool.reserve(T);
      for (int t = 0; t < T; ++t)
        pool.emplace_back([&, t] {
          for (int i = t; i < half; i += T) gl_detail::gl_root(n, i, x.data(), w.data());
        });
      for (auto &th : pool) th.join();
    }
    if (n % 2 == 1) x[n / 2] = 0.5;
  }
} // namespace gbint
