// host_quadrature.cc -- see host_quadrature.hh.
#include "host_quadrature.hh"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace gbint
{
  namespace
  {
    const long double kPiL = 3.141592653589793238462643383279502884L;

    // Solve (J - shift I) y = rhs in place for the symmetric tridiagonal J (diagonal a, squared
    // off-diagonals b) by Gaussian elimination with partial (row) pivoting.  Row interchanges
    // create one extra super-diagonal (u2).  Exactly singular pivots are replaced by a tiny value,
    // which is what inverse iteration at a converged eigenvalue needs.
    void tridiag_solve_pivoted(const std::vector<long double> &a, const std::vector<long double> &b,
                               long double shift, std::vector<long double> &rhs)
    {
      const int n = (int)a.size();
      if (n == 1) {
        const long double d0 = a[0] - shift;
        rhs[0] /= (d0 == 0 ? 1e-300L : d0);
        return;
      }
      std::vector<long double> d(n), lo(n, 0), u1(n, 0), u2(n, 0);
      for (int j = 0; j < n; ++j) d[j] = a[j] - shift;
      for (int j = 0; j + 1 < n; ++j) lo[j] = u1[j] = std::sqrt(b[j]);
      const long double tiny = 1e-300L;
      for (int j = 0; j + 1 < n; ++j) {
        if (std::fabs(d[j]) >= std::fabs(lo[j])) {
          if (d[j] == 0) d[j] = tiny;
          const long double f = lo[j] / d[j];
          d[j + 1] -= f * u1[j];
          rhs[j + 1] -= f * rhs[j];
          u2[j] = 0;
        } else {
          // swap rows j and j+1, then eliminate
          const long double f = d[j] / lo[j];
          d[j] = lo[j];
          const long double t = d[j + 1];
          d[j + 1] = u1[j] - f * t;
          if (j + 2 < n) {
            u2[j] = u1[j + 1];
            u1[j + 1] = -f * u2[j];
          }
          u1[j] = t;
          const long double r = rhs[j];
          rhs[j] = rhs[j + 1];
          rhs[j + 1] = r - f * rhs[j + 1];
        }
      }
      if (d[n - 1] == 0) d[n - 1] = tiny;
      rhs[n - 1] /= d[n - 1];
      rhs[n - 2] = (rhs[n - 2] - u1[n - 2] * rhs[n - 1]) / d[n - 2];
      for (int j = n - 3; j >= 0; --j) rhs[j] = (rhs[j] - u1[j] * rhs[j + 1] - u2[j] * rhs[j + 2]) / d[j];
    }

    // number of eigenvalues of the Jacobi matrix below lambda (Sturm count of the LDL^T pivots)
    int sturm_count(const std::vector<long double> &a, const std::vector<long double> &b, long double lambda)
    {
      const int n = (int)a.size();
      int cnt = 0;
      long double d = 1;
      for (int i = 0; i < n; ++i) {
        const long double off = i > 0 ? b[i - 1] : 0.0L;
        d = (a[i] - lambda) - (i > 0 ? off / d : 0.0L);
        if (d == 0) d = -1e-300L;
        if (d < 0) ++cnt;
      }
      return cnt;
    }
  } // namespace

  void jacobi_gauss(const std::vector<long double> &a, const std::vector<long double> &b, long double mu0,
                    std::vector<long double> &x, std::vector<long double> &w)
  {
    const int n = (int)a.size();
    if ((int)b.size() != n) throw std::invalid_argument("jacobi_gauss: size mismatch");
    x.assign(n, 0);
    w.assign(n, 0);
    // Gershgorin interval
    long double lo = a[0], hi = a[0];
    for (int i = 0; i < n; ++i) {
      long double r = 0;
      if (i > 0) r += std::sqrt(b[i - 1]);
      if (i + 1 < n) r += std::sqrt(b[i]);
      lo = std::min(lo, a[i] - r);
      hi = std::max(hi, a[i] + r);
    }
    for (int k = 0; k < n; ++k) {
      long double l = lo, h = hi;
      for (int it = 0; it < 200; ++it) {
        const long double m = (l + h) / 2;
        if (m == l || m == h) break;
        if (sturm_count(a, b, m) > k)
          h = m;
        else
          l = m;
      }
      const long double lam = (l + h) / 2;
      x[k] = lam;
      // weight = mu0 * (first component of the normalised eigenvector)^2; the eigenvector comes
      // from two steps of inverse iteration with a pivoted tridiagonal solve (the forward
      // three-term recurrence is unstable for the decaying components of this rule)
      const long double shift = lam + (std::fabs(lam) + 1e-30L) * 64 * std::numeric_limits<long double>::epsilon();
      std::vector<long double> v(n, 1.0L);
      for (int it = 0; it < 3; ++it) {
        tridiag_solve_pivoted(a, b, shift, v);
        long double nrm = 0;
        for (int j = 0; j < n; ++j) nrm += v[j] * v[j];
        nrm = std::sqrt(nrm);
        for (int j = 0; j < n; ++j) v[j] /= nrm;
      }
      w[k] = mu0 * v[0] * v[0];
    }
  }

  void fixed_rule(int type, int n, std::vector<double> &x, std::vector<double> &w)
  {
    if (n <= 0) throw std::invalid_argument("quadrature order must be positive");
    switch (type) {
    case RULE_LEGENDRE:
    case RULE_JACOBI:
      gl_rule01(n, x, w);
      return;
    case RULE_CHEBYSHEV:
      // x_i = (1 - cos t_i) / 2 = sin^2(t_i / 2), t_i = (2i+1) pi / (2n); every weight pi / n
      x.resize(n);
      w.assign(n, (double)(kPiL / n));
      for (int i = 0; i < n; ++i) {
        const long double s = std::sin(kPiL * (2 * i + 1) / (4 * n));
        x[i] = (double)(s * s);
      }
      return;
    case RULE_LAGUERRE:
    case RULE_HERMITE: {
      // nodes: eigenvalues of the Jacobi matrix of the monic recurrence (Laguerre a_j = 2j+1,
      // b_j = j^2; Hermite a_j = 0, b_j = j/2), by Sturm bisection.  Weights: the Christoffel
      // function 1 / sum_(k<n) p_k(x_i)^2 of the orthonormal polynomials (Laguerre: L_k itself;
      // Hermite: H_k / sqrt(2^k k! sqrt(pi))), run forward at each node, where they are the
      // growing solution; the tail weights (down to ~1e-170 at n = 100) keep full relative
      // precision, which an eigenvector's first component from inverse iteration does not.
      // Sums beyond the long double range give weight 0 (the true weight is below FP64's).
      std::vector<long double> a(n), b(n, 0.0L), xs, ws;
      for (int j = 0; j < n; ++j) {
        const long double j1 = j + 1;
        a[j] = type == RULE_LAGUERRE ? 2.0L * j + 1 : 0.0L;
        b[j] = type == RULE_LAGUERRE ? j1 * j1 : j1 / 2;
      }
      jacobi_gauss(a, b, type == RULE_LAGUERRE ? 1.0L : std::sqrt(kPiL), xs, ws);
      if (type == RULE_HERMITE && n % 2 == 1) xs[n / 2] = 0.0L;
      x.resize(n);
      w.resize(n);
      const long double h0 = 1.0L / std::sqrt(std::sqrt(kPiL));
      for (int i = 0; i < n; ++i) {
        const long double z = xs[i];
        long double pm = 0.0L, p = type == RULE_LAGUERRE ? 1.0L : h0, sum = p * p;
        for (int k = 0; k + 1 < n; ++k) {
          const long double pn = type == RULE_LAGUERRE
                                     ? ((2 * k + 1 - z) * p - k * pm) / (k + 1)
                                     : std::sqrt(2.0L / (k + 1)) * z * p - std::sqrt((long double)k / (k + 1)) * pm;
          pm = p;
          p = pn;
          sum += p * p;
        }
        x[i] = (double)z;
        w[i] = (double)(1.0L / sum);
      }
      return;
    }
    default:
      throw std::invalid_argument("Unknown quadrature type");
    }
  }

  MatsRule matsubara_rule(double T, double E, int step, int min_size, int max_size, int vacuum_quad_size,
                          int precision_factor)
  {
    MatsRule r;
    if (precision_factor < 0) precision_factor = 1;
    if (vacuum_quad_size <= 6) vacuum_quad_size = 6;
    const bool T_zero = std::fabs(T) <= 1e-12;
    const double rel = std::fabs(E) / std::fabs(T + 1e-16);
    if (T_zero || rel > 1e2) {
      // vacuum: GL split into a linear part on [0, 2|E|] and a log part on [2|E|, 1e6 |E|]
      int m = vacuum_quad_size;
      if (m % 2) ++m;
      const double Ee = std::fabs(E) <= 1e-300 ? 1.0 : std::fabs(E);
      std::vector<double> gx, gw;
      gl_rule01(m / 2, gx, gw);
      r.T_rule = 0;
      r.x.resize(m);
      r.w.resize(m);
      const long double div = 2.0L * Ee, ext = 1e6L * Ee;
      const long double ls = std::log(div), le = std::log(ext / div);
      const double tp = 2.0 * (double)kPiL;
      for (int i = 0; i < m / 2; ++i) {
        r.x[i] = gx[i] * (double)div;
        r.w[i] = gw[i] * (double)div / tp;
        const double xv = (double)std::exp(ls + le * (long double)gx[i]);
        r.x[i + m / 2] = xv;
        r.w[i + m / 2] = gw[i] * (double)le * xv / tp;
      }
      return r;
    }
    const double E_max = (precision_factor + 100) * std::fabs(E);
    int m = 5 + int(std::sqrt(4 * E_max / ((double)(kPiL * kPiL) * std::fabs(T))));
    m = (int)std::ceil(m / (double)step) * step;
    m = std::max(min_size, std::min(max_size, m));
    std::vector<long double> a(m), b(m), xs, ws;
    for (int j = 0; j < m; ++j) {
      const long double j1 = j + 1;
      a[j] = 2 * kPiL * kPiL / ((4 * j + 1) * (long double)(4 * j + 5));
      b[j] = kPiL * kPiL * kPiL * kPiL / ((4 * j1 - 1) * (4 * j1 + 3)) / ((4 * j1 + 1) * (4 * j1 + 1));
    }
    a[0] = kPiL * kPiL / 15;
    jacobi_gauss(a, b, kPiL * kPiL / 6, xs, ws);
    r.T_rule = T;
    r.x.resize(m);
    r.w.resize(m);
    for (int i = 0; i < m; ++i) {
      r.w[i] = (double)((long double)T * ws[i] / xs[i]);
      r.x[i] = (double)(2 * kPiL * (long double)T / std::sqrt(xs[i]));
    }
    return r;
  }
} // namespace gbint
