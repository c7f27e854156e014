// oracle.hh -- TEST INFRASTRUCTURE ONLY.
//
// A plain FP64 CPU restatement of DiFfRG's momentum-loop integrators (the TBB twins),
// its quadrature rules and the benchmark integrands.  It is the checker for the CUDA
// engine in diffrg_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline load it.  Nothing in the product links or calls it.
//
// Parity anchors (paths relative to the DiFfRG project root):
//   * Gauss-Legendre on [0,1]: DiFfRG/src/DiFfRG/common/quadrature/quadrature.cu:12-60
//     (GSL 2.5 gsl_integration_fixed_legendre); pinned against the constexpr tables of
//     DiFfRG/include/DiFfRG/common/quadrature/gauss_legendre.hh (tests/golden/gl_tables.json).
//   * Golub-Welsch from a Jacobi matrix: DiFfRG/include/DiFfRG/common/quadrature/quadrature.hh:28-45
//     with the implicit-QL eigen solver of .../diagonalization.hh:35-145.
//   * Monien bosonic Matsubara rule: DiFfRG/src/DiFfRG/common/quadrature/matsubara.cu:12-161,
//     cache semantics of DiFfRG/src/DiFfRG/common/quadrature/quadrature_provider.cu:12-58.
//   * Integrator families: DiFfRG/include/DiFfRG/physics/integration/*_cpu.hh and
//     DiFfRG/include/DiFfRG/physics/integration_finiteT/*_cpu.hh (cited per function below).
//
// Accumulation is FP64 with a pairwise (blocked) sum so that the oracle's own rounding
// stays far below the 1e-9 tolerances it is used to check.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>

namespace oracle
{
  constexpr double kPi = 3.14159265358979323846264338327950288;

  // ---------------------------------------------------------------------------------------
  // Quadrature rules
  // ---------------------------------------------------------------------------------------

  // Gauss-Legendre nodes/weights on [0,1] by Newton iteration on P_n in long double.
  // Same rule as GSL's fixed Legendre type used by quadrature.cu:45 (nodes ascending).
  inline void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w)
  {
    if (n <= 0) throw std::invalid_argument("gauss_legendre01: order must be positive");
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 0; i < (n + 1) / 2; ++i) {
      // root i of P_n counted from +1 downwards (Tricomi initial guess)
      long double z = std::cos(pi * (i + 0.75L) / (n + 0.5L));
      long double dp = 0;
      for (int it = 0; it < 100; ++it) {
        long double p0 = 1, p1 = z;
        for (int j = 2; j <= n; ++j) {
          long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
          p0 = p1;
          p1 = p2;
        }
        if (n == 1) { p1 = z; p0 = 1; }
        dp = n * (z * p1 - p0) / (z * z - 1);
        const long double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-19L) break;
      }
      // recompute derivative at the converged root
      long double p0 = 1, p1 = z;
      for (int j = 2; j <= n; ++j) {
        long double p2 = ((2 * j - 1) * z * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      dp = (n == 1) ? 1.0L : n * (z * p1 - p0) / (z * z - 1);
      const long double wt = 2 / ((1 - z * z) * dp * dp);
      // map [-1,1] -> [0,1]; ascending order
      x[n - 1 - i] = (double)((1 + z) / 2);
      x[i] = (double)((1 - z) / 2);
      w[n - 1 - i] = (double)(wt / 2);
      w[i] = (double)(wt / 2);
    }
    if (n % 2 == 1) x[n / 2] = 0.5;
  }

  // Symmetric tridiagonal eigen-decomposition by implicit QL with Wilkinson-style shifts,
  // returning eigenvalues ascending and the first component of each normalised eigenvector
  // (all Golub-Welsch needs).  Restates the role of diagonalization.hh:35-145; written from
  // the textbook algorithm (Golub & Van Loan 8.3), accumulating only row 0 of Q.
  template <typename T>
  void tridiag_eig_first_components(std::vector<T> &d, std::vector<T> e_in, std::vector<T> &z0)
  {
    const int n = (int)d.size();
    std::vector<T> e(n, T(0));
    for (int i = 0; i + 1 < n; ++i) e[i] = e_in[i];
    z0.assign(n, T(0));
    z0[0] = 1;
    const T eps = std::numeric_limits<T>::epsilon();
    for (int l = 0; l < n; ++l) {
      int iter = 0;
      for (;;) {
        int m = l;
        for (; m < n - 1; ++m) {
          const T dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
          if (std::fabs(e[m]) <= eps * dd) break;
        }
        if (m == l) break;
        if (++iter > 60) throw std::runtime_error("tridiag_eig: no convergence");
        T g = (d[l + 1] - d[l]) / (2 * e[l]);
        T r = std::hypot(g, T(1));
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
        T s = 1, c = 1, p = 0;
        int i = m - 1;
        for (; i >= l; --i) {
          T f = s * e[i];
          const T b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0) {
            d[i + 1] -= p;
            e[m] = 0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          // rotate the first row of the eigenvector matrix
          f = z0[i + 1];
          z0[i + 1] = s * z0[i] + c * f;
          z0[i] = c * z0[i] - s * f;
        }
        if (r == 0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0;
      }
    }
    // sort ascending, carrying z0
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
    std::vector<T> ds(n), zs(n);
    for (int i = 0; i < n; ++i) {
      ds[i] = d[idx[i]];
      zs[i] = z0[idx[i]];
    }
    d = ds;
    z0 = zs;
  }

  // Golub-Welsch: nodes = eigenvalues of the Jacobi matrix (diag a, off-diag sqrt(b)),
  // weights = mu0 * (first eigenvector component)^2.  Semantics of quadrature.hh:28-45
  // (b[i] holds the squared off-diagonal coupling between i and i+1).
  template <typename T>
  void golub_welsch(const std::vector<T> &a, const std::vector<T> &b, T mu0, std::vector<T> &x, std::vector<T> &w)
  {
    const size_t n = a.size();
    if (b.size() != n) throw std::invalid_argument("golub_welsch: size mismatch");
    std::vector<T> d(a), e(n, T(0)), z0;
    for (size_t i = 0; i + 1 < n; ++i) e[i] = std::sqrt(b[i]);
    if (n == 1) {
      x = {a[0]};
      w = {mu0};
      return;
    }
    tridiag_eig_first_components(d, e, z0);
    x = d;
    w.resize(n);
    for (size_t i = 0; i < n; ++i) w[i] = mu0 * z0[i] * z0[i];
  }

  // Monien's bosonic Matsubara rule: T*sum_{n!=0} f(2 pi T n) ~= sum_i w_i [f(x_i)+f(-x_i)].
  // Size selection: matsubara.cu:12-20 (predict_size) and :54-60 (clamping);
  // recurrence: matsubara.cu:63-76; scaling: matsubara.cu:80-84; T=0 / far-from-T vacuum
  // rule: matsubara.cu:128-160.
  struct MatsubaraRule {
    double T = 0, E = 0;
    std::vector<double> x, w;
  };

  inline int matsubara_predict_size(double T, double E, int step, int precision_factor, int vacuum_quad_size)
  {
    const double rel = std::fabs(E) / std::fabs(T + 1e-16);
    const bool T_zero = std::fabs(T) <= 1e-12 * std::max(1.0, std::fabs(T)) || T == 0.0;
    if (T_zero || rel > 1e2) return -vacuum_quad_size;
    const double E_max = (precision_factor + 100) * std::fabs(E);
    int size = 5 + int(std::sqrt(4 * E_max / (kPi * kPi * std::fabs(T))));
    size = (int)std::ceil(size / (double)step) * step;
    return size;
  }

  inline MatsubaraRule matsubara_rule(double T, double E, int step = 2, int min_size = 0, int max_size = 1024,
                                      int vacuum_quad_size = 48, int precision_factor = 1)
  {
    MatsubaraRule r;
    r.T = T;
    r.E = E;
    if (precision_factor < 0) precision_factor = 1;
    if (vacuum_quad_size <= 6) vacuum_quad_size = 6;
    int m = matsubara_predict_size(T, E, step, precision_factor, vacuum_quad_size);
    if (m < 0) {
      // vacuum rule: half linear GL on [0, 2|E|], half log-mapped GL on [2|E|, 1e6 |E|]
      m = -m;
      if (m % 2) ++m;
      double Ee = std::fabs(E) <= 1e-300 ? 1.0 : E;
      std::vector<double> gx, gw;
      gauss_legendre01(m / 2, gx, gw);
      r.T = 0;
      r.x.resize(m);
      r.w.resize(m);
      const long double div = 2 * std::fabs(Ee);
      const long double ext = 1e6L * std::fabs(Ee);
      const long double ls = std::log(div), le = std::log(ext / div);
      for (int i = 0; i < m / 2; ++i) {
        r.x[i] = gx[i] * (double)div;
        r.w[i] = gw[i] * (double)div / (2 * kPi);
      }
      for (int i = 0; i < m / 2; ++i) {
        const double xv = (double)std::exp(ls + le * gx[i]);
        r.x[i + m / 2] = xv;
        r.w[i + m / 2] = (gw[i] * (double)le * xv) / (2 * kPi);
      }
      return r;
    }
    m = std::max(min_size, std::min(max_size, m));
    // Jacobi matrix of the Monien weight in the variable 1/(pi^2 n^2)-type recurrence,
    // computed in long double, then Golub-Welsch in long double.
    std::vector<long double> a(m), b(m);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int j = 0; j < m; ++j) {
      const long double j1 = j + 1;
      a[j] = 2 * pi * pi / (4 * j + 1) / (4 * j + 5);
      b[j] = pi * pi * pi * pi / ((4 * j1 - 1) * (4 * j1 + 3)) / ((4 * j1 + 1) * (4 * j1 + 1));
    }
    a[0] = pi * pi / 15;
    const long double mu0 = pi * pi / 6;
    std::vector<long double> xs, ws;
    golub_welsch(a, b, mu0, xs, ws);
    r.x.resize(m);
    r.w.resize(m);
    for (int i = 0; i < m; ++i) {
      r.w[i] = (double)((long double)T * ws[i] / xs[i]);
      r.x[i] = (double)(2 * pi * (long double)T / std::sqrt(xs[i]));
    }
    return r;
  }

  // Provider-level selection: MatsubaraStorage::find_E_* uses step 2, max 128,
  // min_matsubara_size (16 from JSON default / 32 without JSON) and passes
  // add_matsubara_size as the precision factor (quadrature_provider.cu:50-52).
  inline MatsubaraRule provider_matsubara(double T, double E, int min_size = 32, int vacuum = 48, int add_size = 0)
  {
    return matsubara_rule(T, E, 2, min_size, 128, vacuum, add_size);
  }

  // ---------------------------------------------------------------------------------------
  // Pairwise accumulator (blocks of 64 FP64 terms, then a binary tree over blocks)
  // ---------------------------------------------------------------------------------------
  struct PairwiseSum {
    std::vector<double> levels;
    std::vector<int> counts;
    double block = 0;
    int nb = 0;
    void add(double v)
    {
      block += v;
      if (++nb == 64) flush();
    }
    void flush()
    {
      double carry = block;
      block = 0;
      nb = 0;
      size_t lv = 0;
      while (true) {
        if (lv == levels.size()) {
          levels.push_back(carry);
          counts.push_back(1);
          return;
        }
        if (counts[lv] == 0) {
          levels[lv] = carry;
          counts[lv] = 1;
          return;
        }
        carry += levels[lv];
        counts[lv] = 0;
        ++lv;
      }
    }
    double total() const
    {
      double t = block;
      for (size_t i = 0; i < levels.size(); ++i)
        if (counts[i]) t += levels[i];
      return t;
    }
  };

  // ---------------------------------------------------------------------------------------
  // Regulator, coordinates, tables
  // ---------------------------------------------------------------------------------------

  // BosonicRegulator<b=1>: RB(k2,q2) = q2/expm1(q2/k2), RBdot = 2 k2 x^2 e^x / expm1(x)^2,
  // x = q2/k2 (DiFfRG/include/DiFfRG/physics/regulators.hh:72-99 with b = 1).
  inline double reg_RB(double k2, double q2)
  {
    const double x = q2 / k2;
    if (x == 0.0) return k2;
    return q2 / std::expm1(x);
  }
  inline double reg_RBdot(double k2, double q2)
  {
    const double x = q2 / k2;
    if (x == 0.0) return 2 * k2;
    const double em = std::expm1(x);
    return 2 * k2 * x * x * std::exp(x) / (em * em);
  }

  // One table axis: log-spaced (index linear in ln x) or linear.
  struct Axis {
    int n = 0;
    int log = 0;
    double lo = 0, hi = 1;
    // continuous grid index, clamped to [0, n-1]
    double index(double v) const
    {
      double u;
      if (log)
        u = std::log(v / lo) / std::log(hi / lo) * (n - 1);
      else
        u = (v - lo) / (hi - lo) * (n - 1);
      if (!(u > 0)) u = 0;  // also maps NaN to the edge
      if (u > n - 1) u = n - 1;
      return u;
    }
  };

  // Row-major table of FP32 values (the engine stores the same FP32 numbers); 1D or 2D.
  struct Table {
    Axis a0, a1;  // a1.n == 0 for a 1D table
    const float *data = nullptr;
    double operator()(double v0) const
    {
      const double u = a0.index(v0);
      int i = (int)u;
      if (i > a0.n - 2) i = a0.n - 2;
      if (i < 0) i = 0;
      const double f = u - i;
      const double y0 = data[i], y1 = data[i + 1];
      return y0 + f * (y1 - y0);
    }
    double operator()(double v0, double v1) const
    {
      const double u = a0.index(v0), t = a1.index(v1);
      int i = (int)u, j = (int)t;
      if (i > a0.n - 2) i = a0.n - 2;
      if (j > a1.n - 2) j = a1.n - 2;
      const double fx = u - i, fy = t - j;
      const int n1 = a1.n;
      const double y00 = data[i * n1 + j], y10 = data[(i + 1) * n1 + j];
      const double y01 = data[i * n1 + j + 1], y11 = data[(i + 1) * n1 + j + 1];
      const double lo = y00 + fx * (y10 - y00);
      const double hi = y01 + fx * (y11 - y01);
      return lo + fy * (hi - lo);
    }
  };
} // namespace oracle
