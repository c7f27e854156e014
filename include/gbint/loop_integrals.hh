// loop_integrals.hh -- DiFfRG's host loop integrals (namespace DiFfRG::LoopIntegrals) and the
// one-dimensional Gauss rule they take, header-only, host C++17 (g++ or nvcc; no CUDA needed).
//
// Same names, arguments and integration measures as
// DiFfRG/include/DiFfRG/physics/loop_integrals.hh:17-656:
//   integrate<NT,d>(fun(q2), x_quadrature, x_extent, k)                               :34-66
//   angle_integrate<NT,d>(fun(q2,cos), ..., cos_quadrature)                           :83-125
//   two_angle_integrate<NT,d>(fun(q2,cos,phi), ..., cos_quadrature)                   :144-194
//   three_angle_integrate<NT,d>(fun(q2,cos1,cos2,phi), ..., cos_quadrature)           :214-275
//   spatial_integrate_and_integrate<NT,d>(fun(q2,q0), ..., m_quadrature, m_extent)    :295-333
//   spatial_angle_integrate_and_integrate<NT,d>(fun(q2,cos,q0), ...)                  :359-409
//   spatial_integrate_and_sum<NT,d>(fun(q2,q0), ..., m_order, m_quadrature, m_extent, T)     :435-504
//   spatial_angle_integrate_and_sum<NT,d>(fun(q2,cos,q0), ..., m_order, ..., T)       :528-616
//   sum<NT>(fun(q0), m_order, m_quadrature, m_extent, T)                               :618-655
// The callables are host functions (lambdas, std::function), so these integrals run on the
// host cores, as the reference's do (there with TBB).  Each term is formed with the reference's
// factors in the reference's order; the rows of the outermost quadrature axis are evaluated on
// up to gbint_loop::max_threads() threads and their partial sums are added in row order, so a
// result does not depend on the number of threads (the reference's TBB reduction order does).
//
// Quadratures: any type with get_points()[i][0] (on [0,1]), get_weights()[i] (summing to 1)
// and size(), e.g. deal.II's QGauss<1>.  Without deal.II, DiFfRG::QGauss<1> below is the n-point
// Gauss-Legendre rule of gbint/gl_rule.hh in that convention.
//
// One deliberate difference: two_angle_integrate weights its phi nodes with the phi rule's
// weights.  The reference multiplies the phi term by the weight of the current cos node
// (loop_integrals.hh:180-181), which turns the phi quadrature into a plain sum of the nodes' values
// and does not compute the integral its documentation states (:129-142); that integral is
// computed here.  Its phi nodes are, as in the reference, those of cos_quadrature on [0, 2 pi].
// Defining GBINT_LOOP_REFERENCE_PHI_WEIGHT before this header restores the reference's weighting,
// for comparisons with results obtained from it.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <exception>
#include <limits>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "gbint/gl_rule.hh"

namespace DiFfRG
{
#ifdef dealii_quadrature_lib_h
  using dealii::QGauss;
#else
  // deal.II's QGauss<1> without deal.II: the n-point Gauss-Legendre rule on [0,1]
  template <int dim> class QGauss;
  template <> class QGauss<1>
  {
  public:
    using point_type = std::array<double, 1>;
    explicit QGauss(const unsigned int n)
    {
      std::vector<double> x;
      gbint::gl_rule01((int)n, x, weights_);
      points_.resize(n);
      for (unsigned int i = 0; i < n; ++i) points_[i][0] = x[i];
    }
    const std::vector<point_type> &get_points() const { return points_; }
    const std::vector<double> &get_weights() const { return weights_; }
    const point_type &point(const unsigned int i) const { return points_[i]; }
    double weight(const unsigned int i) const { return weights_[i]; }
    unsigned int size() const { return (unsigned int)weights_.size(); }

  private:
    std::vector<point_type> points_;
    std::vector<double> weights_;
  };
#endif

  namespace gbint_loop
  {
    constexpr double kPi = 3.141592653589793238462643383279502884;

    // x^n by right-nested products, 1/x^-n for n < 0 (DiFfRG/include/DiFfRG/common/math.hh:40-54)
    template <int n> constexpr double ipow(const double x)
    {
      if constexpr (n == 0)
        return 1.;
      else if constexpr (n < 0)
        return 1. / ipow<-n>(x);
      else if constexpr (n > 1)
        return x * ipow<n - 1>(x);
      else
        return x;
    }

    // a == 0 in the sense of DiFfRG's is_close(a, 0.) (DiFfRG/include/DiFfRG/common/math.hh:160-193)
    inline bool is_zero(const double a) { return std::fabs(a) <= std::numeric_limits<double>::epsilon(); }

    // threads for the host loop integrals: GBINT_HOST_THREADS if set (>= 1), else the hardware's
    inline unsigned max_threads()
    {
      static const unsigned n = [] {
        if (const char *e = std::getenv("GBINT_HOST_THREADS")) {
          const int v = std::atoi(e);
          if (v >= 1) return (unsigned)v;
        }
        const unsigned h = std::thread::hardware_concurrency();
        return h ? h : 1u;
      }();
      return n;
    }

    // integrand calls per thread started: below it, starting a thread costs more than it saves
    constexpr std::size_t kCallsPerThread = std::size_t(1) << 15;

    // sum over r < rows of row(r), the rows' partial sums added in row order; the rows are
    // evaluated on several threads (row r on thread r mod T) when the work is large enough
    template <typename NT, typename ROW> NT reduce_rows(const int rows, const std::size_t calls_per_row, ROW &&row)
    {
      if (rows <= 0) return NT(0);
      std::vector<NT> part((std::size_t)rows, NT(0));
      const std::size_t calls = (std::size_t)rows * calls_per_row;
      const unsigned T = (unsigned)std::min<std::size_t>({(std::size_t)max_threads(), (std::size_t)rows,
                                                           calls / kCallsPerThread + 1});
      if (T <= 1) {
        for (int r = 0; r < rows; ++r) part[(std::size_t)r] = row(r);
      } else {
        std::exception_ptr err;
        std::mutex mu;
        std::vector<std::thread> pool;
        pool.reserve(T);
        for (unsigned t = 0; t < T; ++t)
          pool.emplace_back([&, t] {
            try {
              for (int r = (int)t; r < rows; r += (int)T) part[(std::size_t)r] = row(r);
            } catch (...) {
              std::lock_guard<std::mutex> lk(mu);
              if (!err) err = std::current_exception();
            }
          });
        for (auto &th : pool) th.join();
        if (err) std::rethrow_exception(err);
      }
      NT total(0);
      for (int r = 0; r < rows; ++r) total += part[(std::size_t)r];
      return total;
    }

    // area of the unit sphere in d dimensions, 2 pi^(d/2) / Gamma(d/2)
    inline double sphere_area(const int d) { return 2. * std::pow(kPi, d / 2.) / std::tgamma(d / 2.); }
  } // namespace gbint_loop

  namespace LoopIntegrals
  {
    // int dOmega_d int_0^inf dq q^(d-1) f(q^2) / (2 pi)^d, q^2 = x k^2, x in [0, x_extent]
    template <typename NT, int d, typename FUN, typename QUAD>
    NT integrate(const FUN &fun, const QUAD &x_quadrature, const double x_extent, const double k)
    {
      static_assert(d > 0, "Dimension must be greater than zero");
      using gbint_loop::ipow;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      // the reference takes Gamma(d/2) in long double here (loop_integrals.hh:43)
      const double S_d = (double)(2. * std::pow(gbint_loop::kPi, d / 2.) / std::tgamma((long double)(d / 2.)));
      const double prefactor = S_d * ipow<-d>(2. * gbint_loop::kPi);
      return gbint_loop::reduce_rows<NT>(x_size, 1, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        return x_weight * prefactor * (0.5 * ipow<d>(k) * std::pow(x, (d - 2) / 2.)) * fun(q2);
      });
    }

    // int dOmega_(d-1) int_-1^1 dcos int dq q^(d-1) f(q^2, cos) / (2 pi)^d
    template <typename NT, int d, typename FUN, typename QUAD>
    NT angle_integrate(const FUN &fun, const QUAD &x_quadrature, const double x_extent, const double k,
                       const QUAD &cos_quadrature)
    {
      static_assert(d > 1, "Dimension must be greater than one, otherwise the angular integral not defined.");
      using gbint_loop::ipow;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &cos_q_p = cos_quadrature.get_points();
      const auto &cos_q_w = cos_quadrature.get_weights();
      const int cos_size = (int)cos_quadrature.size();
      const double prefactor = gbint_loop::sphere_area(d) * ipow<-d>(2. * gbint_loop::kPi);
      return gbint_loop::reduce_rows<NT>(x_size, (std::size_t)cos_size, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        NT acc(0);
        for (int cos_it = 0; cos_it < cos_size; ++cos_it) {
          const double cos = (cos_q_p[cos_it][0] - 0.5) * 2.;
          const double cos_weight = cos_q_w[cos_it] * 2.;
          acc += x_weight * prefactor * (0.5 * ipow<d>(k) * std::pow(x, (d - 2) / 2.)) * 0.5 * cos_weight *
                 fun(q2, cos);
        }
        return acc;
      });
    }

    // int dOmega_(d-2) int_-1^1 dcos int_0^2pi dphi int dq q^(d-1) f(q^2, cos, phi) / (2 pi)^d
    template <typename NT, int d, typename FUN, typename QUAD>
    NT two_angle_integrate(const FUN &fun, const QUAD &x_quadrature, const double x_extent, const double k,
                           const QUAD &cos_quadrature)
    {
      static_assert(d > 2, "Dimension must be greater than 2, otherwise the angular integral not defined.");
      using gbint_loop::ipow;
      constexpr double two_pi = 2. * gbint_loop::kPi;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &cos_q_p = cos_quadrature.get_points();
      const auto &cos_q_w = cos_quadrature.get_weights();
      const int cos_size = (int)cos_quadrature.size();
      const double prefactor = gbint_loop::sphere_area(d) * ipow<-d>(two_pi);
      return gbint_loop::reduce_rows<NT>(x_size, (std::size_t)cos_size * cos_size, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        NT acc(0);
        for (int cos_it = 0; cos_it < cos_size; ++cos_it) {
          const double cos = (cos_q_p[cos_it][0] - 0.5) * 2.;
          const double cos_weight = cos_q_w[cos_it] * 2.;
          for (int phi_it = 0; phi_it < cos_size; ++phi_it) {
            const double phi = cos_q_p[phi_it][0] * two_pi;
#ifdef GBINT_LOOP_REFERENCE_PHI_WEIGHT
            const double phi_weight = cos_q_w[cos_it] * two_pi;  // the reference's weighting, opt-in
#else
            const double phi_weight = cos_q_w[phi_it] * two_pi;
#endif
            acc += x_weight * prefactor * (0.5 * ipow<d>(k) * std::pow(x, (d - 2) / 2.)) * 0.5 * cos_weight *
                   phi_weight / two_pi * fun(q2, cos, phi);
          }
        }
        return acc;
      });
    }

    // int dOmega_(d-3) int dcos1 sqrt(1-cos1^2) int dcos2 int dphi int dq q^(d-1) f(q^2,cos1,cos2,phi) / (2 pi)^d
    template <typename NT, int d, typename FUN, typename QUAD>
    NT three_angle_integrate(const FUN &fun, const QUAD &x_quadrature, const double x_extent, const double k,
                             const QUAD &cos_quadrature)
    {
      static_assert(d > 3, "Dimension must be greater than 3, otherwise the angular integral not defined.");
      using gbint_loop::ipow;
      constexpr double two_pi = 2. * gbint_loop::kPi;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &cos_q_p = cos_quadrature.get_points();
      const auto &cos_q_w = cos_quadrature.get_weights();
      const int cos_size = (int)cos_quadrature.size();
      const double S_4 = gbint_loop::sphere_area(4);
      const double prefactor = gbint_loop::sphere_area(d) * ipow<-d>(two_pi);
      return gbint_loop::reduce_rows<NT>(
          x_size, (std::size_t)cos_size * cos_size * cos_size, [&](const int x_it) -> NT {
            const double x = x_q_p[x_it][0] * x_extent;
            const double x_weight = x_q_w[x_it] * x_extent;
            const double q2 = x * ipow<2>(k);
            NT acc(0);
            for (int cos1_it = 0; cos1_it < cos_size; ++cos1_it) {
              const double cos1 = (cos_q_p[cos1_it][0] - 0.5) * 2.;
              const double cos1_weight = cos_q_w[cos1_it] * 2. * std::sqrt(1. - ipow<2>(cos1));
              for (int cos2_it = 0; cos2_it < cos_size; ++cos2_it) {
                const double cos2 = (cos_q_p[cos2_it][0] - 0.5) * 2.;
                const double cos2_weight = cos_q_w[cos2_it] * 2.;
                for (int phi_it = 0; phi_it < cos_size; ++phi_it) {
                  const double phi = cos_q_p[phi_it][0] * two_pi;
                  const double phi_weight = cos_q_w[phi_it] * two_pi;
                  acc += x_weight * prefactor * (0.5 * ipow<d>(k) * std::pow(x, (d - 2) / 2.)) * cos1_weight *
                         cos2_weight * phi_weight / S_4 * fun(q2, cos1, cos2, phi);
                }
              }
            }
            return acc;
          });
    }

    // int_-inf^inf dq0 / (2 pi) int dOmega_(d-1) int dq q^(d-2) f(q^2, q0) / (2 pi)^(d-1),
    // q0 in [0, m_extent] with f(q^2, q0) + f(q^2, -q0)
    template <typename NT, int d, typename FUN, typename QUAD>
    NT spatial_integrate_and_integrate(const FUN &fun, const QUAD &x_quadrature, const double x_extent,
                                       const double k, const QUAD &m_quadrature, const double m_extent)
    {
      static_assert(d > 0, "Dimension must be greater than zero");
      using gbint_loop::ipow;
      constexpr int ds = d - 1;
      constexpr double two_pi = 2. * gbint_loop::kPi;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &m_q_p = m_quadrature.get_points();
      const auto &m_q_w = m_quadrature.get_weights();
      const int m_size = (int)m_quadrature.size();
      const double prefactor = gbint_loop::sphere_area(ds) * ipow<-ds>(two_pi);
      return gbint_loop::reduce_rows<NT>(x_size, 2 * (std::size_t)m_size, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        NT acc(0);
        for (int q0_it = 0; q0_it < m_size; ++q0_it) {
          const double q0 = m_q_p[q0_it][0] * m_extent;
          const double m_weight = m_q_w[q0_it] * m_extent;
          acc += (m_weight / two_pi) * x_weight * prefactor * (0.5 * ipow<ds>(k) * std::pow(x, (ds - 2) / 2.)) *
                 (fun(q2, q0) + fun(q2, -q0));
        }
        return acc;
      });
    }

    // as spatial_integrate_and_integrate with an angle: f(q^2, cos, q0), 0.5 int_-1^1 dcos
    template <typename NT, int d, typename FUN, typename QUAD>
    NT spatial_angle_integrate_and_integrate(const FUN &fun, const QUAD &x_quadrature, const double x_extent,
                                             const double k, const QUAD &cos_quadrature, const QUAD &m_quadrature,
                                             const double m_extent)
    {
      static_assert(d > 0, "Dimension must be greater than zero");
      using gbint_loop::ipow;
      constexpr int ds = d - 1;
      constexpr double two_pi = 2. * gbint_loop::kPi;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &cos_q_p = cos_quadrature.get_points();
      const auto &cos_q_w = cos_quadrature.get_weights();
      const int cos_size = (int)cos_quadrature.size();
      const auto &m_q_p = m_quadrature.get_points();
      const auto &m_q_w = m_quadrature.get_weights();
      const int m_size = (int)m_quadrature.size();
      const double prefactor = gbint_loop::sphere_area(ds) * ipow<-ds>(two_pi);
      return gbint_loop::reduce_rows<NT>(x_size, 2 * (std::size_t)cos_size * m_size, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        NT acc(0);
        for (int cos_it = 0; cos_it < cos_size; ++cos_it) {
          const double cos = (cos_q_p[cos_it][0] - 0.5) * 2.;
          const double cos_weight = cos_q_w[cos_it] * 2.;
          for (int q0_it = 0; q0_it < m_size; ++q0_it) {
            const double q0 = m_q_p[q0_it][0] * m_extent;
            const double m_weight = m_q_w[q0_it] * m_extent;
            acc += (m_weight / two_pi) * x_weight * prefactor * (0.5 * ipow<ds>(k) * std::pow(x, (ds - 2) / 2.)) *
                   0.5 * cos_weight * (fun(q2, cos, q0) + fun(q2, cos, -q0));
          }
        }
        return acc;
      });
    }

    // T sum_(|n| <= m_order) int dOmega_(d-1) int dq q^(d-2) f(q^2, 2 pi T n) / (2 pi)^(d-1), the
    // frequencies above m_order replaced by the q0 integral over the reference's tail interval
    // (nodes 2 pi T m_order + x (m_extent - 2 pi T (m_order + 1)), weights w (m_extent - 2 pi T m_order),
    // loop_integrals.hh:481-499); T == 0 is spatial_integrate_and_integrate
    template <typename NT, int d, typename FUN, typename QUAD>
    NT spatial_integrate_and_sum(const FUN &fun, const QUAD &x_quadrature, const double x_extent, const double k,
                                 const int m_order, const QUAD &m_quadrature, const double m_extent, const double T)
    {
      if (gbint_loop::is_zero(T))
        return spatial_integrate_and_integrate<NT, d>(fun, x_quadrature, x_extent, k, m_quadrature, m_extent);
      static_assert(d > 0, "Dimension must be greater than zero");
      using gbint_loop::ipow;
      constexpr int ds = d - 1;
      constexpr double pi = gbint_loop::kPi;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &m_q_p = m_quadrature.get_points();
      const auto &m_q_w = m_quadrature.get_weights();
      const int m_size = (int)m_quadrature.size();
      const double prefactor = gbint_loop::sphere_area(ds) * ipow<-ds>(2. * pi);

      const NT result_sum = gbint_loop::reduce_rows<NT>(x_size, 2 * (std::size_t)m_order + 1, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        NT acc(0);
        for (int q0_it = -m_order; q0_it <= m_order; ++q0_it) {
          const double q0 = 2. * pi * T * q0_it;
          acc += T * x_weight * prefactor * (0.5 * ipow<ds>(k) * std::pow(x, (ds - 2) / 2.)) * fun(q2, q0);
        }
        return acc;
      });
      const NT result_integral = gbint_loop::reduce_rows<NT>(x_size, 2 * (std::size_t)m_size, [&](const int x_it) -> NT {
        const double x = x_q_p[x_it][0] * x_extent;
        const double x_weight = x_q_w[x_it] * x_extent;
        const double q2 = x * ipow<2>(k);
        NT acc(0);
        for (int q0_it = 0; q0_it < m_size; ++q0_it) {
          const double q0 = (2. * m_order * pi * T) + m_q_p[q0_it][0] * (m_extent - 2. * (m_order + 1) * pi * T);
          const double m_weight = m_q_w[q0_it] * (m_extent - 2. * m_order * pi * T);
          acc += (1. * m_weight / (2. * pi)) * x_weight * prefactor *
                 (0.5 * ipow<ds>(k) * std::pow(x, (ds - 2) / 2.)) * (fun(q2, q0) + fun(q2, -q0));
        }
        return acc;
      });
      return result_sum + result_integral;
    }

    // as spatial_integrate_and_sum with an angle: f(q^2, cos, q0), 0.5 int_-1^1 dcos
    template <typename NT, int d, typename FUN, typename QUAD>
    NT spatial_angle_integrate_and_sum(const FUN &fun, const QUAD &x_quadrature, const double x_extent,
                                       const double k, const QUAD &cos_quadrature, const int m_order,
                                       const QUAD &m_quadrature, const double m_extent, const double T)
    {
      if (gbint_loop::is_zero(T))
        return spatial_angle_integrate_and_integrate<NT, d>(fun, x_quadrature, x_extent, k, cos_quadrature,
                                                            m_quadrature, m_extent);
      static_assert(d > 0, "Dimension must be greater than zero");
      using gbint_loop::ipow;
      constexpr int ds = d - 1;
      constexpr double pi = gbint_loop::kPi;
      const auto &x_q_p = x_quadrature.get_points();
      const auto &x_q_w = x_quadrature.get_weights();
      const int x_size = (int)x_quadrature.size();
      const auto &cos_q_p = cos_quadrature.get_points();
      const auto &cos_q_w = cos_quadrature.get_weights();
      const int cos_size = (int)cos_quadrature.size();
      const auto &m_q_p = m_quadrature.get_points();
      const auto &m_q_w = m_quadrature.get_weights();
      const int m_size = (int)m_quadrature.size();
      const double prefactor = gbint_loop::sphere_area(ds) * ipow<-ds>(2. * pi);

      const NT result_sum = gbint_loop::reduce_rows<NT>(
          x_size, (std::size_t)cos_size * (2 * m_order + 1), [&](const int x_it) -> NT {
            const double x = x_q_p[x_it][0] * x_extent;
            const double x_weight = x_q_w[x_it] * x_extent;
            const double q2 = x * ipow<2>(k);
            NT acc(0);
            for (int cos_it = 0; cos_it < cos_size; ++cos_it) {
              const double cos = (cos_q_p[cos_it][0] - 0.5) * 2.;
              const double cos_weight = cos_q_w[cos_it] * 2.;
              for (int q0_it = -m_order; q0_it <= m_order; ++q0_it) {
                const double q0 = 2. * pi * T * q0_it;
                acc += T * x_weight * prefactor * (0.5 * ipow<ds>(k) * std::pow(x, (ds - 2) / 2.)) * 0.5 *
                       cos_weight * fun(q2, cos, q0);
              }
            }
            return acc;
          });
      const NT result_integral = gbint_loop::reduce_rows<NT>(
          x_size, 2 * (std::size_t)cos_size * m_size, [&](const int x_it) -> NT {
            const double x = x_q_p[x_it][0] * x_extent;
            const double x_weight = x_q_w[x_it] * x_extent;
            const double q2 = x * ipow<2>(k);
            NT acc(0);
            for (int cos_it = 0; cos_it < cos_size; ++cos_it) {
              const double cos = (cos_q_p[cos_it][0] - 0.5) * 2.;
              const double cos_weight = cos_q_w[cos_it] * 2.;
              for (int q0_it = 0; q0_it < m_size; ++q0_it) {
                const double q0 =
                    (2. * m_order * pi * T) + m_q_p[q0_it][0] * (m_extent - 2. * (m_order + 1) * pi * T);
                const double m_weight = m_q_w[q0_it] * (m_extent - 2. * m_order * pi * T);
                acc += (1. * m_weight / (2. * pi)) * x_weight * prefactor *
                       (0.5 * ipow<ds>(k) * std::pow(x, (ds - 2) / 2.)) * 0.5 * cos_weight *
                       (fun(q2, cos, q0) + fun(q2, cos, -q0));
              }
            }
            return acc;
          });
      return result_sum + result_integral;
    }

    // T sum_(|n| <= m_order) f(2 pi T n) (nothing at T == 0) plus the q0 integral of the tail
    // interval of spatial_integrate_and_sum
    template <typename NT, typename FUN, typename QUAD>
    NT sum(const FUN &fun, const int m_order, const QUAD &m_quadrature, const double m_extent, const double T)
    {
      constexpr double pi = gbint_loop::kPi;
      const auto &m_q_p = m_quadrature.get_points();
      const auto &m_q_w = m_quadrature.get_weights();
      const int m_size = (int)m_quadrature.size();
      NT result_sum(0);
      if (!gbint_loop::is_zero(T))
        for (int q0_it = -m_order; q0_it <= m_order; ++q0_it) {
          const double q0 = 2. * pi * T * q0_it;
          result_sum += T * fun(q0);
        }
      NT result_integral(0);
      for (int q0_it = 0; q0_it < m_size; ++q0_it) {
        const double q0 = (2. * m_order * pi * T) + m_q_p[q0_it][0] * (m_extent - 2. * (m_order + 1) * pi * T);
        const double m_weight = m_q_w[q0_it] * (m_extent - 2. * m_order * pi * T);
        result_integral += (1. * m_weight / (2. * pi)) * (fun(q0) + fun(-q0));
      }
      return result_sum + result_integral;
    }
  } // namespace LoopIntegrals
} // namespace DiFfRG
