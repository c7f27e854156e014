// flow_equations.hh -- DiFfRG's FlowEquations / FlowEquationsFiniteT bases: the quadrature
// settings a flow reads from its JSON, the optimisation of the integration extents, and the
// host loop integrals over them.  Header-only host C++17 (g++ or nvcc; no CUDA needed).
//
// Same members and behaviour as DiFfRG/include/DiFfRG/physics/flow_equations.hh:17-320 and
// DiFfRG/src/DiFfRG/physics/flow_equations.cc:13-314:
//   * constructor(json, [T,] optimize_x[, optimize_x0, optimize_q0]) reads
//     /integration/{x,angle,x0,q0}_quadrature_order, jacobian_quadrature_factor,
//     {x,x0,q0}_extent_tolerance, x0_summands, q0_summands and /output/verbosity, then fits the
//     extents (x0 and q0 only when their summand counts are non-zero);
//   * update_x_extent (flow_equations.cc:54-103, 161-206): x_extent = 1.15^n, the smallest n
//     for which the 4D loop integrals of optimize_x over [0, x], [0, 2x] and [0, 10x] (Gauss
//     rules of 5, 10 and 50 times x_quadrature_order points) agree to x_extent_tolerance;
//     1 when optimize_x vanishes at ten probe points; a std::runtime_error when the relative
//     differences grow for more than two steps in a row;
//   * update_q0_extent / update_x0_extent (flow_equations.cc:208-285): the same for the q0 and
//     x0 integrals of LoopIntegrals::sum at T = 0, starting from 0.5 sqrt(x_extent) k and
//     0.5 sqrt(x_extent);
//   * integrate / angle_integrate / ... (and the FiniteT q0 variants): LoopIntegrals over the
//     stored rules and extents at the set k, over the jacobian rules for forward-mode result
//     types (gbint::dual; specialise gbint_detail::uses_jacobian_quadrature for others).
// The JSON object is any type with get_uint / get_double / get_int(path) (DiFfRG's JSONValue).
// print_parameters writes to a std::ostream (std::cout by default) instead of an spdlog logger.
#pragma once

#include <cmath>
#include <functional>
#include <initializer_list>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "gbint/loop_integrals.hh"

namespace gbint
{
  template <typename T> struct dual;
}

namespace DiFfRG
{
  namespace gbint_detail
  {
    // result types whose flows integrate over the jacobian rules (the reference: autodiff::real
    // and autodiff::dual, flow_equations.hh:33-34)
    template <typename NT> struct uses_jacobian_quadrature : std::false_type {};
    template <typename T> struct uses_jacobian_quadrature<gbint::dual<T>> : std::true_type {};

    constexpr unsigned kExtentQuadratureFactor = 5;  // flow_equations.cc:11

    // x_extent and friends: the loop of flow_equations.cc:82-102 around integral(rule, extent)
    // for the rules of 5, 10 and 50 times `order` points; `max_rises` is 2 for x and q0, 1 for x0
    template <typename INTEGRAL>
    double fit_extent(const char *name, const char *order_name, unsigned order, double extent, double tolerance,
                      unsigned max_rises, int verbosity, INTEGRAL &&integral, bool detail_in_error)
    {
      const QGauss<1> quadrature_1(kExtentQuadratureFactor * 1 * order);
      const QGauss<1> quadrature_2(kExtentQuadratureFactor * 2 * order);
      const QGauss<1> quadrature_3(kExtentQuadratureFactor * 10 * order);
      double eps1 = 1., eps2 = 1.;
      unsigned decrease_counter = 0;
      while (eps1 > tolerance || eps2 > tolerance) {
        const double I1 = integral(quadrature_1, extent);
        const double I2 = integral(quadrature_2, 2. * extent);
        const double I3 = integral(quadrature_3, 10. * extent);
        if (std::abs((I2 - I1) / I1) > eps1 && std::abs((I2 - I3) / I2) > eps2)
          decrease_counter++;
        else
          decrease_counter = 0;
        if (decrease_counter > max_rises) {
          std::string msg = std::string("Cannot reach requested precision for ") + name + " - increase " +
                            order_name + " or decrease " + name + "_tolerance.";
          if (detail_in_error)
            msg += " Last eps1: " + std::to_string(eps1) + " Last eps2: " + std::to_string(eps2) + " Last " + name +
                   ": " + std::to_string(extent) + " Last I1: " + std::to_string(I1) +
                   " Last I2: " + std::to_string(I2) + " Last I3: " + std::to_string(I3);
          throw std::runtime_error(msg);
        }
        eps1 = std::abs((I2 - I1) / I1);
        eps2 = std::abs((I2 - I3) / I2);
        if (verbosity > 1)
          std::cout << name << ": " << extent << " I1: " << I1 << " I2: " << I2 << " I3: " << I3 << " eps1: " << eps1
                    << " eps2: " << eps2 << std::endl;
        if (eps1 > tolerance || eps2 > tolerance) extent *= 1.15;
      }
      if (verbosity > 1) std::cout << "Optimizing " << name << " done.\n" << std::endl;
      return extent;
    }

    // the settings a flow base reads: a rule order "/integration/<axis>_quadrature_order", the
    // jacobian rule's order (factor times the order, truncated), a tolerance, the verbosity
    template <class JSON> unsigned rule_order(const JSON &json, const char *axis)
    {
      return json.get_uint(std::string("/integration/") + axis + "_quadrature_order");
    }
    inline unsigned jacobian_order(double factor, unsigned order) { return (unsigned)(factor * order); }
    template <class JSON> double setting(const JSON &json, const char *key)
    {
      return json.get_double(std::string("/integration/") + key);
    }

    // "[logname] <title>:" and one "<label>: <value>" line per row, labels right-aligned in
    // label_width, values in value_width (0: as printed)
    struct ParamRow {
      const char *label;
      std::string value;
    };
    template <typename V> ParamRow row(const char *label, const V &v)
    {
      std::ostringstream o;
      o << v;
      return ParamRow{label, o.str()};
    }
    inline void log_rows(std::ostream &os, const std::string &logname, const char *title,
                         std::initializer_list<ParamRow> rows, int label_width, int value_width)
    {
      std::ostringstream out;
      out << title << ":";
      for (const ParamRow &r : rows) {
        out << "\n" << std::setw(label_width) << (std::string(r.label) + ": ");
        if (value_width > 0)
          out << std::setw(value_width) << r.value;
        else
          out << r.value;
      }
      os << "[" << logname << "] " << out.str() << std::endl;
    }

    // optimize_x vanishes at x = 1 + 1e-3 + (1.5^i - 1), i < 10 (flow_equations.cc:70-79)
    inline bool vanishes_on_probe(const std::function<double(double)> &f)
    {
      for (unsigned i = 0; i < 10; i++) {
        const double x = 1. + 1e-3 + (std::pow(1.5, (double)i) - 1.);
        if (!gbint_loop::is_zero(f(x))) return false;
      }
      return true;
    }
  } // namespace gbint_detail

  class FlowEquations
  {
  protected:
    // members in declaration order: each rule from its order, the jacobian rules from the
    // factor, x_extent starts at 1 and is fitted at once
    template <class JSON>
    FlowEquations(const JSON &json, std::function<double(double)> optimize_x)
        : x_quadrature_order(gbint_detail::rule_order(json, "x")), x_quadrature(x_quadrature_order), x_extent(1.),
          angle_quadrature_order(gbint_detail::rule_order(json, "angle")), angle_quadrature(angle_quadrature_order),
          jacobian_quadrature_factor(gbint_detail::setting(json, "jacobian_quadrature_factor")),
          jac_x_quadrature_order(gbint_detail::jacobian_order(jacobian_quadrature_factor, x_quadrature_order)),
          jac_x_quadrature(jac_x_quadrature_order),
          jac_angle_quadrature_order(gbint_detail::jacobian_order(jacobian_quadrature_factor, angle_quadrature_order)),
          jac_angle_quadrature(jac_angle_quadrature_order),
          x_extent_tolerance(gbint_detail::setting(json, "x_extent_tolerance")), optimize_x(std::move(optimize_x)),
          k(1), unoptimized(true), verbosity(json.get_int("/output/verbosity"))
    {
      update_x_extent();
      unoptimized = false;
      if (verbosity > 1) std::cout << "FlowEquations initialized" << std::endl;
    }

  public:
    void set_k(const double k) { this->k = k; }

    // the reference's log layout: labels right-aligned in 40 columns, values in 10
    void print_parameters(const std::string logname, std::ostream &os = std::cout) const
    {
      using gbint_detail::row;
      gbint_detail::log_rows(os, logname, "FlowEquations",
                             {row("x_quadrature_order", x_quadrature_order),
                              row("jac_x_quadrature_order", jac_x_quadrature_order), row("x_extent", x_extent),
                              row("angle_quadrature_order", angle_quadrature_order),
                              row("jac_angle_quadrature_order", jac_angle_quadrature_order)},
                             40, 10);
    }

    template <typename NT, int d, typename FUN> NT integrate(const FUN &fun) const { return integrate<NT, d>(fun, k); }
    template <typename NT, int d, typename FUN> NT angle_integrate(const FUN &fun) const
    {
      return angle_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT two_angle_integrate(const FUN &fun) const
    {
      return two_angle_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT three_angle_integrate(const FUN &fun) const
    {
      return three_angle_integrate<NT, d>(fun, k);
    }

    template <typename NT, int d, typename FUN> NT integrate(const FUN &fun, const double k) const
    {
      constexpr bool jac = gbint_detail::uses_jacobian_quadrature<NT>::value;
      return LoopIntegrals::integrate<NT, d>(fun, jac ? jac_x_quadrature : x_quadrature, x_extent, k);
    }
    template <typename NT, int d, typename FUN> NT angle_integrate(const FUN &fun, const double k) const
    {
      constexpr bool jac = gbint_detail::uses_jacobian_quadrature<NT>::value;
      return LoopIntegrals::angle_integrate<NT, d>(fun, jac ? jac_x_quadrature : x_quadrature, x_extent, k,
                                                   jac ? jac_angle_quadrature : angle_quadrature);
    }
    template <typename NT, int d, typename FUN> NT two_angle_integrate(const FUN &fun, const double k) const
    {
      constexpr bool jac = gbint_detail::uses_jacobian_quadrature<NT>::value;
      return LoopIntegrals::two_angle_integrate<NT, d>(fun, jac ? jac_x_quadrature : x_quadrature, x_extent, k,
                                                       jac ? jac_angle_quadrature : angle_quadrature);
    }
    template <typename NT, int d, typename FUN> NT three_angle_integrate(const FUN &fun, const double k) const
    {
      constexpr bool jac = gbint_detail::uses_jacobian_quadrature<NT>::value;
      return LoopIntegrals::three_angle_integrate<NT, d>(fun, jac ? jac_x_quadrature : x_quadrature, x_extent, k,
                                                         jac ? jac_angle_quadrature : angle_quadrature);
    }

    void set_jacobian_quadrature_factor(const double jacobian_quadrature_factor)
    {
      jac_x_quadrature_order = jacobian_quadrature_factor * x_quadrature_order;
      jac_x_quadrature = QGauss<1>(jac_x_quadrature_order);
      jac_angle_quadrature_order = jacobian_quadrature_factor * angle_quadrature_order;
      jac_angle_quadrature = QGauss<1>(jac_angle_quadrature_order);
    }

  protected:
    void update_x_extent()
    {
      x_extent = 1.;
      if (verbosity > 1) std::cout << "Optimizing x_extent" << std::endl;
      if (gbint_detail::vanishes_on_probe(optimize_x)) {
        if (verbosity > 1) std::cout << "x_extent is set to 1.\n" << std::endl;
        return;
      }
      // the vacuum flows fit x_extent at k = 1 (flow_equations.cc:83-85)
      x_extent = gbint_detail::fit_extent(
          "x_extent", "x_quadrature_order", x_quadrature_order, 1., x_extent_tolerance, 2, verbosity,
          [&](const QGauss<1> &q, double ext) { return LoopIntegrals::integrate<double, 4>(optimize_x, q, ext, 1.); },
          false);
    }

    const unsigned x_quadrature_order;
    const QGauss<1> x_quadrature;
    double x_extent;

    const unsigned angle_quadrature_order;
    const QGauss<1> angle_quadrature;

    double jacobian_quadrature_factor;

    unsigned jac_x_quadrature_order;
    QGauss<1> jac_x_quadrature;
    unsigned jac_angle_quadrature_order;
    QGauss<1> jac_angle_quadrature;

    const double x_extent_tolerance;

    const std::function<double(double)> optimize_x;

    double k;
    bool unoptimized;
    const int verbosity;
  };

  class FlowEquationsFiniteT
  {
  protected:
    // members in declaration order, as in FlowEquations, with the x0 and q0 axes (summands,
    // rule, extent 0 until fitted) and the temperature
    template <class JSON>
    FlowEquationsFiniteT(const JSON &json, const double T, std::function<double(double)> optimize_x,
                         std::function<double(double)> optimize_x0, std::function<double(double)> optimize_q0)
        : x_quadrature_order(gbint_detail::rule_order(json, "x")), x_quadrature(x_quadrature_order), x_extent(1.),
          x0_summands(json.get_uint("/integration/x0_summands")), x0_quadrature_order(gbint_detail::rule_order(json, "x0")),
          x0_quadrature(x0_quadrature_order), x0_extent(0), q0_summands(json.get_uint("/integration/q0_summands")),
          q0_quadrature_order(gbint_detail::rule_order(json, "q0")), q0_quadrature(q0_quadrature_order), q0_extent(0),
          angle_quadrature_order(gbint_detail::rule_order(json, "angle")), angle_quadrature(angle_quadrature_order),
          jacobian_quadrature_factor(gbint_detail::setting(json, "jacobian_quadrature_factor")),
          jac_x_quadrature_order(gbint_detail::jacobian_order(jacobian_quadrature_factor, x_quadrature_order)),
          jac_x_quadrature(jac_x_quadrature_order),
          jac_x0_quadrature_order(gbint_detail::jacobian_order(jacobian_quadrature_factor, x0_quadrature_order)),
          jac_x0_quadrature(jac_x0_quadrature_order),
          jac_q0_quadrature_order(gbint_detail::jacobian_order(jacobian_quadrature_factor, q0_quadrature_order)),
          jac_q0_quadrature(jac_q0_quadrature_order),
          jac_angle_quadrature_order(gbint_detail::jacobian_order(jacobian_quadrature_factor, angle_quadrature_order)),
          jac_angle_quadrature(jac_angle_quadrature_order),
          x_extent_tolerance(gbint_detail::setting(json, "x_extent_tolerance")),
          x0_extent_tolerance(gbint_detail::setting(json, "x0_extent_tolerance")),
          q0_extent_tolerance(gbint_detail::setting(json, "q0_extent_tolerance")), T(T),
          optimize_x(std::move(optimize_x)), optimize_x0(std::move(optimize_x0)), optimize_q0(std::move(optimize_q0)),
          k(1.), unoptimized(true), verbosity(json.get_int("/output/verbosity"))
    {
      update_x_extent();
      if (x0_summands > 0) update_x0_extent();
      if (q0_summands > 0) update_q0_extent();
      unoptimized = false;
      if (verbosity > 0) std::cout << "FlowEquationsFiniteT initialized" << std::endl;
    }

  public:
    void set_k(const double k) { this->k = k; }

    // the reference's log layout: labels right-aligned in 10 columns, values as printed
    void print_parameters(const std::string logname, std::ostream &os = std::cout) const
    {
      using gbint_detail::row;
      gbint_detail::log_rows(
          os, logname, "FlowEquationsFiniteT",
          {row("x_quadrature_order", x_quadrature_order), row("jac_x_quadrature_order", jac_x_quadrature_order),
           row("x_extent", x_extent), row("x0_quadrature_order", x0_quadrature_order),
           row("jac_x0_quadrature_order", jac_x0_quadrature_order), row("x0_extent", x0_extent),
           row("q0_quadrature_order", q0_quadrature_order), row("jac_q0_quadrature_order", jac_q0_quadrature_order),
           row("q0_extent", q0_extent), row("angle_quadrature_order", angle_quadrature_order),
           row("jac_angle_quadrature_order", jac_angle_quadrature_order), row("T", T)},
          10, 0);
    }

    template <typename NT, int d, typename FUN> NT integrate(const FUN &fun) const { return integrate<NT, d>(fun, k); }
    template <typename NT, int d, typename FUN> NT angle_integrate(const FUN &fun) const
    {
      return angle_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT two_angle_integrate(const FUN &fun) const
    {
      return two_angle_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT three_angle_integrate(const FUN &fun) const
    {
      return three_angle_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT spatial_integrate_and_integrate(const FUN &fun) const
    {
      return spatial_integrate_and_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT spatial_angle_integrate_and_integrate(const FUN &fun) const
    {
      return spatial_angle_integrate_and_integrate<NT, d>(fun, k);
    }
    template <typename NT, int d, typename FUN> NT spatial_integrate_and_sum(const FUN &fun, const double T) const
    {
      return spatial_integrate_and_sum<NT, d>(fun, T, k);
    }
    template <typename NT, int d, typename FUN> NT spatial_angle_integrate_and_sum(const FUN &fun, const double T) const
    {
      return spatial_angle_integrate_and_sum<NT, d>(fun, T, k);
    }
    template <typename NT, typename FUN> NT sum(const FUN &fun, const double T) const { return sum<NT>(fun, T, k); }

    template <typename NT, int d, typename FUN> NT integrate(const FUN &fun, const double k) const
    {
      return LoopIntegrals::integrate<NT, d>(fun, xq<NT>(), x_extent, k);
    }
    template <typename NT, int d, typename FUN> NT angle_integrate(const FUN &fun, const double k) const
    {
      return LoopIntegrals::angle_integrate<NT, d>(fun, xq<NT>(), x_extent, k, aq<NT>());
    }
    template <typename NT, int d, typename FUN> NT two_angle_integrate(const FUN &fun, const double k) const
    {
      return LoopIntegrals::two_angle_integrate<NT, d>(fun, xq<NT>(), x_extent, k, aq<NT>());
    }
    template <typename NT, int d, typename FUN> NT three_angle_integrate(const FUN &fun, const double k) const
    {
      return LoopIntegrals::three_angle_integrate<NT, d>(fun, xq<NT>(), x_extent, k, aq<NT>());
    }
    template <typename NT, int d, typename FUN> NT spatial_integrate_and_integrate(const FUN &fun, const double k) const
    {
      return LoopIntegrals::spatial_integrate_and_integrate<NT, d>(fun, xq<NT>(), x_extent, k, q0q<NT>(), q0_extent);
    }
    template <typename NT, int d, typename FUN>
    NT spatial_angle_integrate_and_integrate(const FUN &fun, const double k) const
    {
      return LoopIntegrals::spatial_angle_integrate_and_integrate<NT, d>(fun, xq<NT>(), x_extent, k, aq<NT>(),
                                                                         q0q<NT>(), q0_extent);
    }
    template <typename NT, int d, typename FUN>
    NT spatial_integrate_and_sum(const FUN &fun, const double T, const double k) const
    {
      return LoopIntegrals::spatial_integrate_and_sum<NT, d>(fun, xq<NT>(), x_extent, k, q0_summands, q0q<NT>(),
                                                             q0_extent, T);
    }
    template <typename NT, int d, typename FUN>
    NT spatial_angle_integrate_and_sum(const FUN &fun, const double T, const double k) const
    {
      return LoopIntegrals::spatial_angle_integrate_and_sum<NT, d>(fun, xq<NT>(), x_extent, k, aq<NT>(), q0_summands,
                                                                   q0q<NT>(), q0_extent, T);
    }
    template <typename NT, typename FUN> NT sum(const FUN &fun, const double T, const double) const
    {
      return LoopIntegrals::sum<NT>(fun, q0_summands, q0q<NT>(), q0_extent, T);
    }

    void set_jacobian_quadrature_factor(const double jacobian_quadrature_factor)
    {
      jac_x_quadrature_order = jacobian_quadrature_factor * x_quadrature_order;
      jac_x_quadrature = QGauss<1>(jac_x_quadrature_order);
      jac_angle_quadrature_order = jacobian_quadrature_factor * angle_quadrature_order;
      jac_angle_quadrature = QGauss<1>(jac_angle_quadrature_order);
      jac_x0_quadrature_order = jacobian_quadrature_factor * x0_quadrature_order;
      jac_x0_quadrature = QGauss<1>(jac_x0_quadrature_order);
      jac_q0_quadrature_order = jacobian_quadrature_factor * q0_quadrature_order;
      jac_q0_quadrature = QGauss<1>(jac_q0_quadrature_order);
    }

  protected:
    template <typename NT> const QGauss<1> &xq() const
    {
      return gbint_detail::uses_jacobian_quadrature<NT>::value ? jac_x_quadrature : x_quadrature;
    }
    template <typename NT> const QGauss<1> &aq() const
    {
      return gbint_detail::uses_jacobian_quadrature<NT>::value ? jac_angle_quadrature : angle_quadrature;
    }
    template <typename NT> const QGauss<1> &q0q() const
    {
      return gbint_detail::uses_jacobian_quadrature<NT>::value ? jac_q0_quadrature : q0_quadrature;
    }

    void update_x_extent()
    {
      x_extent = 1.;
      if (verbosity > 1) std::cout << "Optimizing x_extent" << std::endl;
      if (gbint_detail::vanishes_on_probe(optimize_x)) {
        if (verbosity > 1) std::cout << "x_extent is set to 1.\n" << std::endl;
        return;
      }
      x_extent = gbint_detail::fit_extent(
          "x_extent", "x_quadrature_order", x_quadrature_order, 1., x_extent_tolerance, 2, verbosity,
          [&](const QGauss<1> &q, double ext) { return LoopIntegrals::integrate<double, 4>(optimize_x, q, ext, k); },
          false);
    }
    void update_q0_extent()
    {
      if (verbosity > 1) std::cout << "Optimizing q0_extent" << std::endl;
      q0_extent = gbint_detail::fit_extent(
          "q0_extent", "q0_quadrature_order", q0_quadrature_order, 0.5 * std::sqrt(x_extent) * k, q0_extent_tolerance,
          2, verbosity,
          [&](const QGauss<1> &q, double ext) { return std::abs(LoopIntegrals::sum<double>(optimize_q0, 0, q, ext, 0.)); },
          true);
    }
    void update_x0_extent()
    {
      // the fitted extent is x0_extent; its integrals run over [0, x0_extent k] (flow_equations.cc:275-277)
      if (verbosity > 1) std::cout << "Optimizing x0_extent" << std::endl;
      x0_extent = gbint_detail::fit_extent(
          "x0_extent", "x0_quadrature_order", x0_quadrature_order, 0.5 * std::sqrt(x_extent), x0_extent_tolerance, 1,
          verbosity,
          [&](const QGauss<1> &q, double ext) {
            return std::abs(LoopIntegrals::sum<double>(optimize_x0, 0, q, ext * k, 0.));
          },
          true);
    }

    const unsigned x_quadrature_order;
    const QGauss<1> x_quadrature;
    double x_extent;

    const unsigned x0_summands;
    const unsigned x0_quadrature_order;
    const QGauss<1> x0_quadrature;
    double x0_extent;

    const unsigned q0_summands;
    const unsigned q0_quadrature_order;
    const QGauss<1> q0_quadrature;
    double q0_extent;

    const unsigned angle_quadrature_order;
    const QGauss<1> angle_quadrature;

    double jacobian_quadrature_factor;

    unsigned jac_x_quadrature_order;
    QGauss<1> jac_x_quadrature;
    unsigned jac_x0_quadrature_order;
    QGauss<1> jac_x0_quadrature;
    unsigned jac_q0_quadrature_order;
    QGauss<1> jac_q0_quadrature;
    unsigned jac_angle_quadrature_order;
    QGauss<1> jac_angle_quadrature;

    const double x_extent_tolerance;
    const double x0_extent_tolerance;
    const double q0_extent_tolerance;

    const double T;

    const std::function<double(double)> optimize_x;
    const std::function<double(double)> optimize_x0;
    const std::function<double(double)> optimize_q0;

    double k;
    bool unoptimized;
    const int verbosity;
  };
} // namespace DiFfRG
