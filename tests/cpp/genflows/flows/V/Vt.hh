// Test flow in the generator's layout: a finite-temperature effective-potential flow with value
// (double) and derivative (autodiff::real) integrators.
#pragma once

template <typename REG> class Vt_kernel;
#include "../def.hh"

#include <future>
#include <memory>

namespace DiFfRG
{
  namespace Flows
  {
    class Vt_integrator
    {
    public:
      Vt_integrator(QuadratureProvider &quadrature_provider, std::array<uint, 1> grid_sizes, const double x_extent,
                    const JSONValue &json);
      Vt_integrator(const Vt_integrator &other);
      ~Vt_integrator();

      template <typename NT, typename... T> std::future<NT> request(T &&...t)
      {
        static_assert(std::is_same_v<NT, double> || std::is_same_v<NT, autodiff::real>,
                      "Unknown type requested of Vt_integrator::request");
        if constexpr (std::is_same_v<NT, double>)
          return request_CT(std::forward<T>(t)...);
        else
          return request_AD(std::forward<T>(t)...);
      }
      template <typename NT, typename... T> NT get(T &&...t)
      {
        static_assert(std::is_same_v<NT, double> || std::is_same_v<NT, autodiff::real>,
                      "Unknown type requested of Vt_integrator::get");
        if constexpr (std::is_same_v<NT, double>)
          return get_CT(std::forward<T>(t)...);
        else
          return get_AD(std::forward<T>(t)...);
      }

    private:
      std::future<double> request_CT(const double k, const double N, const double T, const double rhoPhi,
                                     const double m2Pi, const double m2Sigma);
      double get_CT(const double k, const double N, const double T, const double rhoPhi, const double m2Pi,
                    const double m2Sigma);
      std::future<autodiff::real> request_AD(const double k, const double N, const double T, const double rhoPhi,
                                             const autodiff::real m2Pi, const autodiff::real m2Sigma);
      autodiff::real get_AD(const double k, const double N, const double T, const double rhoPhi,
                            const autodiff::real m2Pi, const autodiff::real m2Sigma);

      QuadratureProvider &quadrature_provider;
      const std::array<uint, 1> grid_sizes;
      std::array<uint, 1> jac_grid_sizes;
      const double x_extent;
      const double jacobian_quadrature_factor;
      const JSONValue json;
      std::unique_ptr<DiFfRG::IntegratorTBB<3, double, Vt_kernel<__REGULATOR__>>> integrator;
      std::unique_ptr<DiFfRG::IntegratorTBB<3, autodiff::real, Vt_kernel<__REGULATOR__>>> integrator_AD;
    };
  } // namespace Flows
} // namespace DiFfRG
