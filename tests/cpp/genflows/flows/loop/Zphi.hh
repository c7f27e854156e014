// Test flow in the generator's layout: a two-propagator vertex loop with seven 1D dressing tables.
#pragma once

template <typename REG> class Zphi_kernel;
#include "../def.hh"

#include <future>
#include <memory>

namespace DiFfRG
{
  namespace Flows
  {
    class Zphi_integrator
    {
    public:
      using Tab = TexLinearInterpolator1D<double, LogarithmicCoordinates1D<float>>;
      Zphi_integrator(QuadratureProvider &quadrature_provider, std::array<uint, 2> grid_sizes, const double x_extent,
                      const JSONValue &json);
      Zphi_integrator(const Zphi_integrator &other);
      ~Zphi_integrator();

      template <typename NT, typename... T> std::future<NT> request(T &&...t)
      {
        static_assert(std::is_same_v<NT, double>, "Unknown type requested of Zphi_integrator::request");
        return request_CT(std::forward<T>(t)...);
      }
      template <typename NT, typename... T> NT get(T &&...t)
      {
        static_assert(std::is_same_v<NT, double>, "Unknown type requested of Zphi_integrator::get");
        return get_CT(std::forward<T>(t)...);
      }

    private:
      std::future<double> request_CT(const double k, const double p, const Tab &Zs, const Tab &Zf, const Tab &lam3,
                                     const Tab &lam4, const Tab &dtZs, const Tab &etaS, const Tab &Zv, const double m2);
      double get_CT(const double k, const double p, const Tab &Zs, const Tab &Zf, const Tab &lam3, const Tab &lam4,
                    const Tab &dtZs, const Tab &etaS, const Tab &Zv, const double m2);

      QuadratureProvider &quadrature_provider;
      const std::array<uint, 2> grid_sizes;
      const double x_extent;
      const JSONValue json;
      std::unique_ptr<DiFfRG::IntegratorAngleGPU<4, double, Zphi_kernel<__REGULATOR__>>> integrator;
    };
  } // namespace Flows
} // namespace DiFfRG
