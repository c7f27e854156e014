#define FLOW_CODE

#include "Vt.hh"
#include "Vt.kernel"

namespace DiFfRG
{
  namespace Flows
  {
    Vt_integrator::Vt_integrator(QuadratureProvider &quadrature_provider, std::array<uint, 1> grid_sizes,
                                 const double x_extent, const JSONValue &json)
        : quadrature_provider(quadrature_provider), grid_sizes(grid_sizes), x_extent(x_extent),
          jacobian_quadrature_factor(json.get_double("/integration/jacobian_quadrature_factor")), json(json)
    {
      integrator = std::make_unique<DiFfRG::IntegratorTBB<3, double, Vt_kernel<__REGULATOR__>>>(
          quadrature_provider, grid_sizes, x_extent, json);
      jac_grid_sizes[0] = uint(jacobian_quadrature_factor * grid_sizes[0]);
      integrator_AD = std::make_unique<DiFfRG::IntegratorTBB<3, autodiff::real, Vt_kernel<__REGULATOR__>>>(
          quadrature_provider, jac_grid_sizes, x_extent, json);
    }
    Vt_integrator::Vt_integrator(const Vt_integrator &other)
        : Vt_integrator(other.quadrature_provider, other.grid_sizes, other.x_extent, other.json)
    {
    }
    Vt_integrator::~Vt_integrator() = default;

    std::future<double> Vt_integrator::request_CT(const double k, const double N, const double T, const double rhoPhi,
                                                  const double m2Pi, const double m2Sigma)
    {
      return integrator->request(k, N, T, rhoPhi, m2Pi, m2Sigma);
    }
    double Vt_integrator::get_CT(const double k, const double N, const double T, const double rhoPhi,
                                 const double m2Pi, const double m2Sigma)
    {
      return integrator->get(k, N, T, rhoPhi, m2Pi, m2Sigma);
    }
    std::future<autodiff::real> Vt_integrator::request_AD(const double k, const double N, const double T,
                                                          const double rhoPhi, const autodiff::real m2Pi,
                                                          const autodiff::real m2Sigma)
    {
      return integrator_AD->request(k, N, T, rhoPhi, m2Pi, m2Sigma);
    }
    autodiff::real Vt_integrator::get_AD(const double k, const double N, const double T, const double rhoPhi,
                                         const autodiff::real m2Pi, const autodiff::real m2Sigma)
    {
      return integrator_AD->get(k, N, T, rhoPhi, m2Pi, m2Sigma);
    }
  } // namespace Flows
} // namespace DiFfRG
