#define FLOW_CODE

#include "Zphi.hh"
#include "Zphi.kernel"

namespace DiFfRG
{
  namespace Flows
  {
    Zphi_integrator::Zphi_integrator(QuadratureProvider &quadrature_provider, std::array<uint, 2> grid_sizes,
                                     const double x_extent, const JSONValue &json)
        : quadrature_provider(quadrature_provider), grid_sizes(grid_sizes), x_extent(x_extent), json(json),
          integrator(std::make_unique<DiFfRG::IntegratorAngleGPU<4, double, Zphi_kernel<__REGULATOR__>>>(
              quadrature_provider, grid_sizes, x_extent, json))
    {
    }
    Zphi_integrator::Zphi_integrator(const Zphi_integrator &other)
        : Zphi_integrator(other.quadrature_provider, other.grid_sizes, other.x_extent, other.json)
    {
    }
    Zphi_integrator::~Zphi_integrator() = default;

    std::future<double> Zphi_integrator::request_CT(const double k, const double p, const Tab &Zs, const Tab &Zf,
                                                    const Tab &lam3, const Tab &lam4, const Tab &dtZs, const Tab &etaS,
                                                    const Tab &Zv, const double m2)
    {
      return integrator->request(k, p, Zs, Zf, lam3, lam4, dtZs, etaS, Zv, m2);
    }
    double Zphi_integrator::get_CT(const double k, const double p, const Tab &Zs, const Tab &Zf, const Tab &lam3,
                                   const Tab &lam4, const Tab &dtZs, const Tab &etaS, const Tab &Zv, const double m2)
    {
      return integrator->get(k, p, Zs, Zf, lam3, lam4, dtZs, etaS, Zv, m2);
    }
  } // namespace Flows
} // namespace DiFfRG
