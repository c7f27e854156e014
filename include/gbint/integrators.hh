// integrators.hh -- DiFfRG-compatible integrator class templates on top of libgbint.
//
// Drop-in for the GPU integrator families of DiFfRG (namespace DiFfRG, same class names,
// constructor arguments and get()/request() semantics):
//   IntegratorGPU<d,NT,K>                 DiFfRG/include/DiFfRG/physics/integration/integrator_gpu.hh:21-128
//   IntegratorAngleGPU<d,NT,K>            .../integration/integrator_angle_gpu.hh:21-219
//   Integrator3DGPU<NT,K>                 .../integration/integrator_3D_gpu.hh:21-197
//   Integrator4D2AngGPU<NT,K>             .../integration/integrator_4D_2ang_gpu.hh:21-260
//   Integrator4DGPU<NT,K>                 .../integration/integrator_4D_gpu.hh:21-263
//   Integrator{1,2,3}DCartesianGPU<NT,K>  .../integration/integrator_{1,2,3}D_cartesian_gpu.hh
//   Integrator{2,3}Dp{q,x}0GPU<NT,K>      .../integration/integrator_{2,3}Dp{q,x}0_gpu.hh
//   Integrator{,Angle}FiniteTq0GPU<d,NT,K>, Integrator4DFiniteTq0GPU<NT,K>
//                                         .../integration_finiteT/integrator_*finiteTq0_gpu.hh
//   Integrator{,Angle}FiniteTx0GPU<d,NT,K>, Integrator4DFiniteTx0GPU<NT,K>
//                                         .../integration_finiteT/integrator_*finiteTx0_gpu.hh
//   IntegratorConstant<d,NT,K>            .../integration/integrator_constant.hh:11-73
//   QuadratureProvider                    .../common/quadrature/quadrature_provider.hh:138-248
//
// The user KERNEL (static kernel(...) / constant(...)) is compiled here, in the user's
// translation unit (nvcc), into one fused kernel per family: points are evaluated, reduced in
// FP64 per block and finished by the last block -- no per-point global buffer and no CUB pass.
// NT = double evaluates in FP64; NT = float in FP32 with Kahan-compensated accumulation.
// Everything else goes through the C ABI of libgbint (gbint.h): quadrature storage, streams,
// reduction scratch, result transfer.  Errors throw std::runtime_error, as the reference does.
//
// Differences from the reference, deliberate: angular axes may have different orders;
// request() launches immediately on a pooled stream and its future waits for it (the
// reference defers the reduction to get()); interpolation is exact linear interpolation
// (gbint::Table views), not 8-bit-fraction texture filtering.
#pragma once

#include <array>
#include <cmath>
#include <cstring>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>
#include <cuda/std/complex>

#include "gbint.h"
#include "gbint/device/families.cuh"

namespace DiFfRG
{
  using uint = unsigned int;

  enum class QuadratureType { legendre, chebyshev, laguerre, hermite, jacobi, count };

  namespace get_type
  {
    // coordinate type of a result type NT (the reference's get_type::ctype): NT itself for
    // float/double, the value type for complex numbers; specialise for other NT
    template <typename NT> struct ctype_of {
      using type = NT;
    };
    template <typename T> struct ctype_of<cuda::std::complex<T>> {
      using type = T;
    };
    template <typename NT> using ctype = typename ctype_of<NT>::type;
  } // namespace get_type

  namespace gbint_detail
  {
    // Result types are reduced component by component: C scalar components of type S (float:
    // Kahan-compensated FP32 per thread, double: FP64).  float and double have one component,
    // cuda::std::complex two; specialise nt_traits for other result types (e.g. a dual number
    // holding a value and a derivative) with C, S, get(v, c) and make(double[C]).
    template <typename NT, typename = void> struct nt_traits;
    template <typename NT> struct nt_traits<NT, std::enable_if_t<std::is_arithmetic_v<NT>>> {
      static constexpr int C = 1;
      using S = NT;
      __host__ __device__ static S get(const NT &v, int) { return v; }
      static NT make(const double *c) { return (NT)c[0]; }
    };
    template <typename T> struct nt_traits<cuda::std::complex<T>> {
      static constexpr int C = 2;
      using S = T;
      __host__ __device__ static S get(const cuda::std::complex<T> &v, int c) { return c ? v.imag() : v.real(); }
      static cuda::std::complex<T> make(const double *c) { return cuda::std::complex<T>((T)c[0], (T)c[1]); }
    };
  } // namespace gbint_detail

  namespace gbint_detail
  {
    inline std::string last_error(gb_ctx *ctx)
    {
      char buf[512] = {0};
      if (ctx) gb_last_error(ctx, buf, sizeof(buf));
      return std::string(buf);
    }
    inline void check(gb_ctx *ctx, int rc, const char *what)
    {
      if (rc != GB_OK)
        throw std::runtime_error(std::string(what) + ": " + gb_status_string(rc) + " (" + last_error(ctx) + ")");
    }
    inline void check_cuda(cudaError_t e, const char *what)
    {
      if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
    // JSON accessors in the style of DiFfRG's JSONValue (get_uint/get_double with a path)
    template <class JSON> unsigned json_uint(const JSON &j, const char *path, unsigned dflt)
    {
      try {
        return j.get_uint(path);
      } catch (...) {
        return dflt;
      }
    }
    template <class JSON> double json_double(const JSON &j, const char *path)
    {
      return j.get_double(path);
    }
  } // namespace gbint_detail

  // ---------------------------------------------------------------------------------------
  // QuadratureProvider: process-lifetime owner of quadrature rules (host and device copies)
  // ---------------------------------------------------------------------------------------
  class QuadratureProvider
  {
  public:
    explicit QuadratureProvider(int device = 0)
    {
      gb_ctx *c = nullptr;
      const int rc = gb_ctx_create(device, 0, &c);
      if (rc != GB_OK) throw std::runtime_error(std::string("No CUDA devices found! (") + gb_status_string(rc) + ")");
      ctx_ = std::shared_ptr<gb_ctx>(c, [](gb_ctx *p) { gb_ctx_destroy(p); });
      int dev = 0;
      gb_device_info(c, &dev, &num_sms_);
    }
    // QuadratureProvider(const JSONValue&): /integration/{vacuum_quad_size, add_matsubara_size,
    // min_matsubara_size} with the defaults of quadrature_provider.cu:220-227
    template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>
    explicit QuadratureProvider(const JSON &json) : QuadratureProvider(0)
    {
      using namespace gbint_detail;
      gbint_detail::check(ctx(), gb_quad_config(ctx(), (int)json_uint(json, "/integration/min_matsubara_size", 16),
                                                (int)json_uint(json, "/integration/vacuum_quad_size", 48),
                                                (int)json_uint(json, "/integration/add_matsubara_size", 0)),
                          "QuadratureProvider");
    }

    gb_ctx *ctx() const { return ctx_.get(); }
    int num_sms() const { return num_sms_; }

    // the rules of every QuadratureType (gb_quad_rule: GSL's fixed types with a = 0, b = 1,
    // alpha = beta = 0, as quadrature.cu:12-60 takes them)
    template <typename NT = double>
    const std::vector<NT> &get_points(const size_t order, const QuadratureType type = QuadratureType::legendre)
    {
      return host_rule<NT>(order, type).first;
    }
    template <typename NT = double>
    const std::vector<NT> &get_weights(const size_t order, const QuadratureType type = QuadratureType::legendre)
    {
      return host_rule<NT>(order, type).second;
    }
    template <typename NT = double> const std::vector<NT> &get_matsubara_points(const NT T, const NT E)
    {
      return host_mats<NT>(T, E).first;
    }
    template <typename NT = double> const std::vector<NT> &get_matsubara_weights(const NT T, const NT E)
    {
      return host_mats<NT>(T, E).second;
    }
    template <typename NT = double>
    const NT *get_device_points(const size_t order, const int = 0, const QuadratureType type = QuadratureType::legendre)
    {
      const void *dx = nullptr;
      gbint_detail::check(ctx(), gb_quad_rule(ctx(), (int)type, (int)order, dtype<NT>(), nullptr, nullptr, &dx, nullptr),
                          "get_device_points");
      return static_cast<const NT *>(dx);
    }
    template <typename NT = double>
    const NT *get_device_weights(const size_t order, const int = 0, const QuadratureType type = QuadratureType::legendre)
    {
      const void *dw = nullptr;
      gbint_detail::check(ctx(), gb_quad_rule(ctx(), (int)type, (int)order, dtype<NT>(), nullptr, nullptr, nullptr, &dw),
                          "get_device_weights");
      return static_cast<const NT *>(dw);
    }
    template <typename NT = double> const NT *get_device_matsubara_points(const NT T, const NT E, const int = 0)
    {
      const void *dx = nullptr;
      int n = 0;
      gbint_detail::check(ctx(), gb_quad_matsubara(ctx(), T, E, dtype<NT>(), &n, nullptr, nullptr, &dx, nullptr, nullptr),
                          "get_device_matsubara_points");
      return static_cast<const NT *>(dx);
    }
    template <typename NT = double> const NT *get_device_matsubara_weights(const NT T, const NT E, const int = 0)
    {
      const void *dw = nullptr;
      int n = 0;
      gbint_detail::check(ctx(), gb_quad_matsubara(ctx(), T, E, dtype<NT>(), &n, nullptr, nullptr, nullptr, &dw, nullptr),
                          "get_device_matsubara_weights");
      return static_cast<const NT *>(dw);
    }
    // the rule's own temperature (0 when the vacuum form was chosen) and its size
    double matsubara_rule_T(double T, double E)
    {
      double tr = 0;
      int n = 0;
      gbint_detail::check(ctx(), gb_quad_matsubara(ctx(), T, E, GB_DTYPE_F64, &n, nullptr, nullptr, nullptr, nullptr, &tr),
                          "matsubara");
      return tr;
    }

  private:
    template <typename NT> static int dtype()
    {
      static_assert(std::is_same_v<NT, double> || std::is_same_v<NT, float>, "double or float");
      return std::is_same_v<NT, double> ? GB_DTYPE_F64 : GB_DTYPE_F32;
    }
    template <typename NT>
    const std::pair<std::vector<NT>, std::vector<NT>> &host_rule(size_t order, QuadratureType type)
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto &cache = std::get<std::map<std::pair<int, size_t>, std::pair<std::vector<NT>, std::vector<NT>>>>(gl_);
      const std::pair<int, size_t> key{(int)type, order};
      auto it = cache.find(key);
      if (it != cache.end()) return it->second;
      const double *hx = nullptr, *hw = nullptr;
      gbint_detail::check(ctx(), gb_quad_rule(ctx(), (int)type, (int)order, GB_DTYPE_F64, &hx, &hw, nullptr, nullptr),
                          "get_points");
      auto &e = cache[key];
      e.first.assign(hx, hx + order);
      e.second.assign(hw, hw + order);
      return e;
    }
    template <typename NT> const std::pair<std::vector<NT>, std::vector<NT>> &host_mats(NT T, NT E)
    {
      std::lock_guard<std::mutex> lk(mu_);
      int n = 0;
      const double *hx = nullptr, *hw = nullptr;
      gbint_detail::check(ctx(), gb_quad_matsubara(ctx(), T, E, GB_DTYPE_F64, &n, &hx, &hw, nullptr, nullptr, nullptr),
                          "get_matsubara_points");
      auto &cache = std::get<std::map<std::pair<double, double>, std::pair<std::vector<NT>, std::vector<NT>>>>(mats_);
      auto &e = cache[{(double)T, (double)E}];
      e.first.assign(hx, hx + n);
      e.second.assign(hw, hw + n);
      return e;
    }

    std::shared_ptr<gb_ctx> ctx_;
    int num_sms_ = 1;
    std::mutex mu_;
    std::tuple<std::map<std::pair<int, size_t>, std::pair<std::vector<double>, std::vector<double>>>,
               std::map<std::pair<int, size_t>, std::pair<std::vector<float>, std::vector<float>>>>
        gl_;
    std::tuple<std::map<std::pair<double, double>, std::pair<std::vector<double>, std::vector<double>>>,
               std::map<std::pair<double, double>, std::pair<std::vector<float>, std::vector<float>>>>
        mats_;
  };

  // ---------------------------------------------------------------------------------------
  // the fused kernel and its launch
  // ---------------------------------------------------------------------------------------
  namespace gbint_detail
  {
    // forward declaration: the definition (a kernel launch) is compiled only by nvcc; a host
    // compiler translation unit (e.g. a flow's FlowEquations source, compiled by g++ as in the
    // reference's build) sees the integrator classes complete but cannot launch them
    template <typename NT> class Pending;
    template <class FAM, class KERNEL, typename NT, typename ctype, class... T>
    std::shared_ptr<Pending<NT>> launch(QuadratureProvider &qp, std::shared_ptr<gb_ctx> keep,
                                        const gbint::fam::Params<ctype> &P, NT constant, const T &...t);
  } // namespace gbint_detail

  namespace gbint_detail
  {
    constexpr int kThreads = 256;
    constexpr int kPPT = 4;
    constexpr int kUnit = kThreads * kPPT;

#ifdef __CUDACC__
    __device__ __forceinline__ double warp_sum(double v)
    {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      return v;
    }

    // persistent CTAs pull units of kUnit points; FP64 block sums per unit and component; the
    // last unit to arrive adds the unit partials in order (deterministic) and writes the C result
    // components to partials[n_units * C + c] (component 0 also to *result)
    template <class FAM, class KERNEL, typename NT, typename ctype, class... T>
    __global__ void __launch_bounds__(kThreads)
        k_user(const gbint::fam::Params<ctype> P, long long n_points, int n_units, double *partials, int *counters,
               double *result, T... t)
    {
      using TR = nt_traits<NT>;
      constexpr int C = TR::C;
      using S = typename TR::S;
      __shared__ double red[C][32];
      __shared__ int s_unit, s_last;
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(&counters[0], 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) break;
        const long long begin = (long long)u * kUnit;
        double acc[C];
        if constexpr (std::is_same_v<S, float>) {
          float s[C], c[C];  // Kahan per component
#pragma unroll
          for (int m = 0; m < C; ++m) s[m] = c[m] = 0.f;
#pragma unroll 1
          for (int k = 0; k < kPPT; ++k) {
            const long long idx = begin + threadIdx.x + k * kThreads;
            if (idx < n_points) {
              const NT v = FAM::template eval<KERNEL, NT>(P, idx, t...);
#pragma unroll
              for (int m = 0; m < C; ++m) {
                const float y = __fsub_rn((float)TR::get(v, m), c[m]);
                const float tt = __fadd_rn(s[m], y);
                c[m] = __fsub_rn(__fsub_rn(tt, s[m]), y);
                s[m] = tt;
              }
            }
          }
#pragma unroll
          for (int m = 0; m < C; ++m) acc[m] = (double)s[m] - (double)c[m];
        } else {
#pragma unroll
          for (int m = 0; m < C; ++m) acc[m] = 0.0;
#pragma unroll 1
          for (int k = 0; k < kPPT; ++k) {
            const long long idx = begin + threadIdx.x + k * kThreads;
            if (idx < n_points) {
              const NT v = FAM::template eval<KERNEL, NT>(P, idx, t...);
#pragma unroll
              for (int m = 0; m < C; ++m) acc[m] += (double)TR::get(v, m);
            }
          }
        }
#pragma unroll
        for (int m = 0; m < C; ++m) {
          acc[m] = warp_sum(acc[m]);
          if (lane == 0) red[m][wid] = acc[m];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
          for (int m = 0; m < C; ++m) {
            double s = 0;
            for (int i = 0; i < kThreads / 32; ++i) s += red[m][i];
            partials[(size_t)u * C + m] = s;
          }
          __threadfence();
          s_last = (atomicAdd(&counters[1], 1) == n_units - 1);
        }
        __syncthreads();
        if (s_last) {
          __threadfence();
          double v[C];
#pragma unroll
          for (int m = 0; m < C; ++m) v[m] = 0.0;
          for (int i = threadIdx.x; i < n_units; i += kThreads)
#pragma unroll
            for (int m = 0; m < C; ++m) v[m] += __ldcg(&partials[(size_t)i * C + m]);
#pragma unroll
          for (int m = 0; m < C; ++m) {
            v[m] = warp_sum(v[m]);
            if (lane == 0) red[m][wid] = v[m];
          }
          __syncthreads();
          if (threadIdx.x == 0) {
#pragma unroll
            for (int m = 0; m < C; ++m) {
              double s = 0;
              for (int i = 0; i < kThreads / 32; ++i) s += red[m][i];
              partials[(size_t)n_units * C + m] = s;
              if (m == 0) *result = s;
            }
          }
        }
        __syncthreads();
      }
    }

#endif // __CUDACC__

    // one launched request: resolves to constant + integral
    template <typename NT> class Pending
    {
    public:
      Pending(std::shared_ptr<gb_ctx> ctx, gb_slot slot, NT constant, int n_units)
          : ctx_(std::move(ctx)), slot_(slot), c_(constant), n_units_(n_units)
      {
      }
      NT get()
      {
        constexpr int C = nt_traits<NT>::C;
        double v[C] = {};
        int rc = gb_slot_wait(ctx_.get(), &slot_, &v[0]);
        if (rc == GB_OK && C > 1) {  // the other components, from the partials tail (stream is idle)
          const cudaError_t e = cudaMemcpy(&v[1], slot_.partials + (size_t)n_units_ * C + 1, (C - 1) * sizeof(double),
                                           cudaMemcpyDeviceToHost);
          if (e != cudaSuccess) rc = GB_ECUDA;
        }
        gb_slot_release(ctx_.get(), &slot_);
        check(ctx_.get(), rc, "request");
        return c_ + nt_traits<NT>::make(v);
      }

    private:
      std::shared_ptr<gb_ctx> ctx_;
      gb_slot slot_;
      NT c_;
      int n_units_;
    };

#ifdef __CUDACC__
    template <class FAM, class KERNEL, typename NT, typename ctype, class... T>
    std::shared_ptr<Pending<NT>> launch(QuadratureProvider &qp, std::shared_ptr<gb_ctx> keep,
                                        const gbint::fam::Params<ctype> &P, NT constant, const T &...t)
    {
      constexpr int C = nt_traits<NT>::C;
      const long long n_points = FAM::points(P);
      if (n_points <= 0) throw std::runtime_error("integrator: empty quadrature grid");
      const long long units_ll = (n_points + kUnit - 1) / kUnit;
      if (units_ll > (1ll << 28)) throw std::runtime_error("integrator: grid too large");
      const int n_units = (int)units_ll;
      gb_slot slot;
      check(qp.ctx(), gb_slot_acquire(qp.ctx(), (n_units + 1) * C, &slot), "gb_slot_acquire");
      const int ctas = (int)std::min<long long>(n_units, (long long)qp.num_sms() * 8);
      k_user<FAM, KERNEL, NT, ctype, T...><<<ctas, kThreads, 0, (cudaStream_t)slot.stream>>>(
          P, n_points, n_units, slot.partials, slot.counters, slot.result, t...);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) {
        gb_slot_release(qp.ctx(), &slot);
        check_cuda(e, "integrator kernel launch");
      }
      return std::make_shared<Pending<NT>>(std::move(keep), slot, constant, n_units);
    }
#endif // __CUDACC__

    template <typename NT> std::future<NT> as_future(std::shared_ptr<Pending<NT>> p)
    {
      return std::async(std::launch::deferred, [p]() { return p->get(); });
    }
  } // namespace gbint_detail

  // ---------------------------------------------------------------------------------------
  // base: a family over the provider's GL rules
  // ---------------------------------------------------------------------------------------
  namespace gbint_detail
  {
    template <class FAM, typename NT, typename KERNEL, int NAX> class IntegratorBase
    {
    public:
      using ctype = typename get_type::ctype<NT>;
      static_assert(nt_traits<NT>::C >= 1, "NT needs gbint_detail::nt_traits (float, double, complex built in)");

      IntegratorBase(QuadratureProvider &qp, const std::array<uint, NAX> &gs, ctype x_extent)
          : qp_(&qp), grid_sizes_(gs)
      {
        P_.x_extent = x_extent;
        for (int a = 0; a < NAX; ++a) set_axis(a, gs[a]);
      }

      template <typename... T> NT get(const ctype k, const T &...t) const { return request(k, t...).get(); }
      template <typename... T> std::future<NT> request(const ctype k, const T &...t) const
      {
        gbint::fam::Params<ctype> P = P_;
        P.k = k;
        const NT c = (NT)KERNEL::constant(k, t...);
        return as_future(launch<FAM, KERNEL, NT, ctype>(*qp_, keep(), P, c, t...));
      }

    protected:
      void set_axis(int a, uint n)
      {
        P_.n[a] = (int)n;
        P_.x[a] = qp_->get_device_points<ctype>(n);
        P_.w[a] = qp_->get_device_weights<ctype>(n);
      }
      std::shared_ptr<gb_ctx> keep() const { return std::shared_ptr<gb_ctx>(qp_->ctx(), [](gb_ctx *) {}); }

      QuadratureProvider *qp_;
      std::array<uint, NAX> grid_sizes_;
      gbint::fam::Params<ctype> P_;
    };
  } // namespace gbint_detail

#define GBINT_JSON_CTOR(NAME, NAX)                                                                              \
  template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>                        \
  NAME(QuadratureProvider &qp, const std::array<uint, NAX> grid_sizes, const ctype x_extent, const JSON &json) \
      : NAME(qp, grid_sizes, x_extent, gbint_detail::json_uint(json, "/integration/cudathreadsperblock", 256))  \
  {                                                                                                             \
  }

  template <int d, typename NT, typename KERNEL>
  class IntegratorGPU : public gbint_detail::IntegratorBase<gbint::fam::F1D<d>, NT, KERNEL, 1>
  {
    using B = gbint_detail::IntegratorBase<gbint::fam::F1D<d>, NT, KERNEL, 1>;

  public:
    using ctype = typename B::ctype;
    IntegratorGPU(QuadratureProvider &qp, const std::array<uint, 1> grid_sizes, const ctype x_extent,
                  const uint max_block_size = 256)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
    }
    IntegratorGPU(QuadratureProvider &qp, const uint grid_size, const ctype x_extent, const uint max_block_size = 256)
        : IntegratorGPU(qp, std::array<uint, 1>{{grid_size}}, x_extent, max_block_size)
    {
    }
    GBINT_JSON_CTOR(IntegratorGPU, 1)
  };

  template <int d, typename NT, typename KERNEL>
  class IntegratorAngleGPU : public gbint_detail::IntegratorBase<gbint::fam::FAngle<d>, NT, KERNEL, 2>
  {
    using B = gbint_detail::IntegratorBase<gbint::fam::FAngle<d>, NT, KERNEL, 2>;

  public:
    using ctype = typename B::ctype;
    IntegratorAngleGPU(QuadratureProvider &qp, const std::array<uint, 2> grid_sizes, const ctype x_extent,
                       const uint max_block_size = 256)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
    }
    GBINT_JSON_CTOR(IntegratorAngleGPU, 2)
  };

  template <typename NT, typename KERNEL>
  class Integrator3DGPU : public gbint_detail::IntegratorBase<gbint::fam::F3D, NT, KERNEL, 3>
  {
    using B = gbint_detail::IntegratorBase<gbint::fam::F3D, NT, KERNEL, 3>;

  public:
    using ctype = typename B::ctype;
    Integrator3DGPU(QuadratureProvider &qp, const std::array<uint, 3> grid_sizes, const ctype x_extent,
                    const uint max_block_size = 256)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
    }
    GBINT_JSON_CTOR(Integrator3DGPU, 3)
  };

  template <typename NT, typename KERNEL>
  class Integrator4D2AngGPU : public gbint_detail::IntegratorBase<gbint::fam::F4D2Ang, NT, KERNEL, 3>
  {
    using B = gbint_detail::IntegratorBase<gbint::fam::F4D2Ang, NT, KERNEL, 3>;

  public:
    using ctype = typename B::ctype;
    Integrator4D2AngGPU(QuadratureProvider &qp, const std::array<uint, 3> grid_sizes, const ctype x_extent,
                        const uint max_block_size = 256)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
    }
    GBINT_JSON_CTOR(Integrator4D2AngGPU, 3)
  };

  template <typename NT, typename KERNEL>
  class Integrator4DGPU : public gbint_detail::IntegratorBase<gbint::fam::F4D, NT, KERNEL, 4>
  {
    using B = gbint_detail::IntegratorBase<gbint::fam::F4D, NT, KERNEL, 4>;

  public:
    using ctype = typename B::ctype;
    Integrator4DGPU(QuadratureProvider &qp, const std::array<uint, 4> grid_sizes, const ctype x_extent,
                    const uint max_block_size = 256)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
    }
    GBINT_JSON_CTOR(Integrator4DGPU, 4)
  };

  // Cartesian families: qx in [qx_min, qx_max] etc. (defaults [-pi, pi]), x_extent unused
  template <int dim, typename NT, typename KERNEL>
  class IntegratorCartesianGPU : public gbint_detail::IntegratorBase<gbint::fam::FCart<dim>, NT, KERNEL, dim>
  {
    using B = gbint_detail::IntegratorBase<gbint::fam::FCart<dim>, NT, KERNEL, dim>;

  public:
    using ctype = typename B::ctype;
    IntegratorCartesianGPU(QuadratureProvider &qp, const std::array<uint, dim> grid_sizes, const ctype x_extent = 0,
                           const uint max_block_size = 0)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
      for (int a = 0; a < 3; ++a) {
        qmin_[a] = -(ctype)M_PI;
        qmax_[a] = (ctype)M_PI;
      }
      sync();
    }
    void set_qx_min(ctype v) { qmin_[0] = v; sync(); }
    void set_qy_min(ctype v) { qmin_[1] = v; sync(); }
    void set_qz_min(ctype v) { qmin_[2] = v; sync(); }
    void set_qx_max(ctype v) { qmax_[0] = v; sync(); }
    void set_qy_max(ctype v) { qmax_[1] = v; sync(); }
    void set_qz_max(ctype v) { qmax_[2] = v; sync(); }

  private:
    void sync()
    {
      for (int a = 0; a < 3; ++a) {
        this->P_.qmin[a] = qmin_[a];
        this->P_.qext[a] = qmax_[a] - qmin_[a];
      }
    }
    ctype qmin_[3], qmax_[3];
  };
  template <typename NT, typename KERNEL> using Integrator1DCartesianGPU = IntegratorCartesianGPU<1, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator2DCartesianGPU = IntegratorCartesianGPU<2, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3DCartesianGPU = IntegratorCartesianGPU<3, NT, KERNEL>;

  // explicit q0 / x0 axis at zero temperature
  template <class FAM, int NAX, typename NT, typename KERNEL>
  class IntegratorP0GPU : public gbint_detail::IntegratorBase<FAM, NT, KERNEL, NAX>
  {
    using B = gbint_detail::IntegratorBase<FAM, NT, KERNEL, NAX>;

  public:
    using ctype = typename B::ctype;
    IntegratorP0GPU(QuadratureProvider &qp, const std::array<uint, NAX> grid_sizes, const ctype x_extent,
                    const ctype q0_extent, const uint max_block_size = 256)
        : B(qp, grid_sizes, x_extent)
    {
      (void)max_block_size;
      this->P_.x0_extent = q0_extent;
    }
    template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>
    IntegratorP0GPU(QuadratureProvider &qp, const std::array<uint, NAX> grid_sizes, const ctype x_extent,
                    const ctype q0_extent, const JSON &)
        : IntegratorP0GPU(qp, grid_sizes, x_extent, q0_extent)
    {
    }
  };
  template <typename NT, typename KERNEL> using Integrator2Dpq0GPU = IntegratorP0GPU<gbint::fam::F2Dp0<false>, 3, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator2Dpx0GPU = IntegratorP0GPU<gbint::fam::F2Dp0<true>, 3, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3Dpq0GPU = IntegratorP0GPU<gbint::fam::F3Dp0<false>, 4, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3Dpx0GPU = IntegratorP0GPU<gbint::fam::F3Dp0<true>, 4, NT, KERNEL>;

  // finite temperature, Matsubara rule in q0 (integrator_finiteTq0_gpu.hh)
  template <class FAM, int NSP, typename NT, typename KERNEL> class IntegratorFiniteTq0Base
  {
  public:
    using ctype = typename get_type::ctype<NT>;
    IntegratorFiniteTq0Base(QuadratureProvider &qp, const std::array<uint, NSP> grid_sizes, const ctype x_extent,
                            const ctype T, const uint max_block_size = 256)
        : qp_(&qp), manual_E_(false)
    {
      (void)max_block_size;
      P_.x_extent = x_extent;
      for (int a = 0; a < NSP; ++a) {
        P_.n[a] = (int)grid_sizes[a];
        P_.x[a] = qp.get_device_points<ctype>(grid_sizes[a]);
        P_.w[a] = qp.get_device_weights<ctype>(grid_sizes[a]);
      }
      m_T_ = -1;
      m_E_ = -1;
      set_T(T);
    }
    template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>
    IntegratorFiniteTq0Base(QuadratureProvider &qp, const std::array<uint, NSP> grid_sizes, const ctype x_extent,
                            const JSON &json)
        : IntegratorFiniteTq0Base(qp, grid_sizes, x_extent, (ctype)gbint_detail::json_double(json, "/physical/T"))
    {
    }

    // set_T(T, E): quadrature_provider Matsubara rule for (T, E); E = 0 -> 10 T
    // (integrator_finiteTq0_cpu.hh:48-59)
    void set_T(const ctype T, const ctype E = 0)
    {
      const bool sameT = std::abs(T - m_T_) <= 1e-12 * std::max<ctype>(std::abs(T), 1);
      if (sameT && m_E_ > 0 && std::abs(E - m_E_) / std::max(E, m_E_) < 2.5e-2) return;
      m_T_ = T;
      m_E_ = (std::abs(E) < 1e-300) ? 10 * m_T_ : E;
      manual_E_ = !(std::abs(E) < 1e-300);
      P_.T = m_T_;
      P_.mx = qp_->get_device_matsubara_points<ctype>(m_T_, m_E_);
      P_.mw = qp_->get_device_matsubara_weights<ctype>(m_T_, m_E_);
      P_.nm = (int)qp_->get_matsubara_points<ctype>(m_T_, m_E_).size();
    }
    void set_E(const ctype E) { set_T(m_T_, E); }

    // non-const as in the reference: re-selects the rule when k drifts by more than 2.5 %
    // from the typical energy (integrator_finiteTq0_gpu.hh:142-147)
    template <typename... T> NT get(const ctype k, const T &...t) { return request(k, t...).get(); }
    template <typename... T> std::future<NT> request(const ctype k, const T &...t)
    {
      if (!manual_E_ && std::abs(k - m_E_) / std::max(k, m_E_) > 2.5e-2) {
        set_T(m_T_, k);
        manual_E_ = false;
      }
      gbint::fam::Params<ctype> P = P_;
      P.k = k;
      const NT c = (NT)KERNEL::constant(k, t...);
      return gbint_detail::as_future(gbint_detail::launch<FAM, KERNEL, NT, ctype>(
          *qp_, std::shared_ptr<gb_ctx>(qp_->ctx(), [](gb_ctx *) {}), P, c, t...));
    }

  private:
    QuadratureProvider *qp_;
    gbint::fam::Params<ctype> P_;
    ctype m_T_, m_E_;
    bool manual_E_;
  };
  template <int d, typename NT, typename KERNEL>
  using IntegratorFiniteTq0GPU = IntegratorFiniteTq0Base<gbint::fam::FTq0<d, 0>, 1, NT, KERNEL>;
  template <int d, typename NT, typename KERNEL>
  using IntegratorAngleFiniteTq0GPU = IntegratorFiniteTq0Base<gbint::fam::FTq0<d, 1>, 2, NT, KERNEL>;
  template <typename NT, typename KERNEL>
  using Integrator4DFiniteTq0GPU = IntegratorFiniteTq0Base<gbint::fam::FTq0<4, 2>, 3, NT, KERNEL>;

  // finite temperature, explicit sum + log-mapped tail (integrator_finiteTx0_gpu.hh)
  template <class FAM, int NSP, typename NT, typename KERNEL> class IntegratorFiniteTx0Base
  {
  public:
    using ctype = typename get_type::ctype<NT>;
    // grid_sizes: spatial orders, then the tail order (the reference adds x0_summands to it)
    IntegratorFiniteTx0Base(QuadratureProvider &qp, const std::array<uint, NSP + 1> grid_sizes, const ctype x_extent,
                            const ctype x0_extent, const uint x0_summands, const ctype T,
                            const uint max_block_size = 256)
        : qp_(&qp), tail_order_(grid_sizes[NSP]), original_x0_summands_(x0_summands)
    {
      (void)max_block_size;
      P_.x_extent = x_extent;
      P_.x0_extent = x0_extent;
      for (int a = 0; a < NSP; ++a) {
        P_.n[a] = (int)grid_sizes[a];
        P_.x[a] = qp.get_device_points<ctype>(grid_sizes[a]);
        P_.w[a] = qp.get_device_weights<ctype>(grid_sizes[a]);
      }
      set_T(T);
    }
    template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>
    IntegratorFiniteTx0Base(QuadratureProvider &qp, const std::array<uint, NSP + 1> grid_sizes, const ctype x_extent,
                            const ctype x0_extent, const uint x0_summands, const JSON &json)
        : IntegratorFiniteTx0Base(qp, grid_sizes, x_extent, x0_extent, x0_summands,
                                  (ctype)gbint_detail::json_double(json, "/physical/T"))
    {
    }

    // set_T (integrator_finiteTx0_cpu.hh:41-50): at T = 0 the summands join the tail rule
    void set_T(const ctype T)
    {
      m_T_ = T;
      const bool Tzero = std::abs(T) <= 1e-12;
      x0_summands_ = Tzero ? 0 : original_x0_summands_;
      const uint order = tail_order_ + original_x0_summands_ - x0_summands_;
      P_.T = Tzero ? 0 : T;
      P_.ns = (int)x0_summands_;
      P_.n[NSP] = (int)order;
      if (order > 0) {
        P_.x[NSP] = qp_->get_device_points<ctype>(order);
        P_.w[NSP] = qp_->get_device_weights<ctype>(order);
      }
    }
    void set_x0_extent(const ctype val) { P_.x0_extent = val; }

    template <typename... T> NT get(const ctype k, const T &...t) const { return request(k, t...).get(); }
    template <typename... T> std::future<NT> request(const ctype k, const T &...t) const
    {
      gbint::fam::Params<ctype> P = P_;
      P.k = k;
      const bool Tzero = std::abs(m_T_) <= 1e-12;
      const ctype start = (2 * (ctype)x0_summands_ * (ctype)M_PI * (Tzero ? 0 : m_T_)) / k;
      P.off = Tzero ? (ctype)1e-3 : (ctype)0;
      P.log_start = std::log(start + P.off);
      P.log_ext = std::log(P.x0_extent / (start + P.off));
      const NT c = (NT)KERNEL::constant(k, t...);
      return gbint_detail::as_future(gbint_detail::launch<FAM, KERNEL, NT, ctype>(
          *qp_, std::shared_ptr<gb_ctx>(qp_->ctx(), [](gb_ctx *) {}), P, c, t...));
    }

  private:
    QuadratureProvider *qp_;
    gbint::fam::Params<ctype> P_;
    uint tail_order_, original_x0_summands_, x0_summands_ = 0;
    ctype m_T_ = 0;
  };
  template <int d, typename NT, typename KERNEL>
  using IntegratorFiniteTx0GPU = IntegratorFiniteTx0Base<gbint::fam::FTx0<d, 0>, 1, NT, KERNEL>;
  template <int d, typename NT, typename KERNEL>
  using IntegratorAngleFiniteTx0GPU = IntegratorFiniteTx0Base<gbint::fam::FTx0<d, 1>, 2, NT, KERNEL>;
  template <typename NT, typename KERNEL>
  using Integrator4DFiniteTx0GPU = IntegratorFiniteTx0Base<gbint::fam::FTx0<4, 2>, 3, NT, KERNEL>;

  // IntegratorConstant<d>: constant + kernel(k) S_d/(2 pi)^d, evaluated on the host as the
  // reference does (integrator_constant.hh:47-52)
  template <int d, typename NT, typename KERNEL> class IntegratorConstant
  {
  public:
    using ctype = typename get_type::ctype<NT>;
    IntegratorConstant(QuadratureProvider &, const std::array<uint, 1>, const ctype, const uint = 0) {}
    IntegratorConstant(QuadratureProvider &, const uint, const ctype, const uint = 0) {}
    IntegratorConstant() {}
    template <typename... T> NT get(const ctype k, const T &...t) const
    {
      return KERNEL::constant(k, t...) + KERNEL::kernel(k, t...) * gbint::fam::S_d<ctype>(d) /
                                              gbint::fam::powi<ctype>(2 * (ctype)M_PI, d);
    }
    template <typename... T> std::future<NT> request(const ctype k, const T &...t) const
    {
      const NT v = get(k, t...);
      return std::async(std::launch::deferred, [v]() { return v; });
    }
  };

#undef GBINT_JSON_CTOR

  // The reference's CPU (TBB) integrators have the same constructors, get/request and set_T/set_E
  // as its GPU ones (DiFfRG/include/DiFfRG/physics/integration/*_cpu.hh,
  // .../integration_finiteT/*_cpu.hh); flows written against them run on the GPU classes here
  // (their KERNELs are __host__ __device__ in the generated code).
  template <int d, typename NT, typename KERNEL> using IntegratorTBB = IntegratorGPU<d, NT, KERNEL>;
  template <int d, typename NT, typename KERNEL> using IntegratorAngleTBB = IntegratorAngleGPU<d, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3DTBB = Integrator3DGPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator4D2AngTBB = Integrator4D2AngGPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator4DTBB = Integrator4DGPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator1DCartesianTBB = Integrator1DCartesianGPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator2DCartesianTBB = Integrator2DCartesianGPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3DCartesianTBB = Integrator3DCartesianGPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator2Dpq0TBB = Integrator2Dpq0GPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator2Dpx0TBB = Integrator2Dpx0GPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3Dpq0TBB = Integrator3Dpq0GPU<NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator3Dpx0TBB = Integrator3Dpx0GPU<NT, KERNEL>;
  template <int d, typename NT, typename KERNEL> using IntegratorFiniteTq0TBB = IntegratorFiniteTq0GPU<d, NT, KERNEL>;
  template <int d, typename NT, typename KERNEL>
  using IntegratorAngleFiniteTq0TBB = IntegratorAngleFiniteTq0GPU<d, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator4DFiniteTq0TBB = Integrator4DFiniteTq0GPU<NT, KERNEL>;
  template <int d, typename NT, typename KERNEL> using IntegratorFiniteTx0TBB = IntegratorFiniteTx0GPU<d, NT, KERNEL>;
  template <int d, typename NT, typename KERNEL>
  using IntegratorAngleFiniteTx0TBB = IntegratorAngleFiniteTx0GPU<d, NT, KERNEL>;
  template <typename NT, typename KERNEL> using Integrator4DFiniteTx0TBB = Integrator4DFiniteTx0GPU<NT, KERNEL>;
} // namespace DiFfRG
