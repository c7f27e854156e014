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
// translation unit (nvcc), into one fused persistent kernel per family and argument signature
// (gbint/device/user_batch.cuh): nodes, weights and interpolator tables staged into shared memory
// by TMA bulk copies, points evaluated and reduced in FP64 per work unit, each integral finished
// by its last unit -- no per-point global buffer and no CUB pass.  request() launches at once,
// or, inside a RequestBatch scope (request_data / get_data open one per external grid), joins one
// launch with every other request of the scope.
// NT = double evaluates in FP64; NT = float in FP32 with Kahan-compensated accumulation.
// Everything else goes through the C ABI of libgbint (gbint.h): quadrature storage, streams,
// reduction scratch, result transfer.  Errors throw std::runtime_error, as the reference does.
//
// Differences from the reference, deliberate: angular axes may have different orders;
// request() launches immediately on a pooled stream and its future waits for it (the
// reference defers the reduction to get()); interpolation is exact linear interpolation
// (gbint::Table views), not 8-bit-fraction texture filtering.
#pragma once

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <typeindex>
#include <typeinfo>
#include <vector>

#include <cuda_runtime.h>
#include <cuda/std/complex>

#include "gbint.h"
#include "gbint/device/families.cuh"
#include "gbint/device/user_batch.cuh"

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
    // the owning handle: in-flight launches hold it, so the context outlives them (copying it is
    // an atomic increment, no allocation per request)
    const std::shared_ptr<gb_ctx> &ctx_shared() const { return ctx_; }
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
  // batched launches of the fused kernel (gbint/device/user_batch.cuh)
  // ---------------------------------------------------------------------------------------
  namespace gbint_detail
  {
    constexpr int kMaxBatchItems = 16384;       // a batch launches when it reaches this size
    constexpr unsigned kStageCapBytes = 32768;  // shared memory a launch stages per CTA

    // launches in which a CTA read its staged arrays from global memory instead (staging wait
    // ran out, or an array was not 16-byte aligned) -- results are valid either way
    inline std::atomic<long long> &staging_fallbacks()
    {
      static std::atomic<long long> n{0};
      return n;
    }

    // The device results of one launch.  Their copy to the slot's pinned staging (results and the
    // launch's error word, adjacent in the arena) is queued right behind the kernel; wait()
    // synchronises once, takes the values, releases the request slot and turns a CUDA error into
    // an exception.
    class LaunchResult
    {
    public:
      // queued: the launcher already queued the read-back of results + error word into `pinned`
      LaunchResult(std::shared_ptr<gb_ctx> keep, gb_slot slot, int n_values, const double *d_values, const int *d_err,
                   double *pinned, bool queued = false)
          : keep_(std::move(keep)), slot_(slot), host_(n_values), d_values_(d_values), d_err_(d_err), pinned_(pinned),
            queued_(queued)
      {
      }
      ~LaunchResult()
      {
        if (!done_) {  // never waited for: drain and give the slot back
          cudaStreamSynchronize((cudaStream_t)slot_.stream);
          gb_slot_release(keep_.get(), &slot_);
        }
      }
      const double *wait()
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!done_) {
          cudaStream_t s = (cudaStream_t)slot_.stream;
          int *perr = reinterpret_cast<int *>(pinned_ + host_.size());
          cudaError_t e = cudaSuccess;
          if (!queued_) {
            e = cudaMemcpyAsync(pinned_, d_values_, host_.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(perr, d_err_, sizeof(int), cudaMemcpyDeviceToHost, s);
          }
          if (e == cudaSuccess) e = cudaStreamSynchronize(s);
          if (e == cudaSuccess) {
            std::memcpy(host_.data(), pinned_, host_.size() * sizeof(double));
            // staging that gave up only means the CTA read global memory: results are valid
            if (*perr != 0) staging_fallbacks()++;
          }
          gb_slot_release(keep_.get(), &slot_);
          done_ = true;
          if (e != cudaSuccess) error_ = std::string("integrator kernel: ") + cudaGetErrorString(e);
        }
        if (!error_.empty()) throw std::runtime_error(error_);
        return host_.data();
      }

    private:
      std::shared_ptr<gb_ctx> keep_;
      gb_slot slot_;
      std::vector<double> host_;
      const double *d_values_;
      const int *d_err_;
      double *pinned_;
      bool queued_ = false;
      std::mutex mu_;
      bool done_ = false;
      std::string error_;
    };

    // A batch of integrals of one fused-kernel type (family, KERNEL, result and argument types):
    // add() collects them, launch() runs them all in one persistent launch.
    class BatchBase
    {
    public:
      virtual ~BatchBase() = default;
      virtual void launch() = 0;
      virtual size_t size() const = 0;
      virtual bool launched() const = 0;
      // still taking requests: not launched and below the batch size limit (one lock)
      virtual bool accepting() const = 0;
    };

    template <class FAM, class KERNEL, typename NT, typename ctype, class... T> class UserBatch : public BatchBase
    {
    public:
      using ItemT = gbint::ub::Item<ctype, T...>;
      UserBatch(QuadratureProvider &qp, const std::shared_ptr<gb_ctx> &keep) : qp_(&qp), keep_(keep) {}

      int add(const gbint::fam::Params<ctype> &P, const T &...t)
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (launched_) throw std::logic_error("integrator batch: add after launch");
        const long long n = FAM::points(P);
        if (n <= 0) throw std::runtime_error("integrator: empty quadrature grid");
        const long long per = gbint::ub::unit_points(n);
        const long long u = (n + per - 1) / per;
        if (units_ + u > (1ll << 28)) throw std::runtime_error("integrator: grid too large");
        if (items_.empty()) {  // the staging plan follows the first integral
          if constexpr (sizeof...(T) > 0) tables_ = tables_of(t...);
          // descriptors are ~1 KB with interpolator arguments: no re-copying while a grid's
          // requests arrive
          items_.reserve(256);
          unit_begin_.reserve(256);
        }
        items_.push_back(ItemT{P, gbint::ub::make_pack(t...)});
        unit_begin_.push_back((int)units_);
        units_ += u;
        return (int)items_.size() - 1;
      }
      size_t size() const override
      {
        std::lock_guard<std::mutex> lk(mu_);
        return items_.size();
      }
      bool launched() const override
      {
        std::lock_guard<std::mutex> lk(mu_);
        return launched_;
      }
      bool accepting() const override
      {
        std::lock_guard<std::mutex> lk(mu_);
        return !launched_ && items_.size() < (size_t)kMaxBatchItems;
      }
      void launch() override;
      // the launch's results (launching the batch first if nobody has)
      std::shared_ptr<LaunchResult> result()
      {
        launch();
        return result_;
      }
      // the host values of the launch, C doubles per integral; after the first call a lock-free
      // read (the futures of a grid read them one after another)
      const double *values()
      {
        if (const double *v = values_.load(std::memory_order_acquire)) return v;
        launch();
        const double *v = result_->wait();
        values_.store(v, std::memory_order_release);
        return v;
      }

    private:
      // (device pointer, bytes) of every interpolator argument with a device table
      template <class A> static void table_of(const A &a, std::vector<std::pair<const void *, unsigned>> &out)
      {
        if constexpr (gbint::ub::is_stageable<A>::value) out.emplace_back(a.device_data(), (unsigned)a.table_bytes());
      }
      static std::vector<std::pair<const void *, unsigned>> tables_of(const T &...t)
      {
        std::vector<std::pair<const void *, unsigned>> out;
        (table_of(t, out), ...);
        return out;
      }
      // shared arrays of the launch, from its first integral: rule arrays (axes, Matsubara), then
      // interpolator tables, each once, while they fit the staging budget
      gbint::ub::StagePlan plan() const
      {
        gbint::ub::StagePlan pl;
        const ItemT &it = items_.front();
        auto add = [&](const void *src, size_t bytes) {
          if (!src || bytes == 0 || pl.n >= gbint::ub::kMaxStage) return;
          if (reinterpret_cast<uintptr_t>(src) & 15) return;
          for (int s = 0; s < pl.n; ++s)
            if (pl.src[s] == src) return;
          const unsigned b = (unsigned)((bytes + 15) & ~size_t(15));
          if (pl.total + b > kStageCapBytes) return;
          pl.src[pl.n] = src;
          pl.off[pl.n] = pl.total;
          pl.bytes[pl.n] = b;
          pl.total += b;
          ++pl.n;
        };
        for (int a = 0; a < 4; ++a)
          if (it.P.n[a] > 0) {
            add(it.P.x[a], (size_t)it.P.n[a] * sizeof(ctype));
            add(it.P.w[a], (size_t)it.P.n[a] * sizeof(ctype));
          }
        if (it.P.nm > 0) {
          add(it.P.mx, (size_t)it.P.nm * sizeof(ctype));
          add(it.P.mw, (size_t)it.P.nm * sizeof(ctype));
        }
        for (const auto &t : tables_) add(t.first, t.second);
        return pl;
      }

      QuadratureProvider *qp_;
      std::shared_ptr<gb_ctx> keep_;
      std::vector<ItemT> items_;
      std::vector<std::pair<const void *, unsigned>> tables_;
      std::vector<int> unit_begin_;
      long long units_ = 0;
      mutable std::mutex mu_;
      bool launched_ = false;
      std::shared_ptr<LaunchResult> result_;
      std::atomic<const double *> values_{nullptr};
    };

#ifdef __CUDACC__
    template <class FAM, class KERNEL, typename NT, typename ctype, class... T>
    void UserBatch<FAM, KERNEL, NT, ctype, T...>::launch()
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (launched_) return;
      launched_ = true;
      if (items_.empty()) return;
      using TR = nt_traits<NT>;
      constexpr int C = TR::C;
      const int n = (int)items_.size();
      const int units = (int)units_;
      // the fields that differ between the integrals (the rest travel once, as item 0): compared
      // bytewise against item 0, each varying field 16-byte aligned in a per-integral row
      static_assert(alignof(ItemT) <= 16, "integrator batch: argument types aligned beyond 16 bytes");
      gbint::ub::Varying var{};
      struct FieldAt {
        size_t off, bytes;
      };
      std::array<FieldAt, gbint::ub::kMaxFields> fat{};
      if (n > 1) {
        const char *b0 = reinterpret_cast<const char *>(&items_.front());
        gbint::ub::for_each_field(
            items_.front(),
            [&](int f, const void *p, size_t bytes) {
              fat[f] = FieldAt{(size_t)(static_cast<const char *>(p) - b0), bytes};
              for (int i = 1; i < n; ++i)
                if (std::memcmp(reinterpret_cast<const char *>(&items_[i]) + fat[f].off, p, bytes) != 0) {
                  var.mask |= 1u << f;
                  break;
                }
            },
            std::index_sequence_for<T...>{});
        for (int f = 0; f < gbint::ub::kMaxFields; ++f)
          if ((var.mask >> f) & 1u) {
            var.off[f] = (unsigned short)var.stride;
            var.stride += (unsigned)((fat[f].bytes + 15) / 16 * 16);
          }
        if (var.stride > 60000) throw std::runtime_error("integrator batch: varying arguments too large");
      }
      const bool rowed = n > 1 && var.mask != 0;
      // one slot arena, in doubles: partials | results | error word | arrivals | unit_begin | rows
      const size_t d_part = (size_t)units * C, d_res = (size_t)n * C, d_err = 1;
      const size_t d_arr = ((size_t)n * sizeof(int) + 7) / 8;
      const size_t d_head = d_part + d_res + d_err + d_arr;
      const size_t ub_d = ((size_t)(n + 1) * sizeof(int) + 7) / 8;
      // unit_begin padded so that the rows start on a 16-byte boundary
      const size_t d_ub = n > 1 ? ub_d + ((d_head + ub_d) & 1) : 0;
      const size_t d_items = rowed ? ((size_t)n * var.stride + 7) / 8 : 0;
      const size_t total = d_head + d_ub + d_items;
      if (total > (size_t)(1u << 30)) throw std::runtime_error("integrator batch: too large");
      gb_slot slot;
      check(qp_->ctx(), gb_slot_acquire(qp_->ctx(), (int)total, &slot), "gb_slot_acquire");
      double *base = slot.partials;
      double *partials = base, *results = base + d_part;
      int *err = reinterpret_cast<int *>(base + d_part + d_res);
      int *arrivals = reinterpret_cast<int *>(base + d_part + d_res + d_err);
      int *d_unit_begin = n > 1 ? reinterpret_cast<int *>(base + d_head) : nullptr;
      char *d_rows = rowed ? reinterpret_cast<char *>(base + d_head + d_ub) : nullptr;
      cudaStream_t s = (cudaStream_t)slot.stream;
      // pinned host staging of the slot: [read-back: C doubles per integral + error word | upload:
      // zeroed error word and arrivals, unit_begin, rows] -- error word to rows are adjacent in the
      // arena, so one copy clears the counters and uploads the batch
      const size_t d_zero = d_err + d_arr;
      const size_t up_bytes = n > 1 ? (d_zero + d_ub + d_items) * sizeof(double) : 0;
      const size_t back_bytes = (d_res + 1) * sizeof(double);
      void *pin = nullptr;
      const int rc = gb_slot_host(qp_->ctx(), &slot, back_bytes + up_bytes, &pin);
      if (rc != GB_OK) {
        gb_slot_release(qp_->ctx(), &slot);
        check(qp_->ctx(), rc, "gb_slot_host");
      }
      cudaError_t e = cudaSuccess;
      if (n == 1) {
        e = cudaMemsetAsync(err, 0, d_zero * sizeof(double), s);
      } else {
        char *up = static_cast<char *>(pin) + back_bytes;
        std::memset(up, 0, d_zero * sizeof(double));
        int *ub = reinterpret_cast<int *>(up + d_zero * sizeof(double));
        std::memcpy(ub, unit_begin_.data(), n * sizeof(int));
        ub[n] = units;
        if (rowed) {
          char *rows = up + (d_zero + d_ub) * sizeof(double);
          for (int i = 0; i < n; ++i) {
            const char *src = reinterpret_cast<const char *>(&items_[i]);
            char *row = rows + (size_t)i * var.stride;
            for (int f = 0; f < gbint::ub::kMaxFields; ++f)
              if ((var.mask >> f) & 1u) std::memcpy(row + var.off[f], src + fat[f].off, fat[f].bytes);
          }
        }
        e = cudaMemcpyAsync(err, up, up_bytes, cudaMemcpyHostToDevice, s);
      }
      const gbint::ub::StagePlan pl = plan();
      // persistent grid: a warp per unit, up to as many CTAs as fit on the GPU at once (each
      // stages the shared arrays); the occupancy per staging size is looked up once per kernel
      // type
      auto kern = gbint::ub::k_user_batch<FAM, KERNEL, NT, ctype, TR, T...>;
      static std::mutex occ_mu;
      static std::map<unsigned, int> occ;
      int per_sm = 0;
      {
        std::lock_guard<std::mutex> lk2(occ_mu);
        auto it = occ.find(pl.total);
        if (it != occ.end())
          per_sm = it->second;
        else {
          if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, gbint::ub::kThreads, pl.total) != cudaSuccess ||
              per_sm < 1)
            per_sm = 1;
          occ[pl.total] = per_sm;
        }
      }
      const int per_cta = gbint::ub::kThreads / gbint::ub::kUnitLanes;
      // a grid of equal quadratures: the kernel finds a unit's integral by division
      int upi = units % n == 0 ? units / n : 0;
      for (int i = 1; i < n && upi > 0; ++i)
        if (unit_begin_[i] != i * upi) upi = 0;
      const int ctas = (int)std::min<long long>((units + per_cta - 1) / per_cta, (long long)qp_->num_sms() * per_sm);
      if (e == cudaSuccess) {
        kern<<<ctas, gbint::ub::kThreads, pl.total, s>>>(items_.front(), d_rows, var, d_unit_begin, upi, n, units, pl,
                                                          partials, slot.counters, arrivals, results, err);
        e = cudaGetLastError();
      }
      // the read-back of results and error word (adjacent in the arena) right behind the kernel
      if (e == cudaSuccess) e = cudaMemcpyAsync(pin, results, back_bytes, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) {
        cudaStreamSynchronize(s);
        gb_slot_release(qp_->ctx(), &slot);
        check_cuda(e, "integrator kernel launch");
      }
      result_ = std::make_shared<LaunchResult>(keep_, slot, n * C, results, err, static_cast<double *>(pin), true);
    }
#endif // __CUDACC__

    // the future of integral `idx` of a batch: constant + its components
    template <typename NT, class B> std::future<NT> batch_future(std::shared_ptr<B> b, int idx, NT constant)
    {
      return std::async(std::launch::deferred, [b = std::move(b), idx, constant]() {
        const double *v = b->values() + (size_t)idx * nt_traits<NT>::C;
        return constant + nt_traits<NT>::make(v);
      });
    }
  } // namespace gbint_detail

  // ---------------------------------------------------------------------------------------
  // RequestBatch: the requests a thread issues while one is alive go into one launch per kernel
  // type, launched when the scope ends (or flush(), or a future's get()).  request_data and
  // get_data open one around a whole external grid, so that all its integrals run in a single
  // persistent launch instead of one launch each.  Results are bit-identical to single gets.
  // ---------------------------------------------------------------------------------------
  class RequestBatch;
  namespace gbint_detail
  {
    // the innermost RequestBatch alive on this thread (nullptr: requests launch at once)
    inline RequestBatch *&tl_request_scope_ptr()
    {
      static thread_local RequestBatch *p = nullptr;
      return p;
    }
  } // namespace gbint_detail

  class RequestBatch
  {
  public:
    RequestBatch() : prev_(gbint_detail::tl_request_scope_ptr()) { gbint_detail::tl_request_scope_ptr() = this; }
    ~RequestBatch()
    {
      try {
        flush();
      } catch (...) {
        // a failed launch surfaces again at the futures' get()
      }
      gbint_detail::tl_request_scope_ptr() = prev_;
    }
    RequestBatch(const RequestBatch &) = delete;
    RequestBatch &operator=(const RequestBatch &) = delete;

    // launch everything collected so far
    void flush()
    {
      auto order = std::move(order_);
      order_.clear();
      open_.clear();
      for (auto &b : order) b->launch();
    }

    // the open batch of type B for the provider's context
    template <class B> std::shared_ptr<B> batch(QuadratureProvider &qp, const std::shared_ptr<gb_ctx> &keep)
    {
      // key: the provider's context and a per-batch-type tag address (pointer comparisons only;
      // comparing the types' long mangled names would cost more than the request itself)
      static const char tag = 0;
      const auto key = std::make_pair((const void *)qp.ctx(), (const void *)&tag);
      auto it = open_.find(key);
      // a batch that is full, or that a future's get() already launched, is closed
      if (it != open_.end() && !it->second->accepting()) {
        it->second->launch();
        open_.erase(it);
        it = open_.end();
      }
      if (it == open_.end()) {
        auto b = std::make_shared<B>(qp, keep);
        order_.push_back(b);
        it = open_.emplace(key, b).first;
      }
      return std::static_pointer_cast<B>(it->second);
    }

  private:
    RequestBatch *prev_;
    std::map<std::pair<const void *, const void *>, std::shared_ptr<gbint_detail::BatchBase>> open_;
    std::vector<std::shared_ptr<gbint_detail::BatchBase>> order_;
  };

  namespace gbint_detail
  {
    // one request: into the thread's open RequestBatch if there is one, else launched at once
    template <class FAM, class KERNEL, typename NT, typename ctype, class... T>
    std::future<NT> submit(QuadratureProvider &qp, const std::shared_ptr<gb_ctx> &keep, const gbint::fam::Params<ctype> &P,
                           NT constant, const T &...t)
    {
      using B = UserBatch<FAM, KERNEL, NT, ctype, T...>;
      if (RequestBatch *scope = tl_request_scope_ptr()) {
        auto b = scope->template batch<B>(qp, keep);
        const int idx = b->add(P, t...);
        return batch_future<NT>(std::move(b), idx, constant);
      }
      auto b = std::make_shared<B>(qp, keep);
      const int idx = b->add(P, t...);
      b->launch();
      return batch_future<NT>(std::move(b), idx, constant);
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
        return submit<FAM, KERNEL, NT, ctype>(*qp_, qp_->ctx_shared(), P, c, t...);
      }

    protected:
      void set_axis(int a, uint n)
      {
        P_.n[a] = (int)n;
        P_.x[a] = qp_->get_device_points<ctype>(n);
        P_.w[a] = qp_->get_device_weights<ctype>(n);
      }

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
    // (provider, grid sizes, x_extent, json): the generated wrapper's construction
    // (integrator_2D_cartesian_gpu.hh:70-74)
    template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>
    IntegratorCartesianGPU(QuadratureProvider &qp, const std::array<uint, dim> grid_sizes, const ctype x_extent,
                           const JSON &json)
        : IntegratorCartesianGPU(qp, grid_sizes, x_extent,
                                 gbint_detail::json_uint(json, "/integration/cudathreadsperblock", 256))
    {
    }
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
      return gbint_detail::submit<FAM, KERNEL, NT, ctype>(*qp_, qp_->ctx_shared(), P,
                                                          c, t...);
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
      return gbint_detail::submit<FAM, KERNEL, NT, ctype>(*qp_, qp_->ctx_shared(), P,
                                                          c, t...);
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
    template <class JSON, typename = decltype(std::declval<const JSON &>().get_uint(""))>
    IntegratorConstant(QuadratureProvider &, const std::array<uint, 1>, const ctype, const JSON &)
    {
    }
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
