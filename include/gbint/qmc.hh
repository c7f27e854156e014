// qmc.hh -- the quasi-Monte-Carlo momentum integrators of the drop-in: IntegratorQMC<d>,
// IntegratorAngleQMC<d>, Integrator4DQMC (DiFfRG/include/DiFfRG/physics/integration/
// integrator_qmc.hh, integrator_angle_qmc.hh, integrator_4D_qmc.hh).
//
// The reference hands the integral to the vendored qmc library (DiFfRG/include/qmc/qmc.hpp):
// a rank-1 lattice rule of n points, randomly shifted m times, no periodizing transform
// (transforms::None), the estimate the mean over the shifts and its error the standard error of
// that mean; n or m grows until error <= max(epsabs, epsrel |I|) or maxeval points were spent.
// Here the same estimator and schedule run GB300-first: one launch per sample evaluates all n x m
// lattice points (the KERNEL in NT, one CTA row per shift, FP64 block sums), the host sums each
// shift's blocks in a fixed order and applies the schedule, restated from qmc.hpp's
// Qmc::update / core::reduce: the error ratio min(err / epsabs, |err / (I epsrel)|) capped at 20,
// the expected error scaling n^-0.8, Knuth's online mean and variance over the shifts, the shifts
// of a repeated lattice merged into the previous estimate.
// The lattices are this library's own (the reference's come from its CBC tables): n a prime from
// a geometric ladder (ratio ~1.09 from 1021), Korobov generating vectors (1, a, a^2, ...) mod n
// with a the best of a candidate set under the P_2 figure of merit (product weights 1), chosen
// once per (n, dimension) and cached.  The shifts come from a std::mt19937_64 seeded per
// integrator; the reference seeds its generator from std::random_device, so its own results vary
// from run to run by the error estimate, and parity with it is statistical (as its tests check).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <future>
#include <map>
#include <mutex>
#include <random>
#include <stdexcept>
#include <vector>

#include "gbint/integrators.hh"

namespace gbint
{
  namespace qmc
  {
    // unit-cube point -> weight * KERNEL(coordinates, k, args): the reference's functors
    template <int d> struct Q1 {  // integrator_qmc.hh:29-40
      static constexpr int S = 1;
      template <class K, typename NT, typename ctype, class... A>
      __host__ __device__ static NT eval(const ctype *x, ctype k, ctype xe, const A &...t)
      {
        const ctype q = k * sqrt(x[0] * xe);
        const ctype ie = fam::S_d<ctype>(d) * (fam::powi(q, d - 2) / 2 * k * k) / fam::powi(fam::two_pi<ctype>(), d);
        return ie * xe * K::kernel(q, k, t...);
      }
    };
    template <int d> struct Q2 {  // integrator_angle_qmc.hh:33-48
      static constexpr int S = 2;
      template <class K, typename NT, typename ctype, class... A>
      __host__ __device__ static NT eval(const ctype *x, ctype k, ctype xe, const A &...t)
      {
        const ctype q = k * sqrt(x[0] * xe);
        const ctype cs = 2 * (x[1] - (ctype)0.5);
        const ctype ie = fam::S_d<ctype>(d) * (fam::powi(q, d - 2) / (ctype)2 * k * k) * (1 / (ctype)2) /
                         fam::powi(fam::two_pi<ctype>(), d);
        return ie * (2 * xe) * K::kernel(q, cs, k, t...);
      }
    };
    struct Q4 {  // integrator_4D_qmc.hh:38-58
      static constexpr int S = 4;
      template <class K, typename NT, typename ctype, class... A>
      __host__ __device__ static NT eval(const ctype *x, ctype k, ctype xe, const A &...t)
      {
        const ctype q = k * sqrt(x[0] * xe);
        const ctype c1 = 2 * (x[1] - (ctype)0.5);
        const ctype ie = (q * q * (ctype)0.5 * k * k) * sqrt(1 - c1 * c1) / fam::powi(fam::two_pi<ctype>(), 4);
        const ctype c2 = 2 * (x[2] - (ctype)0.5);
        const ctype phi = fam::two_pi<ctype>() * x[3];
        const ctype wt = fam::two_pi<ctype>() * 2 * 2 * xe;
        return ie * wt * K::kernel(q, c1, c2, phi, k, t...);
      }
    };

    // ------------------------------------------------------------------ lattices (host)
    struct Lattice {
      uint64_t n = 0;
      uint64_t z[4] = {1, 0, 0, 0};
    };

    inline bool is_prime(uint64_t v)
    {
      if (v < 2) return false;
      for (uint64_t p = 2; p * p <= v; ++p)
        if (v % p == 0) return false;
      return true;
    }
    // the lattice sizes: the smallest prime >= 1021 * 1.09^k, up to 2^31
    inline const std::vector<uint64_t> &sizes()
    {
      static const std::vector<uint64_t> v = [] {
        std::vector<uint64_t> s;
        for (double t = 1021; t < 2147483647.0; t *= 1.09) {
          uint64_t c = (uint64_t)t;
          while (!is_prime(c)) ++c;
          if (s.empty() || c > s.back()) s.push_back(c);
        }
        return s;
      }();
      return v;
    }
    // the smallest lattice size >= preferred (the largest one if none is)
    inline uint64_t next_n(uint64_t preferred)
    {
      const auto &s = sizes();
      auto it = std::lower_bound(s.begin(), s.end(), preferred);
      return it == s.end() ? s.back() : *it;
    }
    // P_2 of the Korobov lattice (1, a, a^2, ...) mod n in dim dimensions (smaller is better)
    inline double korobov_p2(uint64_t n, uint64_t a, int dim)
    {
      uint64_t z[4] = {1, 0, 0, 0};
      for (int j = 1; j < dim; ++j) z[j] = (z[j - 1] * a) % n;
      const double c = 2.0 * M_PI * M_PI;
      double sum = 0;
      for (uint64_t i = 0; i < n; ++i) {
        double p = 1;
        for (int j = 0; j < dim; ++j) {
          const double x = (double)((i * z[j]) % n) / (double)n;
          p *= 1.0 + c * (x * x - x + 1.0 / 6.0);
        }
        sum += p;
      }
      return sum / (double)n - 1.0;
    }
    inline const Lattice &lattice(uint64_t n, int dim)
    {
      static std::mutex mu;
      static std::map<std::pair<uint64_t, int>, Lattice> cache;
      std::lock_guard<std::mutex> lk(mu);
      auto it = cache.find({n, dim});
      if (it != cache.end()) return it->second;
      Lattice L;
      L.n = n;
      uint64_t best = 1;
      if (dim > 1) {
        // candidates from a fixed sequence (the choice depends on (n, dim) only); fewer for large n
        const int cands = n <= (1u << 16) ? 48 : (n <= (1u << 20) ? 16 : (n <= (1u << 24) ? 4 : 1));
        double best_p = 1e300;
        uint64_t s = 0x9E3779B97F4A7C15ull ^ (n * 0x100000001B3ull);
        for (int c = 0; c < cands; ++c) {
          s ^= s >> 12;
          s ^= s << 25;
          s ^= s >> 27;
          const uint64_t a = 2 + (s * 2685821657736338717ull) % (n - 3);
          const double p = cands > 1 ? korobov_p2(n, a, dim) : 0.0;
          if (p < best_p) {
            best_p = p;
            best = a;
          }
        }
      }
      for (int j = 1; j < dim; ++j) L.z[j] = (L.z[j - 1] * best) % n;
      return cache.emplace(std::make_pair(n, dim), L).first->second;
    }

    // ------------------------------------------------------------------ the sample kernel
    template <typename ctype> struct QParams {
      ctype k, x_extent;
      unsigned long long n, z[4];
      int m, nblk;
    };

    template <class MAP, class KERNEL, typename NT, typename ctype, class... T, size_t... I>
    __host__ __device__ __forceinline__ NT qmc_apply(const ctype *x, const QParams<ctype> &Q,
                                                     const ub::ArgPack<T...> &a, std::index_sequence<I...>)
    {
      return MAP::template eval<KERNEL, NT>(x, Q.k, Q.x_extent, ub::pget<(int)I>(a)...);
    }

#ifdef __CUDACC__
    constexpr int kQThreads = 256;
    // blockIdx.y = shift; the CTAs of a shift stride over the n lattice points; one FP64 partial
    // per (shift, CTA, component)
    template <class MAP, class KERNEL, typename NT, typename ctype, class COMP, class... T>
    __global__ void __launch_bounds__(kQThreads)
        k_qmc(const QParams<ctype> Q, const ub::ArgPack<T...> args, const double *shifts, double *out)
    {
      constexpr int C = COMP::C, S = MAP::S;
      __shared__ double red[C][32];
      const int k = blockIdx.y;
      ctype d[S];
#pragma unroll
      for (int j = 0; j < S; ++j) d[j] = (ctype)shifts[k * S + j];
      double acc[C];
#pragma unroll
      for (int c = 0; c < C; ++c) acc[c] = 0.0;
      for (unsigned long long i = (unsigned long long)blockIdx.x * kQThreads + threadIdx.x; i < Q.n;
           i += (unsigned long long)gridDim.x * kQThreads) {
        ctype x[S];
#pragma unroll
        for (int j = 0; j < S; ++j) {
          ctype v = (ctype)((i * Q.z[j]) % Q.n) / (ctype)Q.n + d[j];
          x[j] = v >= (ctype)1 ? v - (ctype)1 : v;
        }
        const NT v = qmc_apply<MAP, KERNEL, NT>(x, Q, args, std::index_sequence_for<T...>{});
#pragma unroll
        for (int c = 0; c < C; ++c) acc[c] += (double)COMP::get(v, c);
      }
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[c][wid] = v;
      }
      __syncthreads();
      if (wid == 0) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
          double v = lane < kQThreads / 32 ? red[c][lane] : 0.0;
          for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
          if (lane == 0) out[((size_t)k * Q.nblk + blockIdx.x) * C + c] = v;
        }
      }
    }
#endif
  } // namespace qmc
} // namespace gbint

namespace DiFfRG
{
  namespace gbint_detail
  {
    // the schedule and estimator shared by the three classes
    template <class MAP, typename NT, typename KERNEL> class QMCBase
    {
    public:
      using ctype = typename get_type::ctype<NT>;
      using TR = nt_traits<NT>;
      static constexpr int C = TR::C;

      QMCBase(QuadratureProvider *qp, ctype x_extent, double rel_tol, double abs_tol, unsigned long long maxeval,
              unsigned long long minm = 32, unsigned long long minn = 512)
          : qp_(qp), x_extent_(x_extent), epsrel_(rel_tol), epsabs_(abs_tol), maxeval_(maxeval), minm_(minm),
            minn_(minn)
      {
        if (minm_ < 2) throw std::domain_error("QMC integrator: minm < 2 (at least two random shifts)");
      }

      template <typename... T> NT get(const ctype k, const T &...t) const
      {
        return (NT)KERNEL::constant(k, t...) + integrate(k, t...);
      }
      template <typename... T> std::future<NT> request(const ctype k, const T &...t) const
      {
        const NT constant = (NT)KERNEL::constant(k, t...);
        return std::async(std::launch::deferred, [this, constant, k, t...]() { return constant + integrate(k, t...); });
      }

      // the last integration's lattice size, shifts and points spent (diagnostics)
      struct Stats {
        unsigned long long n = 0, m = 0, evaluations = 0, iterations = 0;
        double error[2] = {0, 0};
      };
      Stats last_stats() const
      {
        std::lock_guard<std::mutex> lk(mu_);
        return stats_;
      }

    protected:
      QuadratureProvider &provider() const
      {
        if (qp_) return *qp_;
        static QuadratureProvider own(0);
        return own;
      }

      template <typename... T> NT integrate(const ctype k, const T &...t) const;

      QuadratureProvider *qp_;
      ctype x_extent_;
      double epsrel_, epsabs_;
      unsigned long long maxeval_, minm_, minn_;
      mutable std::mutex mu_;
      mutable std::mt19937_64 rng_{0x5DEECE66Dull};
      mutable Stats stats_;
    };

#ifdef __CUDACC__
    template <class MAP, typename NT, typename KERNEL>
    template <typename... T>
    NT QMCBase<MAP, NT, KERNEL>::integrate(const ctype k, const T &...t) const
    {
      using gbint::qmc::QParams;
      constexpr int S = MAP::S;
      QuadratureProvider &qp = provider();
      gb_ctx *ctx = qp.ctx();
      const auto args = gbint::ub::make_pack(t...);
      std::uniform_real_distribution<double> uni(0.0, 1.0);
      unsigned long long n = gbint::qmc::next_n(minn_), m = minm_;
      // running estimate of the current lattice size (shifts of the same n merge into it)
      unsigned long long prev_n = 0, prev_m = 0, evaluations = 0, iterations = 0;
      double mean[C] = {}, var[C] = {}, integral[C] = {}, error[C] = {};
      auto ratio = [&]() {
        double r = 0;
        for (int c = 0; c < C; ++c) r = std::max(r, std::min(error[c] / epsabs_, std::abs(error[c] / (integral[c] * epsrel_))));
        return r;
      };
      for (;;) {
        const gbint::qmc::Lattice &L = gbint::qmc::lattice(n, S);
        const int nblk = (int)std::max<unsigned long long>(
            1, std::min<unsigned long long>((n + 4 * gbint::qmc::kQThreads - 1) / (4 * gbint::qmc::kQThreads),
                                            std::max<unsigned long long>(1, 8ull * qp.num_sms() / m)));
        std::vector<double> shifts((size_t)m * S);
        {
          std::lock_guard<std::mutex> lk(mu_);
          for (auto &v : shifts) v = uni(rng_);
        }
        const size_t out_d = (size_t)m * nblk * C, sh_d = shifts.size();
        if (out_d + sh_d > (size_t)(1u << 30)) throw std::runtime_error("QMC integrator: sample too large");
        gb_slot slot;
        check(ctx, gb_slot_acquire(ctx, (int)(out_d + sh_d), &slot), "gb_slot_acquire");
        double *d_out = slot.partials, *d_sh = slot.partials + out_d;
        cudaStream_t s = (cudaStream_t)slot.stream;
        void *pin = nullptr;
        int rc = gb_slot_host(ctx, &slot, (out_d + sh_d) * sizeof(double), &pin);
        if (rc != GB_OK) {
          gb_slot_release(ctx, &slot);
          check(ctx, rc, "gb_slot_host");
        }
        double *h = static_cast<double *>(pin);
        std::memcpy(h + out_d, shifts.data(), sh_d * sizeof(double));
        QParams<ctype> Q{k, x_extent_, L.n, {L.z[0], L.z[1], L.z[2], L.z[3]}, (int)m, nblk};
        cudaError_t e = cudaMemcpyAsync(d_sh, h + out_d, sh_d * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
          gbint::qmc::k_qmc<MAP, KERNEL, NT, ctype, TR, T...>
              <<<dim3((unsigned)nblk, (unsigned)m), gbint::qmc::kQThreads, 0, s>>>(Q, args, d_sh, d_out);
          e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, d_out, out_d * sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
          cudaStreamSynchronize(s);
          gb_slot_release(ctx, &slot);
          check_cuda(e, "QMC sample");
        }
        // per shift: the blocks' partials in block order; then the online mean / variance of the
        // shift sums (continuing the previous estimate when the lattice is the same)
        unsigned long long m0 = 0;
        if (prev_n == n) {
          m0 = prev_m;
          for (int c = 0; c < C; ++c) {
            mean[c] = integral[c] * (double)n;
            var[c] = error[c] * error[c] * (double)(prev_m - 1) * (double)prev_m * (double)n * (double)n;
          }
        } else {
          for (int c = 0; c < C; ++c) mean[c] = var[c] = 0;
        }
        for (unsigned long long kk = 0; kk < m; ++kk)
          for (int c = 0; c < C; ++c) {
            double sum = 0;
            for (int b = 0; b < nblk; ++b) sum += h[((size_t)kk * nblk + b) * C + c];
            const double delta = sum - mean[c];
            mean[c] += delta / (double)(kk + m0 + 1);
            var[c] += delta * (sum - mean[c]);
          }
        gb_slot_release(ctx, &slot);
        const unsigned long long mt = m + m0;
        for (int c = 0; c < C; ++c) {
          integral[c] = mean[c] / (double)n;
          error[c] = std::sqrt(var[c] / ((double)(mt - 1) * (double)mt * (double)n * (double)n));
        }
        evaluations += n * m;
        ++iterations;
        prev_n = n;
        prev_m = mt;
        const double r = ratio();
        if (!(r > 1.0) || evaluations >= maxeval_) break;
        // the next sample (qmc.hpp Qmc::update): grow n by the expected error scaling, or add
        // shifts when that is cheaper or n cannot grow; stay within maxeval
        const double er = std::min(r, 20.0);
        unsigned long long new_m = minm_;
        unsigned long long new_n = gbint::qmc::next_n((unsigned long long)((double)n * std::pow(er, 1.0 / 0.8)));
        if (new_n <= n || er * er - 1.0 < (double)new_n / (double)n) {
          new_n = n;
          new_m = (unsigned long long)((double)m * er * er) + 1 - m;
        }
        if (maxeval_ < evaluations + new_n * new_m)
          new_n = std::max<unsigned long long>(n, gbint::qmc::next_n((maxeval_ - evaluations) / new_m));
        if (n == new_n && maxeval_ < evaluations + new_n * new_m)
          new_m = std::max(1ull, (maxeval_ - evaluations) / new_n);
        n = new_n;
        m = new_m;
      }
      {
        std::lock_guard<std::mutex> lk(mu_);
        stats_.n = prev_n;
        stats_.m = prev_m;
        stats_.evaluations = evaluations;
        stats_.iterations = iterations;
        for (int c = 0; c < C && c < 2; ++c) stats_.error[c] = error[c];
      }
      return TR::make(integral);
    }
#endif
  } // namespace gbint_detail

  // the reference's constructors: (x_extent, rel_tol, abs_tol, maxeval) on a process-wide device
  // context, and the generated code's (provider, grid sizes, x_extent, json) with the JSON keys
  // /integration/{rel_tol, abs_tol, max_eval} and the optional {minm, minn} (cudablocks and
  // cudathreadsperblock are accepted and unused: the launch shape follows the lattice)
#define GBINT_QMC_CTORS(NAME, NGRID)                                                                             \
  NAME(const ctype x_extent, const double rel_tol = 1e-3, const double abs_tol = 1e-14,                          \
       const unsigned long long maxeval = 100000)                                                                \
      : B(nullptr, x_extent, rel_tol, abs_tol, maxeval, 32, 512)                                                 \
  {                                                                                                              \
  }                                                                                                              \
  template <class JSON, typename = decltype(std::declval<const JSON &>().get_double(""))>                       \
  NAME(QuadratureProvider &qp, const std::array<uint, NGRID>, const ctype x_extent, const JSON &json)            \
      : B(&qp, x_extent, json.get_double("/integration/rel_tol"), json.get_double("/integration/abs_tol"),       \
          (unsigned long long)json.get_int("/integration/max_eval"),                                            \
          gbint_detail::json_uint(json, "/integration/minm", 32), gbint_detail::json_uint(json, "/integration/minn", 512)) \
  {                                                                                                              \
  }                                                                                                              \
  template <class JSON, typename = decltype(std::declval<const JSON &>().get_double(""))>                       \
  NAME(const ctype x_extent, const JSON &json)                                                                   \
      : B(nullptr, x_extent, json.get_double("/integration/rel_tol"), json.get_double("/integration/abs_tol"),   \
          (unsigned long long)json.get_int("/integration/max_eval"),                                            \
          gbint_detail::json_uint(json, "/integration/minm", 32), gbint_detail::json_uint(json, "/integration/minn", 512)) \
  {                                                                                                              \
  }

  template <int d, typename NT, typename KERNEL>
  class IntegratorQMC : public gbint_detail::QMCBase<gbint::qmc::Q1<d>, NT, KERNEL>
  {
    using B = gbint_detail::QMCBase<gbint::qmc::Q1<d>, NT, KERNEL>;

  public:
    using ctype = typename B::ctype;
    GBINT_QMC_CTORS(IntegratorQMC, 1)
  };

  template <int d, typename NT, typename KERNEL>
  class IntegratorAngleQMC : public gbint_detail::QMCBase<gbint::qmc::Q2<d>, NT, KERNEL>
  {
    using B = gbint_detail::QMCBase<gbint::qmc::Q2<d>, NT, KERNEL>;

  public:
    using ctype = typename B::ctype;
    GBINT_QMC_CTORS(IntegratorAngleQMC, 2)
  };

  template <typename NT, typename KERNEL>
  class Integrator4DQMC : public gbint_detail::QMCBase<gbint::qmc::Q4, NT, KERNEL>
  {
    using B = gbint_detail::QMCBase<gbint::qmc::Q4, NT, KERNEL>;

  public:
    using ctype = typename B::ctype;
    GBINT_QMC_CTORS(Integrator4DQMC, 4)
  };

#undef GBINT_QMC_CTORS
} // namespace DiFfRG
