// interpolators.hh -- DiFfRG-compatible coordinates and interpolators for user KERNELs.
//
//   LinearCoordinates1D, LogarithmicCoordinates1D, CoordinatePackND (1-3 axes)
//        DiFfRG/include/DiFfRG/discretization/grid/coordinates.hh:28-195
//   IndexStack, BosonicMatsubaraValues, FermionicMatsubaraValues
//        DiFfRG/include/DiFfRG/discretization/grid/stack_coordinates.hh
//   BosonicCoordinates1DFiniteT, FermionicCoordinates1DFiniteT
//        DiFfRG/include/DiFfRG/discretization/grid/combined_coordinates.hh:15-170
//   TexLinearInterpolator1D / 2D / 3D   DiFfRG/include/DiFfRG/physics/interpolation/tex_linear_interpolation_{1D,2D,3D}.hh
//   TexLinearInterpolator1DStack        DiFfRG/include/DiFfRG/physics/interpolation/tex_linear_interpolation_1D_stack.hh
//   LinearInterpolator1D / 2D / 3D      DiFfRG/include/DiFfRG/physics/interpolation/linear_interpolation_{1D,2D,3D}.hh
//
// Objects are trivially copyable views, passed by value into KERNEL::kernel arguments like the
// reference's: a device pointer to the data, a host pointer to the host copy, the sizes and the
// coordinates.  operator() clamps the grid index to the table and interpolates linearly in it
// (bi-/trilinearly in 2D/3D), on the host and on the device alike.  The Tex* variants keep the
// reference's FP32 data but interpolate exactly (the reference's texture filter has an 8-bit
// fraction, ~1e-3 relative, DiFfRG/tests/physics/interpolation/tex_linear_interpolation_1D_gpu.cu:55-57)
// and return NT instead of float; for double-based NT the coordinate map and the interpolation
// run in double (the reference maps in the coordinates' float type), so that the host and the
// device interpolate alike to FP64 rounding.  Device data lives in buffers of the process-wide
// interpolator context until process exit; update() copies the host data in place after the
// device drained, as the reference's update() synchronises.
#pragma once

#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>
#include <cuda/std/complex>

#include "gbint.h"

namespace gbint
{
  template <typename T> struct dual;
}

// Coordinates return std::array / std::tuple from __host__ __device__ members, as the
// reference's do; nvcc needs --expt-relaxed-constexpr for that (DiFfRG's own build passes it,
// DiFfRG/cmake/setup_build_system.cmake:193).
#if defined(__CUDACC__) && !defined(__CUDACC_RELAXED_CONSTEXPR__)
#error "gbint/interpolators.hh: compile with nvcc --expt-relaxed-constexpr (as DiFfRG does)"
#endif

namespace DiFfRG
{
  using uint = unsigned int;

  // ------------------------------------------------------------------ 1D coordinates
  template <typename NT> class LinearCoordinates1D
  {
  public:
    using ctype = NT;
    static constexpr uint dim = 1;
    LinearCoordinates1D(uint grid_extent, double start_, double stop_)
        : start((NT)start_), stop((NT)stop_), grid_extent(grid_extent)
    {
      if (grid_extent == 0) throw std::runtime_error("LinearCoordinates1D: grid_extent must be > 0");
      a = (NT)((stop_ - start_) / (grid_extent - 1.));
    }
    template <typename NT2>
    LinearCoordinates1D(const LinearCoordinates1D<NT2> &other) : LinearCoordinates1D(other.size(), other.start, other.stop)
    {
    }
    __host__ __device__ NT forward(const uint &x) const { return start + a * x; }
    __host__ __device__ NT backward(const NT &y) const { return (y - start) / a; }
    __host__ __device__ uint size() const { return grid_extent; }
    NT start, stop;

  private:
    uint grid_extent;
    NT a;
  };

  // y(i) = start + span (e^(i bias/(n-1)) - 1): n points from start to stop, denser near start
  // for bias > 0; backward(y) = (n-1)/bias * ln(1 + (y - start)/span) is the (fractional) index.
  // backward_derivative keeps the reference's expression (n-1)/(bias (y - start)).
  template <typename NT> class LogarithmicCoordinates1D
  {
  public:
    using ctype = NT;
    static constexpr uint dim = 1;
    LogarithmicCoordinates1D(uint grid_extent, NT start_, NT stop_, NT bias_)
        : start(start_), stop(stop_), bias(bias_), n_(grid_extent)
    {
      if (grid_extent == 0) throw std::runtime_error("LogarithmicCoordinates1D: a grid needs at least one point");
      idx_per_log_ = (NT)((grid_extent - 1.) / bias);
      log_per_idx_ = (NT)(bias / (grid_extent - 1.));
      span_ = (stop - start) / std::expm1(bias);
      inv_span_ = (NT)1 / span_;
    }
    template <typename NT2>
    LogarithmicCoordinates1D(const LogarithmicCoordinates1D<NT2> &other)
        : LogarithmicCoordinates1D(other.size(), (NT)other.start, (NT)other.stop, (NT)other.bias)
    {
    }
    __host__ __device__ NT forward(const uint &x) const { return span_ * expm1(log_per_idx_ * x) + start; }
    __host__ __device__ NT backward(const NT &y) const { return log1p((y - start) * inv_span_) * idx_per_log_; }
    __host__ __device__ NT backward_derivative(const NT &y) const { return idx_per_log_ / (y - start); }
    __host__ __device__ uint size() const { return n_; }
    NT start, stop, bias;

  private:
    uint n_;
    NT idx_per_log_, log_per_idx_, span_, inv_span_;
  };

  // integer stack index and Matsubara frequencies (stack axes of the finite-T coordinates)
  template <typename Idx> class IndexStack
  {
  public:
    using ctype = Idx;
    static constexpr uint dim = 1;
    IndexStack(Idx start, Idx stop) : start(start), stop(stop), m_size((uint)(stop - start))
    {
      if (start > stop) throw std::invalid_argument("IndexStack: start must be smaller than stop");
    }
    __host__ __device__ Idx forward(const Idx x) const { return x + start; }
    __host__ __device__ Idx backward(const Idx y) const { return y - start; }
    __host__ __device__ uint size() const { return m_size; }
    Idx start, stop;

  private:
    uint m_size;
  };

  // omega_n = 2 pi T n (bosonic) or 2 pi T (n + 1/2) (fermionic), n = start .. stop-1;
  // backward rounds to the nearest mode and returns its stack index
  template <typename Idx, typename NT, bool FERMIONIC> class MatsubaraValues
  {
  public:
    using ctype = NT;
    static constexpr uint dim = 1;
    MatsubaraValues(Idx start, Idx stop, NT T) : start(start), stop(stop), T(T), m_size((uint)(stop - start))
    {
      if (start > stop) throw std::invalid_argument("MatsubaraValues: start must be smaller than stop");
    }
    __host__ __device__ NT forward(const Idx &x) const
    {
      return (NT(x + start) + (FERMIONIC ? (NT)0.5 : (NT)0)) * (NT)(2. * M_PI) * T;
    }
    __host__ __device__ Idx backward(const NT &y) const
    {
      const NT s = FERMIONIC ? (y - (NT)M_PI * T) : y;
      return Idx(round(s / ((NT)(2. * M_PI) * T))) - start;
    }
    __host__ __device__ uint size() const { return m_size; }
    Idx start, stop;
    NT T;

  private:
    uint m_size;
  };
  template <typename Idx, typename NT> using BosonicMatsubaraValues = MatsubaraValues<Idx, NT, false>;
  template <typename Idx, typename NT> using FermionicMatsubaraValues = MatsubaraValues<Idx, NT, true>;

  // ------------------------------------------------------------------ packs of 1-3 axes
  template <class... C> class CoordinatePackND;

  template <class C0> class CoordinatePackND<C0>
  {
  public:
    using ctype = typename C0::ctype;
    static constexpr uint dim = 1;
    CoordinatePackND(const C0 &c0) : c0(c0) {}
    __host__ __device__ std::array<ctype, 1> forward(uint i) const { return {{c0.forward(i)}}; }
    __host__ __device__ std::array<ctype, 1> backward(ctype x) const { return {{c0.backward(x)}}; }
    template <uint i> __host__ __device__ const C0 &get_coordinates() const { return c0; }
    uint size() const { return c0.size(); }
    std::array<uint, 1> sizes() const { return {{c0.size()}}; }
    C0 c0;
  };

  template <class C0, class C1> class CoordinatePackND<C0, C1>
  {
  public:
    using ctype = typename C0::ctype;
    static constexpr uint dim = 2;
    CoordinatePackND(const C0 &c0, const C1 &c1) : c0(c0), c1(c1) {}
    __host__ __device__ std::array<ctype, 2> forward(uint i, uint j) const { return {{c0.forward(i), c1.forward(j)}}; }
    __host__ __device__ std::array<ctype, 2> backward(ctype x, ctype y) const
    {
      return {{c0.backward(x), c1.backward(y)}};
    }
    template <uint i> __host__ __device__ const auto &get_coordinates() const
    {
      if constexpr (i == 0)
        return c0;
      else
        return c1;
    }
    uint size() const { return c0.size() * c1.size(); }
    std::array<uint, 2> sizes() const { return {{c0.size(), c1.size()}}; }
    C0 c0;
    C1 c1;
  };

  template <class C0, class C1, class C2> class CoordinatePackND<C0, C1, C2>
  {
  public:
    using ctype = typename C0::ctype;
    static constexpr uint dim = 3;
    CoordinatePackND(const C0 &c0, const C1 &c1, const C2 &c2) : c0(c0), c1(c1), c2(c2) {}
    __host__ __device__ std::array<ctype, 3> forward(uint i, uint j, uint k) const
    {
      return {{c0.forward(i), c1.forward(j), c2.forward(k)}};
    }
    __host__ __device__ std::array<ctype, 3> backward(ctype x, ctype y, ctype z) const
    {
      return {{c0.backward(x), c1.backward(y), c2.backward(z)}};
    }
    template <uint i> __host__ __device__ const auto &get_coordinates() const
    {
      if constexpr (i == 0)
        return c0;
      else if constexpr (i == 1)
        return c1;
      else
        return c2;
    }
    uint size() const { return c0.size() * c1.size() * c2.size(); }
    std::array<uint, 3> sizes() const { return {{c0.size(), c1.size(), c2.size()}}; }
    C0 c0;
    C1 c1;
    C2 c2;
  };

  // ------------------------------------------------------------------ finite-T (mode, |p|) axes
  // Matsubara mode index x log-spaced momentum.  A frequency outside the stored modes is folded
  // onto the nearest stored mode with |p| -> sqrt(p^2 + (omega - omega_edge)^2), as the
  // reference does (combined_coordinates.hh:47-63).
  template <typename Idx, typename NT, bool FERMIONIC> class Coordinates1DFiniteT
  {
  public:
    using ctype = NT;
    static constexpr uint dim = 2;
    Coordinates1DFiniteT(Idx m_start, Idx m_stop, NT m_T, uint grid_extent, NT p_start, NT p_stop, NT p_bias)
        : m_start(m_start), m_stop(m_stop), m_T(m_T), p_start(p_start), p_stop(p_stop), p_bias(p_bias),
          grid_extent(grid_extent), m_size((uint)(m_stop - m_start)), matsubara_values(m_start, m_stop, m_T),
          logarithmic_coordinates(grid_extent, p_start, p_stop, p_bias)
    {
    }
    template <typename NT2>
    Coordinates1DFiniteT(const LogarithmicCoordinates1D<NT2> &lc, Idx m_start, Idx m_stop, NT m_T)
        : Coordinates1DFiniteT(m_start, m_stop, m_T, lc.size(), (NT)lc.start, (NT)lc.stop, (NT)lc.bias)
    {
    }
    // the same axes in another precision
    template <typename NT2>
    explicit Coordinates1DFiniteT(const Coordinates1DFiniteT<Idx, NT2, FERMIONIC> &o)
        : Coordinates1DFiniteT((Idx)o.m_start, (Idx)o.m_stop, (NT)o.m_T, o.sizes()[1], (NT)o.p_start, (NT)o.p_stop,
                               (NT)o.p_bias)
    {
    }
    __host__ __device__ std::array<NT, 2> forward(const uint m, const uint p) const
    {
      return {{matsubara_values.forward((Idx)m), logarithmic_coordinates.forward(p)}};
    }
    __host__ __device__ std::tuple<Idx, NT> backward(const NT m, const NT p) const
    {
      Idx m_idx = matsubara_values.backward(m);
      NT p_idx;
      if (m_idx >= (Idx)m_size || m_idx < 0) {
        m_idx = m_idx < 0 ? 0 : (Idx)m_size - 1;
        const NT dm = m - matsubara_values.forward(m_idx);
        p_idx = logarithmic_coordinates.backward(sqrt(p * p + dm * dm));
      } else
        p_idx = logarithmic_coordinates.backward(p);
      return std::tuple<Idx, NT>(m_idx, p_idx);
    }
    __host__ __device__ uint size() const { return m_size * grid_extent; }
    std::array<uint, 2> sizes() const { return {{m_size, grid_extent}}; }
    NT m_start, m_stop, m_T, p_start, p_stop, p_bias;

  private:
    uint grid_extent, m_size;
    MatsubaraValues<Idx, NT, FERMIONIC> matsubara_values;
    LogarithmicCoordinates1D<NT> logarithmic_coordinates;
  };
  template <typename Idx, typename NT> using BosonicCoordinates1DFiniteT = Coordinates1DFiniteT<Idx, NT, false>;
  template <typename Idx, typename NT> using FermionicCoordinates1DFiniteT = Coordinates1DFiniteT<Idx, NT, true>;

  namespace gbint_detail
  {
    // The precision an interpolator maps coordinates and interpolates in: double whenever the
    // result type is double-based (double, complex<double>, dual<double>), else the coordinates'
    // own type.  The reference maps in the coordinates' type (float for the usual
    // LogarithmicCoordinates1D<float>) and filters with 8-bit texture fractions; mapping in double
    // makes host and device results agree to FP64 rounding.
    template <typename NT> struct scalar_of {
      using type = NT;
    };
    template <typename T> struct scalar_of<::cuda::std::complex<T>> {
      using type = typename scalar_of<T>::type;
    };
    template <typename T> struct scalar_of<gbint::dual<T>> {
      using type = typename scalar_of<T>::type;
    };
    template <typename NT, typename ctype>
    using map_precision = std::conditional_t<std::is_same_v<typename scalar_of<NT>::type, double>, double, ctype>;

    // coordinates C with their floating-point type replaced by W (others unchanged)
    template <class C, typename W> struct at_precision {
      using type = C;
      static const C &make(const C &c) { return c; }
    };
    template <typename T, typename W> struct at_precision<LinearCoordinates1D<T>, W> {
      using type = LinearCoordinates1D<W>;
      static type make(const LinearCoordinates1D<T> &c) { return type(c); }
    };
    template <typename T, typename W> struct at_precision<LogarithmicCoordinates1D<T>, W> {
      using type = LogarithmicCoordinates1D<W>;
      static type make(const LogarithmicCoordinates1D<T> &c) { return type(c); }
    };
    template <typename Idx, typename T, bool F, typename W> struct at_precision<Coordinates1DFiniteT<Idx, T, F>, W> {
      using type = Coordinates1DFiniteT<Idx, W, F>;
      static type make(const Coordinates1DFiniteT<Idx, T, F> &c) { return type(c); }
    };
    template <class C0, typename W> struct at_precision<CoordinatePackND<C0>, W> {
      using type = CoordinatePackND<typename at_precision<C0, W>::type>;
      static type make(const CoordinatePackND<C0> &c) { return type(at_precision<C0, W>::make(c.c0)); }
    };
    template <class C0, class C1, typename W> struct at_precision<CoordinatePackND<C0, C1>, W> {
      using type = CoordinatePackND<typename at_precision<C0, W>::type, typename at_precision<C1, W>::type>;
      static type make(const CoordinatePackND<C0, C1> &c)
      {
        return type(at_precision<C0, W>::make(c.c0), at_precision<C1, W>::make(c.c1));
      }
    };
    template <class C0, class C1, class C2, typename W> struct at_precision<CoordinatePackND<C0, C1, C2>, W> {
      using type = CoordinatePackND<typename at_precision<C0, W>::type, typename at_precision<C1, W>::type,
                                    typename at_precision<C2, W>::type>;
      static type make(const CoordinatePackND<C0, C1, C2> &c)
      {
        return type(at_precision<C0, W>::make(c.c0), at_precision<C1, W>::make(c.c1),
                    at_precision<C2, W>::make(c.c2));
      }
    };
  } // namespace gbint_detail

  namespace gbint_detail
  {
    // process-wide context for interpolator data (device 0), created on first use
    inline gb_ctx *interp_ctx()
    {
      static std::once_flag once;
      static gb_ctx *ctx = nullptr;
      std::call_once(once, [] {
        if (gb_ctx_create(0, 0, &ctx) != GB_OK) ctx = nullptr;
      });
      if (!ctx) throw std::runtime_error("No CUDA devices found! (interpolator context)");
      return ctx;
    }
    // the buffer is a multiple of 16 bytes (zero padding): the fused kernels stage tables into
    // shared memory with TMA bulk copies, whose sizes are multiples of 16 bytes
    inline size_t padded_bytes(size_t bytes) { return (bytes + 15) & ~size_t(15); }
    template <typename T> T *device_copy(const std::vector<T> &h)
    {
      void *d = nullptr;
      gb_ctx *c = interp_ctx();
      const size_t bytes = h.size() * sizeof(T);
      std::vector<char> pad(padded_bytes(bytes), 0);
      if (bytes) std::memcpy(pad.data(), h.data(), bytes);
      if (gb_buffer_create(c, pad.size(), &d) != GB_OK || gb_buffer_upload(c, d, pad.data(), pad.size()) != GB_OK)
        throw std::runtime_error("interpolator: device buffer");
      return static_cast<T *>(d);
    }
    template <typename T> void device_update(T *d, const std::vector<T> &h)
    {
      if (gb_buffer_upload(interp_ctx(), d, h.data(), h.size() * sizeof(T)) != GB_OK)
        throw std::runtime_error("interpolator: update");
    }
    template <typename ctype> __host__ __device__ inline ctype clampc(ctype v, ctype lo, ctype hi)
    {
      return v < lo ? lo : (v > hi ? hi : v);
    }
    // grid cell i in [0, n-2] and fraction of a clamped grid coordinate (n >= 2; n == 1: cell 0)
    template <typename ctype> __host__ __device__ inline void cell(ctype idx, uint n, uint &i, ctype &f)
    {
      if (n < 2) {
        i = 0;
        f = 0;
        return;
      }
      idx = clampc<ctype>(idx, 0, (ctype)(n - 1));
      i = (uint)floor(idx);
      if (i > n - 2) i = n - 2;
      f = idx - (ctype)i;
    }
    // host-side storage of an interpolator (owned for the process lifetime)
    template <typename T> struct Store {
      std::vector<T> host;
      T *dev = nullptr;
    };
    template <typename DT, typename NT> Store<DT> *make_store(const NT *data, size_t n)
    {
      auto *s = new Store<DT>();  // lives until process exit (copies are views)
      s->host.resize(n);
      for (size_t i = 0; i < n; ++i) s->host[i] = data ? (DT)data[i] : (DT)0;
      s->dev = device_copy(s->host);
      return s;
    }
  } // namespace gbint_detail

  // ------------------------------------------------------------------ 1D
  // data[i] at coordinates.forward(i); DT = stored type (float for Tex*, NT for Linear*)
  template <typename NT, typename Coordinates, typename DT> class Interpolator1DBase
  {
  public:
    using ctype = typename Coordinates::ctype;
    using ReturnType = NT;
    Interpolator1DBase(const std::vector<NT> &data, const Coordinates &coordinates)
        : Interpolator1DBase(data.data(), coordinates)
    {
      if (data.size() != coordinates.size()) throw std::runtime_error("interpolator: data size != coordinates size");
    }
    Interpolator1DBase(const NT *data, const Coordinates &coordinates) : coordinates(coordinates), size(coordinates.size())
    {
      store_ = gbint_detail::make_store<DT>(data, size);
      h_data_ = store_->host.data();
      d_data_ = store_->dev;
    }
    explicit Interpolator1DBase(const Coordinates &coordinates) : Interpolator1DBase((const NT *)nullptr, coordinates) {}
    // host-side element access and update (TexLinearInterpolator1D::operator[] / update)
    DT &operator[](const uint i) { return store_->host[i]; }
    const DT &operator[](const uint i) const { return store_->host[i]; }
    template <typename NT2> void update(const NT2 *data)
    {
      for (uint i = 0; i < size; ++i) store_->host[i] = (DT)data[i];
      update();
    }
    void update() { gbint_detail::device_update(store_->dev, store_->host); }
    DT *data() const { return store_->host.data(); }
    const Coordinates &get_coordinates() const { return coordinates; }

    template <typename X> __host__ __device__ NT operator()(const X x) const
    {
#ifdef __CUDA_ARCH__
      const DT *d = d_data_;
#else
      const DT *d = h_data_;
#endif
      uint i;
      W f;
      gbint_detail::cell<W>(coords_w.backward((W)x), size, i, f);
      if (size < 2) return (NT)d[0];
      return (NT)((W)d[i] + f * ((W)d[i + 1] - (W)d[i]));
    }


    // staging interface of the fused kernels (gbint/device/user_batch.cuh): the device table,
    // its size in bytes (a multiple of 16, see device_copy) and a copy reading another buffer
    using gbint_stageable_table = DT;
    __host__ __device__ const void *device_data() const { return d_data_; }
    size_t table_bytes() const { return gbint_detail::padded_bytes(store_->host.size() * sizeof(DT)); }
    __host__ __device__ void retarget(const void *p) { d_data_ = static_cast<const DT *>(p); }

  protected:
    using W = gbint_detail::map_precision<NT, ctype>;
    Coordinates coordinates;
    typename gbint_detail::at_precision<Coordinates, W>::type coords_w =
        gbint_detail::at_precision<Coordinates, W>::make(coordinates);
    uint size;
    gbint_detail::Store<DT> *store_;
    const DT *h_data_;
    const DT *d_data_;
  };
  template <typename NT, typename Coordinates>
  using TexLinearInterpolator1D = Interpolator1DBase<NT, Coordinates, float>;
  template <typename NT, typename Coordinates>
  using LinearInterpolator1D = Interpolator1DBase<NT, Coordinates, NT>;

  // ------------------------------------------------------------------ 2D
  // data row-major [size0][size1], bilinear in the two grid indices
  template <typename NT, typename Coordinates, typename DT> class Interpolator2DBase
  {
  public:
    using ctype = typename Coordinates::ctype;
    using ReturnType = NT;
    Interpolator2DBase(const std::vector<NT> &data, const Coordinates &coordinates)
        : Interpolator2DBase(data.data(), coordinates)
    {
      if (data.size() != (size_t)coordinates.size()) throw std::runtime_error("interpolator: data size != coordinates size");
    }
    Interpolator2DBase(const NT *data, const Coordinates &coordinates)
        : coordinates(coordinates), n0(coordinates.sizes()[0]), n1(coordinates.sizes()[1])
    {
      store_ = gbint_detail::make_store<DT>(data, (size_t)n0 * n1);
      h_data_ = store_->host.data();
      d_data_ = store_->dev;
    }
    explicit Interpolator2DBase(const Coordinates &coordinates) : Interpolator2DBase((const NT *)nullptr, coordinates) {}
    DT &operator[](const uint i) { return store_->host[i]; }
    const DT &operator[](const uint i) const { return store_->host[i]; }
    template <typename NT2> void update(const NT2 *data)
    {
      for (size_t i = 0; i < store_->host.size(); ++i) store_->host[i] = (DT)data[i];
      update();
    }
    void update() { gbint_detail::device_update(store_->dev, store_->host); }
    DT *data() const { return store_->host.data(); }
    const Coordinates &get_coordinates() const { return coordinates; }

    template <typename X, typename Y> __host__ __device__ NT operator()(const X x, const Y y) const
    {
#ifdef __CUDA_ARCH__
      const DT *d = d_data_;
#else
      const DT *d = h_data_;
#endif
      const auto idx = coords_w.backward((W)x, (W)y);
      uint i, j;
      W fx, fy;
      gbint_detail::cell<W>(idx[0], n0, i, fx);
      gbint_detail::cell<W>(idx[1], n1, j, fy);
      const uint i1 = n0 > 1 ? i + 1 : i, j1 = n1 > 1 ? j + 1 : j;
      const W y00 = d[(size_t)i * n1 + j], y10 = d[(size_t)i1 * n1 + j];
      const W y01 = d[(size_t)i * n1 + j1], y11 = d[(size_t)i1 * n1 + j1];
      const W lo = y00 + fx * (y10 - y00), hi = y01 + fx * (y11 - y01);
      return (NT)(lo + fy * (hi - lo));
    }


    // staging interface of the fused kernels (gbint/device/user_batch.cuh): the device table,
    // its size in bytes (a multiple of 16, see device_copy) and a copy reading another buffer
    using gbint_stageable_table = DT;
    __host__ __device__ const void *device_data() const { return d_data_; }
    size_t table_bytes() const { return gbint_detail::padded_bytes(store_->host.size() * sizeof(DT)); }
    __host__ __device__ void retarget(const void *p) { d_data_ = static_cast<const DT *>(p); }

  protected:
    using W = gbint_detail::map_precision<NT, ctype>;
    Coordinates coordinates;
    typename gbint_detail::at_precision<Coordinates, W>::type coords_w =
        gbint_detail::at_precision<Coordinates, W>::make(coordinates);
    uint n0, n1;
    gbint_detail::Store<DT> *store_;
    const DT *h_data_;
    const DT *d_data_;
  };
  template <typename NT, typename Coordinates>
  using TexLinearInterpolator2D = Interpolator2DBase<NT, Coordinates, float>;
  template <typename NT, typename Coordinates>
  using LinearInterpolator2D = Interpolator2DBase<NT, Coordinates, NT>;

  // ------------------------------------------------------------------ 3D
  // data row-major [size0][size1][size2], trilinear (x first, then y, then z)
  template <typename NT, typename Coordinates, typename DT> class Interpolator3DBase
  {
  public:
    using ctype = typename Coordinates::ctype;
    using ReturnType = NT;
    Interpolator3DBase(const std::vector<NT> &data, const Coordinates &coordinates)
        : Interpolator3DBase(data.data(), coordinates)
    {
      if (data.size() != (size_t)coordinates.size()) throw std::runtime_error("interpolator: data size != coordinates size");
    }
    Interpolator3DBase(const NT *data, const Coordinates &coordinates)
        : coordinates(coordinates), n0(coordinates.sizes()[0]), n1(coordinates.sizes()[1]), n2(coordinates.sizes()[2])
    {
      store_ = gbint_detail::make_store<DT>(data, (size_t)n0 * n1 * n2);
      h_data_ = store_->host.data();
      d_data_ = store_->dev;
    }
    explicit Interpolator3DBase(const Coordinates &coordinates) : Interpolator3DBase((const NT *)nullptr, coordinates) {}
    DT &operator[](const uint i) { return store_->host[i]; }
    const DT &operator[](const uint i) const { return store_->host[i]; }
    template <typename NT2> void update(const NT2 *data)
    {
      for (size_t i = 0; i < store_->host.size(); ++i) store_->host[i] = (DT)data[i];
      update();
    }
    void update() { gbint_detail::device_update(store_->dev, store_->host); }
    DT *data() const { return store_->host.data(); }
    const Coordinates &get_coordinates() const { return coordinates; }

    template <typename X, typename Y, typename Z> __host__ __device__ NT operator()(const X x, const Y y, const Z z) const
    {
#ifdef __CUDA_ARCH__
      const DT *d = d_data_;
#else
      const DT *d = h_data_;
#endif
      const auto idx = coords_w.backward((W)x, (W)y, (W)z);
      uint i, j, l;
      W fx, fy, fz;
      gbint_detail::cell<W>(idx[0], n0, i, fx);
      gbint_detail::cell<W>(idx[1], n1, j, fy);
      gbint_detail::cell<W>(idx[2], n2, l, fz);
      const uint i1 = n0 > 1 ? i + 1 : i, j1 = n1 > 1 ? j + 1 : j, l1 = n2 > 1 ? l + 1 : l;
      auto at = [&](uint a, uint b, uint c) -> W { return (W)d[((size_t)a * n1 + b) * n2 + c]; };
      auto lx = [&](uint b, uint c) -> W {
        const W v0 = at(i, b, c);
        return v0 + fx * (at(i1, b, c) - v0);
      };
      const W c00 = lx(j, l), c10 = lx(j1, l), c01 = lx(j, l1), c11 = lx(j1, l1);
      const W c0 = c00 + fy * (c10 - c00), c1 = c01 + fy * (c11 - c01);
      return (NT)(c0 + fz * (c1 - c0));
    }


    // staging interface of the fused kernels (gbint/device/user_batch.cuh): the device table,
    // its size in bytes (a multiple of 16, see device_copy) and a copy reading another buffer
    using gbint_stageable_table = DT;
    __host__ __device__ const void *device_data() const { return d_data_; }
    size_t table_bytes() const { return gbint_detail::padded_bytes(store_->host.size() * sizeof(DT)); }
    __host__ __device__ void retarget(const void *p) { d_data_ = static_cast<const DT *>(p); }

  protected:
    using W = gbint_detail::map_precision<NT, ctype>;
    Coordinates coordinates;
    typename gbint_detail::at_precision<Coordinates, W>::type coords_w =
        gbint_detail::at_precision<Coordinates, W>::make(coordinates);
    uint n0, n1, n2;
    gbint_detail::Store<DT> *store_;
    const DT *h_data_;
    const DT *d_data_;
  };
  template <typename NT, typename Coordinates>
  using TexLinearInterpolator3D = Interpolator3DBase<NT, Coordinates, float>;
  template <typename NT, typename Coordinates>
  using LinearInterpolator3D = Interpolator3DBase<NT, Coordinates, NT>;

  // ------------------------------------------------------------------ 1D stack (finite T)
  // A stack of 1D tables, one per Matsubara mode: data [mode s][p i] (FP32), Coordinates with
  // dim 2 whose backward(m, p) gives (stack index, p grid coordinate), e.g.
  // BosonicCoordinates1DFiniteT; linear in p within the selected stack entry.
  template <typename NT, typename Coordinates, uint max_stack_size = 64> class TexLinearInterpolator1DStack
  {
    static_assert(Coordinates::dim == 2, "TexLinearInterpolator1DStack requires 2D coordinates");

  public:
    using ctype = typename Coordinates::ctype;
    using ReturnType = NT;
    TexLinearInterpolator1DStack(const std::vector<NT> &data, const Coordinates &coordinates)
        : TexLinearInterpolator1DStack(data.data(), coordinates)
    {
      if (data.size() != (size_t)coordinates.size()) throw std::runtime_error("interpolator: data size != coordinates size");
    }
    TexLinearInterpolator1DStack(const NT *data, const Coordinates &coordinates)
        : coordinates(coordinates), stack_size(coordinates.sizes()[0]), p_size(coordinates.sizes()[1])
    {
      if (stack_size > max_stack_size) throw std::runtime_error("TexLinearInterpolator1DStack: stack too large");
      store_ = gbint_detail::make_store<float>(data, (size_t)stack_size * p_size);
      h_data_ = store_->host.data();
      d_data_ = store_->dev;
    }
    explicit TexLinearInterpolator1DStack(const Coordinates &coordinates)
        : TexLinearInterpolator1DStack((const NT *)nullptr, coordinates)
    {
    }
    template <typename Coordinates2>
    TexLinearInterpolator1DStack(const Coordinates2 &coordinates, const uint m_start, const uint m_end, const double T)
        : TexLinearInterpolator1DStack(Coordinates(coordinates, m_start, m_end, T))
    {
    }
    template <typename NT2> void update(const NT2 *data)
    {
      for (size_t i = 0; i < store_->host.size(); ++i) store_->host[i] = (float)data[i];
      update();
    }
    void update() { gbint_detail::device_update(store_->dev, store_->host); }
    // host data of stack entry i
    float *data(const uint i) const { return store_->host.data() + (size_t)i * p_size; }
    float &operator[](const uint i) { return store_->host[i]; }
    const float &operator[](const uint i) const { return store_->host[i]; }
    const Coordinates &get_coordinates() const { return coordinates; }

    template <typename M, typename P> __host__ __device__ NT operator()(const M m, const P p) const
    {
#ifdef __CUDA_ARCH__
      const float *d = d_data_;
#else
      const float *d = h_data_;
#endif
      const auto mp = coords_w.backward((W)m, (W)p);
      int s = (int)std::get<0>(mp);
      s = s < 0 ? 0 : (s >= (int)stack_size ? (int)stack_size - 1 : s);
      uint i;
      W f;
      gbint_detail::cell<W>((W)std::get<1>(mp), p_size, i, f);
      const float *row = d + (size_t)s * p_size;
      if (p_size < 2) return (NT)row[0];
      return (NT)((W)row[i] + f * ((W)row[i + 1] - (W)row[i]));
    }


    // staging interface of the fused kernels (gbint/device/user_batch.cuh): the device table,
    // its size in bytes (a multiple of 16, see device_copy) and a copy reading another buffer
    using gbint_stageable_table = float;
    __host__ __device__ const void *device_data() const { return d_data_; }
    size_t table_bytes() const { return gbint_detail::padded_bytes(store_->host.size() * sizeof(float)); }
    __host__ __device__ void retarget(const void *p) { d_data_ = static_cast<const float *>(p); }

  protected:
    using W = gbint_detail::map_precision<NT, ctype>;
    Coordinates coordinates;
    typename gbint_detail::at_precision<Coordinates, W>::type coords_w =
        gbint_detail::at_precision<Coordinates, W>::make(coordinates);
    uint stack_size, p_size;
    gbint_detail::Store<float> *store_;
    const float *h_data_;
    const float *d_data_;
  };
} // namespace DiFfRG
