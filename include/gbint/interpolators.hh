// interpolators.hh -- DiFfRG-compatible coordinates and interpolators for user KERNELs.
//
//   LinearCoordinates1D, LogarithmicCoordinates1D, CoordinatePackND (2 axes)
//        DiFfRG/include/DiFfRG/discretization/grid/coordinates.hh:28-195
//   TexLinearInterpolator1D / 2D        DiFfRG/include/DiFfRG/physics/interpolation/tex_linear_interpolation_{1D,2D}.hh
//   LinearInterpolator1D / 2D           DiFfRG/include/DiFfRG/physics/interpolation/linear_interpolation_{1D,2D}.hh
//
// Objects are trivially copyable views, passed by value into KERNEL::kernel arguments like the
// reference's: a device pointer to the data, a host pointer to the host copy, the size and the
// coordinates.  operator() clamps the grid index to the table and interpolates linearly in it,
// on the host and on the device alike.  The Tex* variants keep the reference's FP32 data but
// interpolate exactly (the reference's texture filter has an 8-bit fraction, ~1e-3 relative,
// DiFfRG/tests/physics/interpolation/tex_linear_interpolation_1D_gpu.cu:55-57).  Device data lives
// in buffers of the process-wide interpolator context until process exit; update() copies the
// host data in place after the device drained, as the reference's update() synchronises.
#pragma once

#include <cmath>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbint.h"

namespace DiFfRG
{
  using uint = unsigned int;

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
    __host__ __device__ NT forward(const uint &x) const { return start + a * x; }
    __host__ __device__ NT backward(const NT &y) const { return (y - start) / a; }
    __host__ __device__ uint size() const { return grid_extent; }
    NT start, stop;

  private:
    uint grid_extent;
    NT a;
  };

  template <typename NT> class LogarithmicCoordinates1D
  {
  public:
    using ctype = NT;
    static constexpr uint dim = 1;
    LogarithmicCoordinates1D(uint grid_extent, NT start_, NT stop_, NT bias_)
        : start(start_), stop(stop_), bias(bias_), grid_extent(grid_extent), gem1((NT)(grid_extent - 1.)),
          gem1inv((NT)(1. / (grid_extent - 1.)))
    {
      if (grid_extent == 0) throw std::runtime_error("LogarithmicCoordinates1D: grid_extent must be > 0");
      a = bias;
      b = (stop - start) / std::expm1(a);
      c = start;
    }
    __host__ __device__ NT forward(const uint &x) const { return b * expm1(a * x * gem1inv) + c; }
    __host__ __device__ NT backward(const NT &y) const { return log1p((y - c) / b) * gem1 / a; }
    __host__ __device__ uint size() const { return grid_extent; }
    NT start, stop, bias;

  private:
    uint grid_extent;
    NT gem1, gem1inv;
    NT a, b, c;
  };

  // two coordinate axes (the reference's CoordinatePackND for the 2D interpolators)
  template <class C0, class C1> class CoordinatePackND
  {
  public:
    using ctype = typename C0::ctype;
    static constexpr uint dim = 2;
    CoordinatePackND(const C0 &c0, const C1 &c1) : c0(c0), c1(c1) {}
    __host__ __device__ void backward(ctype x, ctype y, ctype &ix, ctype &iy) const
    {
      ix = c0.backward(x);
      iy = c1.backward(y);
    }
    __host__ __device__ uint size0() const { return c0.size(); }
    __host__ __device__ uint size1() const { return c1.size(); }
    C0 c0;
    C1 c1;
  };

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
    template <typename T> T *device_copy(const std::vector<T> &h)
    {
      void *d = nullptr;
      gb_ctx *c = interp_ctx();
      if (gb_buffer_create(c, h.size() * sizeof(T), &d) != GB_OK ||
          gb_buffer_upload(c, d, h.data(), h.size() * sizeof(T)) != GB_OK)
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
    // host-side storage of an interpolator (owned for the process lifetime)
    template <typename T> struct Store {
      std::vector<T> host;
      T *dev = nullptr;
    };
  } // namespace gbint_detail

  // 1D: data[i] at coordinates.forward(i); DT = stored type (float for Tex*, NT for Linear*)
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
      auto *s = new gbint_detail::Store<DT>();  // lives until process exit (copies are views)
      s->host.resize(size);
      for (uint i = 0; i < size; ++i) s->host[i] = (DT)data[i];
      s->dev = gbint_detail::device_copy(s->host);
      store_ = s;
      h_data_ = s->host.data();
      d_data_ = s->dev;
    }
    // host-side element access and update (TexLinearInterpolator1D::operator[] / update)
    DT &operator[](const uint i) { return store_->host[i]; }
    const DT &operator[](const uint i) const { return store_->host[i]; }
    void update() { gbint_detail::device_update(store_->dev, store_->host); }
    DT *data() const { return store_->host.data(); }

    __host__ __device__ NT operator()(const ctype x) const
    {
      ctype idx = coordinates.backward(x);
      idx = gbint_detail::clampc<ctype>(idx, 0, (ctype)(size - 1));
#ifdef __CUDA_ARCH__
      const DT *d = d_data_;
#else
      const DT *d = h_data_;
#endif
      uint i = (uint)floor(idx);
      if (i > size - 2) i = size - 2;
      const ctype f = idx - (ctype)i;
      return (NT)((ctype)d[i] + f * ((ctype)d[i + 1] - (ctype)d[i]));
    }

  protected:
    Coordinates coordinates;
    uint size;
    gbint_detail::Store<DT> *store_;
    const DT *h_data_;
    const DT *d_data_;
  };
  template <typename NT, typename Coordinates>
  using TexLinearInterpolator1D = Interpolator1DBase<NT, Coordinates, float>;
  template <typename NT, typename Coordinates>
  using LinearInterpolator1D = Interpolator1DBase<NT, Coordinates, NT>;

  // 2D: data row-major [size0][size1], bilinear in the two grid indices
  template <typename NT, typename Coordinates, typename DT> class Interpolator2DBase
  {
  public:
    using ctype = typename Coordinates::ctype;
    using ReturnType = NT;
    Interpolator2DBase(const std::vector<NT> &data, const Coordinates &coordinates)
        : Interpolator2DBase(data.data(), coordinates)
    {
      if (data.size() != (size_t)coordinates.size0() * coordinates.size1())
        throw std::runtime_error("interpolator: data size != coordinates size");
    }
    Interpolator2DBase(const NT *data, const Coordinates &coordinates)
        : coordinates(coordinates), n0(coordinates.size0()), n1(coordinates.size1())
    {
      auto *s = new gbint_detail::Store<DT>();
      s->host.resize((size_t)n0 * n1);
      for (size_t i = 0; i < s->host.size(); ++i) s->host[i] = (DT)data[i];
      s->dev = gbint_detail::device_copy(s->host);
      store_ = s;
      h_data_ = s->host.data();
      d_data_ = s->dev;
    }
    DT &operator[](const uint i) { return store_->host[i]; }
    void update() { gbint_detail::device_update(store_->dev, store_->host); }

    __host__ __device__ NT operator()(const ctype x, const ctype y) const
    {
      ctype ix, iy;
      coordinates.backward(x, y, ix, iy);
      ix = gbint_detail::clampc<ctype>(ix, 0, (ctype)(n0 - 1));
      iy = gbint_detail::clampc<ctype>(iy, 0, (ctype)(n1 - 1));
#ifdef __CUDA_ARCH__
      const DT *d = d_data_;
#else
      const DT *d = h_data_;
#endif
      uint i = (uint)floor(ix), j = (uint)floor(iy);
      if (i > n0 - 2) i = n0 - 2;
      if (j > n1 - 2) j = n1 - 2;
      const ctype fx = ix - (ctype)i, fy = iy - (ctype)j;
      const ctype y00 = d[(size_t)i * n1 + j], y10 = d[(size_t)(i + 1) * n1 + j];
      const ctype y01 = d[(size_t)i * n1 + j + 1], y11 = d[(size_t)(i + 1) * n1 + j + 1];
      const ctype lo = y00 + fx * (y10 - y00), hi = y01 + fx * (y11 - y01);
      return (NT)(lo + fy * (hi - lo));
    }

  protected:
    Coordinates coordinates;
    uint n0, n1;
    gbint_detail::Store<DT> *store_;
    const DT *h_data_;
    const DT *d_data_;
  };
  template <typename NT, typename Coordinates>
  using TexLinearInterpolator2D = Interpolator2DBase<NT, Coordinates, float>;
  template <typename NT, typename Coordinates>
  using LinearInterpolator2D = Interpolator2DBase<NT, Coordinates, NT>;
} // namespace DiFfRG
