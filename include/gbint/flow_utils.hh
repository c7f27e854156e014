// flow_utils.hh -- the fan-out helpers flow equations use around the integrators, with the
// names and arguments of DiFfRG/include/DiFfRG/physics/utils.hh:31-220 and make_grid of
// DiFfRG/include/DiFfRG/discretization/grid/coordinates.hh:200-225:
//   make_grid(coordinates)                        the coordinates' points (1D values, 2D/3D arrays)
//   request_data<NT>(fun, coordinates|grid, k, args... | std::tuple<args...>)
//                                                 fun.request<NT>(k, point..., args...) for each point
//   update_data(futures, dest)                    dest[i] = futures[i].get()
//   update_interpolator(futures, interpolator)    interpolator[i] = futures[i].get(); update()
//   get_data<NT>(dest, fun, grid, k, args... | std::tuple<args...>)
//                                                 dest[i] = fun.get<NT>(k, point..., args...)
// request_data opens a RequestBatch (gbint/integrators.hh) around the grid: every request() of
// the drop-in integrators issued for the grid -- also through the wrapper classes of generated
// flows -- joins one persistent launch per kernel type, launched before request_data returns
// (the reference launches one kernel and runs one reduction with its synchronisation per point).
// get_data issues all requests before it collects (the reference runs the gets on TBB threads
// instead).  Results equal single get()s bit for bit.  C++17: the reference's IsCoordinate /
// IsContainer constraints are checked with traits.
#pragma once

#include <array>
#include <future>
#include <memory>
#include <stdexcept>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "gbint/integrators.hh"
#include "gbint/interpolators.hh"

namespace DiFfRG
{
  namespace gbint_detail
  {
    // a coordinates object: has dim and forward(...) (the reference's IsCoordinate)
    template <typename T, typename = void> struct is_coordinates : std::false_type {};
    template <typename T>
    struct is_coordinates<T, std::void_t<decltype(T::dim), typename T::ctype>> : std::true_type {};
    template <typename P> constexpr bool is_scalar_point = std::is_arithmetic_v<std::decay_t<P>>;

    template <typename NT, typename FUN, typename P, typename... T>
    std::future<NT> request_point(FUN &fun, double k, const P &p, const T &...args)
    {
      if constexpr (is_scalar_point<P>)
        return fun.template request<NT>(k, p, args...);
      else
        return std::apply([&](auto... c) { return fun.template request<NT>(k, c..., args...); }, p);
    }
  } // namespace gbint_detail

  template <typename Coordinates> auto make_grid(const Coordinates &coordinates)
  {
    using ctype = typename Coordinates::ctype;
    if constexpr (Coordinates::dim == 1) {
      std::vector<ctype> grid(coordinates.size());
      for (uint i = 0; i < coordinates.size(); ++i) {
        const auto v = coordinates.forward(i);
        if constexpr (std::is_arithmetic_v<decltype(v)>)
          grid[i] = v;
        else
          grid[i] = v[0];  // a one-axis pack returns std::array<ctype, 1>
      }
      return grid;
    } else if constexpr (Coordinates::dim == 2) {
      const auto n = coordinates.sizes();
      std::vector<std::array<ctype, 2>> grid(coordinates.size());
      for (uint i = 0; i < n[0]; ++i)
        for (uint j = 0; j < n[1]; ++j) grid[i * n[1] + j] = coordinates.forward(i, j);
      return grid;
    } else {
      static_assert(Coordinates::dim == 3, "make_grid: 1D, 2D or 3D coordinates");
      const auto n = coordinates.sizes();
      std::vector<std::array<ctype, 3>> grid(coordinates.size());
      for (uint i = 0; i < n[0]; ++i)
        for (uint j = 0; j < n[1]; ++j)
          for (uint l = 0; l < n[2]; ++l) grid[(i * n[1] + j) * n[2] + l] = coordinates.forward(i, j, l);
      return grid;
    }
  }

  // fun.request<NT>(k, point..., args...) for every point of a coordinates object or a grid
  // (a container of scalars or of std::array / tuple-like points)
  template <typename NT, typename FUN, typename GRID, typename... T>
  std::shared_ptr<std::vector<std::future<NT>>> request_data(FUN &fun, const GRID &grid, const double k, T... args)
  {
    auto futures = std::make_shared<std::vector<std::future<NT>>>();
    RequestBatch batch;  // one launch for the grid, at the end of this scope
    if constexpr (gbint_detail::is_coordinates<GRID>::value) {
      const auto points = make_grid(grid);
      futures->reserve(points.size());
      for (const auto &p : points) futures->emplace_back(gbint_detail::request_point<NT>(fun, k, p, args...));
    } else {
      futures->reserve(grid.size());
      for (std::size_t i = 0; i < grid.size(); ++i)
        futures->emplace_back(gbint_detail::request_point<NT>(fun, k, grid[i], args...));
    }
    return futures;
  }
  template <typename NT, typename FUN, typename GRID, typename... T>
  std::shared_ptr<std::vector<std::future<NT>>> request_data(FUN &fun, const GRID &grid, const double k,
                                                             std::tuple<T...> args)
  {
    return std::apply([&](auto... a) { return request_data<NT>(fun, grid, k, a...); }, args);
  }

  template <typename NT1, typename NT2, typename... T>
  void update_data(std::shared_ptr<std::vector<std::future<NT1>>> futures, NT2 *destination)
  {
    for (std::size_t i = 0; i < futures->size(); ++i) destination[i] = static_cast<NT2>((*futures)[i].get());
  }

  template <typename NT, typename INT, typename... T>
  void update_interpolator(std::shared_ptr<std::vector<std::future<NT>>> futures, INT &destination)
  {
    for (std::size_t i = 0; i < futures->size(); ++i) destination[i] = (*futures)[i].get();
    destination.update();
  }

  template <typename NT, typename FUN, typename GRID, typename... T>
  void get_data(NT *dest, FUN &fun, const GRID &grid, const double k, T... args)
  {
    update_data(request_data<NT>(fun, grid, k, args...), dest);
  }
  template <typename NT, typename FUN, typename GRID, typename... T>
  void get_data(NT *dest, FUN &fun, const GRID &grid, const double k, std::tuple<T...> args)
  {
    std::apply([&](auto... a) { get_data<NT>(dest, fun, grid, k, a...); }, args);
  }
} // namespace DiFfRG
