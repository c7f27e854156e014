// utils_compat.hh -- the host utilities of DiFfRG/include/DiFfRG/common/utils.hh that generated
// flows and their drivers can name (the header every generated flows/def.hh includes first),
// without spdlog: header-only, same names and results.
//   constexpr_for<Start, End, Inc>(f)   f(std::integral_constant<...>) for Start, Start+Inc, ... < End
//   strip_name(s)                       s without blanks and the punctuation ^$#%&*-+=~`!@?<>,.:;'"|\/(){}[]
//   string_to_double_array("1,2.5,3")   {1, 2.5, 3}
//   getWithPrecision(p, x)              fixed notation with p decimals
//   to_string_with_digits(x, d)         fixed notation with d significant digits before rounding
//   file_exists, make_folder (adds '/'), create_folder (with parents), has_suffix
//   time_format(s)                      "59s", "2min5s", "1h2min3s" (below 120 s plain seconds)
//   time_format_ms(ms)                  "999ms", "1s250ms", "2min5s", "1h2min"
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "gbint/json.hh"
#include "gbint/math_compat.hh"

namespace DiFfRG
{
  using uint = unsigned int;

  template <auto Start, auto End, auto Inc, class F> constexpr void constexpr_for(F &&f)
  {
    if constexpr (Start < End) {
      f(std::integral_constant<decltype(Start), Start>());
      constexpr_for<Start + Inc, End, Inc>(f);
    }
  }

  inline std::string strip_name(const std::string &name)
  {
    static const std::string drop = " ^$#%&*-+=~`!@?<>,.:;'\"|\\/(){}[]";
    std::string out;
    out.reserve(name.size());
    for (char c : name)
      if (drop.find(c) == std::string::npos) out += c;
    return out;
  }

  inline std::vector<double> string_to_double_array(const std::string &str)
  {
    std::vector<double> out;
    size_t b = 0;
    while (b <= str.size()) {
      const size_t e = std::min(str.find(',', b), str.size());
      if (e > b || e < str.size()) out.push_back(std::stod(str.substr(b, e - b)));
      b = e + 1;
    }
    return out;
  }

  template <typename T> std::string getWithPrecision(uint precision, T number)
  {
    std::ostringstream os;
    os << std::fixed << std::setprecision((int)precision) << number;
    return os.str();
  }

  template <typename T> std::string to_string_with_digits(const T number, const int digits)
  {
    if (digits <= 0) throw std::runtime_error("to_string_with_digits: digits must be > 0");
    const int lead = (int)std::ceil(std::log10(std::fabs((double)number)));
    std::ostringstream os;
    os << std::fixed << std::setprecision(std::max(digits - lead, 0)) << number;
    return os.str();
  }

  inline bool file_exists(const std::string &name) { return std::ifstream(name).good(); }

  inline std::string make_folder(const std::string &path)
  {
    return (!path.empty() && path.back() == '/') ? path : path + '/';
  }

  inline bool create_folder(const std::string &path_)
  {
    std::error_code ec;
    std::filesystem::create_directories(make_folder(path_), ec);
    return !ec && std::filesystem::is_directory(make_folder(path_));
  }

  inline std::string time_format(size_t s)
  {
    using std::to_string;
    if (s < 120) return to_string(s) + "s";
    if (s < 3600) return to_string(s / 60) + "min" + to_string(s % 60) + "s";
    return to_string(s / 3600) + "h" + to_string((s % 3600) / 60) + "min" + to_string(s % 60) + "s";
  }

  inline std::string time_format_ms(size_t ms)
  {
    using std::to_string;
    if (ms < 1000) return to_string(ms) + "ms";
    if (ms < 60000) return to_string(ms / 1000) + "s" + to_string(ms % 1000) + "ms";
    if (ms < 3600000) return to_string(ms / 60000) + "min" + to_string((ms % 60000) / 1000) + "s";
    return to_string(ms / 3600000) + "h" + to_string((ms % 3600000) / 60000) + "min";
  }

  inline bool has_suffix(const std::string &str, const std::string &suffix)
  {
    return str.size() >= suffix.size() && str.compare(str.size() - suffix.size(), suffix.size(), suffix) == 0;
  }
} // namespace DiFfRG
