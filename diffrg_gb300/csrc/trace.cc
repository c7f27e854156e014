// trace.cc -- the JSON-lines event log (see trace.hh).
#include "trace.hh"

#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace gbint
{
  namespace
  {
    std::once_flag g_once;
    std::mutex g_mu;
    FILE *g_out = nullptr;
    std::chrono::steady_clock::time_point g_t0;

    void open_log()
    {
      const char *p = std::getenv("GBINT_LOG");
      if (!p || !*p) return;
      g_out = std::strcmp(p, "stderr") == 0 ? stderr : std::fopen(p, "a");
      g_t0 = std::chrono::steady_clock::now();
    }
  } // namespace

  bool log_enabled()
  {
    std::call_once(g_once, open_log);
    return g_out != nullptr;
  }

  void log_event(const char *event, const std::string &fields)
  {
    if (!log_enabled()) return;
    const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - g_t0).count();
    std::lock_guard<std::mutex> lk(g_mu);
    std::fprintf(g_out, "{\"t\": %.6f, \"event\": \"%s\"%s%s}\n", t, event, fields.empty() ? "" : ", ",
                 fields.c_str());
    std::fflush(g_out);
  }

  std::string jfields(const char *fmt, ...)
  {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return buf;
  }
} // namespace gbint
