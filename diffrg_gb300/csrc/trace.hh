// trace.hh -- NVTX ranges and the optional JSON-lines event log of libgbint.
//
// NVTX ranges (header-only NVTX v3: inert unless a profiler is attached) mark every batch run,
// table update, serving launch and the reference-pattern path.  The event log is off unless
// the environment variable GBINT_LOG names a file (or "stderr"); each line is one JSON object
// {"t": seconds since the first event, "event": name, ...fields}.
#pragma once

#include <string>

#include <nvtx3/nvToolsExt.h>

namespace gbint
{
  struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
  };

  bool log_enabled();
  // fields: the inside of a JSON object without braces, e.g. "\"n\": 3, \"ms\": 1.5" (may be empty)
  void log_event(const char *event, const std::string &fields);
  // printf-style helper for the fields
  std::string jfields(const char *fmt, ...) __attribute__((format(printf, 1, 2)));
} // namespace gbint
