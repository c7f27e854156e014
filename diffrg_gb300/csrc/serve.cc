// serve.cc -- request loop of libgbint (continuous batching).
#include "engine.hh"

namespace gbint
{
  int serve_start(gb_ctx *ctx, int, int) { return set_error(ctx, GB_EINVAL, "serving not available"); }
  int serve_stop(gb_ctx *) { return GB_OK; }
  int serve_submit(gb_ctx *ctx, const gb_integral *, int, gb_table *const *, int, int, gb_ticket *)
  {
    return set_error(ctx, GB_EINVAL, "serving not started");
  }
  int serve_poll(gb_ctx *ctx, gb_ticket, double *, bool, double) { return set_error(ctx, GB_EINVAL, "no ticket"); }
  int serve_cancel(gb_ctx *ctx, gb_ticket) { return set_error(ctx, GB_EINVAL, "no ticket"); }
  int serve_stats(gb_ctx *ctx, gb_stats *out)
  {
    if (!ctx || !out) return GB_EINVAL;
    *out = gb_stats{};
    return GB_OK;
  }
  int serve_reset_stats(gb_ctx *) { return GB_OK; }
} // namespace gbint
