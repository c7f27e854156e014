// serve.cc -- the request loop of libgbint (continuous batching).
//
// request() calls from time steppers become gb_submit tickets.  A dispatcher thread forms
// device batches from the queue in arrival order (consecutive requests of one precision are
// merged up to max_items integrals; each request keeps its own tables), and launches a batch
// as soon as one of the max_inflight slots is free and its buffers fit the context's HBM
// budget.  Batches of different slots overlap on the device and requests keep being admitted
// while others run.  Each slot owns a device arena (descriptors, units, partials, results)
// and pinned staging, grown only when a batch needs more, so the steady state allocates
// nothing.  Serving grids are not persistent (one CTA per work unit) and small batches run on
// high-priority streams, so the block scheduler hands them SMs as soon as CTAs of a large
// batch retire instead of after the whole large batch.  Completion is detected with CUDA
// events; results arrive in pinned host memory on the batch stream.  Every result is
// independent of what it was batched with (the per-integral finish sums its units in a fixed
// order), which the tests check bit for bit.  Latency = submit -> result ready (p50/p99).
//
// Table updates are ordered against serving: a batch's stream waits for the last table update
// before it starts, and a table update waits for in-flight batches before it overwrites the
// back buffer, so each batch reads one consistent epoch of every table.
#include "engine.hh"
#include "kernels.hh"
#include "trace.hh"

#include <algorithm>
#include <chrono>
#include <cmath>

namespace gbint
{
  namespace
  {
    double now_s()
    {
      return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }

    enum ReqState { RQ_QUEUED = 0, RQ_RUNNING = 1, RQ_DONE = 2, RQ_FAILED = 3, RQ_CANCELED = 4 };

    struct Request {
      gb_ticket id = 0;
      std::vector<gb_integral> items;
      std::vector<gb_table *> tables;
      int precision = GB_PREC_FP32C;
      double t_submit = 0;
      std::vector<double> results;
      int state = RQ_QUEUED;
      int rc = GB_OK;
      std::string err;
    };

    // batches below this many quadrature points go to the high-priority stream of their slot
    constexpr uint64_t kSmallBatchPoints = 1ull << 27;

    struct Slot {
      cudaStream_t s_hi = nullptr, s_lo = nullptr;
      cudaEvent_t done = nullptr;
      // device arena (bytes counted in the context's in_use)
      size_t cap_items = 0, cap_units = 0, cap_segs = 0, cap_seg = 0, cap_aux = 0, bytes = 0;
      ItemDev *d_items = nullptr;
      UnitDev *d_units = nullptr;
      ExpandDev *d_expand = nullptr;
      SegDev *d_segs = nullptr;
      double *d_seg = nullptr, *d_partials = nullptr, *d_out = nullptr;
      float4 *d_aux = nullptr;
      int *d_item_count = nullptr, *d_counters = nullptr;
      // pinned staging of the same capacities
      ItemDev *h_items = nullptr;
      UnitDev *h_units = nullptr;
      ExpandDev *h_expand = nullptr;
      SegDev *h_segs = nullptr;
      float4 *h_aux = nullptr;
      double *h_out = nullptr;
      gb_batch *plan = nullptr;
      std::vector<Request *> reqs;
      bool busy = false;
      double t_launch = 0;
    };

    constexpr int kMaxRunsPerBatch = 16;
  } // namespace

  struct ServeState {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<Request *> queue;
    std::map<gb_ticket, Request *> all;
    std::vector<Slot> slots;
    int max_items = 2048;
    bool stop = false;
    gb_ticket next_id = 1;
    // statistics
    uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0, points = 0;
    double busy_s = 0, busy_since = -1;
    std::vector<double> lat;
  };

  namespace
  {
    void free_arena(gb_ctx *ctx, Slot &sl)
    {
      cudaFree(sl.d_items);
      cudaFree(sl.d_units);
      cudaFree(sl.d_expand);
      cudaFree(sl.d_segs);
      cudaFree(sl.d_seg);
      cudaFree(sl.d_aux);
      cudaFree(sl.d_partials);
      cudaFree(sl.d_out);
      cudaFree(sl.d_item_count);
      cudaFree(sl.d_counters);
      cudaFreeHost(sl.h_items);
      cudaFreeHost(sl.h_units);
      cudaFreeHost(sl.h_expand);
      cudaFreeHost(sl.h_segs);
      cudaFreeHost(sl.h_aux);
      cudaFreeHost(sl.h_out);
      ctx->in_use -= sl.bytes;
      const cudaStream_t a = sl.s_hi, b = sl.s_lo;
      const cudaEvent_t d = sl.done;
      sl = Slot{};
      sl.s_hi = a;
      sl.s_lo = b;
      sl.done = d;
    }

    size_t arena_bytes(size_t items, size_t units, size_t segs, size_t seg, size_t aux)
    {
      return items * (sizeof(ItemDev) + sizeof(ExpandDev) + sizeof(double) + sizeof(int)) +
             units * (sizeof(UnitDev) + sizeof(double)) +
             segs * sizeof(SegDev) + seg * sizeof(double) + aux * sizeof(float4) + kMaxRunsPerBatch * sizeof(int);
    }

    // make the slot's arena hold a batch of the given sizes; GB_EBUDGET if the budget is short.
    // Caller holds ctx->mu and the slot is idle.
    int reserve(gb_ctx *ctx, Slot &sl, size_t items, size_t units, size_t segs, size_t seg, size_t aux)
    {
      if (items <= sl.cap_items && units <= sl.cap_units && segs <= sl.cap_segs && seg <= sl.cap_seg &&
          aux <= sl.cap_aux)
        return GB_OK;
      auto grow = [](size_t need, size_t cap) { return need <= cap ? cap : std::max(need, cap + cap / 2); };
      const size_t ni = grow(items, sl.cap_items), nu = grow(units, sl.cap_units), ns = grow(segs, sl.cap_segs),
                   nseg = grow(seg, sl.cap_seg), na = grow(aux, sl.cap_aux);
      const size_t nb = arena_bytes(ni, nu, ns, nseg, na);
      if (ctx->in_use - sl.bytes + nb > ctx->budget)
        return set_error(ctx, GB_EBUDGET, "serving batch does not fit the HBM budget now");
      free_arena(ctx, sl);
      cudaError_t e = cudaSuccess;
      auto dev = [&](void **p, size_t sz) {
        if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(sz, 16));
      };
      auto host = [&](void **p, size_t sz) {
        if (e == cudaSuccess) e = cudaMallocHost(p, std::max<size_t>(sz, 16));
      };
      dev((void **)&sl.d_items, ni * sizeof(ItemDev));
      dev((void **)&sl.d_units, nu * sizeof(UnitDev));
      dev((void **)&sl.d_expand, ni * sizeof(ExpandDev));
      dev((void **)&sl.d_segs, ns * sizeof(SegDev));
      dev((void **)&sl.d_seg, nseg * sizeof(double));
      dev((void **)&sl.d_aux, na * sizeof(float4));
      dev((void **)&sl.d_partials, nu * sizeof(double));
      dev((void **)&sl.d_out, ni * sizeof(double));
      dev((void **)&sl.d_item_count, ni * sizeof(int));
      dev((void **)&sl.d_counters, kMaxRunsPerBatch * sizeof(int));
      host((void **)&sl.h_items, ni * sizeof(ItemDev));
      host((void **)&sl.h_units, nu * sizeof(UnitDev));
      host((void **)&sl.h_expand, ni * sizeof(ExpandDev));
      host((void **)&sl.h_segs, ns * sizeof(SegDev));
      host((void **)&sl.h_aux, na * sizeof(float4));
      host((void **)&sl.h_out, ni * sizeof(double));
      sl.bytes = nb;
      ctx->in_use += nb;
      if (e != cudaSuccess) {
        free_arena(ctx, sl);
        return cuda_fail(ctx, e, "serving arena");
      }
      sl.cap_items = ni;
      sl.cap_units = nu;
      sl.cap_segs = ns;
      sl.cap_seg = nseg;
      sl.cap_aux = na;
      return GB_OK;
    }

    // the requests of a finished (or failed) slot get their results; the slot becomes free
    void finish_slot(gb_ctx *ctx, ServeState *S, Slot &sl, bool ok, const std::string &err)
    {
      const double t = now_s();
      if (log_enabled()) {
        size_t n = 0;
        double oldest = t;
        for (Request *r : sl.reqs) {
          n += r->items.size();
          oldest = std::min(oldest, r->t_submit);
        }
        log_event("serve_done", jfields("\"slot\": %d, \"ok\": %d, \"requests\": %zu, \"integrals\": %zu, "
                                        "\"gpu_ms\": %.3f, \"max_latency_ms\": %.3f",
                                        (int)(&sl - S->slots.data()), ok ? 1 : 0, sl.reqs.size(), n,
                                        (t - sl.t_launch) * 1e3, (t - oldest) * 1e3));
      }
      {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        free_batch(ctx, sl.plan);  // arena batch: releases the held axes only
        sl.plan = nullptr;
      }
      std::lock_guard<std::mutex> lk(S->mu);
      size_t off = 0;
      for (Request *r : sl.reqs) {
        if (ok) {
          r->results.assign(sl.h_out + off, sl.h_out + off + r->items.size());
          r->state = RQ_DONE;
          S->lat.push_back(t - r->t_submit);
          S->completed++;
        } else {
          r->state = RQ_FAILED;
          r->rc = GB_EDEVICE;
          r->err = err;
        }
        off += r->items.size();
      }
      sl.reqs.clear();
      sl.busy = false;
      bool any = false;
      for (auto &s2 : S->slots) any |= s2.busy;
      if (!any && S->busy_since >= 0) {
        S->busy_s += t - S->busy_since;
        S->busy_since = -1;
      }
      S->cv_done.notify_all();
    }

    // consecutive queued requests of the head's precision, up to max_items integrals
    std::vector<Request *> take_group(ServeState *S)
    {
      std::vector<Request *> g;
      // canceled requests leave the queue here (and are freed if their ticket was polled)
      auto drop = [&](Request *r) {
        S->queue.pop_front();
        if (!S->all.count(r->id)) delete r;
      };
      while (!S->queue.empty() && S->queue.front()->state == RQ_CANCELED) drop(S->queue.front());
      if (S->queue.empty()) return g;
      const int prec = S->queue.front()->precision;
      size_t items = 0;
      while (!S->queue.empty()) {
        Request *r = S->queue.front();
        if (r->state == RQ_CANCELED) {
          drop(r);
          continue;
        }
        if (r->precision != prec || (!g.empty() && items + r->items.size() > (size_t)S->max_items)) break;
        g.push_back(r);
        items += r->items.size();
        S->queue.pop_front();
      }
      return g;
    }

    // plan the group's integrals and launch them on the slot (caller: dispatcher thread)
    int launch_group(gb_ctx *ctx, ServeState *S, Slot &sl, const std::vector<Request *> &g)
    {
      TraceRange tr("gbint serve_launch");
      std::vector<gb_integral> items;
      std::vector<gb_table *const *> tl;
      std::vector<int> tn;
      for (Request *r : g)
        for (const auto &it : r->items) {
          items.push_back(it);
          tl.push_back(r->tables.data());
          tn.push_back((int)r->tables.size());
        }
      const int n = (int)items.size();
      std::lock_guard<std::recursive_mutex> lk(ctx->mu);
      // a group of table updates is in progress: launch after it, so that the batch sees all
      // of the group or none of it
      if (ctx->update_depth > 0) return GB_EAGAIN;
      cudaSetDevice(ctx->device);
      gb_batch *b = new gb_batch();
      int rc = plan_batch(ctx, items.data(), n, tl.data(), tn.data(), g[0]->precision, b);
      if (rc == GB_OK && b->runs.size() > (size_t)kMaxRunsPerBatch) rc = set_error(ctx, GB_EINVAL, "too many kind runs");
      if (rc == GB_OK) rc = reserve(ctx, sl, n, b->n_units_total, b->segs.size(), b->seg_total, b->aux.size());
      if (rc) {
        free_batch(ctx, b);
        return rc;
      }
      // bind the arena, stage the descriptors, order after the last table update, run
      b->arena = true;
      b->d_items = sl.d_items;
      b->d_units = sl.d_units;
      b->d_expand = sl.d_expand;
      b->d_segs = sl.d_segs;
      b->d_seg = sl.d_seg;
      b->d_aux = sl.d_aux;
      b->d_partials = sl.d_partials;
      b->d_item_count = sl.d_item_count;
      b->d_counters = sl.d_counters;
      b->d_out = sl.d_out;
      // not persistent: one CTA per unit that retires after it, so SMs free up per unit
      b->single = true;
      for (auto &run : b->runs) run.ctas = run.n_units;
      std::memcpy(sl.h_items, b->items.data(), n * sizeof(ItemDev));
      // the units themselves are written on the device from one range per integral (or, for a
      // cost-ordered run, uploaded as built)
      if (b->host_units)
        std::memcpy(sl.h_units, b->units.data(), b->units.size() * sizeof(UnitDev));
      else
        std::memcpy(sl.h_expand, b->expand.data(), b->expand.size() * sizeof(ExpandDev));
      if (!b->segs.empty()) std::memcpy(sl.h_segs, b->segs.data(), b->segs.size() * sizeof(SegDev));
      if (!b->aux.empty()) std::memcpy(sl.h_aux, b->aux.data(), b->aux.size() * sizeof(float4));
      const cudaStream_t s = b->points < kSmallBatchPoints ? sl.s_hi : sl.s_lo;
      cudaError_t e = cudaStreamWaitEvent(s, ctx->tables_event, 0);
      if (e == cudaSuccess) e = cudaMemcpyAsync(sl.d_items, sl.h_items, n * sizeof(ItemDev), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess && b->host_units)
        e = cudaMemcpyAsync(sl.d_units, sl.h_units, b->units.size() * sizeof(UnitDev), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess && !b->host_units) {
        e = cudaMemcpyAsync(sl.d_expand, sl.h_expand, b->expand.size() * sizeof(ExpandDev), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = launch_expand_units(sl.d_expand, (int)b->expand.size(), sl.d_units, s);
      }
      if (e == cudaSuccess && !b->segs.empty())
        e = cudaMemcpyAsync(sl.d_segs, sl.h_segs, b->segs.size() * sizeof(SegDev), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess && !b->aux.empty())
        e = cudaMemcpyAsync(sl.d_aux, sl.h_aux, b->aux.size() * sizeof(float4), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(sl.d_item_count, 0, n * sizeof(int), s);
      if (e != cudaSuccess) {
        cudaStreamSynchronize(s);
        free_batch(ctx, b);
        return cuda_fail(ctx, e, "serving batch upload");
      }
      rc = run_batch(ctx, b, nullptr, s);
      if (rc == GB_OK) {
        e = cudaMemcpyAsync(sl.h_out, sl.d_out, n * sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaEventRecord(sl.done, s);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "serving batch launch");
      }
      if (rc) {
        // work may be queued on s: let it drain before the arena is reused
        cudaStreamSynchronize(s);
        free_batch(ctx, b);
        return rc;
      }
      sl.plan = b;
      sl.reqs = g;
      sl.t_launch = now_s();
      if (log_enabled())
        log_event("serve_launch", jfields("\"slot\": %d, \"requests\": %zu, \"integrals\": %d, \"points\": %llu, "
                                          "\"high_priority\": %d, \"queue_ms\": %.3f",
                                          (int)(&sl - S->slots.data()), g.size(), n, (unsigned long long)b->points,
                                          s == sl.s_hi ? 1 : 0, (sl.t_launch - g[0]->t_submit) * 1e3));
      std::lock_guard<std::mutex> lk2(S->mu);
      sl.busy = true;
      S->batches++;
      S->points += b->points;
      return GB_OK;
    }

    void loop(gb_ctx *ctx)
    {
      ServeState *S = ctx->serve;
      cudaSetDevice(ctx->device);
      for (;;) {
        // completions
        for (auto &sl : S->slots) {
          bool busy;
          {
            std::lock_guard<std::mutex> lk(S->mu);
            busy = sl.busy;
          }
          if (!busy) continue;
          const cudaError_t q = cudaEventQuery(sl.done);
          if (q == cudaSuccess)
            finish_slot(ctx, S, sl, true, "");
          else if (q != cudaErrorNotReady)
            finish_slot(ctx, S, sl, false, cudaGetErrorString(q));
        }
        // admission: the queue head takes the first free slot
        std::vector<Request *> g;
        Slot *slot = nullptr;
        bool any_busy = false;
        {
          std::unique_lock<std::mutex> lk(S->mu);
          if (S->stop) break;
          for (auto &sl : S->slots) {
            any_busy |= sl.busy;
            if (!sl.busy && !slot) slot = &sl;
          }
          if (slot) g = take_group(S);
          if (g.empty()) {
            // poll completions every 20 us while the GPU works, else sleep until a submit
            if (any_busy)
              S->cv.wait_for(lk, std::chrono::microseconds(20));
            else
              S->cv.wait_for(lk, std::chrono::milliseconds(50));
            continue;
          }
          for (Request *r : g) r->state = RQ_RUNNING;
          if (S->busy_since < 0) S->busy_since = now_s();
        }
        int rc = launch_group(ctx, S, *slot, g);
        if (rc == GB_EAGAIN) {
          // table-update group open: the requests go back to the head of the queue
          std::unique_lock<std::mutex> lk(S->mu);
          for (auto it = g.rbegin(); it != g.rend(); ++it) {
            (*it)->state = RQ_QUEUED;
            S->queue.push_front(*it);
          }
          S->cv.wait_for(lk, std::chrono::microseconds(50));
          continue;
        }
        if (rc == GB_EBUDGET) {
          if (any_busy) {
            // wait for memory: the group goes back to the head of the queue
            std::unique_lock<std::mutex> lk(S->mu);
            for (auto it = g.rbegin(); it != g.rend(); ++it) {
              (*it)->state = RQ_QUEUED;
              S->queue.push_front(*it);
            }
            S->cv_done.wait_for(lk, std::chrono::milliseconds(1));
            continue;
          }
          // nothing in flight: give back the idle arenas and try once more
          {
            std::lock_guard<std::recursive_mutex> lk(ctx->mu);
            for (auto &sl : S->slots)
              if (&sl != slot) free_arena(ctx, sl);
          }
          rc = launch_group(ctx, S, *slot, g);
        }
        if (rc) {
          std::lock_guard<std::mutex> lk(S->mu);
          for (Request *r : g) {
            r->state = RQ_FAILED;
            r->rc = rc;
            r->err = ctx->last_error;
          }
          if (rc == GB_EBUDGET) S->rejected += g.size();
          bool busy = false;
          for (auto &sl : S->slots) busy |= sl.busy;
          if (!busy && S->busy_since >= 0) {
            S->busy_s += now_s() - S->busy_since;
            S->busy_since = -1;
          }
          S->cv_done.notify_all();
        }
      }
      // drain what is in flight
      for (auto &sl : S->slots)
        if (sl.busy) {
          const cudaError_t e = cudaEventSynchronize(sl.done);
          finish_slot(ctx, S, sl, e == cudaSuccess, e == cudaSuccess ? "" : cudaGetErrorString(e));
        }
    }
  } // namespace

  int serve_fence_tables(gb_ctx *ctx, cudaStream_t s)
  {
    for (auto &sl : ctx->serve->slots) GB_CUDA(cudaStreamWaitEvent(s, sl.done, 0));
    return GB_OK;
  }

  int serve_start(gb_ctx *ctx, int max_inflight, int max_items)
  {
    if (!ctx) return GB_EINVAL;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (ctx->serve) return set_error(ctx, GB_EINVAL, "serving already started");
    if (max_inflight < 1 || max_inflight > 64 || max_items < 1)
      return set_error(ctx, GB_EINVAL, "gb_serve_start: max_inflight must be 1..64 and max_items >= 1");
    GB_CUDA(cudaSetDevice(ctx->device));
    int lo = 0, hi = 0;
    GB_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));  // hi is the numerically smaller one
    auto S = std::make_unique<ServeState>();
    S->max_items = max_items;
    S->slots.resize(max_inflight);
    for (auto &sl : S->slots) {
      cudaError_t e = cudaStreamCreateWithPriority(&sl.s_hi, cudaStreamNonBlocking, hi);
      if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&sl.s_lo, cudaStreamNonBlocking, lo);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
      if (e != cudaSuccess) {
        for (auto &s2 : S->slots) {
          if (s2.s_hi) cudaStreamDestroy(s2.s_hi);
          if (s2.s_lo) cudaStreamDestroy(s2.s_lo);
          if (s2.done) cudaEventDestroy(s2.done);
        }
        return cuda_fail(ctx, e, "serving streams");
      }
    }
    ctx->serve = S.release();
    ctx->serve->th = std::thread(loop, ctx);
    return GB_OK;
  }

  int serve_stop(gb_ctx *ctx)
  {
    if (!ctx || !ctx->serve) return GB_OK;
    ServeState *S = ctx->serve;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
    }
    S->cv.notify_all();
    if (S->th.joinable()) S->th.join();
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    for (auto &sl : S->slots) {
      free_arena(ctx, sl);
      cudaStreamDestroy(sl.s_hi);
      cudaStreamDestroy(sl.s_lo);
      cudaEventDestroy(sl.done);
    }
    // canceled requests already polled are referenced by the queue only
    for (Request *r : S->queue)
      if (!S->all.count(r->id)) delete r;
    for (auto &kv : S->all) delete kv.second;
    ctx->serve = nullptr;
    delete S;
    return GB_OK;
  }

  int serve_submit(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                   gb_ticket *out)
  {
    if (!ctx) return GB_EINVAL;
    if (!items || n <= 0 || !out || n_tables < 0 || (n_tables > 0 && !tables))
      return set_error(ctx, GB_EINVAL, "gb_submit: bad arguments");
    if (precision < GB_PREC_FP32C || precision > GB_PREC_FP32A) return set_error(ctx, GB_EINVAL, "bad precision");
    ServeState *S = ctx->serve;
    if (!S) return set_error(ctx, GB_EINVAL, "serving not started (gb_serve_start)");
    // a request whose descriptors alone exceed the budget can never be admitted
    if (arena_bytes(n, n, 0, 0, 0) > ctx->budget) {
      std::lock_guard<std::mutex> lk(S->mu);
      S->rejected++;
      return set_error(ctx, GB_EBUDGET, "request can never fit the HBM budget");
    }
    auto *r = new Request();
    r->items.assign(items, items + n);
    if (n_tables > 0) r->tables.assign(tables, tables + n_tables);
    else r->tables.push_back(nullptr);
    r->precision = precision;
    r->t_submit = now_s();
    {
      std::lock_guard<std::mutex> lk(S->mu);
      r->id = S->next_id++;
      S->all[r->id] = r;
      S->queue.push_back(r);
      S->submitted++;
    }
    S->cv.notify_all();
    *out = r->id;
    return GB_OK;
  }

  int serve_poll(gb_ctx *ctx, gb_ticket t, double *out, bool wait, double timeout_s)
  {
    if (!ctx) return GB_EINVAL;
    ServeState *S = ctx->serve;
    if (!S) return set_error(ctx, GB_EINVAL, "serving not started");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(t);
    if (it == S->all.end()) return set_error(ctx, GB_EINVAL, "unknown ticket");
    Request *r = it->second;
    auto pending = [&] { return r->state == RQ_QUEUED || r->state == RQ_RUNNING; };
    if (wait && pending()) {
      const auto deadline =
          std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9);
      if (!S->cv_done.wait_until(lk, deadline, [&] { return !pending(); }))
        return set_error(ctx, GB_ETIMEDOUT, "gb_wait timed out");
    }
    if (pending()) return GB_EAGAIN;
    const int state = r->state, rc = r->rc;
    if (state == RQ_DONE && out) std::copy(r->results.begin(), r->results.end(), out);
    const std::string err = r->err;
    S->all.erase(it);
    // a canceled request may still sit in the queue; the dispatcher drops it there
    bool queued = false;
    if (state == RQ_CANCELED)
      for (Request *q : S->queue) queued |= q == r;
    if (!queued) delete r;
    lk.unlock();
    if (state == RQ_CANCELED) return GB_ECANCELED;
    if (state == RQ_FAILED) return set_error(ctx, rc ? rc : GB_EDEVICE, err);
    return GB_OK;
  }

  int serve_cancel(gb_ctx *ctx, gb_ticket t)
  {
    if (!ctx) return GB_EINVAL;
    ServeState *S = ctx->serve;
    if (!S) return set_error(ctx, GB_EINVAL, "serving not started");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(t);
    if (it == S->all.end()) return set_error(ctx, GB_EINVAL, "unknown ticket");
    if (it->second->state != RQ_QUEUED) return GB_EAGAIN;  // already on the GPU (or done)
    it->second->state = RQ_CANCELED;
    S->cv_done.notify_all();
    return GB_OK;
  }

  int serve_stats(gb_ctx *ctx, gb_stats *out)
  {
    if (!ctx || !out) return GB_EINVAL;
    *out = gb_stats{};
    out->bytes_in_use = ctx->in_use;
    out->bytes_budget = ctx->budget;
    ServeState *S = ctx->serve;
    if (!S) return GB_OK;
    std::lock_guard<std::mutex> lk(S->mu);
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->rejected = S->rejected;
    out->batches_launched = S->batches;
    out->points_evaluated = S->points;
    out->busy_seconds = S->busy_s + (S->busy_since >= 0 ? now_s() - S->busy_since : 0.0);
    if (!S->lat.empty()) {
      std::vector<double> v = S->lat;
      std::sort(v.begin(), v.end());
      // nearest-rank percentile
      auto pct = [&](double q) {
        const size_t r = (size_t)std::ceil(q * (double)v.size());
        return v[std::min(v.size(), std::max<size_t>(r, 1)) - 1];
      };
      out->p50_latency_s = pct(0.50);
      out->p99_latency_s = pct(0.99);
      out->max_latency_s = v.back();
    }
    return GB_OK;
  }

  int serve_reset_stats(gb_ctx *ctx)
  {
    if (!ctx || !ctx->serve) return GB_OK;
    ServeState *S = ctx->serve;
    std::lock_guard<std::mutex> lk(S->mu);
    S->submitted = S->completed = S->rejected = S->batches = S->points = 0;
    S->busy_s = 0;
    S->busy_since = -1;
    for (auto &sl : S->slots)
      if (sl.busy) S->busy_since = now_s();
    S->lat.clear();
    return GB_OK;
  }
} // namespace gbint
