// slots.cu -- request slots for user-kernel launches from the C++ class templates.
//
// A slot bundles what one reference request() takes from RMM and the stream pool
// (integrator_4D_gpu.hh:173-197): a pooled stream, a device buffer of FP64 unit partials, the
// work-unit / arrival counters, a device result and a pinned host landing place.  Slots are
// recycled: acquire picks a free slot whose capacity fits (or grows one), release returns it.
#include "engine.hh"

#include <algorithm>

namespace gbint
{
  struct SlotRec {
    gb_slot pub{};
    cudaStream_t stream = nullptr;
    double *host_result = nullptr;  // pinned
    void *host_staging = nullptr;   // pinned, grown on demand (gb_slot_host)
    size_t host_staging_bytes = 0;
    bool busy = false;
  };
  struct SlotPool {
    std::mutex mu;
    std::vector<SlotRec *> all;
  };

  SlotPool *slot_pool(gb_ctx *ctx)
  {
    static std::mutex create_mu;
    std::lock_guard<std::mutex> lk(create_mu);
    if (!ctx->slotpool) ctx->slotpool = new SlotPool();
    return ctx->slotpool;
  }

  void destroy_slots(gb_ctx *ctx)
  {
    if (!ctx->slotpool) return;
    for (SlotRec *s : ctx->slotpool->all) {
      cudaStreamSynchronize(s->stream);
      cudaFree(s->pub.partials);
      cudaFree(s->pub.counters);
      cudaFreeHost(s->host_result);
      if (s->host_staging) cudaFreeHost(s->host_staging);
      cudaStreamDestroy(s->stream);
      delete s;
    }
    delete ctx->slotpool;
    ctx->slotpool = nullptr;
  }
} // namespace gbint

using namespace gbint;

extern "C" {

int gb_slot_acquire(gb_ctx *ctx, int units, gb_slot *out)
{
  if (!ctx || !out || units <= 0) return set_error(ctx, GB_EINVAL, "bad slot request");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  SlotPool *P = slot_pool(ctx);
  SlotRec *pick = nullptr;
  {
    std::lock_guard<std::mutex> lk(P->mu);
    for (SlotRec *s : P->all)
      if (!s->busy && s->pub.capacity_units >= units) {
        pick = s;
        break;
      }
    if (!pick)
      for (SlotRec *s : P->all)
        if (!s->busy) {
          pick = s;
          break;
        }
    if (pick) pick->busy = true;
  }
  if (!pick) {
    pick = new SlotRec();
    e = cudaStreamCreateWithFlags(&pick->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&pick->pub.counters, 4 * sizeof(int) + sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&pick->host_result, sizeof(double));
    if (e != cudaSuccess) {
      delete pick;
      return cuda_fail(ctx, e, "slot creation");
    }
    pick->pub.result = reinterpret_cast<double *>(pick->pub.counters + 2);
    pick->pub.stream = pick->stream;
    pick->busy = true;
    std::lock_guard<std::mutex> lk(P->mu);
    pick->pub.id = (int)P->all.size();
    P->all.push_back(pick);
  }
  if (pick->pub.capacity_units < units) {
    cudaStreamSynchronize(pick->stream);
    cudaFree(pick->pub.partials);
    const int cap = std::max(units, 2 * pick->pub.capacity_units);
    e = cudaMalloc(&pick->pub.partials, (size_t)cap * sizeof(double));
    if (e != cudaSuccess) {
      pick->pub.partials = nullptr;
      pick->pub.capacity_units = 0;
      std::lock_guard<std::mutex> lk(P->mu);
      pick->busy = false;
      return cuda_fail(ctx, e, "slot partials");
    }
    pick->pub.capacity_units = cap;
  }
  e = cudaMemsetAsync(pick->pub.counters, 0, 2 * sizeof(int), pick->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "slot reset");
  *out = pick->pub;
  return GB_OK;
}

int gb_slot_wait(gb_ctx *ctx, const gb_slot *slot, double *out)
{
  if (!ctx || !slot || !out || !ctx->slotpool) return set_error(ctx, GB_EINVAL, "bad slot");
  SlotRec *s = nullptr;
  {
    std::lock_guard<std::mutex> lk(ctx->slotpool->mu);
    if (slot->id < 0 || slot->id >= (int)ctx->slotpool->all.size()) return set_error(ctx, GB_EINVAL, "bad slot id");
    s = ctx->slotpool->all[slot->id];
  }
  cudaError_t e = cudaMemcpyAsync(s->host_result, s->pub.result, sizeof(double), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "slot wait");
  *out = *s->host_result;
  return GB_OK;
}

int gb_slot_host(gb_ctx *ctx, const gb_slot *slot, size_t bytes, void **host)
{
  if (!ctx || !slot || !host || !ctx->slotpool) return set_error(ctx, GB_EINVAL, "bad slot");
  SlotRec *s = nullptr;
  {
    std::lock_guard<std::mutex> lk(ctx->slotpool->mu);
    if (slot->id < 0 || slot->id >= (int)ctx->slotpool->all.size()) return set_error(ctx, GB_EINVAL, "bad slot id");
    s = ctx->slotpool->all[slot->id];
  }
  if (s->host_staging_bytes < bytes) {
    // the slot's previous work has drained (the slot is held by its caller); grow 1.5x
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (s->host_staging) cudaFreeHost(s->host_staging);
    s->host_staging = nullptr;
    s->host_staging_bytes = 0;
    const size_t cap = std::max(bytes, (size_t)64 << 10) + bytes / 2;
    if (e == cudaSuccess) e = cudaMallocHost(&s->host_staging, cap);
    if (e != cudaSuccess) {
      s->host_staging = nullptr;
      return cuda_fail(ctx, e, "slot host staging");
    }
    s->host_staging_bytes = cap;
  }
  *host = s->host_staging;
  return GB_OK;
}

int gb_slot_release(gb_ctx *ctx, const gb_slot *slot)
{
  if (!ctx || !slot || !ctx->slotpool) return GB_EINVAL;
  std::lock_guard<std::mutex> lk(ctx->slotpool->mu);
  if (slot->id < 0 || slot->id >= (int)ctx->slotpool->all.size()) return GB_EINVAL;
  ctx->slotpool->all[slot->id]->busy = false;
  return GB_OK;
}

int gb_buffer_create(gb_ctx *ctx, size_t bytes, void **d_ptr)
{
  if (!ctx || !d_ptr || bytes == 0) return set_error(ctx, GB_EINVAL, "bad buffer request");
  if (ctx->in_use + bytes > ctx->budget) return set_error(ctx, GB_EBUDGET, "buffer exceeds the HBM budget");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(d_ptr, bytes);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gb_buffer_create");
  ctx->in_use += bytes;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  ctx->buffers[*d_ptr] = bytes;
  return GB_OK;
}

int gb_buffer_upload(gb_ctx *ctx, void *d_ptr, const void *host, size_t bytes)
{
  if (!ctx || !d_ptr || !host) return GB_EINVAL;
  {
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    auto it = ctx->buffers.find(d_ptr);
    if (it == ctx->buffers.end() || it->second < bytes) return set_error(ctx, GB_EINVAL, "unknown buffer or too many bytes");
  }
  // in place, after the device drained: kernels in flight on pooled streams may read the buffer
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(d_ptr, host, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gb_buffer_upload");
  return GB_OK;
}

int gb_buffer_destroy(gb_ctx *ctx, void *d_ptr)
{
  if (!ctx || !d_ptr) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  auto it = ctx->buffers.find(d_ptr);
  if (it == ctx->buffers.end()) return GB_EINVAL;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();  // in-flight kernels may still read it
  cudaFree(d_ptr);
  ctx->in_use -= it->second;
  ctx->buffers.erase(it);
  return GB_OK;
}

int gb_device_info(gb_ctx *ctx, int *device, int *num_sms)
{
  if (!ctx) return GB_EINVAL;
  if (device) *device = ctx->device;
  if (num_sms) *num_sms = ctx->num_sms;
  return GB_OK;
}

} // extern "C"
