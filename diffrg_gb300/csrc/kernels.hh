// kernels.hh -- host-side launchers of the gbint kernels (implemented in kernels_*.cu).
#pragma once

#include <cuda_runtime.h>

#include "engine_types.hh"

namespace gbint
{
  // generic FP64 kernel: points per unit
  constexpr int kGenericThreads = 256;
  constexpr int kGenericPPT = 4;
  constexpr int kGenericUnitPoints = kGenericThreads * kGenericPPT;

  cudaError_t launch_generic(const RunParams &P, int ctas, cudaStream_t s);
  // also zeroes the n_counters (<= 64) work counters of the batch's kind runs
  cudaError_t launch_seg(const SegDev *segs, int n_segs, int total_entries, const double *pv, const double *pw,
                         const float4 *aux, const TableDev *tabs, double *seg_out, int *counters, int n_counters,
                         cudaStream_t s);
  // writes the UnitDev records of n integrals' unit ranges, in stream order
  cudaError_t launch_expand_units(const ExpandDev *ex, int n, UnitDev *units, cudaStream_t s);
  // rebuilds a 1D table's per-cell records (TableDev::cr_off, gr_off) from its data (table, laid
  // out as D describes), in stream order
  cudaError_t launch_cell_records(float *table, const TableDev &D, cudaStream_t s);
  // writes one table directory entry in stream order (the entry travels as a kernel parameter)
  cudaError_t launch_dir_set(TableDev *dst, const TableDev &v, cudaStream_t s);
  // writes n directory entries dir[slot[i]] = v[i] in stream order (chunks travel as parameters)
  cudaError_t launch_dir_set_many(TableDev *dir, const int *slot, const TableDev *v, int n, cudaStream_t s);
  // FP32-compensated persistent kernels (kinds K_S1..K_S5); threads in {128, 256, 512}
  cudaError_t launch_fp32c(int kind, const RunParams &P, int threads, int ctas, int tab_bytes_cap, int rec_cap,
                           cudaStream_t s);
  // resident CTAs per SM for that configuration (0 if it cannot launch)
  int fp32c_occupancy(int kind, int threads, int tab_bytes_cap, int rec_cap);
  int kind_default_threads(int kind);
  // the schedule of a kind when nothing is set (every field filled in)
  gb_schedule kind_default_schedule(int kind);

  // reference execution pattern: one value per (row of) point(s) into dest
  cudaError_t launch_plain(const ItemDev *item_dev, long long n_threads, int loop_axis, const double *pv,
                           const double *pw, const TableDev *tabs, double *dest, cudaStream_t s);

  // plain FFMA / MUFU throughput probes (peaks for the roofline)
  cudaError_t launch_peak_ffma(float *out, int ctas, int threads, int iters, cudaStream_t s);
  cudaError_t launch_peak_mufu(float *out, int ctas, int threads, int iters, cudaStream_t s);
  cudaError_t launch_peak_dfma(double *out, int ctas, int threads, int iters, cudaStream_t s);
  // one bounded mbarrier wait that nothing completes (records ERR_MBAR_TIMEOUT after `limit` cycles)
  cudaError_t launch_wait_selftest(int *err, long long limit, cudaStream_t s);
} // namespace gbint
