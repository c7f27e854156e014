// kernels_generic.cu -- FP64 kernels: the generic fused kernel (any family x any catalogue
// integrand), the reference-pattern per-point kernel, the hoisted-factor (segment) kernel and
// the FFMA/MUFU/DFMA peak probes used as roofline denominators.
#include "device_common.cuh"
#include "integrands.cuh"
#include "kernels.hh"

namespace gbint
{
  using namespace dev;

  // ------------------------------------------------------------------------------------------
  // Generic fused FP64 kernel.  Persistent CTAs take work units (item, point range) from an
  // atomic counter; each thread evaluates kGenericPPT points of the flattened tensor grid,
  // partials are reduced in FP64 and the last unit of an item finishes it (unit_finish).
  // Replaces gridreduce_* + thrust::reduce (e.g. integrator_4D_gpu.hh:21-49,141-158) with one
  // launch for a whole batch and no per-point global buffer.
  // ------------------------------------------------------------------------------------------
  __global__ void __launch_bounds__(kGenericThreads) k_generic(const RunParams P)
  {
    __shared__ double red[32];
    __shared__ int s_unit, s_flag;
    __shared__ TableDev sT[4];
    for (int iter = 0;; ++iter) {
      if (threadIdx.x == 0)
        s_unit = P.single ? (iter == 0 ? (int)blockIdx.x : P.n_units) : atomicAdd(P.unit_counter, 1);
      __syncthreads();
      const int u = s_unit;
      if (u >= P.n_units) break;
      const UnitDev U = P.units[u];
      const ItemDev &it = P.items[U.item];
      if (threadIdx.x < 4) {
        const int slot = it.tab[threadIdx.x];
        if (slot >= 0) sT[threadIdx.x] = P.tabs[slot];
      }
      __syncthreads();
      double acc = 0.0;
#pragma unroll 1
      for (int k = 0; k < kGenericPPT; ++k) {
        const int local = threadIdx.x + k * blockDim.x;
        if (local < U.row_count) acc += eval_point_fp64(it, (long long)U.row_begin + local, P.pv, P.pw, sT);
      }
      const double tot = block_sum(acc, red);
      unit_finish(P, U.slot, U.item, tot, red, &s_flag);
    }
  }

  cudaError_t launch_generic(const RunParams &P, int ctas, cudaStream_t s)
  {
    k_generic<<<ctas, kGenericThreads, 0, s>>>(P);
    return cudaGetLastError();
  }

  // ------------------------------------------------------------------------------------------
  // Reference execution pattern (the FP64 denominator): one thread per point -- or per point of
  // the other axes with an in-thread loop over `loop_axis`, as gridreduce_4d loops over cos2
  // (integrator_4D_gpu.hh:42-47) and gridreduce_4d_finiteT* over q0 -- writing one FP64 value to
  // global memory for a later device-wide reduction.
  // ------------------------------------------------------------------------------------------
  __global__ void __launch_bounds__(256) k_plain(const ItemDev *itp, long long n_threads, int loop_axis,
                                                 const double *pv, const double *pw, const TableDev *tabs,
                                                 double *dest)
  {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_threads) return;
    const ItemDev &it = *itp;
    TableDev T[4];
    for (int i = 0; i < 4; ++i)
      if (it.tab[i] >= 0) T[i] = tabs[it.tab[i]];
    const int nloop = loop_axis >= 0 ? it.ax[loop_axis].n : 1;
    double acc = 0.0;
    for (int l = 0; l < nloop; ++l) {
      Pt P{0, 0, 0, 0, 0, 0, 0, 0, it.k};
      double w = 1.0;
      bool pm = false;
      long long rem = t;
      for (int a = it.n_axes - 1; a >= 0; --a) {
        const AxisRef ax = it.ax[a];
        int idx;
        if (a == loop_axis)
          idx = l;
        else {
          idx = (int)(rem % ax.n);
          rem /= ax.n;
        }
        const int node = ax.off + idx;
        set_role(P, ax.role, pv[node]);
        w *= pw[node];
        if (idx >= ax.pm_from) pm = true;
      }
      double f = ig_eval64(it.integrand, it.family, P, it.args, T);
      if (pm) {
        P.q0 = -P.q0;
        f += ig_eval64(it.integrand, it.family, P, it.args, T);
      }
      acc += w * f;
    }
    dest[t] = acc;
  }

  cudaError_t launch_plain(const ItemDev *item_dev, long long n_threads, int loop_axis, const double *pv,
                           const double *pw, const TableDev *tabs, double *dest, cudaStream_t s)
  {
    const long long blocks = (n_threads + 255) / 256;
    k_plain<<<(unsigned)blocks, 256, 0, s>>>(item_dev, n_threads, loop_axis, pv, pw, tabs, dest);
    return cudaGetLastError();
  }

  // ------------------------------------------------------------------------------------------
  // Hoisted FP64 factors of the FP32-compensated kernels: one-axis (or two-axis) parts of the
  // integrand that many points share, evaluated once per node in FP64.
  // ------------------------------------------------------------------------------------------
  __global__ void __launch_bounds__(256) k_seg(const SegDev *segs, const double *pv, const double *pw,
                                               const float4 *aux, const TableDev *tabs, double *out, int *counters,
                                               int n_counters)
  {
    // the work counters of the kernels that follow in stream order start from zero
    if (blockIdx.x == 0 && blockIdx.y == 0 && (int)threadIdx.x < n_counters) counters[threadIdx.x] = 0;
    const SegDev S = segs[blockIdx.y];
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= S.n0 * S.n1) return;
    const TableDev &T = tabs[S.tab];
    double F = 0.0;
    switch (S.kind) {
    case SEG_S1: {
      const int i = S.ax0.off + e;
      const double q = pv[i], q2 = q * q;
      F = pw[i] * S.par[0] * G1_64(T, q2) * reg_Rdot(q2);
      break;
    }
    case SEG_S2: {
      // F_{m,i} = w_m w_q Rdot(q^2) / (Z(|w_m| / 2 pi T, |q|) (w_m^2 + q^2) + R(q^2)); the q-only
      // factors come from the host (FP64, per q node: w_q Rdot(q^2), R(q^2), q^2, |q| fraction
      // and cell on the table), so an entry is one bilinear lookup and one division
      const int m = e / S.n1, i = e % S.n1;
      const double *Q = reinterpret_cast<const double *>(aux + S.aux_off) + 6 * i;
      const double w = pv[S.ax0.off + m];
      int jw;
      const double fw = dev::axis_frac64(T.a0, fabs(w) / (2 * 3.14159265358979323846 * S.par[0]), jw);
      const int jq = (int)Q[4], n1 = T.n1;
      const float *d0 = T.data + (size_t)jw * n1 + jq, *d1 = d0 + n1;
      const double lo = dev::lerp64(d0[0], d1[0], fw), hi = dev::lerp64(d0[1], d1[1], fw);
      const double z = dev::lerp64(lo, hi, Q[3]);
      F = pw[S.ax0.off + m] * Q[0] / (z * (w * w + Q[2]) + Q[1]);
      // the S2 kernel multiplies this factor per point: stored as a double-float pair
      const dev::df f = dev::df_from(F);
      reinterpret_cast<float2 *>(out)[S.off + e] = make_float2(f.hi, f.lo);
      return;
    }
    case SEG_AX1: {
      // node k of the axis, first-axis cell ix: the table lerped along its second axis at rows ix
      // and ix + 1, stored as {z, dz = z' - z} double-float pairs
      const int k = e / S.n1, ix = e % S.n1;
      int jc;
      const double fc = dev::axis_frac64(T.a1, pv[S.ax0.off + k], jc);
      const float *d0 = T.data + (size_t)ix * T.n1 + jc, *d1 = d0 + T.n1;
      const double z0 = dev::lerp64(d0[0], d0[1], fc), z1 = dev::lerp64(d1[0], d1[1], fc);
      const dev::df a = dev::df_from(z0), b = dev::df_from(z1 - z0);
      reinterpret_cast<float4 *>(out + S.off)[e] = make_float4(a.hi, a.lo, b.hi, b.lo);
      return;
    }
    case SEG_S2Z: {
      // record r = 2 m + sign at frequency +-w_m + W, |q| cell jq: the table lerped along its mode
      // axis at columns jq and jq + 1, stored as {z, dz = z' - z} double-float pairs
      const int r = e / S.n1, jq = e % S.n1;
      const double w = pv[S.ax0.off + (r >> 1)];
      const double ws = ((r & 1) ? -w : w) + S.par[0];
      int j;
      const double f = dev::axis_frac64(T.a0, fabs(ws) * S.par[1], j);
      const float *d0 = T.data + (size_t)j * T.n1 + jq, *d1 = d0 + T.n1;
      const double z0 = dev::lerp64(d0[0], d1[0], f), z1 = dev::lerp64(d0[1], d1[1], f);
      const dev::df a = dev::df_from(z0), b = dev::df_from(z1 - z0);
      reinterpret_cast<float4 *>(out + S.off)[e] = make_float4(a.hi, a.lo, b.hi, b.lo);
      return;
    }
    case SEG_S3: {
      const int i = S.ax0.off + e;
      const double q = pv[i], q2 = q * q;
      F = pw[i] * reg_Rdot(q2) * G1_64(T, q2);
      break;
    }
    case SEG_S5: {
      const int i = e / S.n1, j = e % S.n1;
      const int ni = S.ax0.off + i, nj = S.ax1.off + j;
      const double q = pv[ni], q2 = q * q;
      F = pw[ni] * pw[nj] * reg_Rdot(q2) * G2_64(T, q2, pv[nj]);
      break;
    }
    }
    out[S.off + e] = F;
  }

  cudaError_t launch_seg(const SegDev *segs, int n_segs, int max_entries, const double *pv, const double *pw,
                         const float4 *aux, const TableDev *tabs, double *seg_out, int *counters, int n_counters,
                         cudaStream_t s)
  {
    if (n_counters > 64) return cudaErrorInvalidValue;
    if (n_segs == 0) return cudaSuccess;
    // each entry is a chain of FP64 operations on the low-rate FP64 pipe: small CTAs spread the
    // entries over all SMs instead of queueing them on a few
    constexpr int kSegThreads = 64;
    dim3 grid((max_entries + kSegThreads - 1) / kSegThreads, n_segs);
    k_seg<<<grid, kSegThreads, 0, s>>>(segs, pv, pw, aux, tabs, seg_out, counters, n_counters);
    return cudaGetLastError();
  }
  __global__ void k_dir_set(TableDev *dst, const TableDev v) { *dst = v; }

  // one CTA per integral (grid-stride), its threads over the integral's units
  __global__ void k_expand_units(const ExpandDev *ex, int n, UnitDev *units)
  {
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
      const ExpandDev e = ex[i];
      for (int u = threadIdx.x; u < e.n_units; u += blockDim.x) {
        UnitDev U;
        U.item = e.item;
        U.row_begin = u * e.rpu;
        U.row_count = min(e.rpu, e.rows - u * e.rpu);
        U.slot = e.slot0 + u;
        units[(size_t)e.unit0 + u] = U;
      }
    }
  }

  cudaError_t launch_expand_units(const ExpandDev *ex, int n, UnitDev *units, cudaStream_t s)
  {
    if (n <= 0) return cudaSuccess;
    k_expand_units<<<n < 4096 ? n : 4096, 256, 0, s>>>(ex, n, units);
    return cudaGetLastError();
  }

  // Per-cell records of a 1D log table, one thread a cell.  Value record: {1/c_j hi, lo, y_j,
  // hi(d_j)} and lo(d_j), d_j = y_{j+1} - y_j split exactly into two floats.  Within cell j the
  // table value is linear in the log index, so in t = x / c_j - 1 (c_j the cell centre) it is
  // Z = z0 + z1 ln(1 + t), z0 = (y_j + y_{j+1}) / 2, z1 = d_j kln.  Propagator record (with the
  // regulator's FP64 coefficients a_k of R(c_j (1 + t))), in FP64: the Taylor series of 1 / D,
  // D = c_j (1 + t) Z + R, from D's coefficients d_k = c_j (w_k + w_{k-1}) + a_k (w_k those of Z,
  // w_0 = z0, w_k = (-1)^(k+1) z1 / k) by the recursion
  // g_0 = 1 / d_0, g_k = -g_0 sum_{i=1..k} d_i g_{k-i}, in four float4 arrays of a float4 per
  // cell: {1/c_j hi, lo, g0 hi, lo}, {g1 hi, lo, g2 hi, lo}, {g3, g4, g5, g6}, {g7, g8, el, +-eh}.  (el, eh): the cell's edges in t,
  // 2^(-+1/(2 scale)) - 1, moved inwards by 4e-7 (more than the FP32 error of the kernels' t):
  // a t outside them sends the kernel to an exact decision of the cell.  eh is negative where the
  // series is not trusted over the cell (its tail, estimated from the ratio of the last two
  // coefficients, above 1e-12 of g_0); the kernels evaluate such cells from the value record and
  // the regulator.
  __global__ void k_cell_records(float *table, const int rc_off, const int cr_off, const int gr_off,
                                 const int rd_off, const int cells, const double scale, const double shift)
  {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cells) return;
    const float y0 = table[j], y1 = table[j + 1];
    const double d = (double)y1 - (double)y0;  // exact
    const double kln = scale / 0.69314718055994530942;
    const double z0 = (double)y0 + 0.5 * d, z1 = d * kln;
    const double hl = 0.34657359027997265471 / scale;  // ln 2 / (2 scale): half a cell in ln x
    const float el = __fadd_rn((float)expm1(-hl), 4e-7f), eh = __fsub_rn((float)expm1(hl), 4e-7f);
    const float2 r = reinterpret_cast<const float2 *>(table + rc_off)[j];
    const dev::df dd = dev::two_sum(y1, -y0);
    reinterpret_cast<float4 *>(table + cr_off)[j] = make_float4(r.x, r.y, y0, dd.hi);
    table[cr_off + 4 * cells + j] = dd.lo;
    if (!gr_off) return;
    const double *a = reinterpret_cast<const double *>(table + rd_off) + 10 * j;
    const double c = exp2(((double)j + 0.5 - shift) / scale);
    constexpr int K = 9;  // coefficients g0..g8
    double w[K], D[K], g[K];
    w[0] = z0;
    for (int k = 1; k < K; ++k) w[k] = z1 * ((k & 1) ? 1.0 : -1.0) / k;
    D[0] = c * w[0] + a[0];
    for (int k = 1; k < K; ++k) D[k] = c * (w[k] + w[k - 1]) + a[k];
    g[0] = 1.0 / D[0];
    for (int k = 1; k < K; ++k) {
      double s = 0.0;
      for (int i = 1; i <= k; ++i) s += D[i] * g[k - i];
      g[k] = -s * g[0];
    }
    // the cell spans |t| <= 2^(1/(2 scale)) - 1
    const double h = expm1(hl);
    const double rt = g[K - 2] != 0.0 ? fabs(g[K - 1] / g[K - 2]) * h : 1.0;
    double hk = h;
    for (int k = 1; k < K - 1; ++k) hk *= h;
    bool ok = D[0] > 0.0 && rt < 0.5 && fabs(g[K - 1]) * hk * rt / (1.0 - rt) <= 1e-12 * fabs(g[0]);
    for (int k = 0; k < K; ++k) ok = ok && isfinite(g[k]);
    const dev::df G0 = dev::df_from(g[0]), G1 = dev::df_from(g[1]), G2 = dev::df_from(g[2]);
    // four float4 arrays of `cells` entries (a lookup's 16-byte loads at different cells then
    // fall on different shared-memory banks)
    float4 *gr = reinterpret_cast<float4 *>(table + gr_off) + j;
    gr[0] = make_float4(r.x, r.y, G0.hi, G0.lo);
    gr[cells] = make_float4(G1.hi, G1.lo, G2.hi, G2.lo);
    gr[2 * cells] = make_float4((float)g[3], (float)g[4], (float)g[5], (float)g[6]);
    gr[3 * cells] = make_float4((float)g[7], (float)g[8], el, ok ? eh : -eh);
  }

  cudaError_t launch_cell_records(float *table, const TableDev &D, cudaStream_t s)
  {
    const int cells = D.n0 - 1;
    if (cells <= 0 || !D.cr_off) return cudaSuccess;
    k_cell_records<<<(cells + 127) / 128, 128, 0, s>>>(table, D.rc_off, D.cr_off, D.gr_off, D.rd_off, cells,
                                                        D.a0.scale64, D.a0.shift64);
    return cudaGetLastError();
  }

  cudaError_t launch_dir_set(TableDev *dst, const TableDev &v, cudaStream_t s)
  {
    k_dir_set<<<1, 1, 0, s>>>(dst, v);
    return cudaGetLastError();
  }

  constexpr int kDirChunk = 24;
  struct DirChunk {
    int n;
    int slot[kDirChunk];
    TableDev v[kDirChunk];
  };
  static_assert(sizeof(DirChunk) <= 4096, "directory chunk exceeds the kernel parameter limit");
  __global__ void k_dir_set_many(TableDev *dir, const DirChunk c)
  {
    if ((int)threadIdx.x < c.n) dir[c.slot[threadIdx.x]] = c.v[threadIdx.x];
  }

  cudaError_t launch_dir_set_many(TableDev *dir, const int *slot, const TableDev *v, int n, cudaStream_t s)
  {
    for (int i = 0; i < n; i += kDirChunk) {
      DirChunk c{};
      c.n = n - i < kDirChunk ? n - i : kDirChunk;
      for (int j = 0; j < c.n; ++j) {
        c.slot[j] = slot[i + j];
        c.v[j] = v[i + j];
      }
      k_dir_set_many<<<1, kDirChunk, 0, s>>>(dir, c);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }


  // ------------------------------------------------------------------------------------------
  // Throughput probes: 8 independent dependency chains per thread.
  // ------------------------------------------------------------------------------------------
  __global__ void k_peak_ffma(float *out, int iters)
  {
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-7f + i;
    const float b = 0.9999f, c = 1e-6f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int r = 0; r < 16; ++r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = __fmaf_rn(a[i], b, c);
      }
    }
    float s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == 123.456f) out[0] = s;
  }
  __global__ void k_peak_mufu(float *out, int iters)
  {
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = 1.0f + threadIdx.x * 1e-7f + i * 1e-3f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = __log2f(a[i] + 2.0f);
      }
    }
    float s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == 123.456f) out[0] = s;
  }
  __global__ void k_peak_dfma(double *out, int iters)
  {
    double a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-7 + i;
    const double b = 0.9999, c = 1e-6;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = fma(a[i], b, c);
      }
    }
    double s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == 123.456) out[0] = s;
  }
  cudaError_t launch_peak_ffma(float *out, int ctas, int threads, int iters, cudaStream_t s)
  {
    k_peak_ffma<<<ctas, threads, 0, s>>>(out, iters);
    return cudaGetLastError();
  }
  cudaError_t launch_peak_mufu(float *out, int ctas, int threads, int iters, cudaStream_t s)
  {
    k_peak_mufu<<<ctas, threads, 0, s>>>(out, iters);
    return cudaGetLastError();
  }
  // Self-test of the bounded waits: an mbarrier that expects one arrival nobody makes.  The
  // wait gives up after `limit` cycles and records ERR_MBAR_TIMEOUT, as a stalled TMA copy would.
  __global__ void k_wait_selftest(int *err, long long limit)
  {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
      dev::mbar_init(&bar, 1);
      dev::mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) dev::mbar_wait_bounded(&bar, 0, err, limit);
    __syncthreads();
  }

  cudaError_t launch_wait_selftest(int *err, long long limit, cudaStream_t s)
  {
    k_wait_selftest<<<1, 32, 0, s>>>(err, limit);
    return cudaGetLastError();
  }

  cudaError_t launch_peak_dfma(double *out, int ctas, int threads, int iters, cudaStream_t s)
  {
    k_peak_dfma<<<ctas, threads, 0, s>>>(out, iters);
    return cudaGetLastError();
  }
} // namespace gbint
