// engine.cu -- C ABI of libgbint: context, QuadratureProvider, dressing tables, batch planning
// and execution, and the reference-pattern FP64 path.
#include "engine.hh"
#include "kernels.hh"
#include "trace.hh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <new>
#include <set>
#include <stdexcept>

#include <cub/device/device_reduce.cuh>

using namespace gbint;

namespace gbint
{
  int set_error(gb_ctx *ctx, int code, const std::string &msg)
  {
    if (ctx) ctx->last_error = msg;
    return code;
  }
  int cuda_fail(gb_ctx *ctx, cudaError_t e, const char *what)
  {
    return set_error(ctx, GB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
} // namespace gbint


namespace
{
  constexpr double kPi = 3.14159265358979323846;
  constexpr int kPoolCapacity = 1 << 21;  // nodes (about 112 MB of device memory)
  constexpr int kPoolStreams = 16;

  double S_d(int d) { return 2.0 * std::pow(kPi, d / 2.0) / std::tgamma(d / 2.0); }
  double powi(double x, int n)
  {
    if (n < 0) return 1.0 / powi(x, -n);
    double r = 1;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
  }

  dev::AxisDev make_axis(int n, int log, double lo, double hi)
  {
    dev::AxisDev a{};
    a.n = n;
    a.log = log;
    if (n < 2) {
      a.scale64 = 0;
      a.shift64 = 0;
    } else if (log) {
      a.scale64 = (n - 1) / std::log2(hi / lo);
      a.shift64 = -std::log2(lo) * a.scale64;
    } else {
      a.scale64 = (n - 1) / (hi - lo);
      a.shift64 = -lo * a.scale64;
    }
    a.scale = dev::df_from(a.scale64);
    a.shift = dev::df_from(a.shift64);
    a.kln = dev::df_from(a.scale64 / std::log(2.0));
    return a;
  }

  const GLRule &gl_host(gb_ctx *ctx, int n)
  {
    auto it = ctx->gl.find(n);
    if (it != ctx->gl.end()) return it->second;
    GLRule &r = ctx->gl[n];
    gl_rule01(n, r.x, r.w);
    return r;
  }

  // Matsubara cache with the reference's relative 1e-6 match on T and E
  // (MatsubaraStorage::find_T_d / find_E_d, quadrature_provider.cu:12-58)
  MatsEntry &mats_host(gb_ctx *ctx, double T, double E)
  {
    auto close = [](double a, double b) { return std::fabs(a - b) <= 1e-6 * std::fabs(b) || a == b; };
    for (auto &m : ctx->mats)
      if (close(T, m->T) && close(E, m->E)) return *m;
    auto e = std::make_unique<MatsEntry>();
    e->T = T;
    e->E = E;
    e->rule = matsubara_rule(T, E, 2, ctx->mats_min, 128, ctx->mats_vacuum, ctx->mats_add);
    ctx->mats.push_back(std::move(e));
    return *ctx->mats.back();
  }

  // ------------------------------------------------------------------ axes
  enum AxisKind : int {
    AK_XRAD = 1,   // q = k sqrt(t x_ext), w = w_t x_ext C q^pw
    AK_QRAD = 2,   // q = qmax t, w = qmax w_t C q^pw
    AK_COS = 3,    // c = 2(t - 1/2), w = 2 w_t C [sqrt(1-c^2)]
    AK_PHI = 4,    // phi = 2 pi t, w = 2 pi w_t C
    AK_CART = 5,   // v = qmin + ext t, w = ext w_t C
    AK_PQ0 = 6,    // q0 = s t ext, w = w_t ext, all nodes +-
    AK_MATS = 7,   // [0 (w = T)] + Monien nodes, +- from 1
    AK_FTX0 = 8,   // explicit sum (w = T) + log-mapped tail
    AK_MODES = 9,  // w_m = 2 pi T m, m = 0..M, w = C, +- from 1
    AK_ONE = 10    // single node 0 with weight C
  };

  // first fit in the free list, else the bump region
  bool pool_take(NodePool &P, int n, int &off)
  {
    for (auto it = P.free_ranges.begin(); it != P.free_ranges.end(); ++it)
      if (it->second >= n) {
        off = it->first;
        const int rest = it->second - n;
        P.free_ranges.erase(it);
        if (rest) P.free_ranges[off + n] = rest;
        return true;
      }
    if (P.used + n > P.capacity) return false;
    off = P.used;
    P.used += n;
    return true;
  }

  // drop every axis no batch holds; its range joins the free list (coalesced)
  void pool_evict_unheld(gb_ctx *ctx)
  {
    NodePool &P = ctx->pool;
    const uint64_t ev0 = P.evictions;
    for (auto it = ctx->axis_cache.begin(); it != ctx->axis_cache.end();) {
      if (it->second.refs == 0) {
        P.free_ranges[it->second.ref.off] = it->second.ref.n;
        P.evictions++;
        it = ctx->axis_cache.erase(it);
      } else
        ++it;
    }
    for (auto it = P.free_ranges.begin(); it != P.free_ranges.end();) {
      auto nx = std::next(it);
      if (nx != P.free_ranges.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        P.free_ranges.erase(nx);
        continue;
      }
      ++it;
    }
    if (!P.free_ranges.empty()) {  // a free tail returns to the bump region
      auto last = std::prev(P.free_ranges.end());
      if (last->first + last->second == P.used) {
        P.used = last->first;
        P.free_ranges.erase(last);
      }
    }
    if (log_enabled())
      log_event("node_pool_evict", jfields("\"axes\": %llu, \"used\": %d, \"free_ranges\": %zu",
                                           (unsigned long long)(P.evictions - ev0), P.used, P.free_ranges.size()));
  }

  int pool_append(gb_ctx *ctx, const HostAxis &h, AxisRef &ref)
  {
    const int n = (int)h.v.size();
    int off = 0;
    if (!pool_take(ctx->pool, n, off)) {
      pool_evict_unheld(ctx);
      if (!pool_take(ctx->pool, n, off))
        return set_error(ctx, GB_ENOMEM, "node pool exhausted (all axes held by live batches)");
    }
    std::vector<NodeRec> rec(n);
    for (int i = 0; i < n; ++i) {
      const dev::df v = dev::df_from(h.v[i]), w = dev::df_from(h.w[i]), a = dev::df_from(h.a[i]),
                    aw = dev::df_from(h.w[i] * h.a[i]);
      rec[i] = NodeRec{v.hi, v.lo, w.hi, w.lo, a.hi, a.lo, aw.hi, aw.lo};
    }
    // stream-ordered copies on the context's own (non-blocking) stream, then a wait on that
    // stream only: the nodes are in place before any later launch on any stream reads them,
    // and the legacy default stream is never touched
    cudaStream_t s = ctx->stream;
    GB_CUDA(cudaMemcpyAsync(ctx->pool.d_v + off, h.v.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaMemcpyAsync(ctx->pool.d_w + off, h.w.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaMemcpyAsync(ctx->pool.d_a + off, h.a.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaMemcpyAsync(ctx->pool.d_rec + off, rec.data(), n * sizeof(NodeRec), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaStreamSynchronize(s));
    ref.off = off;
    ref.n = n;
    ref.pm_from = std::min(h.pm_from, n);
    return GB_OK;
  }

  int build_axis(gb_ctx *ctx, const AxisKey &key, HostAxis &h)
  {
    const int n = key.n;
    const double *p = key.p;
    auto gl = [&](int order) -> const GLRule & { return gl_host(ctx, order); };
    switch (key.kind) {
    case AK_XRAD: {  // p: x_ext, k, pw, C
      const GLRule &R = gl(n);
      for (int i = 0; i < n; ++i) {
        const double q = p[1] * std::sqrt(R.x[i] * p[0]);
        h.v.push_back(q);
        h.w.push_back(R.w[i] * p[0] * p[3] * powi(q, (int)p[2]));
        h.a.push_back(q * q);
      }
      break;
    }
    case AK_QRAD: {  // p: qmax, pw, C
      const GLRule &R = gl(n);
      for (int i = 0; i < n; ++i) {
        const double q = p[0] * R.x[i];
        h.v.push_back(q);
        h.w.push_back(p[0] * R.w[i] * p[2] * powi(q, (int)p[1]));
        h.a.push_back(q * q);
      }
      break;
    }
    case AK_COS: {  // p: jac, C
      const GLRule &R = gl(n);
      for (int i = 0; i < n; ++i) {
        const double t = R.x[i];
        const double c = 2 * (t - 0.5);
        const double s = 2.0 * std::sqrt(t * (1.0 - t));  // sqrt(1 - c^2) without cancellation
        h.v.push_back(c);
        h.w.push_back(2 * R.w[i] * p[1] * (p[0] != 0 ? s : 1.0));
        h.a.push_back(s);
      }
      break;
    }
    case AK_PHI: {  // p: C
      const GLRule &R = gl(n);
      for (int i = 0; i < n; ++i) {
        const double ph = 2 * kPi * R.x[i];
        h.v.push_back(ph);
        h.w.push_back(2 * kPi * R.w[i] * p[0]);
        h.a.push_back(std::cos(ph));
      }
      break;
    }
    case AK_CART: {  // p: qmin, ext, C
      const GLRule &R = gl(n);
      for (int i = 0; i < n; ++i) {
        const double v = p[0] + p[1] * R.x[i];
        h.v.push_back(v);
        h.w.push_back(p[1] * R.w[i] * p[2]);
        h.a.push_back(v * v);
      }
      break;
    }
    case AK_PQ0: {  // p: ext, scale
      const GLRule &R = gl(n);
      for (int i = 0; i < n; ++i) {
        const double q0 = p[1] * R.x[i] * p[0];
        h.v.push_back(q0);
        h.w.push_back(R.w[i] * p[0]);
        h.a.push_back(q0 * q0);
      }
      h.pm_from = 0;
      break;
    }
    case AK_MATS: {  // p: T, E
      const MatsEntry &M = mats_host(ctx, p[0], p[1]);
      const bool zero = p[0] > 0;  // the integrator's m_T decides (integrator_finiteTq0_cpu.hh:107-108)
      if (zero) {
        h.v.push_back(0.0);
        h.w.push_back(p[0]);
        h.a.push_back(0.0);
      }
      for (size_t i = 0; i < M.rule.x.size(); ++i) {
        h.v.push_back(M.rule.x[i]);
        h.w.push_back(M.rule.w[i]);
        h.a.push_back(M.rule.x[i] * M.rule.x[i]);
      }
      h.pm_from = zero ? 1 : 0;
      break;
    }
    case AK_FTX0: {  // n = tail order; p: T, k, x0_ext, ns, C_int
      const double T = p[0], k = p[1], x0e = p[2];
      const int ns = (int)p[3];
      for (int m = 0; m < ns; ++m) {
        const double q0 = 2 * kPi * T * m;
        h.v.push_back(q0);
        h.w.push_back(T);
        h.a.push_back(q0 * q0);
      }
      const bool Tzero = std::fabs(T) <= 1e-12;
      const double off = Tzero ? 1e-3 : 0.0;
      const double start = (2 * ns * kPi * (Tzero ? 0.0 : T)) / k;
      const double ls = std::log(start + off), le = std::log(x0e / (start + off));
      if (n > 0) {
        const GLRule &R = gl(n);
        for (int i = 0; i < n; ++i) {
          const double q0 = k * (std::exp(ls + le * R.x[i]) - off);
          h.v.push_back(q0);
          h.w.push_back(p[4] * R.w[i] * le * q0 / k);
          h.a.push_back(q0 * q0);
        }
      }
      h.pm_from = ns > 0 ? 1 : 0;
      break;
    }
    case AK_MODES: {  // n = M + 1; p: T, C
      for (int m = 0; m < n; ++m) {
        const double w = 2 * kPi * p[0] * m;
        h.v.push_back(w);
        h.w.push_back(p[1]);
        h.a.push_back(w * w);
      }
      h.pm_from = 1;
      break;
    }
    case AK_ONE: {
      h.v.push_back(0.0);
      h.w.push_back(p[0]);
      h.a.push_back(0.0);
      break;
    }
    default:
      return set_error(ctx, GB_EINVAL, "unknown axis kind");
    }
    return GB_OK;
  }

  // the axis of `key` (built and copied into the pool on first use); `hold` (if given) takes a
  // reference that keeps it from eviction until release_axes
  int get_axis(gb_ctx *ctx, const AxisKey &key, int role, AxisRef &ref, std::vector<AxisKey> *hold)
  {
    auto it = ctx->axis_cache.find(key);
    if (it == ctx->axis_cache.end()) {
      HostAxis h;
      int rc = build_axis(ctx, key, h);
      if (rc) return rc;
      if (h.v.empty()) return set_error(ctx, GB_EINVAL, "empty quadrature axis");
      AxisRef r{};
      rc = pool_append(ctx, h, r);
      if (rc) return rc;
      it = ctx->axis_cache.emplace(key, AxisEntry{r, 0, std::move(h.v), std::move(h.w)}).first;
    }
    ref = it->second.ref;
    ref.role = role;
    if (hold) {
      it->second.refs++;
      hold->push_back(key);
    }
    return GB_OK;
  }

  AxisKey K(int kind, int n, std::initializer_list<double> ps)
  {
    AxisKey k;
    k.kind = kind;
    k.n = n;
    int i = 0;
    for (double v : ps) k.p[i++] = v;
    return k;
  }

  // Family -> axes.  Every reference int_element / weight factor is folded into the axes
  // (constants into the radial axis).  Sources per family in gbint.h.
  int family_axes(gb_ctx *ctx, const gb_integral &g, AxisRef ax[4], int &na, std::vector<AxisKey> *hold)
  {
    const double k = g.k, xe = g.x_extent, tp = 2 * kPi;
    const int d = g.d;
    for (int i = 0; i < 4; ++i) ax[i] = AxisRef{0, 0, R_NONE, 1 << 30};
    na = 0;
    auto add = [&](const AxisKey &key, int role) -> int {
      if (key.kind != AK_MATS && key.kind != AK_FTX0 && key.kind != AK_ONE && key.kind != AK_MODES &&
          (key.n <= 0 || key.n > 4096))
        return set_error(ctx, GB_EINVAL, "quadrature order out of range (1..4096)");
      int rc = get_axis(ctx, key, role, ax[na], hold);
      if (rc) return rc;
      ++na;
      return GB_OK;
    };
    const int *n = g.n;
    int rc = GB_OK;
    switch (g.family) {
    case GB_FAM_1D:
      rc = add(K(AK_XRAD, n[0], {xe, k, double(d - 2), S_d(d) * k * k / 2 / powi(tp, d)}), R_Q);
      break;
    case GB_FAM_ANGLE:
      if ((rc = add(K(AK_XRAD, n[0], {xe, k, double(d - 2), S_d(d) * k * k / 2 * 0.5 / powi(tp, d)}), R_Q))) break;
      rc = add(K(AK_COS, n[1], {0, 1}), R_C1);
      break;
    case GB_FAM_3D:
      if ((rc = add(K(AK_XRAD, n[0], {xe, k, 1, k * k / 2 / powi(tp, 3)}), R_Q))) break;
      if ((rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
      rc = add(K(AK_PHI, n[2], {1}), R_PHI);
      break;
    case GB_FAM_4D2ANG:
      if ((rc = add(K(AK_XRAD, n[0], {xe, k, 2, tp * 0.5 * k * k / powi(tp, 4)}), R_Q))) break;
      if ((rc = add(K(AK_COS, n[1], {1, 1}), R_C1))) break;
      rc = add(K(AK_COS, n[2], {0, 1}), R_C2);
      break;
    case GB_FAM_4D:
      if ((rc = add(K(AK_XRAD, n[0], {xe, k, 2, 0.5 * k * k / powi(tp, 4)}), R_Q))) break;
      if ((rc = add(K(AK_COS, n[1], {1, 1}), R_C1))) break;
      if ((rc = add(K(AK_COS, n[2], {0, 1}), R_C2))) break;
      rc = add(K(AK_PHI, n[3], {1}), R_PHI);
      break;
    case GB_FAM_CART1:
    case GB_FAM_CART2:
    case GB_FAM_CART3: {
      const int dim = g.family - GB_FAM_CART1 + 1;
      const int roles[3] = {R_QX, R_QY, R_QZ};
      for (int a = 0; a < dim && !rc; ++a)
        rc = add(K(AK_CART, n[a], {g.qmin[a], g.qmax[a] - g.qmin[a], a == 0 ? powi(tp, -dim) : 1.0}), roles[a]);
      break;
    }
    case GB_FAM_2DPQ0:
    case GB_FAM_2DPX0: {
      const bool px = g.family == GB_FAM_2DPX0;
      if ((rc = add(K(AK_XRAD, n[0], {xe, k, 0, 0.5 * k * k * tp * 0.5 * (px ? k : 1.0) / powi(tp, 3)}), R_Q))) break;
      if ((rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
      rc = add(K(AK_PQ0, n[2], {g.x0_extent, px ? k : 1.0}), R_Q0);
      break;
    }
    case GB_FAM_3DPQ0:
    case GB_FAM_3DPX0: {
      const bool px = g.family == GB_FAM_3DPX0;
      if ((rc = add(K(AK_XRAD, n[0], {xe, k, 1, 0.5 * k * k * (px ? k : 1.0) / powi(tp, 4)}), R_Q))) break;
      if ((rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
      if ((rc = add(K(AK_PHI, n[2], {1}), R_PHI))) break;
      rc = add(K(AK_PQ0, n[3], {g.x0_extent, px ? k : 1.0}), R_Q0);
      break;
    }
    case GB_FAM_FTQ0:
    case GB_FAM_ANGLE_FTQ0:
    case GB_FAM_4D_FTQ0: {
      // E: given, else the reference rule (E = 10T, re-selected to k if |k-E|/max > 2.5%)
      double E = g.E;
      if (!(E > 0)) {
        E = 10 * g.T;
        if (std::fabs(k - E) / std::max(k, E) > 2.5e-2) E = k;
      }
      if (g.family == GB_FAM_4D_FTQ0) {
        if ((rc = add(K(AK_XRAD, n[0], {xe, k, 1, 0.5 * k * k / powi(tp, 3)}), R_Q))) break;
        if ((rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
        if ((rc = add(K(AK_PHI, n[2], {1}), R_PHI))) break;
      } else {
        const double half = g.family == GB_FAM_ANGLE_FTQ0 ? 0.5 : 1.0;
        if ((rc = add(K(AK_XRAD, n[0], {xe, k, double(d - 3), S_d(d - 1) * 0.5 * k * k * half / powi(tp, d - 1)}), R_Q)))
          break;
        if (g.family == GB_FAM_ANGLE_FTQ0 && (rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
      }
      rc = add(K(AK_MATS, 0, {g.T, E, (double)ctx->mats_min, (double)ctx->mats_vacuum, (double)ctx->mats_add}), R_Q0);
      break;
    }
    case GB_FAM_FTX0:
    case GB_FAM_ANGLE_FTX0:
    case GB_FAM_4D_FTX0: {
      const bool Tzero = std::fabs(g.T) <= 1e-12;
      const int ns = Tzero ? 0 : g.x0_summands;
      int tail;
      if (g.family == GB_FAM_4D_FTX0) {
        if ((rc = add(K(AK_XRAD, n[0], {xe, k, 1, 0.5 * k * k / powi(tp, 3)}), R_Q))) break;
        if ((rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
        if ((rc = add(K(AK_PHI, n[2], {1}), R_PHI))) break;
        tail = n[3];
      } else {
        const double half = g.family == GB_FAM_ANGLE_FTX0 ? 0.5 : 1.0;
        if ((rc = add(K(AK_XRAD, n[0], {xe, k, double(d - 3), S_d(d - 1) * 0.5 * k * k * half / powi(tp, d - 1)}), R_Q)))
          break;
        if (g.family == GB_FAM_ANGLE_FTX0) {
          if ((rc = add(K(AK_COS, n[1], {0, 1}), R_C1))) break;
          tail = n[2];
        } else
          tail = n[1];
      }
      tail += g.x0_summands - ns;  // at T = 0 the summands join the tail (integrator_finiteTx0_cpu.hh:41-50)
      if (tail < 0 || tail > 4096) return set_error(ctx, GB_EINVAL, "x0 quadrature order out of range");
      rc = add(K(AK_FTX0, tail, {Tzero ? 0.0 : g.T, k, g.x0_extent, (double)ns, k / tp}), R_Q0);
      break;
    }
    case GB_FAM_CONST:
      rc = add(K(AK_ONE, 1, {S_d(d) / powi(tp, d)}), R_NONE);
      break;
    case GB_FAM_QLOOP:
      if ((rc = add(K(AK_QRAD, n[0], {xe, 3, 4 * kPi / powi(tp, 4)}), R_Q))) break;
      rc = add(K(AK_COS, n[1], {0, 1}), R_C1);
      break;
    case GB_FAM_QLOOP_T: {
      const int M = g.x0_summands;
      if (M < 0 || M > 4095) return set_error(ctx, GB_EINVAL, "mode count out of range");
      if ((rc = add(K(AK_MODES, M + 1, {g.T, g.T * tp / powi(tp, 3)}), R_Q0))) break;
      if ((rc = add(K(AK_QRAD, n[0], {xe, 2, 1.0}), R_Q))) break;
      rc = add(K(AK_COS, n[1], {0, 1}), R_C1);
      break;
    }
    default:
      return set_error(ctx, GB_EINVAL, "unknown family");
    }
    return rc;
  }

  int tables_needed(int integrand)
  {
    switch (integrand) {
    case GB_IG_PROP1:
    case GB_IG_FTLOOP:
      return 1;
    case GB_IG_PROP3:
      return 4;
    case GB_IG_VERT4:
      return 2;
    }
    return 0;
  }
} // namespace

// ============================================================================ batches
namespace gbint
{
  void release_axes(gb_ctx *ctx, std::vector<AxisKey> &held)
  {
    for (const AxisKey &k : held) {
      auto it = ctx->axis_cache.find(k);
      if (it != ctx->axis_cache.end() && it->second.refs > 0) it->second.refs--;
    }
    held.clear();
  }

  void free_batch(gb_ctx *ctx, gb_batch *b)
  {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->h_err) cudaFreeHost(b->h_err);
    if (!b->arena) {
      cudaFree(b->d_items);
      cudaFree(b->d_units);
      cudaFree(b->d_expand);
      cudaFree(b->d_segs);
      cudaFree(b->d_seg);
      cudaFree(b->d_aux);
      cudaFree(b->d_partials);
      cudaFree(b->d_item_count);
      cudaFree(b->d_counters);
      cudaFree(b->d_out);
      if (ctx) ctx->in_use -= b->bytes;
    }
    if (ctx) release_axes(ctx, b->held);
    delete b;
  }

  size_t batch_device_bytes(const gb_batch *b)
  {
    const size_t n = b->n, nu = b->n_units_total;
    return n * sizeof(ItemDev) + nu * sizeof(UnitDev) + b->expand.size() * sizeof(ExpandDev) +
           b->segs.size() * sizeof(SegDev) +
           b->seg_total * sizeof(double) + b->aux.size() * sizeof(float4) + nu * sizeof(double) + n * sizeof(int) +
           b->runs.size() * sizeof(int) + n * sizeof(double);
  }

  // Per-item double-float constants of the S kinds, formed on the host in FP64 by the same
  // expressions the kernels would otherwise evaluate for every row on the (1/64-rate) FP64
  // pipe; for S2 also one record per (mode, sign): {cell, fraction, (+-w_m + W)^2 hi, lo} on
  // the table's mode axis.  `modes` are the host node values of the item's mode axis.
  void item_aux(const gb_ctx *ctx, const gb_integral &g, ItemDev &it, const std::vector<double> *modes,
                std::vector<float4> &aux)
  {
    auto df2 = [](double a, double b) {
      const dev::df x = dev::df_from(a), y = dev::df_from(b);
      return make_float4(x.hi, x.lo, y.hi, y.lo);
    };
    it.aux_off = (int)aux.size();
    const double p = g.args[1];
    switch (kind_base(it.kind)) {
    case K_S1:
      aux.push_back(df2(p * p, 2.0 * p));
      break;
    case K_S2: {
      aux.push_back(df2(p * p, 2.0 * p));
      const double T = g.args[2], Om = g.args[3];
      const double inv2piT = 1.0 / (2.0 * 3.14159265358979323846 * T);
      const dev::AxisDev &a0 = ctx->h_dir[it.tab[0]].a0;
      for (int m = 0; m < it.ax[0].n; ++m)
        for (int sg = 0; sg < 2; ++sg) {
          const double w = (*modes)[m];
          const double ws = (sg == 0 ? w : -w) + Om;
          int jj = 0;
          const float f = (float)dev::axis_frac64(a0, std::fabs(ws) * inv2piT, jj);
          const dev::df w2 = dev::df_from(ws * ws);
          float jf;
          std::memcpy(&jf, &jj, sizeof(jf));
          aux.push_back(make_float4(jf, f, w2.hi, w2.lo));
        }
      break;
    }
    case K_S3:
    case K_S3R:
      aux.push_back(df2(p, g.args[2]));                   // P, cos(theta)
      aux.push_back(df2(p * p, 0.25 * p * p));           // P^2, P^2 / 4
      aux.push_back(df2(g.args[3], 0.0));                 // sin(theta)
      break;
    case K_S5:
    case K_S5Z:
      aux.push_back(df2(p, p * p));                       // P, P^2
      aux.push_back(df2(g.args[2], g.args[3]));           // cos(alpha), sin(alpha)
      break;
    default:
      break;
    }
  }

  constexpr size_t kS5zSmemLimit = 200 * 1024;

  // Shared memory of the S5Z kernel at rpu rows per unit: table A's cell-centre reciprocals
  // (staged per item), then two per-unit buffers, each with the node records of c2 and phi and
  // table A's slices at the unit's c1 nodes (rows are ordered (c1, q), so a unit spans at most
  // (rpu - 1) / nq + 2 c1 nodes).
  int s5z_tab_bytes(const gb_ctx *ctx, const ItemDev &it)
  {
    const TableDev &A = ctx->h_dir[it.tab[0]];
    return A.rc_off ? A.bytes - 4 * A.rc_off : 0;
  }
  int s5z_rec_cap(const gb_ctx *ctx, const ItemDev &it, int rpu)
  {
    const int ns0 = ctx->h_dir[it.tab[0]].n0 - 1;
    const int jspan = std::min(it.ax[1].n, (rpu - 1) / it.ax[0].n + 2);
    return it.ax[2].n + it.ax[3].n + (jspan * ns0 + 1) / 2;  // NodeRec units (32 B = 2 slice entries)
  }
  // S3R: whether table B carries propagator records and C, D value records, and the bytes
  // staged (B's propagator records, then C's and D's value records and difference low words)
  bool s3r_ready(const gb_ctx *ctx, const ItemDev &it)
  {
    for (int t = 1; t < 4; ++t) {
      if (it.tab[t] < 0) return false;
      const TableDev &D = ctx->h_dir[it.tab[t]];
      if (!D.cr_off || D.n1 != 0) return false;
    }
    return ctx->h_dir[it.tab[1]].gr_off > 0;
  }
  int s3r_tab_bytes(const gb_ctx *ctx, const ItemDev &it)
  {
    int b = 64 * (ctx->h_dir[it.tab[1]].n0 - 1);
    for (int t = 2; t < 4; ++t) {
      const int c = ctx->h_dir[it.tab[t]].n0 - 1;
      b += 16 * c + (4 * c + 15) / 16 * 16;
    }
    return b;
  }
  size_t s5z_smem_bytes(const gb_ctx *ctx, const ItemDev &it, int rpu)
  {
    const size_t tab = ((size_t)s5z_tab_bytes(ctx, it) + 127) / 128 * 128;
    const size_t rec = ((size_t)s5z_rec_cap(ctx, it, rpu) + 3) / 4 * 4;
    return tab + 2 * rec * sizeof(NodeRec);
  }

  gb_schedule resolve_schedule(const gb_ctx *ctx, int kind)
  {
    gb_schedule s = ctx->sched[kind_base(kind) + (kind_acc(kind) ? 8 : 0)];
    const gb_schedule d = kind_default_schedule(kind);
    if (s.threads <= 0) s.threads = d.threads;
    if (s.rows_per_thread <= 0) s.rows_per_thread = d.rows_per_thread;
    if (s.inner_split <= 0) s.inner_split = d.inner_split;
    const int kb = kind_base(kind);
    if (kb != K_S3 && kb != K_S3R && kb != K_S5Z) s.inner_split = 1;
    if (s.unit_order != GB_ORDER_COST) s.unit_order = GB_ORDER_ITEM;
    return s;
  }

  namespace
  {
    int log2_exact(int v)
    {
      int l = 0;
      while ((1 << l) < v) ++l;
      return l;
    }

    // quadrature rows a work unit of the schedule spans (before the inner split)
    int base_rows_per_unit(const gb_schedule &s) { return s.threads * s.rows_per_thread / s.inner_split; }
  } // namespace

  int plan_batch(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *const *item_tables,
                 const int *item_ntables, int precision, gb_batch *b)
  {
    if (!ctx || n <= 0 || !items) return set_error(ctx, GB_EINVAL, "bad batch arguments");
    if (precision < GB_PREC_FP32C || precision > GB_PREC_FP32A) return set_error(ctx, GB_EINVAL, "bad precision");
    b->n = n;
    b->precision = precision;
    b->src.assign(items, items + n);
    b->items.resize(n);
    std::map<std::tuple<int, int, int, int, double>, int> seg_index;  // dedupe
    std::map<std::tuple<int, int, int, double, double>, int> slice_index;
    std::map<std::tuple<int, int, int>, int> ax1_index;  // SEG_AX1 slices by (table, axis)
    std::vector<int> item_kind(n);
    for (int i = 0; i < n; ++i) {
      const gb_integral &g = items[i];
      ItemDev &it = b->items[i];
      std::memset(&it, 0, sizeof(it));
      it.integrand = g.integrand;
      it.family = g.family;
      it.k = g.k;
      std::memcpy(it.args, g.args, sizeof(it.args));
      if (g.integrand != GB_IG_POLY && g.integrand != GB_IG_PROP1 && g.integrand != GB_IG_PROP3 &&
          g.integrand != GB_IG_VERT4 && g.integrand != GB_IG_FTLOOP)
        return set_error(ctx, GB_EINVAL, "unknown integrand");
      const size_t held0 = b->held.size();
      int rc = family_axes(ctx, g, it.ax, it.n_axes, &b->held);
      if (rc) return rc;
      // tables
      if (g.table_base < 0 || g.table_base > item_ntables[i])
        return set_error(ctx, GB_EINVAL, "table_base outside the table list");
      gb_table *const *tables = item_tables[i] ? item_tables[i] + g.table_base : nullptr;
      const int n_tables = item_ntables[i] - g.table_base;
      const int nt = tables_needed(g.integrand);
      if (nt > n_tables) return set_error(ctx, GB_EINVAL, "integrand needs more tables than given");
      for (int t = 0; t < 4; ++t) it.tab[t] = -1;
      for (int t = 0; t < nt; ++t) {
        if (!tables || !tables[t] || tables[t]->slot < 0) return set_error(ctx, GB_EINVAL, "null table");
        it.tab[t] = tables[t]->slot;
      }
      if (g.integrand == GB_IG_FTLOOP && (tables[0]->spec.n1 < 2 || !(g.args[2] > 0)))
        return set_error(ctx, GB_EINVAL, "FTLOOP needs a 2D table and T > 0");
      if (g.integrand == GB_IG_VERT4) {
        const gb_table_spec &a = tables[0]->spec, &c = tables[1]->spec;
        if (a.n1 < 2 || std::memcmp(&a, &c, sizeof(a)) != 0)
          return set_error(ctx, GB_EINVAL, "VERT4 needs two 2D tables with identical axes");
      }
      for (int t = 0; t < nt; ++t)
        if (g.integrand != GB_IG_FTLOOP && g.integrand != GB_IG_VERT4 && tables[t]->spec.n1 != 0)
          return set_error(ctx, GB_EINVAL, "integrand needs 1D tables");
      // points (integrand evaluations, +-q0 counted twice)
      uint64_t pts = 1;
      for (int a = 0; a < it.n_axes; ++a) {
        const AxisRef &A = it.ax[a];
        const uint64_t single = (uint64_t)std::min(A.pm_from, A.n);
        pts *= single + 2 * (uint64_t)(A.n - single);
      }
      b->points += pts;
      // kind
      int kind = K_GENERIC;
      if (precision != GB_PREC_FP64) {
        if (g.integrand == GB_IG_PROP1 && it.n_axes == 2 && it.ax[0].role == R_Q && it.ax[1].role == R_C1 &&
            it.ax[1].pm_from >= it.ax[1].n)
          kind = K_S1;
        else if (g.integrand == GB_IG_FTLOOP && g.family == GB_FAM_QLOOP_T)
          kind = K_S2;
        else if (g.integrand == GB_IG_PROP3 && g.family == GB_FAM_3D)
          kind = K_S3;
        else if (g.integrand == GB_IG_VERT4 && g.family == GB_FAM_4D)
          kind = K_S5;
        // The fast form has ~5e-8 rms error per point and factor and a residual small-x bias of
        // ~1e-9 (measured on GB300), so it can miss 1e-9 on integrals whose weight sits on a few
        // thousand points; FP32C therefore uses the accurate double-float form (per-point error
        // ~2e-9, no measurable bias).  FP32F selects the fast form explicitly.
        if (kind != K_GENERIC && precision != GB_PREC_FP32F) kind |= K_ACC;
      }
      // table bytes of S kinds must fit shared memory
      if (kind != K_GENERIC) {
        int tb = 0;
        for (int t = 0; t < nt; ++t) tb += tables[t]->bytes;
        if (tb > 160 * 1024) kind = K_GENERIC;
      }
      // 4D vertex, accurate form: the 2D tables read through slices along their cos axis when
      // table A's slices at the c1 nodes of one work unit (double buffered) fit shared memory at
      // the widest CTA
      if (kind == (K_S5 | K_ACC) &&
          s5z_smem_bytes(ctx, it, base_rows_per_unit(resolve_schedule(ctx, K_S5Z | K_ACC))) <= kS5zSmemLimit)
        kind = K_S5Z | K_ACC;
      // 3D loop, accurate form: the three point-dependent tables through their cell records
      // when all three carry them and table B its regulator coefficients
      if (kind == (K_S3 | K_ACC) && s3r_ready(ctx, it)) kind = K_S3R | K_ACC;
      it.kind = kind;
      item_kind[i] = kind;
      long long rows;
      const int kb = kind_base(kind);
      switch (kb) {
      case K_S1: rows = it.ax[0].n; break;
      case K_S2: rows = (long long)it.ax[1].n * it.ax[2].n; break;  // (q, cos); inner: modes
      case K_S3:
      case K_S3R: rows = (long long)it.ax[0].n * it.ax[1].n; break;
      case K_S5:
      case K_S5Z: rows = (long long)it.ax[0].n * it.ax[1].n; break;  // S5Z: ordered (c1, q)
      default: {
        rows = 1;
        for (int a = 0; a < it.n_axes; ++a) rows *= it.ax[a].n;
      }
      }
      if (rows > (1ll << 30)) return set_error(ctx, GB_EINVAL, "integral too large for one item (split it)");
      it.rows = (int)rows;
      // hoisted segment
      if (kind != K_GENERIC) {
        SegDev S{};
        S.kind = kb == K_S5Z ? SEG_S5 : kb == K_S3R ? SEG_S3 : kb;  // SEG_S* == K_S*
        S.tab = it.tab[0];
        S.ax0 = it.ax[0];
        S.n0 = it.ax[0].n;
        S.n1 = 1;
        double par = 0;
        if (kb == K_S1) par = g.args[2];
        if (kb == K_S2) {
          S.ax1 = it.ax[1];
          S.n1 = it.ax[1].n;
          par = g.args[2];
        }
        if (kb == K_S5 || kb == K_S5Z) {
          S.ax1 = it.ax[1];
          S.n1 = it.ax[1].n;
        }
        S.par[0] = par;
        auto key = std::make_tuple(S.kind, S.ax0.off, S.kind == SEG_S2 || S.kind == SEG_S5 ? S.ax1.off : -1, S.tab, par);
        auto f = seg_index.find(key);
        if (f == seg_index.end()) {
          if (kb == K_S2) {
            // q-only FP64 factors of the S2 segment, per q node: w_q Rdot(q^2), R(q^2), q^2 and
            // the |q| fraction and cell on the table's second axis (6 doubles in 3 float4 slots)
            const AxisEntry &qa = ctx->axis_cache.at(b->held[held0 + 1]);
            if ((int)qa.v.size() != S.n1 || qa.w.size() != qa.v.size())
              return set_error(ctx, GB_EINVAL, "S2 segment: unexpected q axis");
            const TableDev &D = ctx->h_dir[S.tab];
            S.aux_off = (int)b->aux.size();
            for (int q = 0; q < S.n1; ++q) {
              const double x2 = qa.v[q] * qa.v[q];
              int jq = 0;
              const double fq = dev::axis_frac64(D.a1, std::sqrt(x2), jq);
              const double rec[6] = {qa.w[q] * dev::reg_Rdot(x2), dev::reg_R(x2), x2, fq, (double)jq, 0.0};
              float4 f4[3];
              std::memcpy(f4, rec, sizeof(rec));
              b->aux.insert(b->aux.end(), f4, f4 + 3);
            }
          }
          S.off = (int)b->seg_total;
          b->seg_total += (size_t)S.n0 * S.n1;
          b->seg_max_entries = std::max(b->seg_max_entries, S.n0 * S.n1);
          seg_index[key] = (int)b->segs.size();
          b->segs.push_back(S);
          it.seg_off = S.off;
        } else
          it.seg_off = b->segs[f->second].off;
      }
      // S2, accurate form: the table interpolated along its mode axis at each (mode, sign)
      // frequency, per |q| cell, so that a point lerps along |q| only; shared by the items with
      // the same table, mode axis, T and external frequency
      if (kind == (K_S2 | K_ACC)) {
        const double Tt = g.args[2], Om = g.args[3];
        auto key = std::make_tuple(it.tab[0], it.ax[0].off, it.ax[0].n, Tt, Om);
        auto f = slice_index.find(key);
        if (f == slice_index.end()) {
          SegDev S{};
          S.kind = SEG_S2Z;
          S.tab = it.tab[0];
          S.ax0 = it.ax[0];
          S.n0 = 2 * it.ax[0].n;               // (mode, sign) records
          S.n1 = tables[0]->spec.n1 - 1;        // |q| cells
          S.par[0] = Om;
          S.par[1] = 1.0 / (2.0 * 3.14159265358979323846 * Tt);
          b->seg_total += b->seg_total & 1;    // float4 entries: 16-byte aligned
          S.off = (int)b->seg_total;
          b->seg_total += 2 * (size_t)S.n0 * S.n1;
          b->seg_max_entries = std::max(b->seg_max_entries, S.n0 * S.n1);
          slice_index[key] = S.off;
          b->segs.push_back(S);
          it.slice_off = S.off;
        } else
          it.slice_off = f->second;
      }
      // S5Z: tables A and B interpolated along their cos axis at the c1 and c2 nodes (shared by
      // the items with the same table and axis)
      if (kind == (K_S5Z | K_ACC)) {
        const int ns0 = tables[0]->spec.n0 - 1;
        auto ax1_slice = [&](int slot, const AxisRef &ax) -> int {
          const auto key = std::make_tuple(slot, ax.off, ax.n);
          auto f = ax1_index.find(key);
          if (f != ax1_index.end()) return f->second;
          SegDev S{};
          S.kind = SEG_AX1;
          S.tab = slot;
          S.ax0 = ax;
          S.n0 = ax.n;
          S.n1 = ns0;
          b->seg_total += b->seg_total & 1;  // float4 entries: 16-byte aligned
          S.off = (int)b->seg_total;
          b->seg_total += 2 * (size_t)S.n0 * S.n1;
          b->seg_max_entries = std::max(b->seg_max_entries, S.n0 * S.n1);
          b->segs.push_back(S);
          ax1_index[key] = S.off;
          return S.off;
        };
        it.slice_off = ax1_slice(it.tab[0], it.ax[1]);
        it.slice_off2 = ax1_slice(it.tab[1], it.ax[2]);
        it.slice_off3 = ax1_slice(it.tab[0], it.ax[2]);
      }
      if (kind != K_GENERIC) item_aux(ctx, g, it, &ctx->axis_cache.at(b->held[held0]).v, b->aux);
      // reference-pattern geometry
      int loop_axis = -1;
      if (g.family == GB_FAM_4D) loop_axis = 2;
      if (g.family == GB_FAM_4D_FTQ0 || g.family == GB_FAM_4D_FTX0) loop_axis = 3;
      long long pt = 1;
      for (int a = 0; a < it.n_axes; ++a)
        if (a != loop_axis) pt *= it.ax[a].n;
      b->plain_loop_axis.push_back(loop_axis);
      b->plain_threads.push_back(pt);
    }
    // units grouped by kind; built on the host only when a run goes out in cost order (a
    // permutation), else expanded on the device from one range per integral
    b->host_units = false;
    for (int i = 0; i < n; ++i)
      if (item_kind[i] != K_GENERIC && resolve_schedule(ctx, item_kind[i]).unit_order == GB_ORDER_COST)
        b->host_units = true;
    long long nunits = 0;
    const int kinds[11] = {K_S1,         K_S2,         K_S3,          K_S5,          K_S1 | K_ACC, K_S2 | K_ACC,
                           K_S3 | K_ACC, K_S3R | K_ACC, K_S5 | K_ACC, K_S5Z | K_ACC, K_GENERIC};
    for (int kind : kinds) {
      gb_batch::KindRun run;
      run.kind = kind;
      run.unit_begin = (int)nunits;
      const int kb = kind_base(kind);
      const gb_schedule sc = kind == K_GENERIC ? gb_schedule{kGenericThreads, kGenericPPT, 1, GB_ORDER_ITEM}
                                               : resolve_schedule(ctx, kind);
      const int rpu = kind == K_GENERIC ? kGenericUnitPoints : sc.threads * sc.rows_per_thread;
      const int split_log2 = log2_exact(sc.inner_split);
      int tab_cap = 0, rec_cap = 0;
      bool any = false;
      for (int i = 0; i < n; ++i) {
        if (item_kind[i] != kind) continue;
        any = true;
        ItemDev &it = b->items[i];
        if (kind != K_GENERIC) {
          // every row becomes inner_split rows (one part of its inner loop each)
          if (((long long)it.rows << split_log2) > (1ll << 30))
            return set_error(ctx, GB_EINVAL, "integral too large for one item (split it)");
          it.split_log2 = split_log2;
          it.rows <<= split_log2;
        }
        const int nu = (it.rows + rpu - 1) / rpu;
        if (nunits + nu > (long long)INT32_MAX) return set_error(ctx, GB_EINVAL, "batch has more than 2^31 work units");
        it.unit_begin = (int)(nunits - run.unit_begin);
        it.n_units = nu;
        if (b->host_units) {
          for (int u = 0; u < nu; ++u) {
            UnitDev U{};
            U.item = i;
            U.row_begin = u * rpu;
            U.row_count = std::min(rpu, it.rows - u * rpu);
            U.slot = it.unit_begin + u;
            b->units.push_back(U);
          }
        } else {
          b->expand.push_back(ExpandDev{i, (int)nunits, nu, it.rows, rpu, it.unit_begin});
        }
        nunits += nu;
        if (kind != K_GENERIC) {
          int tb = 0;
          for (int t = 0; t < tables_needed(it.integrand); ++t) {
            const TableDev &D = ctx->h_dir[it.tab[t]];
            // S2 accurate form: only the cell-centre reciprocals are staged
            tb += kind == (K_S2 | K_ACC) ? (D.rc_off ? D.bytes - 4 * D.rc_off : 0) : ctx->slots[it.tab[t]]->bytes;
          }
          if (kb == K_S5Z) tb = s5z_tab_bytes(ctx, it);
          if (kb == K_S3R) tb = s3r_tab_bytes(ctx, it);
          tab_cap = std::max(tab_cap, tb);
          int rc_n = 0;
          if (kb == K_S1) rc_n = it.ax[1].n;
          if (kb == K_S2 || kb == K_S3 || kb == K_S3R) rc_n = it.ax[2].n;
          if (kb == K_S5) rc_n = it.ax[2].n + it.ax[3].n;
          if (kb == K_S5Z) rc_n = s5z_rec_cap(ctx, it, rpu >> split_log2);
          rec_cap = std::max(rec_cap, rc_n);
        }
      }
      if (!any) continue;
      run.n_units = (int)(nunits - run.unit_begin);
      if (b->host_units && sc.unit_order == GB_ORDER_COST && kind != K_GENERIC) {
        // largest cost (rows x points per row) first; ties keep item order
        std::vector<double> per_row(n, 0.0);
        for (int i = 0; i < n; ++i)
          if (item_kind[i] == kind) {
            const ItemDev &it = b->items[i];
            double pts = 1;
            for (int a = 0; a < it.n_axes; ++a) pts *= it.ax[a].n;
            per_row[i] = pts / it.rows;
          }
        std::stable_sort(b->units.begin() + run.unit_begin, b->units.end(), [&](const UnitDev &x, const UnitDev &y) {
          return x.row_count * per_row[x.item] > y.row_count * per_row[y.item];
        });
      }
      run.tab_cap = (tab_cap + 127) / 128 * 128;
      run.rec_cap = (rec_cap + 3) / 4 * 4;
      if (kind == K_GENERIC) {
        run.threads = kGenericThreads;
        run.ctas = std::min(run.n_units, ctx->num_sms * 8);
      } else {
        run.threads = sc.threads;
        const int occ = fp32c_occupancy(kind, sc.threads, run.tab_cap, run.rec_cap);
        if (occ <= 0) return set_error(ctx, GB_EINVAL, "FP32 kernel cannot launch with this table/record size");
        run.ctas = std::min(run.n_units, ctx->num_sms * occ);
      }
      b->runs.push_back(run);
    }
    b->n_units_total = (size_t)nunits;
    return GB_OK;
  }

  int build_batch(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                  gb_batch **out)
  {
    if (!ctx || !out || n <= 0 || !items) return set_error(ctx, GB_EINVAL, "bad batch arguments");
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    GB_CUDA(cudaSetDevice(ctx->device));
    std::vector<gb_table *const *> tl(n, tables);
    std::vector<int> tn(n, n_tables);
    gb_batch *b = new gb_batch();
    int rc = plan_batch(ctx, items, n, tl.data(), tn.data(), precision, b);
    if (rc) {
      free_batch(ctx, b);
      return rc;
    }
    // device buffers
    const size_t nu = b->n_units_total;
    const size_t bytes = batch_device_bytes(b);
    if (ctx->in_use + bytes > ctx->budget) {
      free_batch(ctx, b);
      return set_error(ctx, GB_EBUDGET, "batch exceeds the HBM budget");
    }
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t sz) {
      if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(sz, 16));
    };
    alloc((void **)&b->d_items, n * sizeof(ItemDev));
    alloc((void **)&b->d_units, nu * sizeof(UnitDev));
    alloc((void **)&b->d_expand, b->expand.size() * sizeof(ExpandDev));
    alloc((void **)&b->d_segs, b->segs.size() * sizeof(SegDev));
    alloc((void **)&b->d_seg, b->seg_total * sizeof(double));
    alloc((void **)&b->d_aux, b->aux.size() * sizeof(float4));
    alloc((void **)&b->d_partials, nu * sizeof(double));
    alloc((void **)&b->d_item_count, n * sizeof(int));
    alloc((void **)&b->d_counters, b->runs.size() * sizeof(int));
    alloc((void **)&b->d_out, n * sizeof(double));
    b->bytes = bytes;
    ctx->in_use += bytes;
    if (e == cudaSuccess) e = cudaMemcpy(b->d_items, b->items.data(), n * sizeof(ItemDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && b->host_units)
      e = cudaMemcpy(b->d_units, b->units.data(), nu * sizeof(UnitDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !b->host_units) {
      e = cudaMemcpy(b->d_expand, b->expand.data(), b->expand.size() * sizeof(ExpandDev), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = launch_expand_units(b->d_expand, (int)b->expand.size(), b->d_units, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    if (e == cudaSuccess && !b->segs.empty())
      e = cudaMemcpy(b->d_segs, b->segs.data(), b->segs.size() * sizeof(SegDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !b->aux.empty())
      e = cudaMemcpy(b->d_aux, b->aux.data(), b->aux.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->d_item_count, 0, n * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_out, 0, n * sizeof(double));
    if (e != cudaSuccess) {
      free_batch(ctx, b);
      return cuda_fail(ctx, e, "batch device buffers");
    }
    if (log_enabled())
      log_event("batch_create", jfields("\"integrals\": %d, \"units\": %zu, \"points\": %llu, \"bytes\": %zu, "
                                        "\"precision\": %d, \"runs\": %zu",
                                        n, nu, (unsigned long long)b->points, bytes, precision, b->runs.size()));
    *out = b;
    return GB_OK;
  }

  int run_batch(gb_ctx *ctx, gb_batch *b, double *d_out, cudaStream_t s)
  {
    TraceRange tr("gbint run_batch");
    RunParams P{};
    P.items = b->d_items;
    P.n_items = b->n;
    P.pv = ctx->pool.d_v;
    P.pw = ctx->pool.d_w;
    P.pa = ctx->pool.d_a;
    P.prec = ctx->pool.d_rec;
    P.tabs = ctx->d_dir;
    P.seg = b->d_seg;
    P.aux = b->d_aux;
    P.item_count = b->d_item_count;
    P.out = d_out ? d_out : b->d_out;
    P.err = ctx->d_err;
    P.single = b->single ? 1 : 0;
    // the segment kernel zeroes the run counters; without segments a memset does
    if (!b->segs.empty())
      GB_CUDA(launch_seg(b->d_segs, (int)b->segs.size(), b->seg_max_entries, P.pv, P.pw, P.aux, P.tabs, b->d_seg,
                         b->d_counters, (int)b->runs.size(), s));
    else
      GB_CUDA(cudaMemsetAsync(b->d_counters, 0, b->runs.size() * sizeof(int), s));
    for (size_t r = 0; r < b->runs.size(); ++r) {
      const auto &run = b->runs[r];
      P.units = b->d_units + run.unit_begin;
      P.n_units = run.n_units;
      P.partials = b->d_partials + run.unit_begin;
      P.unit_counter = b->d_counters + r;
      if (run.kind == K_GENERIC)
        GB_CUDA(launch_generic(P, run.ctas, s));
      else
        GB_CUDA(launch_fp32c(run.kind, P, run.threads, run.ctas, run.tab_cap, run.rec_cap, s));
    }
    return GB_OK;
  }

  // Device descriptor of one integral for the generic FP64 kernel: axes from the context's node
  // pool (pre-allocated; new quadrature orders are copied in, nothing is allocated on the device)
  // and table directory slots.  Caller holds ctx->mu.
  int prepare_item_fp64(gb_ctx *ctx, const gb_integral &g, gb_table *const *tables, int n_tables, ItemDev &it,
                        uint64_t &grid_points, std::vector<AxisKey> &hold)
  {
    std::memset(&it, 0, sizeof(it));
    if (g.integrand != GB_IG_POLY && g.integrand != GB_IG_PROP1 && g.integrand != GB_IG_PROP3 &&
        g.integrand != GB_IG_VERT4 && g.integrand != GB_IG_FTLOOP)
      return set_error(ctx, GB_EINVAL, "unknown integrand");
    if (g.table_base < 0 || g.table_base > n_tables) return set_error(ctx, GB_EINVAL, "table_base outside the table list");
    if (tables) tables += g.table_base;
    n_tables -= g.table_base;
    it.kind = K_GENERIC;
    it.integrand = g.integrand;
    it.family = g.family;
    it.k = g.k;
    std::memcpy(it.args, g.args, sizeof(it.args));
    int rc = family_axes(ctx, g, it.ax, it.n_axes, &hold);
    if (rc) return rc;
    const int nt = tables_needed(g.integrand);
    if (nt > n_tables) return set_error(ctx, GB_EINVAL, "integrand needs more tables than given");
    for (int t = 0; t < 4; ++t) it.tab[t] = -1;
    for (int t = 0; t < nt; ++t) {
      if (!tables || !tables[t] || tables[t]->slot < 0) return set_error(ctx, GB_EINVAL, "null table");
      it.tab[t] = tables[t]->slot;
    }
    if (g.integrand == GB_IG_FTLOOP && (tables[0]->spec.n1 < 2 || !(g.args[2] > 0)))
      return set_error(ctx, GB_EINVAL, "FTLOOP needs a 2D table and T > 0");
    if (g.integrand == GB_IG_VERT4 && tables[0]->spec.n1 < 2)
      return set_error(ctx, GB_EINVAL, "VERT4 needs 2D tables");
    grid_points = 1;
    for (int a = 0; a < it.n_axes; ++a) grid_points *= (uint64_t)it.ax[a].n;
    return GB_OK;
  }
} // namespace gbint

namespace gbint
{
  // Device copy of a rule array, allocated and zero-filled to a multiple of 16 bytes: the C++
  // layer's fused kernel stages these arrays into shared memory with TMA bulk copies, whose size
  // must be a multiple of 16 bytes and stay inside the allocation.
  template <typename T> int rule_device_copy(gb_ctx *ctx, const std::vector<double> &h, T **d)
  {
    const size_t bytes = h.size() * sizeof(T), padded = (bytes + 15) & ~size_t(15);
    std::vector<T> v(padded / sizeof(T), T(0));
    for (size_t i = 0; i < h.size(); ++i) v[i] = (T)h[i];
    GB_CUDA(cudaMalloc(d, padded));
    GB_CUDA(cudaMemcpy(*d, v.data(), padded, cudaMemcpyHostToDevice));
    return GB_OK;
  }
} // namespace gbint

// ============================================================================ C ABI
extern "C" {

int gb_version(void) { return GBINT_ABI_VERSION; }

const char *gb_status_string(int s)
{
  switch (s) {
  case GB_OK: return "ok";
  case GB_EINVAL: return "invalid argument";
  case GB_ENOMEM: return "out of memory";
  case GB_EBUDGET: return "HBM budget exceeded";
  case GB_ETIMEDOUT: return "timed out";
  case GB_ECUDA: return "CUDA error";
  case GB_ENODEV: return "no CUDA device";
  case GB_EAGAIN: return "not ready";
  case GB_EDEVICE: return "device-side error flag";
  case GB_ECANCELED: return "canceled";
  }
  return "unknown status";
}

int gb_ctx_create(int device, size_t budget, gb_ctx **out)
{
  if (!out) return GB_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GB_ENODEV;
  if (device < 0 || device >= ndev) return GB_ENODEV;
  auto ctx = std::make_unique<gb_ctx>();
  ctx->device = device;
  ctx->budget = budget ? budget : ((size_t)8 << 30);
  gb_ctx *c = ctx.get();
#define CK(call)                                       \
  do {                                                 \
    cudaError_t e__ = (call);                          \
    if (e__ != cudaSuccess) return GB_ECUDA;           \
  } while (0)
  CK(cudaSetDevice(device));
  CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&c->tables_event, cudaEventDisableTiming));
  c->pool_streams.resize(kPoolStreams);
  for (auto &s : c->pool_streams) CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  c->pool.capacity = kPoolCapacity;
  CK(cudaMalloc(&c->pool.d_v, kPoolCapacity * sizeof(double)));
  CK(cudaMalloc(&c->pool.d_w, kPoolCapacity * sizeof(double)));
  CK(cudaMalloc(&c->pool.d_a, kPoolCapacity * sizeof(double)));
  CK(cudaMalloc(&c->pool.d_rec, kPoolCapacity * sizeof(NodeRec)));
  CK(cudaMalloc(&c->d_dir, kMaxTables * sizeof(TableDev)));
  CK(cudaMemset(c->d_dir, 0, kMaxTables * sizeof(TableDev)));
  c->h_dir.assign(kMaxTables, TableDev{});
  c->slots.assign(kMaxTables, nullptr);
  CK(cudaMalloc(&c->d_err, sizeof(int)));
  CK(cudaMemset(c->d_err, 0, sizeof(int)));
  CK(cudaMalloc(&c->plain_res, kPoolStreams * sizeof(double)));
  CK(cudaMallocHost(&c->plain_res_h, kPoolStreams * sizeof(double)));
  c->plain_buf.assign(kPoolStreams, nullptr);
  c->plain_buf_elems.assign(kPoolStreams, 0);
  c->plain_tmp.assign(kPoolStreams, nullptr);
  c->plain_tmp_bytes.assign(kPoolStreams, 0);
#undef CK
  *out = ctx.release();
  return GB_OK;
}

int gb_ctx_destroy(gb_ctx *ctx)
{
  if (!ctx) return GB_EINVAL;
  if (ctx->serve) serve_stop(ctx);
  if (ctx->dloop) dloop_stop(ctx);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  destroy_slots(ctx);
  for (auto &kv : ctx->buffers) cudaFree(kv.first);
  ctx->buffers.clear();
  for (auto &kv : ctx->gl) {
    cudaFree(kv.second.d64x);
    cudaFree(kv.second.d64w);
    cudaFree(kv.second.d32x);
    cudaFree(kv.second.d32w);
  }
  for (auto &kv : ctx->rules) {
    cudaFree(kv.second.d64x);
    cudaFree(kv.second.d64w);
    cudaFree(kv.second.d32x);
    cudaFree(kv.second.d32w);
  }
  for (auto &m : ctx->mats) {
    cudaFree(m->d64x);
    cudaFree(m->d64w);
    cudaFree(m->d32x);
    cudaFree(m->d32w);
  }
  for (auto *t : ctx->slots)
    if (t) {
      cudaFree(t->buf[0]);
      cudaFree(t->buf[1]);
      delete t;
    }
  for (size_t i = 0; i < ctx->plain_buf.size(); ++i) {
    cudaFree(ctx->plain_buf[i]);
    cudaFree(ctx->plain_tmp[i]);
  }
  cudaFree(ctx->plain_res);
  cudaFreeHost(ctx->plain_res_h);
  cudaFree(ctx->pool.d_v);
  cudaFree(ctx->pool.d_w);
  cudaFree(ctx->pool.d_a);
  cudaFree(ctx->pool.d_rec);
  cudaFree(ctx->d_dir);
  cudaFree(ctx->d_err);
  for (auto s : ctx->pool_streams) cudaStreamDestroy(s);
  cudaStreamDestroy(ctx->stream);
  cudaEventDestroy(ctx->tables_event);
  delete ctx;
  return GB_OK;
}

int gb_last_error(gb_ctx *ctx, char *buf, size_t len)
{
  if (!ctx || !buf || len == 0) return GB_EINVAL;
  std::snprintf(buf, len, "%s", ctx->last_error.c_str());
  return GB_OK;
}

// ------------------------------------------------------------------ provider
// a cached rule's host arrays, and its device copies of dtype (made on first request)
static int rule_out(gb_ctx *ctx, GLRule &r, int order, int dtype, const double **hx, const double **hw,
                    const void **dx, const void **dw)
{
  if (hx) *hx = r.x.data();
  if (hw) *hw = r.w.data();
  if (dx || dw) {
    GB_CUDA(cudaSetDevice(ctx->device));
    if (dtype == GB_DTYPE_F64) {
      if (!r.d64x) {
        int rc = rule_device_copy(ctx, r.x, &r.d64x);
        if (!rc) rc = rule_device_copy(ctx, r.w, &r.d64w);
        if (rc) return rc;
      }
      if (dx) *dx = r.d64x;
      if (dw) *dw = r.d64w;
    } else {
      if (!r.d32x) {
        int rc = rule_device_copy(ctx, r.x, &r.d32x);
        if (!rc) rc = rule_device_copy(ctx, r.w, &r.d32w);
        if (rc) return rc;
      }
      if (dx) *dx = r.d32x;
      if (dw) *dw = r.d32w;
    }
  }
  return GB_OK;
}

int gb_quad_gl(gb_ctx *ctx, int order, int dtype, const double **hx, const double **hw, const void **dx,
               const void **dw)
{
  if (!ctx || order <= 0 || order > 4096) return set_error(ctx, GB_EINVAL, "bad GL order");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  return rule_out(ctx, const_cast<GLRule &>(gl_host(ctx, order)), order, dtype, hx, hw, dx, dw);
}

int gb_quad_rule(gb_ctx *ctx, int type, int order, int dtype, const double **hx, const double **hw, const void **dx,
                 const void **dw)
{
  if (type == GB_QUAD_LEGENDRE) return gb_quad_gl(ctx, order, dtype, hx, hw, dx, dw);
  if (!ctx || order <= 0 || order > 4096) return set_error(ctx, GB_EINVAL, "bad quadrature order");
  if (type < GB_QUAD_LEGENDRE || type > GB_QUAD_JACOBI) return set_error(ctx, GB_EINVAL, "Unknown quadrature type");
  {
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    auto it = ctx->rules.find({type, order});
    if (it != ctx->rules.end()) return rule_out(ctx, it->second, order, dtype, hx, hw, dx, dw);
  }
  // A cold rule is built without the context lock (Laguerre and Hermite bisect every node on the
  // Jacobi matrix: up to ~1 s at order 4096), so serving and other callers are not held up; a
  // rule built twice by racing callers is the same rule, and the first one inserted is kept.
  GLRule r;
  try {
    fixed_rule(type, order, r.x, r.w);
  } catch (const std::bad_alloc &) {
    return set_error(ctx, GB_ENOMEM, "quadrature rule: host memory");
  } catch (const std::exception &ex) {
    return set_error(ctx, GB_EINVAL, std::string("quadrature rule: ") + ex.what());
  }
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  auto it = ctx->rules.find({type, order});
  if (it == ctx->rules.end()) {
    try {
      it = ctx->rules.emplace(std::make_pair(type, order), std::move(r)).first;
    } catch (const std::bad_alloc &) {
      return set_error(ctx, GB_ENOMEM, "quadrature rule: host memory");
    }
  }
  return rule_out(ctx, it->second, order, dtype, hx, hw, dx, dw);
}

int gb_quad_rule_host(int type, int order, double *nodes, double *weights)
{
  if (order <= 0 || order > 4096 || !nodes || !weights || type < GB_QUAD_LEGENDRE || type > GB_QUAD_JACOBI)
    return GB_EINVAL;
  try {
    std::vector<double> x, w;
    fixed_rule(type, order, x, w);
    std::memcpy(nodes, x.data(), order * sizeof(double));
    std::memcpy(weights, w.data(), order * sizeof(double));
  } catch (...) {
    return GB_EINVAL;
  }
  return GB_OK;
}

int gb_quad_matsubara(gb_ctx *ctx, double T, double E, int dtype, int *size, const double **hx, const double **hw,
                      const void **dx, const void **dw, double *T_rule)
{
  if (!ctx || !(T >= 0) || !(E >= 0)) return set_error(ctx, GB_EINVAL, "bad Matsubara parameters");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  MatsEntry &m = mats_host(ctx, T, E);
  const int n = (int)m.rule.x.size();
  if (size) *size = n;
  if (hx) *hx = m.rule.x.data();
  if (hw) *hw = m.rule.w.data();
  if (T_rule) *T_rule = m.rule.T_rule;
  if (dx || dw) {
    GB_CUDA(cudaSetDevice(ctx->device));
    if (dtype == GB_DTYPE_F64) {
      if (!m.d64x) {
        int rc = rule_device_copy(ctx, m.rule.x, &m.d64x);
        if (!rc) rc = rule_device_copy(ctx, m.rule.w, &m.d64w);
        if (rc) return rc;
      }
      if (dx) *dx = m.d64x;
      if (dw) *dw = m.d64w;
    } else {
      if (!m.d32x) {
        int rc = rule_device_copy(ctx, m.rule.x, &m.d32x);
        if (!rc) rc = rule_device_copy(ctx, m.rule.w, &m.d32w);
        if (rc) return rc;
      }
      if (dx) *dx = m.d32x;
      if (dw) *dw = m.d32w;
    }
  }
  return GB_OK;
}

int gb_quad_config(gb_ctx *ctx, int min_size, int vacuum, int add)
{
  if (!ctx) return GB_EINVAL;
  // QuadratureProvider(json) / MatsubaraStorage setters (quadrature_provider.cu:112-126,220-227)
  if (min_size <= 0) return set_error(ctx, GB_EINVAL, "min_matsubara_size must be positive");
  if (vacuum <= 0) return set_error(ctx, GB_EINVAL, "vacuum_quad_size must be positive");
  if (add < 0) return set_error(ctx, GB_EINVAL, "add_matsubara_size must be non-negative");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  ctx->mats_min = min_size;
  ctx->mats_vacuum = vacuum;
  ctx->mats_add = add;
  return GB_OK;
}

// ------------------------------------------------------------------ tables
namespace gbint
{
  // Taylor coefficients of R(x) = x / expm1(x) about the centres c_j of a log axis's cells, in
  // t = x / c_j - 1: R(c (1 + t)) = sum_k a_k t^k, k <= 7, from the power-series quotient
  // c (1 + t) / (expm1(c) + e^c sum_{k>=1} (c t)^k / k!) in long double (the divisor's higher
  // terms are small against its constant, so the recurrence is stable for every c).  12 floats
  // per cell: a0 and a1 as double-float pairs, a2..a7, two zeros.
  std::vector<float> regulator_cell_coeffs(const dev::AxisDev &ax)
  {
    const int nc = ax.n - 1;
    std::vector<float> out(12 * (size_t)nc, 0.f);
    for (int j = 0; j < nc; ++j) {
      const long double l2c = ((long double)j + 0.5L - (long double)ax.shift64) / (long double)ax.scale64;
      const long double c = exp2l(l2c);
      long double d[8], a[8];
      d[0] = expm1l(c);
      long double pw = 1.0L;
      for (int k = 1; k < 8; ++k) {
        pw *= c / k;
        d[k] = expl(c) * pw;
      }
      for (int k = 0; k < 8; ++k) {
        long double nk = k < 2 ? c : 0.0L;
        for (int i = 0; i < k; ++i) nk -= a[i] * d[k - i];
        a[k] = nk / d[0];
      }
      float *o = out.data() + 12 * (size_t)j;
      for (int h = 0; h < 2; ++h) {
        const dev::df v = dev::df_from((double)a[h]);
        o[2 * h] = v.hi;
        o[2 * h + 1] = v.lo;
      }
      for (int k = 2; k < 8; ++k) o[2 + k] = (float)a[k];
    }
    return out;
  }
  // the same expansion through t^9 in FP64 (10 a cell): the propagator records are built from it
  std::vector<double> regulator_cell_coeffs64(const dev::AxisDev &ax)
  {
    const int nc = ax.n - 1;
    std::vector<double> out(10 * (size_t)nc, 0.0);
    for (int j = 0; j < nc; ++j) {
      const long double l2c = ((long double)j + 0.5L - (long double)ax.shift64) / (long double)ax.scale64;
      const long double c = exp2l(l2c);
      long double d[10], a[10];
      d[0] = expm1l(c);
      long double pw = 1.0L;
      for (int k = 1; k < 10; ++k) {
        pw *= c / k;
        d[k] = expl(c) * pw;
      }
      for (int k = 0; k < 10; ++k) {
        long double nk = k < 2 ? c : 0.0L;
        for (int i = 0; i < k; ++i) nk -= a[i] * d[k - i];
        a[k] = nk / d[0];
        out[10 * (size_t)j + k] = (double)a[k];
      }
    }
    return out;
  }
} // namespace gbint

int gb_table_create(gb_ctx *ctx, const gb_table_spec *spec, gb_table **out)
{
  if (!ctx || !spec || !out) return set_error(ctx, GB_EINVAL, "bad table arguments");
  if (spec->n0 < 2 || (spec->n1 != 0 && spec->n1 < 2)) return set_error(ctx, GB_EINVAL, "table axes need >= 2 points");
  if ((spec->log0 && !(spec->lo0 > 0 && spec->hi0 > spec->lo0)) || (!spec->log0 && !(spec->hi0 > spec->lo0)))
    return set_error(ctx, GB_EINVAL, "bad table axis 0 range");
  if (spec->n1 && ((spec->log1 && !(spec->lo1 > 0 && spec->hi1 > spec->lo1)) || (!spec->log1 && !(spec->hi1 > spec->lo1))))
    return set_error(ctx, GB_EINVAL, "bad table axis 1 range");
  const long long elems = (long long)spec->n0 * std::max(spec->n1, 1);
  if (elems > (1 << 24)) return set_error(ctx, GB_EINVAL, "table too large");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  int slot = -1;
  for (int i = 0; i < kMaxTables; ++i)
    if (!ctx->slots[i]) {
      slot = i;
      break;
    }
  if (slot < 0) return set_error(ctx, GB_ENOMEM, "table directory full");
  auto t = std::make_unique<gb_table>();
  t->spec = *spec;
  t->elems = (int)elems;
  const int data_bytes = (int)((elems * 4 + 15) / 16 * 16);
  // Tables with a log axis whose cells are at most 25 % wide carry, after the data, 1/c_j for
  // that axis's cell centres c_j = sqrt(x_j x_{j+1}) as double-float pairs: the FP32 kernels
  // take a point's fraction relative to its cell centre (ln(x / c_j), a short series) instead
  // of forming a double-float log2 of x.
  const dev::AxisDev ax0 = make_axis(spec->n0, spec->log0, spec->lo0, spec->hi0);
  const dev::AxisDev ax1 = spec->n1 ? make_axis(spec->n1, spec->log1, spec->lo1, spec->hi1) : dev::AxisDev{};
  const double kMinScale = 1.0 / std::log2(1.25), kMinScaleSq = 1.0 / std::log2(1.12);
  int rc_axis = -1;
  if (spec->log0 && ax0.scale64 >= kMinScale)
    rc_axis = 0;
  else if (spec->n1 && spec->log1 && ax1.scale64 >= kMinScale)
    rc_axis = 1;
  std::vector<float> rc;
  if (rc_axis >= 0) {
    const dev::AxisDev &ax = rc_axis == 0 ? ax0 : ax1;
    rc.resize(2 * (ax.n - 1));
    for (int j = 0; j + 1 < ax.n; ++j) {
      // log2 c_j = (j + 1/2 - shift) / scale
      const long double l2c = ((long double)j + 0.5L - (long double)ax.shift64) / (long double)ax.scale64;
      const dev::df r = dev::df_from((double)exp2l(-l2c));
      rc[2 * j] = r.hi;
      rc[2 * j + 1] = r.lo;
    }
  }
  t->bytes = data_bytes + (int)((rc.size() * 4 + 15) / 16 * 16);
  // With the reciprocals, the Taylor coefficients of the regulator R(x) = x / expm1(x) about each
  // cell centre in t = x / c_j - 1 (through t^7), behind them in global memory (not staged): a
  // propagator 1 / (Z(x) x + R(x)) looked up at x gets R from the t of its table fraction.
  // (cells at most 12 % wide, |t| <= 0.06: truncation < 1e-11 of the denominator)
  const bool with_rq = rc_axis >= 0 && (rc_axis == 0 ? ax0 : ax1).scale64 >= kMinScaleSq;
  const std::vector<float> rq = with_rq ? regulator_cell_coeffs(rc_axis == 0 ? ax0 : ax1) : std::vector<float>{};
  // 1D tables with reciprocals also carry per-cell records (built from the data on every update):
  // a value lookup reads the cell's reciprocal, value and difference with one 16-byte load; with
  // the regulator, a propagator lookup reads the cell's series of 1 / (Z(x) x + R(x)) with four
  // (the FP64 regulator coefficients they are built from sit behind them)
  const int cells = spec->n0 - 1;
  const bool with_cr = rc_axis == 0 && spec->n1 == 0;
  const bool with_gr = with_cr && with_rq;
  const std::vector<double> rd = with_gr ? regulator_cell_coeffs64(ax0) : std::vector<double>{};
  const size_t cr_bytes = with_cr ? (size_t)cells * 16 + ((size_t)cells * 4 + 15) / 16 * 16 : 0;
  const size_t gr_bytes = with_gr ? (size_t)cells * 64 : 0;
  const size_t cr_at = (size_t)t->bytes + rq.size() * 4;  // 16-byte multiple
  const size_t gr_at = cr_at + cr_bytes, rd_at = gr_at + gr_bytes;
  const size_t alloc = rd_at + rd.size() * 8;
  GB_CUDA(cudaSetDevice(ctx->device));
  GB_CUDA(cudaMalloc(&t->buf[0], alloc));
  GB_CUDA(cudaMalloc(&t->buf[1], alloc));
  GB_CUDA(cudaMemset(t->buf[0], 0, alloc));
  GB_CUDA(cudaMemset(t->buf[1], 0, alloc));
  for (int b = 0; b < 2; ++b) {
    if (!rc.empty())
      GB_CUDA(cudaMemcpy(reinterpret_cast<char *>(t->buf[b]) + data_bytes, rc.data(), rc.size() * 4,
                         cudaMemcpyHostToDevice));
    if (!rq.empty())
      GB_CUDA(cudaMemcpy(reinterpret_cast<char *>(t->buf[b]) + t->bytes, rq.data(), rq.size() * 4,
                         cudaMemcpyHostToDevice));
    if (!rd.empty())
      GB_CUDA(cudaMemcpy(reinterpret_cast<char *>(t->buf[b]) + rd_at, rd.data(), rd.size() * 8,
                         cudaMemcpyHostToDevice));
  }
  TableDev &D = ctx->h_dir[slot];
  D = TableDev{};
  D.data = t->buf[0];
  D.n0 = spec->n0;
  D.n1 = spec->n1;
  D.bytes = t->bytes;
  D.rc_off = rc.empty() ? 0 : data_bytes / 4;
  D.rq_off = rq.empty() ? 0 : t->bytes / 4;
  D.rc_axis = std::max(rc_axis, 0);
  D.rc_sq = rc_axis >= 0 && (rc_axis == 0 ? ax0 : ax1).scale64 >= kMinScaleSq;
  D.cr_off = with_cr ? (int)(cr_at / 4) : 0;
  D.gr_off = with_gr ? (int)(gr_at / 4) : 0;
  D.rd_off = with_gr ? (int)(rd_at / 4) : 0;
  D.e_lo = std::expm1(-std::log(2.0) / (2.0 * ax0.scale64));
  D.e_hi = std::expm1(std::log(2.0) / (2.0 * ax0.scale64));
  D.a0 = ax0;
  D.a1 = ax1;
  if (with_cr) {
    for (int b = 0; b < 2; ++b)
      GB_CUDA(launch_cell_records(static_cast<float *>(t->buf[b]), D, ctx->stream));
    GB_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  GB_CUDA(cudaMemcpy(ctx->d_dir + slot, &D, sizeof(TableDev), cudaMemcpyHostToDevice));
  t->slot = slot;
  ctx->slots[slot] = t.get();
  *out = t.release();
  return GB_OK;
}

static int table_update_impl(gb_ctx *ctx, gb_table *t, const float *src, cudaMemcpyKind kind, void *stream)
{
  TraceRange tr("gbint table_update");
  if (!ctx || !t || !src || t->slot < 0) return set_error(ctx, GB_EINVAL, "bad table update");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  GB_CUDA(cudaSetDevice(ctx->device));
  {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone)
      return set_error(ctx, GB_EINVAL, "table updates cannot be captured in a graph (update before gb_graph_launch)");
  }
  const int back = t->front ^ 1;
  // serving batches still reading the back buffer (an older epoch) finish first
  if (ctx->serve) {
    const int rc = serve_fence_tables(ctx, s);
    if (rc) return rc;
  }
  if (ctx->dloop) {
    const int rc = dloop_fence_tables(ctx);
    if (rc) return rc;
  }
  GB_CUDA(cudaMemcpyAsync(t->buf[back], src, (size_t)t->elems * 4, kind, s));
  if (ctx->h_dir[t->slot].cr_off)
    GB_CUDA(launch_cell_records(static_cast<float *>(t->buf[back]), ctx->h_dir[t->slot], s));
  // publish the new buffer in the directory, ordered after the data on the same stream (the
  // host copy of the entry changes only once the device write is enqueued)
  TableDev D = ctx->h_dir[t->slot];
  D.data = t->buf[back];
  GB_CUDA(launch_dir_set(ctx->d_dir + t->slot, D, s));
  ctx->h_dir[t->slot] = D;
  t->front = back;
  t->epoch++;
  GB_CUDA(cudaEventRecord(ctx->tables_event, s));
  return GB_OK;
}

int gb_table_group_begin(gb_ctx *ctx)
{
  if (!ctx) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  ctx->update_depth++;
  return GB_OK;
}

int gb_table_group_end(gb_ctx *ctx)
{
  if (!ctx) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (ctx->update_depth <= 0) return set_error(ctx, GB_EINVAL, "gb_table_group_end without gb_table_group_begin");
  ctx->update_depth--;
  return GB_OK;
}

int gb_table_update(gb_ctx *ctx, gb_table *t, const float *host_data, void *stream)
{
  return table_update_impl(ctx, t, host_data, cudaMemcpyHostToDevice, stream);
}

int gb_table_update_device(gb_ctx *ctx, gb_table *t, const float *device_data, void *stream)
{
  return table_update_impl(ctx, t, device_data, cudaMemcpyDeviceToDevice, stream);
}

int gb_table_update_many(gb_ctx *ctx, int n, gb_table *const *tables, const float *const *host_data, void *stream)
{
  TraceRange tr("gbint table_update_many");
  if (!ctx || n < 0 || (n > 0 && (!tables || !host_data))) return set_error(ctx, GB_EINVAL, "bad table update list");
  if (n == 0) return GB_OK;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  GB_CUDA(cudaSetDevice(ctx->device));
  {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone)
      return set_error(ctx, GB_EINVAL, "table updates cannot be captured in a graph (update before gb_graph_launch)");
  }
  std::vector<int> slots(n);
  for (int i = 0; i < n; ++i) {
    if (!tables[i] || tables[i]->slot < 0 || !host_data[i]) return set_error(ctx, GB_EINVAL, "bad table update list");
    slots[i] = tables[i]->slot;
    for (int j = 0; j < i; ++j)
      if (slots[j] == slots[i]) return set_error(ctx, GB_EINVAL, "a table appears twice in one update list");
  }
  // serving batches still reading the back buffers (an older epoch) finish first
  if (ctx->serve) {
    const int rc = serve_fence_tables(ctx, s);
    if (rc) return rc;
  }
  if (ctx->dloop) {
    const int rc = dloop_fence_tables(ctx);
    if (rc) return rc;
  }
  std::vector<TableDev> dir(n);
  for (int i = 0; i < n; ++i) {
    gb_table *t = tables[i];
    const int back = t->front ^ 1;
    GB_CUDA(cudaMemcpyAsync(t->buf[back], host_data[i], (size_t)t->elems * 4, cudaMemcpyHostToDevice, s));
    if (ctx->h_dir[t->slot].cr_off)
      GB_CUDA(launch_cell_records(static_cast<float *>(t->buf[back]), ctx->h_dir[t->slot], s));
    dir[i] = ctx->h_dir[t->slot];
    dir[i].data = t->buf[back];
  }
  GB_CUDA(launch_dir_set_many(ctx->d_dir, slots.data(), dir.data(), n, s));
  for (int i = 0; i < n; ++i) {
    ctx->h_dir[slots[i]] = dir[i];
    tables[i]->front ^= 1;
    tables[i]->epoch++;
  }
  GB_CUDA(cudaEventRecord(ctx->tables_event, s));
  return GB_OK;
}

int gb_table_epoch(gb_ctx *ctx, gb_table *t, uint64_t *epoch)
{
  if (!ctx || !t || !epoch) return GB_EINVAL;
  *epoch = t->epoch;
  return GB_OK;
}

int gb_table_destroy(gb_ctx *ctx, gb_table *t)
{
  if (!ctx || !t) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  if (t->slot >= 0) ctx->slots[t->slot] = nullptr;
  cudaFree(t->buf[0]);
  cudaFree(t->buf[1]);
  delete t;
  return GB_OK;
}

// ------------------------------------------------------------------ batches
int gb_batch_create(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                    gb_batch **out)
{
  return build_batch(ctx, items, n, tables, n_tables, precision, out);
}

int gb_batch_run(gb_ctx *ctx, gb_batch *b, double *d_out, void *stream)
{
  if (!ctx || !b) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  GB_CUDA(cudaSetDevice(ctx->device));
  return run_batch(ctx, b, d_out, stream ? (cudaStream_t)stream : ctx->stream);
}

int gb_batch_run_graph(gb_ctx *ctx, gb_batch *b, void *stream)
{
  if (!ctx || !b) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  GB_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (!b->graph) {
    cudaStream_t cap;
    GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    GB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    const int rc = run_batch(ctx, b, nullptr, cap);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  }
  GB_CUDA(cudaGraphLaunch(b->graph, s));
  return GB_OK;
}

// ------------------------------------------------------------------ CUDA-graph sweeps
struct gb_graph {
  cudaGraphExec_t exec = nullptr;
  int launches = 0;  // kernel launches per replay
};

static bool capturing(cudaStream_t s)
{
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
}

int gb_graph_capture_begin(gb_ctx *ctx, void *stream)
{
  if (!ctx) return GB_EINVAL;
  GB_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (capturing(s)) return set_error(ctx, GB_EINVAL, "stream is already capturing");
  GB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  return GB_OK;
}

int gb_graph_capture_end(gb_ctx *ctx, void *stream, gb_graph **out)
{
  if (!ctx || !out) return set_error(ctx, GB_EINVAL, "bad gb_graph_capture_end arguments");
  GB_CUDA(cudaSetDevice(ctx->device));
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(stream ? (cudaStream_t)stream : ctx->stream, &g);
  if (e != cudaSuccess || !g) return cuda_fail(ctx, e != cudaSuccess ? e : cudaErrorStreamCaptureInvalidated,
                                               "cudaStreamEndCapture (a captured call failed or was not capturable)");
  auto G = std::make_unique<gb_graph>();
  size_t nn = 0;
  if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
    std::vector<cudaGraphNode_t> nodes(nn);
    if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
      for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) G->launches++;
      }
  }
  e = cudaGraphInstantiate(&G->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  *out = G.release();
  return GB_OK;
}

int gb_graph_launch(gb_ctx *ctx, gb_graph *g, void *stream)
{
  if (!ctx || !g) return GB_EINVAL;
  GB_CUDA(cudaSetDevice(ctx->device));
  GB_CUDA(cudaGraphLaunch(g->exec, stream ? (cudaStream_t)stream : ctx->stream));
  return GB_OK;
}

int gb_graph_info(gb_ctx *ctx, gb_graph *g, int *kernel_launches)
{
  if (!ctx || !g || !kernel_launches) return GB_EINVAL;
  *kernel_launches = g->launches;
  return GB_OK;
}

int gb_graph_destroy(gb_ctx *ctx, gb_graph *g)
{
  if (!ctx || !g) return GB_EINVAL;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  delete g;
  return GB_OK;
}

int gb_batch_results(gb_ctx *ctx, gb_batch *b, double *host_out, void *stream)
{
  if (!ctx || !b || !host_out) return GB_EINVAL;
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (capturing(s)) return set_error(ctx, GB_EINVAL, "gb_batch_results cannot be captured in a graph");
  GB_CUDA(cudaSetDevice(ctx->device));
  // the results and the error word come back on the caller's stream behind the batch's kernels,
  // with one synchronisation (the error word lands in the batch's pinned word, allocated once)
  if (!b->h_err) GB_CUDA(cudaMallocHost(&b->h_err, sizeof(int)));
  GB_CUDA(cudaMemcpyAsync(host_out, b->d_out, b->n * sizeof(double), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(b->h_err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  const int err = *b->h_err;
  if (err) {
    cudaMemset(ctx->d_err, 0, sizeof(int));
    return set_error(ctx, GB_EDEVICE, "kernel reported error flags " + std::to_string(err));
  }
  return GB_OK;
}

int gb_batch_get(gb_ctx *ctx, gb_batch *b, double *host_out, void *stream)
{
  int rc = gb_batch_run(ctx, b, nullptr, stream);
  if (rc) return rc;
  return gb_batch_results(ctx, b, host_out, stream);
}

int gb_batch_info(gb_ctx *ctx, gb_batch *b, uint64_t *points, int *n_units, int *n_items)
{
  if (!ctx || !b) return GB_EINVAL;
  if (points) *points = b->points;
  if (n_units) *n_units = (int)b->n_units_total;
  if (n_items) *n_items = b->n;
  return GB_OK;
}

int gb_batch_destroy(gb_ctx *ctx, gb_batch *b)
{
  if (!ctx || !b) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  free_batch(ctx, b);
  return GB_OK;
}

// Reference execution pattern: request() launches the per-point kernel for every integral on a
// pooled stream; get() then reduces each integral's buffer with CUB, copies the value to the
// host and synchronises (integrator_4D_gpu.hh:141-197).  In-flight buffers are bounded to 4 GiB.
int gb_batch_run_plain(gb_ctx *ctx, gb_batch *b, double *host_out, int n_streams)
{
  TraceRange tr("gbint run_plain (reference pattern)");
  if (!ctx || !b || !host_out) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  GB_CUDA(cudaSetDevice(ctx->device));
  const int S = std::max(1, std::min(n_streams, (int)ctx->pool_streams.size()));
  const size_t cap_bytes = (size_t)4 << 30;
  int i0 = 0;
  std::vector<double *> bufs;
  std::vector<size_t> buf_elems;
  std::vector<void *> tmps;
  std::vector<size_t> tmp_bytes;
  int rc = GB_OK;
  while (i0 < b->n && rc == GB_OK) {
    // chunk of integrals whose buffers fit the cap
    int i1 = i0;
    size_t bytes = 0;
    while (i1 < b->n && (i1 == i0 || bytes + b->plain_threads[i1] * sizeof(double) <= cap_bytes)) {
      bytes += b->plain_threads[i1] * sizeof(double);
      ++i1;
    }
    const int m = i1 - i0;
    if ((int)bufs.size() < m) {
      bufs.resize(m, nullptr);
      buf_elems.resize(m, 0);
      tmps.resize(m, nullptr);
      tmp_bytes.resize(m, 0);
    }
    // request(): allocate + launch
    for (int j = 0; j < m && rc == GB_OK; ++j) {
      const int i = i0 + j;
      cudaStream_t s = ctx->pool_streams[i % S];
      const size_t ne = (size_t)b->plain_threads[i];
      if (buf_elems[j] < ne) {
        cudaFree(bufs[j]);
        if (cudaMalloc(&bufs[j], ne * sizeof(double)) != cudaSuccess) {
          rc = set_error(ctx, GB_ENOMEM, "plain buffer");
          break;
        }
        buf_elems[j] = ne;
      }
      cudaError_t e = launch_plain(b->d_items + i, (long long)ne, b->plain_loop_axis[i], ctx->pool.d_v,
                                   ctx->pool.d_w, ctx->d_dir, bufs[j], s);
      if (e != cudaSuccess) rc = cuda_fail(ctx, e, "plain kernel");
    }
    // get(): reduce + D2H + sync, one integral at a time
    for (int j = 0; j < m && rc == GB_OK; ++j) {
      const int i = i0 + j;
      const int si = i % S;
      cudaStream_t s = ctx->pool_streams[si];
      const size_t ne = (size_t)b->plain_threads[i];
      size_t need = 0;
      cub::DeviceReduce::Sum(nullptr, need, bufs[j], ctx->plain_res + si, (int)ne, s);
      if (tmp_bytes[j] < need) {
        cudaFree(tmps[j]);
        if (cudaMalloc(&tmps[j], need) != cudaSuccess) {
          rc = set_error(ctx, GB_ENOMEM, "cub temp");
          break;
        }
        tmp_bytes[j] = need;
      }
      cudaError_t e = cub::DeviceReduce::Sum(tmps[j], need, bufs[j], ctx->plain_res + si, (int)ne, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->plain_res_h + si, ctx->plain_res + si, sizeof(double),
                                                cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        rc = cuda_fail(ctx, e, "plain reduce");
        break;
      }
      host_out[i] = b->src[i].args[0] + ctx->plain_res_h[si];
    }
    i0 = i1;
  }
  cudaDeviceSynchronize();
  for (size_t j = 0; j < bufs.size(); ++j) {
    cudaFree(bufs[j]);
    cudaFree(tmps[j]);
  }
  return rc;
}

int gb_get(gb_ctx *ctx, const gb_integral *item, gb_table *const *tables, int n_tables, int precision, double *out)
{
  if (!ctx || !item || !out) return GB_EINVAL;
  gb_batch *b = nullptr;
  int rc = build_batch(ctx, item, 1, tables, n_tables, precision, &b);
  if (rc) return rc;
  rc = gb_batch_get(ctx, b, out, nullptr);
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaStreamSynchronize(ctx->stream);
  free_batch(ctx, b);
  return rc;
}

// ------------------------------------------------------------------ serving
int gb_serve_start(gb_ctx *ctx, int max_inflight, int max_items)
{
  if (ctx && ctx->dloop) return set_error(ctx, GB_EINVAL, "serving already started");
  return serve_start(ctx, max_inflight, max_items);
}
int gb_serve_start_device(gb_ctx *ctx, int ring_slots, int max_items, long long max_units, double idle_seconds)
{
  return dloop_start(ctx, ring_slots, max_items, max_units, idle_seconds);
}
int gb_serve_device_info(gb_ctx *ctx, long long *launches, int *idle_exits, int *running)
{
  if (!ctx) return GB_EINVAL;
  if (!ctx->dloop) return set_error(ctx, GB_EINVAL, "device request loop not started (gb_serve_start_device)");
  return dloop_info(ctx, launches, idle_exits, running);
}
int gb_serve_stop(gb_ctx *ctx)
{
  if (ctx && ctx->dloop) return dloop_stop(ctx);
  return serve_stop(ctx);
}
int gb_submit(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
              gb_ticket *out)
{
  if (ctx && ctx->dloop) return dloop_submit(ctx, items, n, tables, n_tables, precision, out);
  return serve_submit(ctx, items, n, tables, n_tables, precision, out);
}
int gb_poll(gb_ctx *ctx, gb_ticket t, double *out)
{
  if (ctx && ctx->dloop) return dloop_poll(ctx, t, out, false, 0.0);
  return serve_poll(ctx, t, out, false, 0.0);
}
int gb_wait(gb_ctx *ctx, gb_ticket t, double *out, double timeout_s)
{
  if (ctx && ctx->dloop) return dloop_poll(ctx, t, out, true, timeout_s);
  return serve_poll(ctx, t, out, true, timeout_s);
}
int gb_cancel(gb_ctx *ctx, gb_ticket t)
{
  if (ctx && ctx->dloop) return GB_EAGAIN;  // published at submit: already on the GPU
  return serve_cancel(ctx, t);
}
int gb_get_stats(gb_ctx *ctx, gb_stats *out)
{
  if (ctx && ctx->dloop && out) {
    *out = gb_stats{};
    out->bytes_in_use = ctx->in_use;
    out->bytes_budget = ctx->budget;
    return dloop_stats(ctx, out);
  }
  return serve_stats(ctx, out);
}
int gb_reset_stats(gb_ctx *ctx)
{
  if (ctx && ctx->dloop) return dloop_reset_stats(ctx);
  return serve_reset_stats(ctx);
}

int gb_selftest_wait(gb_ctx *ctx, long long max_cycles)
{
  if (!ctx) return GB_EINVAL;
  if (max_cycles < 1 || max_cycles > (1ll << 31)) return set_error(ctx, GB_EINVAL, "max_cycles must be 1..2^31");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  GB_CUDA(cudaSetDevice(ctx->device));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  int before = 0;
  GB_CUDA(cudaMemcpy(&before, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  GB_CUDA(launch_wait_selftest(ctx->d_err, max_cycles, ctx->stream));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  int err = 0;
  GB_CUDA(cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  GB_CUDA(cudaMemcpy(ctx->d_err, &before, sizeof(int), cudaMemcpyHostToDevice));
  if (err & ~before & kErrMbarTimeout)
    return set_error(ctx, GB_ETIMEDOUT, "bounded mbarrier wait gave up after " + std::to_string(max_cycles) + " cycles");
  return GB_OK;
}

int gb_measure_peaks(gb_ctx *ctx, double *fp32_tflops, double *mufu_gops, double *fp64_tflops)
{
  if (!ctx) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  GB_CUDA(cudaSetDevice(ctx->device));
  void *buf = nullptr;
  GB_CUDA(cudaMalloc(&buf, 64));
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  cudaStream_t s = ctx->stream;
  const int threads = 256, ctas = ctx->num_sms * 8;
  auto timeit = [&](int which, int iters, double &ms) -> int {
    for (int rep = 0; rep < 2; ++rep) {  // warm-up + timed
      GB_CUDA(cudaEventRecord(e0, s));
      cudaError_t e = which == 0   ? launch_peak_ffma((float *)buf, ctas, threads, iters, s)
                      : which == 1 ? launch_peak_mufu((float *)buf, ctas, threads, iters, s)
                                   : launch_peak_dfma((double *)buf, ctas, threads, iters, s);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "peak probe");
      GB_CUDA(cudaEventRecord(e1, s));
      GB_CUDA(cudaEventSynchronize(e1));
      float f = 0;
      GB_CUDA(cudaEventElapsedTime(&f, e0, e1));
      ms = f;
    }
    return GB_OK;
  };
  const double nthreads = (double)threads * ctas;
  double ms = 0;
  int rc = timeit(0, 4096, ms);
  if (!rc && fp32_tflops) *fp32_tflops = nthreads * 4096.0 * 16 * 8 * 2 / (ms * 1e-3) / 1e12;
  if (!rc) rc = timeit(1, 2048, ms);
  if (!rc && mufu_gops) *mufu_gops = nthreads * 2048.0 * 4 * 8 / (ms * 1e-3) / 1e9;
  if (!rc) rc = timeit(2, 64, ms);
  if (!rc && fp64_tflops) *fp64_tflops = nthreads * 64.0 * 4 * 8 * 2 / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  return rc;
}

} // extern "C"
