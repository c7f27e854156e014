// dropin_bench.cu -- throughput of the C++ drop-in path on a generated-layout flow: the seven-
// table vertex loop of tests/cpp/genflows/flows/loop (IntegratorAngleGPU<4, double>, seven
// TexLinearInterpolator1D tables, RationalExpRegulator) over 128 external momenta, FP64, at the
// quadrature the reference's examples run (x_quadrature_order 32, angle 2 x 8: 32 x 16 points,
// Examples/YangMills/SP/parameter.json with flows.cc's grid_sizes_angle_int) and at 64 x 32.
//
// Three ways to get the 128 integrals, each timed end to end on the host clock (steps of all
// 128, after warm-up; results read back to host memory every step):
//   batched    get_data: one RequestBatch, one persistent launch with staged nodes and tables
//   per_request  128 request() calls, each its own launch, then 128 get()
//   reference_pattern  the reference's IntegratorAngleGPU::request / future::get
//              (integrator_angle_gpu.hh:141-160): request() launches one kernel per integral on
//              a pooled stream (16 streams) writing every point's value to a device buffer (from a
//              pre-allocated pool, as its RMM pool), get() runs thrust::reduce on that stream
// Prints one JSON object.  The device time of the batched step is bracketed by CUDA events.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/reduce.h>

#include "flows/loop/Zphi.cu"

#include <DiFfRG/physics/utils.hh>

namespace
{
  using Clock = std::chrono::steady_clock;
  double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }
  using Tab = TexLinearInterpolator1D<double, LogarithmicCoordinates1D<float>>;
  using K = Zphi_kernel<__REGULATOR__>;
  using FAM = gbint::fam::FAngle<4>;

  // the reference pattern's per-point kernel: value * weight of every grid point to a buffer
  __global__ void k_points(gbint::fam::Params<double> P, long long n, double *out, double p, Tab a, Tab b, Tab c,
                           Tab d, Tab e, Tab f, Tab g, double m2)
  {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = FAM::eval<K, double>(P, i, p, a, b, c, d, e, f, g, m2);
  }

  std::vector<double> seeded(unsigned n, unsigned seed, double base, double amp)
  {
    std::vector<double> v(n);
    unsigned long long s = 88172645463325252ull ^ (seed * 0x9E3779B97F4A7C15ull);
    for (unsigned i = 0; i < n; ++i) {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      v[i] = base + amp * (double)(s >> 11) * (1.0 / 9007199254740992.0);
    }
    return v;
  }

  struct Result {
    double batched, batched_dev, per_request, reference, maxdiff_single, maxdiff_ref;
    long long points;
  };

  Result run_config(QuadratureProvider &qp, const JSONValue &json, std::array<uint, 2> gs, const std::vector<Tab> &T,
                    int steps, int warm)
  {
    const double x_extent = 3.0, k = 1.2, m2 = 0.15;
    Flows::Zphi_integrator flow(qp, gs, x_extent, json);
    const int NP = 128;
    std::vector<double> p(NP);
    for (int i = 0; i < NP; ++i) p[i] = 1e-2 * std::pow(1e3, i / (NP - 1.0));
    const auto args = std::make_tuple(T[0], T[1], T[2], T[3], T[4], T[5], T[6], m2);
    std::vector<double> batched(NP), single(NP), plain(NP);

    auto run_batched = [&]() { get_data<double>(batched.data(), flow, p, k, args); };
    auto run_single = [&]() {
      std::vector<std::future<double>> f;
      f.reserve(NP);
      for (int i = 0; i < NP; ++i)
        f.push_back(flow.request<double>(k, p[i], T[0], T[1], T[2], T[3], T[4], T[5], T[6], m2));
      for (int i = 0; i < NP; ++i) single[i] = f[i].get();
    };
    // the reference's request/get: one point kernel per request on a pooled stream, the
    // reduction (thrust::reduce on the same stream) when the future is read
    gbint::fam::Params<double> P;
    P.x_extent = x_extent;
    P.k = k;
    for (int a = 0; a < 2; ++a) {
      P.n[a] = (int)gs[a];
      P.x[a] = qp.get_device_points<double>(gs[a]);
      P.w[a] = qp.get_device_weights<double>(gs[a]);
    }
    const long long npts = FAM::points(P);
    constexpr int NS = 16;
    std::vector<cudaStream_t> st(NS);
    for (auto &x : st) cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking);
    std::vector<double *> buf(NP);
    for (auto &b : buf) cudaMalloc(&b, npts * sizeof(double));
    auto run_reference = [&]() {
      for (int i = 0; i < NP; ++i)
        k_points<<<(unsigned)((npts + 255) / 256), 256, 0, st[i % NS]>>>(P, npts, buf[i], p[i], T[0], T[1], T[2], T[3],
                                                                        T[4], T[5], T[6], m2);
      for (int i = 0; i < NP; ++i)
        plain[i] = K::constant(k, p[i], T[0], T[1], T[2], T[3], T[4], T[5], T[6], m2) +
                   thrust::reduce(thrust::cuda::par.on(st[i % NS]), buf[i], buf[i] + npts, 0.0, thrust::plus<double>());
    };

    auto timed = [&](auto &&fn) {
      for (int w = 0; w < warm; ++w) fn();
      cudaDeviceSynchronize();
      const auto t0 = Clock::now();
      for (int s = 0; s < steps; ++s) fn();
      cudaDeviceSynchronize();
      return secs(t0, Clock::now()) / steps;
    };
    Result r{};
    r.points = npts;
    r.batched = timed(run_batched);
    r.per_request = timed(run_single);
    r.reference = timed(run_reference);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double dev = 0;
    for (int s = 0; s < steps; ++s) {
      cudaDeviceSynchronize();
      cudaEventRecord(e0);
      run_batched();
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      dev += ms * 1e-3;
    }
    r.batched_dev = dev / steps;
    for (int i = 0; i < NP; ++i) {
      r.maxdiff_single = std::fmax(r.maxdiff_single, std::fabs(batched[i] - single[i]));
      r.maxdiff_ref = std::fmax(r.maxdiff_ref, std::fabs(batched[i] - plain[i]) / std::fabs(plain[i]));
    }
    for (auto &b : buf) cudaFree(b);
    for (auto &x : st) cudaStreamDestroy(x);
    return r;
  }

  void print_config(const char *name, const Result &r, int steps, bool last)
  {
    const int NP = 128;
    std::printf("\"%s\": {\"points_per_integral\": %lld, \"steps\": %d, "
                "\"batched\": {\"value\": %.6g, \"ms_per_step\": %.6g, \"device_ms_per_step\": %.6g}, "
                "\"per_request\": {\"value\": %.6g, \"ms_per_step\": %.6g}, "
                "\"reference_pattern\": {\"value\": %.6g, \"ms_per_step\": %.6g, \"streams\": 16}, "
                "\"batched_over_reference_pattern\": %.6g, \"batched_over_per_request\": %.6g, "
                "\"batched_equals_per_request_bitwise\": %s, \"max_rel_diff_vs_reference_pattern\": %.3e}%s",
                name, r.points, steps, NP / r.batched, r.batched * 1e3, r.batched_dev * 1e3, NP / r.per_request,
                r.per_request * 1e3, NP / r.reference, r.reference * 1e3, r.reference / r.batched,
                r.per_request / r.batched, r.maxdiff_single == 0 ? "true" : "false", r.maxdiff_ref, last ? "" : ", ");
  }
} // namespace

int main(int argc, char **argv)
{
  const int steps = argc > 1 ? std::atoi(argv[1]) : 20;
  const int warm = argc > 2 ? std::atoi(argv[2]) : 3;
  const JSONValue json(std::string(R"({"integration": {"cudathreadsperblock": 256}})"));
  QuadratureProvider qp(json);
  const LogarithmicCoordinates1D<float> coords(64, 1e-3f, 40.f, 5.f);
  std::vector<Tab> T;
  const double base[7] = {1.0, 0.8, 1.2, 0.05, 1.0, -0.1, 1.1}, amp[7] = {0.6, 0.5, 0.4, 0.1, 0.5, 0.2, 0.5};
  for (int t = 0; t < 7; ++t) T.emplace_back(seeded(64, 5 + t, base[t], amp[t]), coords);
  const Result ex = run_config(qp, json, {{32, 16}}, T, steps, warm);
  const Result big = run_config(qp, json, {{64, 32}}, T, steps, warm);
  std::printf("{\"workload\": \"generator-layout vertex loop (tests/cpp/genflows/flows/loop/Zphi): IntegratorAngleGPU<4, "
              "double>, seven 64-point TexLinearInterpolator1D tables, RationalExpRegulator, 128 external momenta per "
              "step\", \"integrals_per_step\": 128, \"unit\": \"integrals/s\", \"value\": %.6g, "
              "\"vs_reference_pattern\": %.6g, \"config_of_value\": \"examples_32x16\", ",
              128 / ex.batched, ex.reference / ex.batched);
  print_config("examples_32x16", ex, steps, false);
  print_config("grid_64x32", big, steps, true);
  std::printf("}\n");
  return 0;
}
