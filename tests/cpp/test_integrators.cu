// Test driver of the DiFfRG-compatible class templates (include/gbint/integrators.hh).
//
// Like the reference's integrator tests (e.g. DiFfRG/tests/physics/integration/integrator_4D_gpu.cu),
// each family integrates a product of polynomials (a rational function in q0 for the finite-T
// q0 families).  Cases come on stdin, one per line:
//   family d n0 n1 n2 n3 x_extent x0_extent x0_summands T k prec a0 .. a23
// (prec 0 = NT double, 1 = NT float; family numbers as GB_FAM_* in gbint.h); this program prints
// one value per case with 17 significant digits.  tests/test_gpu_cpp_api.py compares them with
// the FP64 oracle and with the closed forms.
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "gbint/autodiff.hh"
#include "gbint/integrators.hh"
#include "gbint/interpolators.hh"
#include "gbint/regulators.hh"
#include "gbint/flow_utils.hh"
#include "gbint/kernel_math.hh"

using namespace DiFfRG;

// KERNEL reading two dressing functions through interpolator objects passed as arguments,
// the way generated DiFfRG kernels do (e.g. ZA.kernel): G(x) = 1/(Z(x) x + R(x)), R = x/expm1(x)
using ZTex = TexLinearInterpolator1D<double, LogarithmicCoordinates1D<float>>;
using ZLin = LinearInterpolator1D<double, LinearCoordinates1D<double>>;
struct KInterp {
  static __host__ __device__ double kernel(double q, double c, double k, const ZTex &Z, const ZLin &W, double p)
  {
    const double q2 = q * q, x2 = q2 + p * p + 2 * p * q * c;
    const double R1 = q2 > 0 ? q2 / expm1(q2) : 1.0, R2 = x2 > 0 ? x2 / expm1(x2) : 1.0;
    return W(q2) / ((Z((float)q2) * q2 + R1) * (Z((float)x2) * x2 + R2));
  }
  static __host__ __device__ double constant(double, const ZTex &, const ZLin &, double) { return 0.0; }
};

struct Coeffs {
  double a[24];
};

template <typename NT> __host__ __device__ inline NT pv(const double *c, int n, NT x)
{
  NT r = 0;
  for (int i = n - 1; i >= 0; --i) r = r * x + (NT)c[i];
  return r;
}
template <typename NT> __host__ __device__ inline NT pq0(const Coeffs &C, NT q0)
{
  const NT v = pv<NT>(C.a + 19, 4, q0);
  return C.a[23] != 0 ? (NT)1 / v : v;
}

template <typename NT> struct K1 {  // (q)
  static __host__ __device__ NT kernel(NT q, NT, const Coeffs &C) { return pv<NT>(C.a + 1, 6, q); }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct K2 {  // (q, cos) -- angle; Cartesian 2D (qx, qy)
  static __host__ __device__ NT kernel(NT q, NT c, NT, const Coeffs &C) { return pv<NT>(C.a + 1, 6, q) * pv<NT>(C.a + 7, 4, c); }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct K3 {  // (q, c1, x3): 3D (phi), 4D2Ang (cos2), Cartesian 3D (qz)
  static __host__ __device__ NT kernel(NT q, NT c, NT z, NT, const Coeffs &C)
  {
    return pv<NT>(C.a + 1, 6, q) * pv<NT>(C.a + 7, 4, c) * pv<NT>(C.a + 11, 4, z);
  }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct K4 {  // 4D (q, c1, c2, phi)
  static __host__ __device__ NT kernel(NT q, NT c1, NT c2, NT phi, NT, const Coeffs &C)
  {
    return pv<NT>(C.a + 1, 6, q) * pv<NT>(C.a + 7, 4, c1) * pv<NT>(C.a + 11, 4, c2) * pv<NT>(C.a + 15, 4, phi);
  }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct KT1 {  // (q, q0)
  static __host__ __device__ NT kernel(NT q, NT q0, NT, const Coeffs &C) { return pv<NT>(C.a + 1, 6, q) * pq0<NT>(C, q0); }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct KT2 {  // (q, cos, q0)
  static __host__ __device__ NT kernel(NT q, NT c, NT q0, NT, const Coeffs &C)
  {
    return pv<NT>(C.a + 1, 6, q) * pv<NT>(C.a + 7, 4, c) * pq0<NT>(C, q0);
  }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct KT3 {  // (q, cos, phi, q0)
  static __host__ __device__ NT kernel(NT q, NT c, NT phi, NT q0, NT, const Coeffs &C)
  {
    return pv<NT>(C.a + 1, 6, q) * pv<NT>(C.a + 7, 4, c) * pv<NT>(C.a + 11, 4, phi) * pq0<NT>(C, q0);
  }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};
template <typename NT> struct KC {  // constant integrator: kernel(k)
  static __host__ __device__ NT kernel(NT k, const Coeffs &C) { return pv<NT>(C.a + 1, 6, k); }
  static __host__ __device__ NT constant(NT, const Coeffs &C) { return (NT)C.a[0]; }
};

struct Case {
  int fam, d, n[4], ns, prec;
  double xe, x0e, T, k;
  Coeffs C;
};

template <typename NT, int d> double run_d(QuadratureProvider &qp, const Case &c)
{
  const NT xe = (NT)c.xe, k = (NT)c.k;
  const uint n0 = c.n[0], n1 = c.n[1], n2 = c.n[2], n3 = c.n[3];
  switch (c.fam) {
  case GB_FAM_1D: return IntegratorGPU<d, NT, K1<NT>>(qp, {{n0}}, xe).get(k, c.C);
  case GB_FAM_ANGLE: return IntegratorAngleGPU<d, NT, K2<NT>>(qp, {{n0, n1}}, xe).get(k, c.C);
  case GB_FAM_FTQ0: return IntegratorFiniteTq0GPU<d, NT, KT1<NT>>(qp, {{n0}}, xe, (NT)c.T).get(k, c.C);
  case GB_FAM_ANGLE_FTQ0: return IntegratorAngleFiniteTq0GPU<d, NT, KT2<NT>>(qp, {{n0, n1}}, xe, (NT)c.T).get(k, c.C);
  case GB_FAM_FTX0:
    return IntegratorFiniteTx0GPU<d, NT, KT1<NT>>(qp, {{n0, n1}}, xe, (NT)c.x0e, c.ns, (NT)c.T).get(k, c.C);
  case GB_FAM_ANGLE_FTX0:
    return IntegratorAngleFiniteTx0GPU<d, NT, KT2<NT>>(qp, {{n0, n1, n2}}, xe, (NT)c.x0e, c.ns, (NT)c.T).get(k, c.C);
  case GB_FAM_CONST: return IntegratorConstant<d, NT, KC<NT>>(qp, {{n0}}, xe).get(k, c.C);
  }
  throw std::runtime_error("family without dimension template");
}

template <typename NT> double run(QuadratureProvider &qp, const Case &c)
{
  const NT xe = (NT)c.xe, k = (NT)c.k;
  const uint n0 = c.n[0], n1 = c.n[1], n2 = c.n[2], n3 = c.n[3];
  switch (c.fam) {
  case GB_FAM_3D: return Integrator3DGPU<NT, K3<NT>>(qp, {{n0, n1, n2}}, xe).get(k, c.C);
  case GB_FAM_4D2ANG: return Integrator4D2AngGPU<NT, K3<NT>>(qp, {{n0, n1, n2}}, xe).get(k, c.C);
  case GB_FAM_4D: return Integrator4DGPU<NT, K4<NT>>(qp, {{n0, n1, n2, n3}}, xe).get(k, c.C);
  case GB_FAM_CART1: {
    Integrator1DCartesianGPU<NT, K1<NT>> I(qp, {{n0}});
    I.set_qx_min(-1.0), I.set_qx_max(1.5);
    return I.get(k, c.C);
  }
  case GB_FAM_CART2: {
    Integrator2DCartesianGPU<NT, K2<NT>> I(qp, {{n0, n1}});
    I.set_qx_min(-1.0), I.set_qx_max(1.5), I.set_qy_min(-0.5), I.set_qy_max(0.5);
    return I.get(k, c.C);
  }
  case GB_FAM_CART3: {
    Integrator3DCartesianGPU<NT, K3<NT>> I(qp, {{n0, n1, n2}});
    I.set_qx_min(-1.0), I.set_qx_max(1.5), I.set_qy_min(-0.5), I.set_qy_max(0.5), I.set_qz_min(-2.0),
        I.set_qz_max(1.0);
    return I.get(k, c.C);
  }
  case GB_FAM_2DPQ0: return Integrator2Dpq0GPU<NT, KT2<NT>>(qp, {{n0, n1, n2}}, xe, (NT)c.x0e).get(k, c.C);
  case GB_FAM_2DPX0: return Integrator2Dpx0GPU<NT, KT2<NT>>(qp, {{n0, n1, n2}}, xe, (NT)c.x0e).get(k, c.C);
  case GB_FAM_3DPQ0: return Integrator3Dpq0GPU<NT, KT3<NT>>(qp, {{n0, n1, n2, n3}}, xe, (NT)c.x0e).get(k, c.C);
  case GB_FAM_3DPX0: return Integrator3Dpx0GPU<NT, KT3<NT>>(qp, {{n0, n1, n2, n3}}, xe, (NT)c.x0e).get(k, c.C);
  case GB_FAM_4D_FTQ0: return Integrator4DFiniteTq0GPU<NT, KT3<NT>>(qp, {{n0, n1, n2}}, xe, (NT)c.T).get(k, c.C);
  case GB_FAM_4D_FTX0:
    return Integrator4DFiniteTx0GPU<NT, KT3<NT>>(qp, {{n0, n1, n2, n3}}, xe, (NT)c.x0e, c.ns, (NT)c.T).get(k, c.C);
  }
  if (c.d == 3) return run_d<NT, 3>(qp, c);
  if (c.d == 4) return run_d<NT, 4>(qp, c);
  throw std::runtime_error("unsupported d");
}

// complex result type: real part = the K2 polynomial with coefficients A, imaginary part = with B
struct KComplex {
  using CT = cuda::std::complex<double>;
  static __host__ __device__ CT kernel(double q, double c, double k, const Coeffs &A, const Coeffs &B)
  {
    return CT(K2<double>::kernel(q, c, k, A), K2<double>::kernel(q, c, k, B));
  }
  static __host__ __device__ CT constant(double k, const Coeffs &A, const Coeffs &B) { return CT(A.a[0], B.a[0]); }
};
struct KComplexF {
  using CT = cuda::std::complex<float>;
  static __host__ __device__ CT kernel(float q, float c, float k, const Coeffs &A, const Coeffs &B)
  {
    return CT(K2<float>::kernel(q, c, k, A), K2<float>::kernel(q, c, k, B));
  }
  static __host__ __device__ CT constant(float k, const Coeffs &A, const Coeffs &B) { return CT((float)A.a[0], (float)B.a[0]); }
};

int complex_cases()
{
  QuadratureProvider qp;
  Coeffs A{}, B{};
  A.a[0] = 0.25;
  A.a[1] = 1.0;
  A.a[3] = 0.5;
  A.a[7] = 1.0;
  A.a[8] = 0.3;
  B.a[0] = -0.5;
  B.a[2] = 2.0;
  B.a[7] = 0.2;
  B.a[9] = 1.0;
  IntegratorAngleGPU<4, cuda::std::complex<double>, KComplex> IC(qp, {{48, 16}}, 1.7);
  IntegratorAngleGPU<4, double, K2<double>> ID(qp, {{48, 16}}, 1.7);
  IntegratorAngleGPU<4, cuda::std::complex<float>, KComplexF> IF(qp, {{48, 16}}, 1.7);
  for (double k : {0.5, 1.0, 1.3}) {
    const auto z = IC.get(k, A, B);
    const auto zf = IF.request((float)k, A, B).get();
    std::printf("CPLX %.17g %.17g %.17g %.17g %.9g %.9g\n", z.real(), z.imag(), ID.get(k, A), ID.get(k, B),
                (double)zf.real(), (double)zf.imag());
  }
  return 0;
}

// dual result type (the role of autodiff::real): the polynomial integrands times e^{-s u},
// u = q^2/k^2 (Cartesian: qx^2/k^2), with s the seeded variable.  The value and the
// s-derivative are compared with two plain FP64 integrals of e^{-s u} f and -u e^{-s u} f.
template <typename T> struct KDualAngle {
  using R = gbint::dual<T>;
  static __host__ __device__ R kernel(T q, T c, T k, const Coeffs &C, const R &s)
  {
    return K2<T>::kernel(q, c, k, C) * exp(-s * (q * q / (k * k)));
  }
  static __host__ __device__ R constant(T, const Coeffs &C, const R &) { return R(C.a[0]); }
};
struct KDualCart {
  using R = autodiff::real;
  static __host__ __device__ R kernel(double qx, double k, const Coeffs &C, const R &s)
  {
    return K1<double>::kernel(qx, k, C) * exp(-s * (qx * qx / (k * k)));
  }
  static __host__ __device__ R constant(double, const Coeffs &C, const R &) { return R(C.a[0]); }
};
struct KDualFT {
  using R = autodiff::real;
  static __host__ __device__ R kernel(double q, double c, double q0, double k, const Coeffs &C, const R &s)
  {
    return KT2<double>::kernel(q, c, q0, k, C) * exp(-s * (q * q / (k * k)));
  }
  static __host__ __device__ R constant(double, const Coeffs &C, const R &) { return R(C.a[0]); }
};
template <int DER> __host__ __device__ inline double damped(double f, double u, double s)
{
  const double e = ::exp(-s * u) * f;
  return DER ? -u * e : e;
}
template <int DER> struct PDualAngle {
  static __host__ __device__ double kernel(double q, double c, double k, const Coeffs &C, double s)
  {
    return damped<DER>(K2<double>::kernel(q, c, k, C), q * q / (k * k), s);
  }
  static __host__ __device__ double constant(double, const Coeffs &C, double) { return DER ? 0.0 : C.a[0]; }
};
template <int DER> struct PDualCart {
  static __host__ __device__ double kernel(double qx, double k, const Coeffs &C, double s)
  {
    return damped<DER>(K1<double>::kernel(qx, k, C), qx * qx / (k * k), s);
  }
  static __host__ __device__ double constant(double, const Coeffs &C, double) { return DER ? 0.0 : C.a[0]; }
};
template <int DER> struct PDualFT {
  static __host__ __device__ double kernel(double q, double c, double q0, double k, const Coeffs &C, double s)
  {
    return damped<DER>(KT2<double>::kernel(q, c, q0, k, C), q * q / (k * k), s);
  }
  static __host__ __device__ double constant(double, const Coeffs &C, double) { return DER ? 0.0 : C.a[0]; }
};

// prints "DUAL <family> value derivative plain_value plain_derivative" per case
int dual_cases()
{
  QuadratureProvider qp;
  Coeffs A{};
  A.a[0] = 0.25;
  A.a[1] = 1.0;
  A.a[3] = 0.5;
  A.a[7] = 1.0;
  A.a[8] = 0.3;
  A.a[19] = 1.0;  // q0 factor 1 + q0^2 (finite T)
  A.a[21] = 1.0;
  IntegratorAngleGPU<4, autodiff::real, KDualAngle<double>> IA(qp, {{48, 16}}, 1.7);
  IntegratorAngleGPU<4, gbint::dual<float>, KDualAngle<float>> IAf(qp, {{48, 16}}, 1.7);
  IntegratorAngleGPU<4, double, PDualAngle<0>> PA0(qp, {{48, 16}}, 1.7);
  IntegratorAngleGPU<4, double, PDualAngle<1>> PA1(qp, {{48, 16}}, 1.7);
  Integrator1DCartesianGPU<autodiff::real, KDualCart> IC(qp, {{32}});
  Integrator1DCartesianGPU<double, PDualCart<0>> PC0(qp, {{32}});
  Integrator1DCartesianGPU<double, PDualCart<1>> PC1(qp, {{32}});
  PC0.set_qx_min(-1.5), PC0.set_qx_max(1.2);
  PC1.set_qx_min(-1.5), PC1.set_qx_max(1.2);
  IC.set_qx_min(-1.5), IC.set_qx_max(1.2);
  IntegratorAngleFiniteTq0GPU<4, autodiff::real, KDualFT> IT(qp, {{32, 12}}, 1.5, 0.2);
  IntegratorAngleFiniteTq0GPU<4, double, PDualFT<0>> PT0(qp, {{32, 12}}, 1.5, 0.2);
  IntegratorAngleFiniteTq0GPU<4, double, PDualFT<1>> PT1(qp, {{32, 12}}, 1.5, 0.2);
  for (double k : {0.6, 1.1}) {
    for (double s : {0.3, 1.7}) {
      const autodiff::real sd = gbint::seed(s);
      const autodiff::real a = IA.get(k, A, sd);
      const gbint::dual<float> af = IAf.request((float)k, A, gbint::seed((float)s)).get();
      std::printf("DUAL ANGLE %.17g %.17g %.17g %.17g\n", val(a), derivative(a), PA0.get(k, A, s), PA1.get(k, A, s));
      std::printf("DUAL ANGLEF %.9g %.9g %.17g %.17g\n", (double)val(af), (double)derivative(af), PA0.get(k, A, s),
                  PA1.get(k, A, s));
      const autodiff::real c = IC.request(k, A, sd).get();
      std::printf("DUAL CART1 %.17g %.17g %.17g %.17g\n", val(c), derivative(c), PC0.get(k, A, s), PC1.get(k, A, s));
      const autodiff::real t = IT.get(k, A, sd);
      std::printf("DUAL FTQ0 %.17g %.17g %.17g %.17g\n", val(t), derivative(t), PT0.get(k, A, s), PT1.get(k, A, s));
    }
  }
  return 0;
}

// regulator shapes (gbint/regulators.hh): each function on the host and on the device, and the
// derivatives once more by forward differentiation with gbint::dual (dq2RB: q^2 seeded;
// RBdot = 2 k^2 dR/dk^2: k^2 seeded with derivative 2 k^2).  Prints
// "REG <name> <k2> <q2> <fn> <host> <device> <dual>" (dual: nan where not applicable).
constexpr int kRegFns = 6;  // RB, RBdot, dq2RB, RF, RFdot, dq2RF
template <class R, bool DQ2> __host__ __device__ void reg_eval(double k2, double q2, double *o)
{
  o[0] = R::RB(k2, q2);
  o[1] = R::RBdot(k2, q2);
  o[3] = R::RF(k2, q2);
  o[4] = R::RFdot(k2, q2);
  if constexpr (DQ2) {
    o[2] = R::dq2RB(k2, q2);
    o[5] = R::dq2RF(k2, q2);
  } else
    o[2] = o[5] = NAN;
}
template <class R, bool DQ2> __global__ void reg_kernel(const double *kq, int n, double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) reg_eval<R, DQ2>(kq[2 * t], kq[2 * t + 1], out + kRegFns * t);
}
struct Bos1 {
  static constexpr double b = 1.;
};
struct Exp3 {
  static constexpr double b = 3.;
};
struct Poly3 {
  static constexpr int order = 3;
};
struct Rat5 {
  static constexpr int order = 5;
  constexpr static double c = 1.5;
  constexpr static double b0 = 0.25;
};
template <class R, bool DQ2> int reg_case(const char *name)
{
  std::vector<double> kq;
  for (double k2 : {0.3, 1.0, 2.5})
    for (double q2 : {1e-3, 0.2, 0.9, 1.7, 4.0}) kq.push_back(k2), kq.push_back(q2);
  const int n = (int)kq.size() / 2;
  double *dkq = nullptr, *dout = nullptr;
  if (cudaMalloc(&dkq, kq.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dout, n * kRegFns * sizeof(double)) != cudaSuccess)
    return 1;
  cudaMemcpy(dkq, kq.data(), kq.size() * sizeof(double), cudaMemcpyHostToDevice);
  reg_kernel<R, DQ2><<<1, 64>>>(dkq, n, dout);
  std::vector<double> dev(n * kRegFns);
  if (cudaMemcpy(dev.data(), dout, dev.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  cudaFree(dkq);
  cudaFree(dout);
  for (int t = 0; t < n; ++t) {
    const double k2 = kq[2 * t], q2 = kq[2 * t + 1];
    double h[kRegFns];
    reg_eval<R, DQ2>(k2, q2, h);
    double ad[kRegFns];
    for (double &v : ad) v = NAN;
    ad[1] = gbint::derivative(R::RB(autodiff::real(k2, 2 * k2), q2));
    if constexpr (DQ2) ad[2] = gbint::derivative(R::RB(k2, gbint::seed(q2)));
    ad[4] = gbint::derivative(R::RF(autodiff::real(k2, 2 * k2), q2));
    if constexpr (DQ2) ad[5] = gbint::derivative(R::RF(k2, gbint::seed(q2)));
    for (int f = 0; f < kRegFns; ++f)
      std::printf("REG %s %.17g %.17g %d %.17g %.17g %.17g\n", name, k2, q2, f, h[f], dev[t * kRegFns + f], ad[f]);
  }
  return 0;
}
int regulator_cases()
{
  int rc = 0;
  rc |= reg_case<LitimRegulator<>, false>("litim");
  rc |= reg_case<BosonicRegulator<>, true>("bosonic2");
  rc |= reg_case<BosonicRegulator<Bos1>, true>("bosonic1");
  rc |= reg_case<ExponentialRegulator<>, true>("exp2");
  rc |= reg_case<ExponentialRegulator<Exp3>, true>("exp3");
  rc |= reg_case<SmoothedLitimRegulator<>, false>("smoothlitim");
  rc |= reg_case<PolynomialExpRegulator<>, true>("polyexp8");
  rc |= reg_case<PolynomialExpRegulator<Poly3>, true>("polyexp3");
  rc |= reg_case<RationalExpRegulator<>, true>("ratexp8");
  rc |= reg_case<RationalExpRegulator<Rat5>, true>("ratexp5");
  return rc;
}

// fan-out helpers (gbint/flow_utils.hh): request_data over a grid of external momenta (a
// std::vector and a 2D coordinate pack), update_data, update_interpolator, get_data; every value
// must equal the direct get() bit for bit.  Prints "FAN <what> <max abs diff> <n>".
struct KExt1 {  // the K2 polynomial times (1 + p q^2): one external argument p per grid point
  static __host__ __device__ double kernel(double q, double c, double k, double p, const Coeffs &C)
  {
    return K2<double>::kernel(q, c, k, C) * (1 + p * q * q);
  }
  static __host__ __device__ double constant(double, double p, const Coeffs &C) { return C.a[0] + p; }
};
struct KExt2 {  // two external arguments (p1, p2) from a 2D coordinate pack
  static __host__ __device__ double kernel(double q, double c, double k, double p1, double p2, const Coeffs &C)
  {
    return K2<double>::kernel(q, c, k, C) * (1 + p1 * q * q + p2 * c);
  }
  static __host__ __device__ double constant(double, double, double, const Coeffs &C) { return C.a[0]; }
};
struct KTabArg {  // two interpolator arguments (their tables are staged in shared memory)
  template <class TAB>
  static __host__ __device__ double kernel(double q, double c, double k, double p, const TAB &Z, const TAB &Y)
  {
    const double r = sqrt(q * q + p * p - 2 * p * q * c);
    return Z(q) * Y(r) * q * q / (1 + q * q * q * q) * (1 + 0.5 * c * k);
  }
  template <class TAB> static __host__ __device__ double constant(double, double p, const TAB &Z, const TAB &) { return Z(p); }
};
struct KTabDual {  // dual result: the seeded argument s enters through exp(-s q^2)
  template <class TAB>
  static __host__ __device__ autodiff::real kernel(double q, double c, double k, const autodiff::real &s, const TAB &Z)
  {
    return Z(q) * exp(-s * q * q) * (1 + c * c) * k;
  }
  template <class TAB> static __host__ __device__ autodiff::real constant(double, const autodiff::real &, const TAB &)
  {
    return autodiff::real(0.0);
  }
};
int fanout_cases()
{
  QuadratureProvider qp;
  Coeffs A{};
  A.a[0] = 0.25;
  A.a[1] = 1.0;
  A.a[3] = 0.5;
  A.a[7] = 1.0;
  A.a[8] = 0.3;
  const double k = 0.8;
  IntegratorAngleGPU<4, double, KExt1> I1(qp, {{32, 16}}, 1.5);
  IntegratorAngleGPU<4, double, KExt2> I2(qp, {{32, 16}}, 1.5);
  auto report = [](const char *what, const std::vector<double> &a, const std::vector<double> &b) {
    double m = a.size() == b.size() ? 0.0 : 1e300;
    for (size_t i = 0; i < a.size() && i < b.size(); ++i) m = std::max(m, std::fabs(a[i] - b[i]));
    std::printf("FAN %s %.17g %zu\n", what, m, a.size());
  };
  // 1D grid (std::vector) and a 1D coordinates object
  LogarithmicCoordinates1D<double> pc(24, 1e-3, 10.0, 0.0);
  const auto grid = make_grid(pc);
  std::vector<double> direct(grid.size()), viafut(grid.size()), viaget(grid.size()), viacoord(grid.size());
  for (size_t i = 0; i < grid.size(); ++i) direct[i] = I1.get(k, grid[i], A);
  update_data(request_data<double>(I1, grid, k, A), viafut.data());
  report("request_data_vector", viafut, direct);
  update_data(request_data<double>(I1, pc, k, std::make_tuple(A)), viacoord.data());
  report("request_data_coordinates_tuple", viacoord, direct);
  get_data<double>(viaget.data(), I1, grid, k, A);
  report("get_data", viaget, direct);
  // into an interpolator over the same coordinates
  LinearInterpolator1D<double, LogarithmicCoordinates1D<double>> Zi(pc);
  update_interpolator(request_data<double>(I1, grid, k, A), Zi);
  std::vector<double> back(grid.size());
  for (size_t i = 0; i < grid.size(); ++i) back[i] = Zi[i];
  report("update_interpolator", back, direct);
  // 2D coordinate pack
  using LC = LinearCoordinates1D<double>;
  CoordinatePackND<LC, LC> pack(LC(5, 0.0, 1.0), LC(4, -1.0, 1.0));
  const auto g2 = make_grid(pack);
  std::vector<double> d2(g2.size()), v2(g2.size());
  for (size_t i = 0; i < g2.size(); ++i) d2[i] = I2.get(k, g2[i][0], g2[i][1], A);
  update_data(request_data<double>(I2, pack, k, A), v2.data());
  report("request_data_pack2d", v2, d2);

  // RequestBatch scope: integrals of two integrators of one type with different grids and of
  // several k in one launch; a get() inside the scope launches the open batch, later requests
  // start a new one; a kernel with TexLinearInterpolator1D arguments (staged tables) and a dual
  // result type alongside.  Every value bit-identical to its single get().
  IntegratorAngleGPU<4, double, KExt1> I1b(qp, {{48, 12}}, 1.2);
  IntegratorAngleGPU<4, double, KTabArg> IT(qp, {{40, 20}}, 2.0);
  IntegratorAngleGPU<4, autodiff::real, KTabDual> ID(qp, {{24, 8}}, 1.7);
  IntegratorAngleGPU<4, double, KExt1> IB(qp, {{160, 128}}, 1.4);  // 20480 points: two points per thread
  const LogarithmicCoordinates1D<float> tc(48, 1e-3f, 20.f, 4.f);
  std::vector<double> zv(48), yv(48);
  for (int i = 0; i < 48; ++i) zv[i] = 1.0 + 0.3 * std::sin(0.37 * i), yv[i] = 0.5 + 0.01 * i * i;
  const TexLinearInterpolator1D<double, LogarithmicCoordinates1D<float>> Z(zv, tc), Y(yv, tc);
  std::vector<std::future<double>> fs;
  std::vector<std::future<autodiff::real>> fd;
  std::vector<double> want;
  std::vector<autodiff::real> wantd;
  for (int i = 0; i < 10; ++i) want.push_back(I1.get(0.5 + 0.05 * i, grid[i], A));
  for (int i = 0; i < 10; ++i) want.push_back(I1b.get(0.7, grid[i], A));
  for (int i = 0; i < 4; ++i) want.push_back(I1.get(0.9, grid[i], A));
  for (int i = 0; i < 3; ++i) want.push_back(IB.get(0.8, grid[i], A));
  for (int i = 0; i < 8; ++i) want.push_back(IT.get(1.1, grid[i], Z, Y));
  for (int i = 0; i < 6; ++i) wantd.push_back(ID.get(1.0, autodiff::real(0.2 + 0.1 * i, 1.0), Z));
  double early = 0;
  {
    RequestBatch rb;
    for (int i = 0; i < 10; ++i) fs.push_back(I1.request(0.5 + 0.05 * i, grid[i], A));
    for (int i = 0; i < 10; ++i) fs.push_back(I1b.request(0.7, grid[i], A));
    early = fs[3].get();  // launches the open batch of this kernel type
    for (int i = 0; i < 4; ++i) fs.push_back(I1.request(0.9, grid[i], A));
    for (int i = 0; i < 3; ++i) fs.push_back(IB.request(0.8, grid[i], A));
    for (int i = 0; i < 8; ++i) fs.push_back(IT.request(1.1, grid[i], Z, Y));
    for (int i = 0; i < 6; ++i) fd.push_back(ID.request(1.0, autodiff::real(0.2 + 0.1 * i, 1.0), Z));
  }
  std::vector<double> got, wd, gd;
  for (size_t i = 0; i < fs.size(); ++i) got.push_back(i == 3 ? early : fs[i].get());
  for (size_t i = 0; i < fd.size(); ++i) {
    const autodiff::real v = fd[i].get();
    gd.push_back(autodiff::val(v)), gd.push_back(autodiff::derivative(v));
    wd.push_back(autodiff::val(wantd[i])), wd.push_back(autodiff::derivative(wantd[i]));
  }
  report("request_batch_scope", got, want);
  report("request_batch_scope_dual", gd, wd);
  std::printf("FAN staging_fallbacks %lld 1\n", (long long)gbint_detail::staging_fallbacks().load());
  return 0;
}

// a KERNEL in the shape the reference's code generator writes (template on the regulator,
// templated argument types, powr / complex / real, private RB.. forwarding to REG), used through
// a CPU (TBB) class name, against the same integrand in plain real arithmetic on the GPU class:
// Rdot(q^2) Re[(q^2 + R + m2 + (q0 + i mu)^2)^-2].  Prints "GEN <T> <generated> <plain>".
template <typename REG> class GenKernel
{
public:
  template <typename T1, typename T2>
  static __forceinline__ __host__ __device__ auto kernel(const double q, const double q0, const double k, const T1 m2,
                                                         const T2 mu)
  {
    const double R = RB(powr<2>(k), powr<2>(q));
    const double Rd = RBdot(powr<2>(k), powr<2>(q));
    return real(Rd * powr<-2>(complex<double>(powr<2>(q) + R + m2, 0.) + powr<2>(q0 + complex<double>(0., mu))));
  }
  template <typename T1, typename T2>
  static __forceinline__ __host__ __device__ auto constant(const double k, const T1 m2, const T2 mu)
  {
    return 0.1 * m2 + 0. * k * mu;
  }

private:
  static __forceinline__ __device__ __host__ auto RB(const double k2, const double p2) { return REG::RB(k2, p2); }
  static __forceinline__ __device__ __host__ auto RBdot(const double k2, const double p2) { return REG::RBdot(k2, p2); }
};
struct PlainKernel {
  static __host__ __device__ double kernel(double q, double q0, double k, double m2, double mu)
  {
    const double k2 = k * k, q2 = q * q;
    const double R = BosonicRegulator<>::RB(k2, q2), Rd = BosonicRegulator<>::RBdot(k2, q2);
    const double a = q2 + R + m2 + q0 * q0 - mu * mu, b = 2 * q0 * mu;
    return Rd * (a * a - b * b) / ((a * a + b * b) * (a * a + b * b));
  }
  static __host__ __device__ double constant(double, double m2, double) { return 0.1 * m2; }
};
int generated_cases()
{
  QuadratureProvider qp;
  for (double T : {0.15, 0.6}) {
    IntegratorFiniteTq0TBB<4, double, GenKernel<BosonicRegulator<>>> G(qp, {{40}}, 2.5, T);
    IntegratorFiniteTq0GPU<4, double, PlainKernel> P(qp, {{40}}, 2.5, T);
    for (double mu : {0.0, 0.3}) std::printf("GEN %.3g %.17g %.17g\n", T, G.get(0.9, 0.4, mu), P.get(0.9, 0.4, mu));
  }
  return 0;
}

// device evaluation of an interpolator at host-given points (checks the device branch)
template <typename I> __global__ void eval_pts3(I f, const double *x, int n, double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = (double)f(x[3 * t], x[3 * t + 1], x[3 * t + 2]);
}
template <typename I> __global__ void eval_pts2(I f, const double *x, int n, double *out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = (double)f(x[2 * t], x[2 * t + 1]);
}
template <int D, typename I> std::vector<double> on_device(const I &f, const std::vector<double> &x)
{
  const int n = (int)x.size() / D;
  double *dx = nullptr, *dout = nullptr;
  if (cudaMalloc(&dx, x.size() * sizeof(double)) != cudaSuccess || cudaMalloc(&dout, n * sizeof(double)) != cudaSuccess)
    throw std::runtime_error("cudaMalloc");
  cudaMemcpy(dx, x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice);
  if constexpr (D == 3)
    eval_pts3<<<(n + 127) / 128, 128>>>(f, dx, n, dout);
  else
    eval_pts2<<<(n + 127) / 128, 128>>>(f, dx, n, dout);
  std::vector<double> out(n);
  if (cudaMemcpy(out.data(), dout, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    throw std::runtime_error("device evaluation failed");
  cudaFree(dx);
  cudaFree(dout);
  return out;
}

// 3D and stacked interpolators: device branch vs host branch vs the closed form they must
// reproduce (multilinear data are interpolated exactly)
int interp3_cases()
{
  using L = LinearCoordinates1D<double>;
  using P3 = CoordinatePackND<L, L, L>;
  const uint n0 = 9, n1 = 7, n2 = 5;
  P3 pk(L(n0, -1.0, 3.0), L(n1, 0.0, 2.0), L(n2, -2.0, 2.0));
  auto tri = [](double x, double y, double z) {
    return 1 + 0.5 * x - 0.3 * y + 0.2 * z + 0.1 * x * y - 0.05 * y * z + 0.02 * x * z + 0.01 * x * y * z;
  };
  std::vector<double> data((size_t)n0 * n1 * n2);
  for (uint i = 0; i < n0; ++i)
    for (uint j = 0; j < n1; ++j)
      for (uint l = 0; l < n2; ++l) {
        const auto v = pk.forward(i, j, l);
        data[((size_t)i * n1 + j) * n2 + l] = tri(v[0], v[1], v[2]);
      }
  LinearInterpolator3D<double, P3> lin(data, pk);
  TexLinearInterpolator3D<double, P3> tex(data, pk);
  std::vector<double> pts;
  for (int t = 0; t < 40; ++t) {
    const double u = std::sin(1.3 * t + 0.2), v = std::cos(0.7 * t), w = std::sin(2.1 * t + 1.0);
    pts.push_back(1.0 + 1.9 * u);
    pts.push_back(1.0 + 0.95 * v);
    pts.push_back(1.9 * w);
  }
  const auto dl = on_device<3>(lin, pts), dt = on_device<3>(tex, pts);
  for (size_t t = 0; t < dl.size(); ++t) {
    const double x = pts[3 * t], y = pts[3 * t + 1], z = pts[3 * t + 2];
    std::printf("LIN3 %.17g %.17g %.17g\n", dl[t], lin(x, y, z), tri(x, y, z));
    std::printf("TEX3 %.17g %.17g %.17g\n", dt[t], tex(x, y, z), tri(x, y, z));
  }
  // clamping outside the box: the value at the nearest face
  const std::vector<double> out_pts{-5.0, 1.0, 0.5, 10.0, -3.0, 0.0};
  const auto dcl = on_device<3>(lin, out_pts);
  std::printf("CLAMP3 %.17g %.17g\n", dcl[0], tri(-1.0, 1.0, 0.5));
  std::printf("CLAMP3 %.17g %.17g\n", dcl[1], tri(3.0, 0.0, 0.0));
  // finite-T stack: modes n = 0..7 at T, 40 log-spaced p in [1e-3, 10]; data linear in the p
  // grid index per mode, so the lookup equals a_s + b_s * backward(p) exactly
  const double T = 0.15;
  using FT = BosonicCoordinates1DFiniteT<int, double>;
  FT fc(0, 8, T, 40, 1e-3, 10.0, 4.0);
  std::vector<double> sd(8 * 40);
  for (int s2 = 0; s2 < 8; ++s2)
    for (int i = 0; i < 40; ++i) sd[s2 * 40 + i] = 0.5 + 0.1 * s2 + 0.02 * (s2 + 1) * i;
  TexLinearInterpolator1DStack<double, FT> st(sd, fc);
  LogarithmicCoordinates1D<double> lc(40, 1e-3, 10.0, 4.0);
  std::vector<double> mp;
  for (int t = 0; t < 24; ++t) {
    const int mode = t % 10;  // modes 8, 9 lie above the stack: folded onto mode 7
    mp.push_back(2 * M_PI * T * mode);
    mp.push_back(std::exp(-6.0 + 0.35 * t));
  }
  const auto ds = on_device<2>(st, mp);
  for (size_t t = 0; t < ds.size(); ++t) {
    const double m = mp[2 * t], p = mp[2 * t + 1];
    int s2 = (int)std::lround(m / (2 * M_PI * T));
    double pp = p;
    if (s2 > 7) {
      const double dm = m - 2 * M_PI * T * 7;
      pp = std::sqrt(p * p + dm * dm);
      s2 = 7;
    }
    double idx = lc.backward(pp);
    idx = idx < 0 ? 0 : (idx > 39 ? 39 : idx);
    std::printf("STACK %.17g %.17g %.17g\n", ds[t], st(m, p), 0.5 + 0.1 * s2 + 0.02 * (s2 + 1) * idx);
  }
  return 0;
}

int main(int argc, char **argv)
{
  if (argc > 1 && std::string(argv[1]) == "--interp3") return interp3_cases();
  if (argc > 1 && std::string(argv[1]) == "--complex") return complex_cases();
  if (argc > 1 && std::string(argv[1]) == "--dual") return dual_cases();
  if (argc > 1 && std::string(argv[1]) == "--regulators") return regulator_cases();
  if (argc > 1 && std::string(argv[1]) == "--fanout") return fanout_cases();
  if (argc > 1 && std::string(argv[1]) == "--generated") return generated_cases();
  QuadratureProvider qp;
  std::string line;
  std::vector<Case> cases;
  while (std::getline(std::cin, line)) {
    if (line.empty()) continue;
    std::istringstream is(line);
    Case c{};
    is >> c.fam >> c.d >> c.n[0] >> c.n[1] >> c.n[2] >> c.n[3] >> c.xe >> c.x0e >> c.ns >> c.T >> c.k >> c.prec;
    for (int i = 0; i < 24; ++i) is >> c.C.a[i];
    cases.push_back(c);
  }
  // first all values through get(), then the same through request() launched back to back
  std::vector<double> got(cases.size());
  for (size_t i = 0; i < cases.size(); ++i) {
    try {
      got[i] = cases[i].prec ? run<float>(qp, cases[i]) : run<double>(qp, cases[i]);
    } catch (const std::exception &e) {
      std::printf("ERROR %s\n", e.what());
      return 2;
    }
    std::printf("%.17g\n", got[i]);
  }
  if (argc > 1 && std::string(argv[1]) == "--interp") {
    // device interpolation inside a user KERNEL vs the same quadrature summed on the host with
    // the interpolators' host branch
    std::vector<double> z(64), wv(33);
    for (int i = 0; i < 64; ++i) z[i] = 1.0 + 0.3 * std::sin(0.37 * i);
    for (int i = 0; i < 33; ++i) wv[i] = 0.5 + 0.01 * i * i;
    ZTex Z(z, LogarithmicCoordinates1D<float>(64, 1e-4f, 50.f, 3.f));
    ZLin W(wv, LinearCoordinates1D<double>(33, 0.0, 4.0));
    const uint nx = 48, nc = 16;
    const double xe = 3.0, k = 1.1;
    IntegratorAngleGPU<4, double, KInterp> I(qp, {{nx, nc}}, xe);
    for (double p : {0.01, 0.5, 2.0}) {
      const double got = I.get(k, Z, W, p);
      const auto &X = qp.get_points<double>(nx), &Xw = qp.get_weights<double>(nx);
      const auto &A = qp.get_points<double>(nc), &Aw = qp.get_weights<double>(nc);
      const double Sd = 2 * M_PI * M_PI;
      double ref = 0;
      for (uint i = 0; i < nx; ++i) {
        const double q = k * std::sqrt(X[i] * xe);
        const double ie = Sd * (q * q / 2 * k * k) * 0.5 / std::pow(2 * M_PI, 4);
        for (uint j = 0; j < nc; ++j) {
          const double c = 2 * (A[j] - 0.5);
          ref += ie * 2 * Aw[j] * Xw[i] * xe * KInterp::kernel(q, c, k, Z, W, p);
        }
      }
      std::printf("INTERP %.17g %.17g\n", got, ref);
    }
    // update(): new host values become visible to the next launch
    for (int i = 0; i < 64; ++i) Z[i] = 2.0f;
    Z.update();
    const double after = I.get(k, Z, W, 0.5);
    double ref2 = 0;
    {
      const auto &X = qp.get_points<double>(nx), &Xw = qp.get_weights<double>(nx);
      const auto &A = qp.get_points<double>(nc), &Aw = qp.get_weights<double>(nc);
      for (uint i = 0; i < nx; ++i) {
        const double q = k * std::sqrt(X[i] * xe);
        const double ie = 2 * M_PI * M_PI * (q * q / 2 * k * k) * 0.5 / std::pow(2 * M_PI, 4);
        for (uint j = 0; j < nc; ++j)
          ref2 += ie * 2 * Aw[j] * Xw[i] * xe * KInterp::kernel(q, 2 * (A[j] - 0.5), k, Z, W, 0.5);
      }
    }
    std::printf("INTERP %.17g %.17g\n", after, ref2);
    return 0;
  }
  if (argc > 1 && std::string(argv[1]) == "--requests") {
    // futures in flight together (pooled streams), then resolved
    IntegratorAngleGPU<4, double, K2<double>> I(qp, {{64, 12}}, 1.5);
    std::vector<std::future<double>> fs;
    Coeffs C{};
    C.a[1] = 1.0;
    C.a[7] = 1.0;
    for (int j = 0; j < 32; ++j) {
      C.a[2] = 0.01 * j;
      fs.push_back(I.request(0.8, C));
    }
    for (int j = 0; j < 32; ++j) {
      C.a[2] = 0.01 * j;
      const double a = fs[j].get(), b = I.get(0.8, C);
      std::printf("REQ %.17g %.17g\n", a, b);
    }
  }
  return 0;
}
