// selftest.cc -- TEST INFRASTRUCTURE ONLY: drives every entry point of the FP64 oracle once on
// small cases, built together with oracle_capi.cc under AddressSanitizer and
// UndefinedBehaviorSanitizer (`make -C oracle sanitize`).  Exit status 0 and "selftest ok" mean
// no sanitizer report and finite results; tests/test_oracle_sanitized.py runs it.
#include <cmath>
#include <cstdio>
#include <vector>

extern "C" {
typedef struct {
  int n0, log0;
  double lo0, hi0;
  int n1, log1;
  double lo1, hi1;
  const float *data;
} orc_table;
typedef struct {
  int family, d;
  int n[4];
  double x_extent, x0_extent;
  int x0_summands;
  double T, E;
  int mats_min, mats_vacuum, mats_add;
  double qmin[3], qmax[3];
} orc_family_desc;
int orc_gauss_legendre(int n, double *x, double *w);
int orc_golub_welsch(int n, const double *a, const double *b, double mu0, double *x, double *w);
int orc_matsubara(double T, double E, int step, int min_size, int max_size, int vacuum, int prec, double *x,
                  double *w, int cap, double *T_used);
int orc_family(const orc_family_desc *descs, int integrand, int n_int, const double *k, const double *args,
               const orc_table *tables, int n_tables, double *out, int threads);
int orc_w1(int n_int, const int *nq, const int *nc, const double *qmax, const double *p, const orc_table *z,
           double *out, int threads);
int orc_w2(int n_int, int M, int nq, int nc, double qmax, const double *p, const double *Tv, const double *Om,
           const orc_table *z, double *out, int threads);
int orc_table_eval(const orc_table *t, int n, const double *x0, const double *x1, double *out);
int orc_regulator(int n, const double *q2, double *rb, double *rbdot);
}

static int fails = 0;
static void check(bool ok, const char *what)
{
  if (!ok) {
    std::printf("FAIL %s\n", what);
    ++fails;
  }
}

int main()
{
  // Gauss-Legendre and Golub-Welsch
  for (int n : {1, 2, 7, 64, 257}) {
    std::vector<double> x(n), w(n);
    check(orc_gauss_legendre(n, x.data(), w.data()) == 0, "gauss_legendre");
    double s = 0;
    for (double v : w) s += v;
    check(std::fabs(s - 1.0) < 1e-13, "GL weight sum");
    std::vector<double> a(n, 0.0), b(n, 0.0);
    for (int i = 1; i < n; ++i) b[i] = i / std::sqrt(4.0 * i * i - 1.0);
    std::vector<double> xg(n), wg(n);
    check(orc_golub_welsch(n, a.data(), b.data(), 2.0, xg.data(), wg.data()) == 0, "golub_welsch");
  }
  // Matsubara rules
  for (double T : {0.0, 0.01, 0.3, 2.0}) {
    std::vector<double> x(256), w(256);
    double Tu = -1;
    const int n = orc_matsubara(T, 1.0, 2, 32, 128, 48, 0, x.data(), w.data(), 256, &Tu);
    check(n > 0 && n <= 256 && Tu >= 0, "matsubara");
  }
  // tables
  std::vector<float> z1(128), z2(64 * 128);
  for (int i = 0; i < 128; ++i) z1[i] = 1.0f + 0.3f * std::sin(0.1f * i);
  for (int i = 0; i < 64 * 128; ++i) z2[i] = 1.0f + 0.2f * std::cos(0.01f * i);
  orc_table t1{128, 1, 1e-4, 100.0, 0, 0, 0, 1, z1.data()};
  orc_table t2{64, 0, 0.0, 64.0, 128, 1, 1e-3, 20.0, z2.data()};
  {
    std::vector<double> x0{1e-6, 1e-3, 0.5, 50.0, 1e5}, x1{1e-4, 0.01, 1.0, 19.0, 30.0}, out(5), out2(5);
    check(orc_table_eval(&t1, 5, x0.data(), nullptr, out.data()) == 0, "table_eval 1D");
    check(orc_table_eval(&t2, 5, x0.data(), x1.data(), out.data()) == 0, "table_eval 2D");
    check(orc_regulator(5, x0.data(), out.data(), out2.data()) == 0, "regulator");
  }
  // every family with the polynomial integrand, small orders
  const int fams[][7] = {
      // family, d, n0, n1, n2, n3, x0_summands
      {1, 4, 16, 0, 0, 0, 0},   {2, 4, 16, 6, 0, 0, 0},  {3, 3, 16, 6, 8, 0, 0},  {4, 4, 16, 6, 6, 0, 0},
      {5, 4, 16, 8, 6, 4, 0},   {6, 1, 8, 0, 0, 0, 0},   {7, 2, 8, 6, 0, 0, 0},   {8, 3, 8, 6, 4, 0, 0},
      {9, 3, 16, 6, 6, 0, 0},   {10, 3, 16, 6, 6, 0, 0}, {11, 4, 16, 6, 8, 6, 0}, {12, 4, 16, 6, 8, 6, 0},
      {13, 4, 16, 0, 0, 0, 0},  {14, 4, 16, 6, 0, 0, 0}, {15, 4, 16, 8, 8, 0, 0}, {16, 4, 16, 16, 0, 0, 8},
      {17, 4, 16, 6, 16, 0, 8}, {18, 4, 8, 6, 6, 12, 4}, {19, 4, 1, 0, 0, 0, 0}};
  for (const auto &f : fams) {
    orc_family_desc d{};
    d.family = f[0];
    d.d = f[1];
    for (int i = 0; i < 4; ++i) d.n[i] = f[2 + i];
    d.x_extent = 1.5;
    d.x0_extent = 1.3;
    d.x0_summands = f[6];
    d.T = (f[0] >= 13 && f[0] <= 18) ? 0.2 : 0.0;
    d.mats_min = 32;
    d.mats_vacuum = 48;
    for (int i = 0; i < 3; ++i) {
      d.qmin[i] = -1.0;
      d.qmax[i] = 1.0;
    }
    if (f[0] >= 16 && f[0] <= 18) d.x0_extent = 8 * 10 * 2 * M_PI * 0.2 * 1.5 + 1000.0;
    double args[24] = {0.1, 1.0, 0.5, 0.0, 0.0, 0.0, 0.0, 1.0, 0.2, 0, 0, 1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0, 0, 0, 0, 0};
    const double k = 0.7;
    double out = 0;
    check(orc_family(&d, 0, 1, &k, args, nullptr, 0, &out, 1) == 0 && std::isfinite(out), "family");
  }
  // benchmark loops
  {
    int nq = 16, nc = 8;
    double qmax = 2.0, p = 0.3, out = 0, T = 0.2, Om = 0.0;
    check(orc_w1(1, &nq, &nc, &qmax, &p, &t1, &out, 1) == 0 && std::isfinite(out), "w1");
    check(orc_w2(1, 8, 16, 8, 2.0, &p, &T, &Om, &t2, &out, 1) == 0 && std::isfinite(out), "w2");
  }
  if (fails) return 1;
  std::printf("selftest ok\n");
  return 0;
}
