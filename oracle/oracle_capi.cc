// oracle_capi.cc -- TEST INFRASTRUCTURE ONLY (see oracle.hh).
//
// extern "C" surface of the FP64 CPU oracle, loaded with ctypes by tests/ and by bench.py's
// CPU-baseline leg.  OpenMP parallelises over integrals; within one integral the sum is a
// sequential pairwise FP64 sum (deterministic for any thread count).
#include "integrands.hh"

#include <cstring>
#include <exception>
#include <omp.h>

using namespace oracle;

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

int orc_version(void) { return 1; }

int orc_gauss_legendre(int n, double *x, double *w)
{
  try {
    std::vector<double> xs, ws;
    gauss_legendre01(n, xs, ws);
    std::memcpy(x, xs.data(), sizeof(double) * n);
    std::memcpy(w, ws.data(), sizeof(double) * n);
    return 0;
  } catch (...) {
    return -1;
  }
}

int orc_golub_welsch(int n, const double *a, const double *b, double mu0, double *x, double *w)
{
  try {
    std::vector<long double> av(a, a + n), bv(b, b + n), xs, ws;
    golub_welsch(av, bv, (long double)mu0, xs, ws);
    for (int i = 0; i < n; ++i) {
      x[i] = (double)xs[i];
      w[i] = (double)ws[i];
    }
    return 0;
  } catch (...) {
    return -1;
  }
}

// returns the rule size (<= cap) or a negative error; *T_used = 0 for the vacuum rule
int orc_matsubara(double T, double E, int step, int min_size, int max_size, int vacuum, int prec, double *x,
                  double *w, int cap, double *T_used)
{
  try {
    MatsubaraRule r = matsubara_rule(T, E, step, min_size, max_size, vacuum, prec);
    if ((int)r.x.size() > cap) return -2;
    std::memcpy(x, r.x.data(), sizeof(double) * r.x.size());
    std::memcpy(w, r.w.data(), sizeof(double) * r.w.size());
    if (T_used) *T_used = r.T;
    return (int)r.x.size();
  } catch (...) {
    return -1;
  }
}

static Table to_table(const orc_table &t)
{
  Table r;
  r.a0 = Axis{t.n0, t.log0, t.lo0, t.hi0};
  r.a1 = Axis{t.n1, t.log1, t.lo1, t.hi1};
  r.data = t.data;
  return r;
}

static Tables to_tables(const orc_table *tables, int n_tables)
{
  Tables T;
  for (int i = 0; i < n_tables && i < 4; ++i) T.t[i] = to_table(tables[i]);
  return T;
}

static FamilyDesc to_desc(const orc_family_desc &d)
{
  FamilyDesc f;
  f.family = d.family;
  f.d = d.d;
  for (int i = 0; i < 4; ++i) f.n[i] = d.n[i];
  f.x_extent = d.x_extent;
  f.x0_extent = d.x0_extent;
  f.x0_summands = d.x0_summands;
  f.T = d.T;
  f.E = d.E;
  f.mats_min = d.mats_min;
  f.mats_vacuum = d.mats_vacuum;
  f.mats_add = d.mats_add;
  for (int i = 0; i < 3; ++i) {
    f.qmin[i] = d.qmin[i];
    f.qmax[i] = d.qmax[i];
  }
  return f;
}

// One integral per (desc[i], k[i], args[i*24 ...]); result = constant args[i*24] + quadrature.
int orc_family(const orc_family_desc *descs, int integrand, int n_int, const double *k, const double *args,
               const orc_table *tables, int n_tables, double *out, int threads)
{
  const Tables T = to_tables(tables, n_tables);
  int err = 0;
  if (threads > 0) omp_set_num_threads(threads);
  // warm the rule cache serially (it is mutex-guarded, this only avoids contention)
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int i = 0; i < n_int; ++i) {
    try {
      const FamilyDesc f = to_desc(descs[i]);
      const double *a = args + (size_t)i * kArgs;
      out[i] = integrate(f, k[i], a[0],
                         [&](const Point &P) { return eval_kernel(integrand, f.family, T, P, a); });
    } catch (...) {
      err |= 1;
    }
  }
  return err ? -1 : 0;
}

int orc_w1(int n_int, const int *nq, const int *nc, const double *qmax, const double *p, const orc_table *z,
           double *out, int threads)
{
  const Tables T = to_tables(z, 1);
  int err = 0;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int i = 0; i < n_int; ++i) {
    try {
      out[i] = w1(T, nq[i], nc[i], qmax[i], p[i]);
    } catch (...) {
      err |= 1;
    }
  }
  return err ? -1 : 0;
}

int orc_w2(int n_int, int M, int nq, int nc, double qmax, const double *p, const double *Tv, const double *Om,
           const orc_table *z, double *out, int threads)
{
  const Tables T = to_tables(z, 1);
  int err = 0;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : err)
  for (int i = 0; i < n_int; ++i) {
    try {
      out[i] = w2(T, M, nq, nc, qmax, p[i], Tv[i], Om ? Om[i] : 0.0);
    } catch (...) {
      err |= 1;
    }
  }
  return err ? -1 : 0;
}

// Table evaluation (1D if x1 == nullptr) -- used by the interpolation known-answer tests.
int orc_table_eval(const orc_table *t, int n, const double *x0, const double *x1, double *out)
{
  const Table T = to_table(*t);
  for (int i = 0; i < n; ++i) out[i] = x1 ? T(x0[i], x1[i]) : T(x0[i]);
  return 0;
}

int orc_regulator(int n, const double *q2, double *rb, double *rbdot)
{
  for (int i = 0; i < n; ++i) {
    rb[i] = reg_RB(1.0, q2[i]);
    rbdot[i] = reg_RBdot(1.0, q2[i]);
  }
  return 0;
}

int orc_max_threads(void) { return omp_get_max_threads(); }
}
