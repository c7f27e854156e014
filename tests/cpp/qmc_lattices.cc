// qmc_lattices.cc -- host-side lattice construction of the QMC integrators (gbint/qmc.hh):
// prints the lattice-size ladder, next_n at a few preferred sizes and the chosen Korobov
// generating vectors with their P_2 figure of merit; tests/test_qmc_lattices.py checks them.
#include <cstdio>

#include "gbint/qmc.hh"

int main()
{
  using namespace gbint::qmc;
  const auto &s = sizes();
  std::printf("SIZES %zu", s.size());
  for (size_t i = 0; i < 12 && i < s.size(); ++i) std::printf(" %llu", (unsigned long long)s[i]);
  std::printf(" LAST %llu\n", (unsigned long long)s.back());
  for (unsigned long long p : {1ull, 512ull, 1021ull, 1022ull, 100000ull, 5000000000ull})
    std::printf("NEXT %llu %llu\n", p, (unsigned long long)next_n(p));
  for (int dim : {1, 2, 4})
    for (unsigned long long n : {1021ull, 8191ull, 65537ull}) {
      const unsigned long long nn = next_n(n);
      const Lattice &L = lattice(nn, dim);
      const Lattice &L2 = lattice(nn, dim);  // cached
      const double p2 = dim > 1 ? korobov_p2(nn, L.z[1], dim) : 0.0;
      // a few other multipliers for comparison
      double worst_other = 0;
      for (unsigned long long a : {2ull, 3ull, nn / 2, nn / 3}) worst_other = std::max(worst_other, dim > 1 ? korobov_p2(nn, a, dim) : 0.0);
      std::printf("LAT %d %llu %llu %llu %llu %llu %.6e %.6e %d\n", dim, nn, (unsigned long long)L.z[0], (unsigned long long)L.z[1],
                  (unsigned long long)L.z[2], (unsigned long long)L.z[3], p2, worst_other, &L == &L2 ? 1 : 0);
    }
  return 0;
}
