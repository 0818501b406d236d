// Runs the reference's sequential CPU m-Cubes (cuda/mcubes/mcubesSeq.hh,
// seq_mcubes_integrate) on a few integrands and prints one JSON line per run.
// TEST INFRASTRUCTURE, host code only, built from the reference sources by
// oracle/ref/build_ref.sh into oracle/_ref/mcubes_seq_run; its output becomes
// tests/golden/mcubes_ref.json (tests/golden/make_mcubes_ref_golden.py).
//
// Usage: mcubes_seq_run <case> <ncall> <itmx> <seed>
//   case 0: 6-D Gaussian sigma 0.01 normalised to 1 (the m-Cubes configuration)
//   case 1: 3-D corner peak (1 + 3x + 2y + z)^-4 (cuda/mcubes/demos/seqGenz3_3D.cpp)
//   case 2: 4-D C0 exp(-sum a_i |x_i - u_i|), a = (2, 3, 1, 2), u = (.5, .2, .7, .4)
// The reference seeds its ran2 generator from the global idum (seqCodesDefs.hh:15-16);
// <seed> sets it (idum = -seed) before the run.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "cuda/mcubes/mcubesSeq.hh"

struct Gauss6 {
  double operator()(double a, double b, double c, double d, double e, double f) const {
    const double s = 0.01, k = 1.0 / (s * std::sqrt(2.0 * M_PI));
    const double x[6] = {a, b, c, d, e, f};
    double v = 1.0;
    for (double xi : x) v *= k * std::exp(-(xi - 0.5) * (xi - 0.5) / (2 * s * s));
    return v;
  }
};

struct Corner3 {
  double operator()(double x, double y, double z) const { return std::pow(1 + 3 * x + 2 * y + z, -4); }
};

struct C0_4 {
  double operator()(double a, double b, double c, double d) const {
    return std::exp(-(2 * std::fabs(a - .5) + 3 * std::fabs(b - .2) + 1 * std::fabs(c - .7) + 2 * std::fabs(d - .4)));
  }
};

template <class F, int N>
void run(const char* name, unsigned long ncall, int itmx) {
  quad::Volume<double, N> vol;
  auto r = seq_mcubes_integrate<F, N>(F{}, N, 1e-9, 1e-20, ncall, &vol, itmx);
  std::printf("{\"case\": \"%s\", \"estimate\": %.17g, \"errorest\": %.17g, \"chi_sq\": %.17g}\n", name, r.estimate,
              r.errorest, r.chi_sq);
}

int main(int argc, char** argv) {
  if (argc != 5) return 2;
  const int c = std::atoi(argv[1]);
  const unsigned long ncall = std::strtoul(argv[2], nullptr, 10);
  const int itmx = std::atoi(argv[3]);
  idum = -std::atol(argv[4]);
  if (c == 0) run<Gauss6, 6>("gauss6_sigma0.01", ncall, itmx);
  if (c == 1) run<Corner3, 3>("corner3", ncall, itmx);
  if (c == 2) run<C0_4, 4>("c0_4", ncall, itmx);
  return 0;
}
