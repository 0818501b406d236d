// Dumps the reference's own degree-9 rule tables (host side of
// cuda/pagani/quad/GPUquad/Rule.cuh) so the oracle and the GB300 library can be
// pinned against them bit for bit.  TEST INFRASTRUCTURE: compiled from the
// reference sources where they lie by oracle/ref/build_ref.sh, output only into
// oracle/_ref/.  Runs without a GPU: the reference's device copies at the end of
// Rule::Init fail and are reported, the host tables are complete before that.
//
// Output: one line per table, "<ndim> <name> <hex-float or int> ...".
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "cuda/pagani/quad/GPUquad/Rule.cuh"

// Rule's tables are private members.  Explicit instantiation may name private
// members, which gives this dumper read access without touching the reference.
template <typename Tag, typename Tag::type M>
struct Expose {
  friend typename Tag::type get(Tag) { return M; }
};
#define EXPOSE(NAME, TYPE)                                        \
  struct NAME {                                                   \
    typedef TYPE quad::Rule<double>::*type;                       \
    friend type get(NAME);                                        \
  };                                                              \
  template struct Expose<NAME, &quad::Rule<double>::NAME>;
EXPOSE(CPURuleWt, double*)
EXPOSE(CPUScale, double*)
EXPOSE(CPUNorm, double*)
EXPOSE(cpuG, double*)
EXPOSE(cpuGenPermGIndex, int*)
EXPOSE(cpuGenPermVarStart, int*)
EXPOSE(genPtr, int*)
#define M(obj, NAME) ((obj).*get(NAME()))

int main(int argc, char** argv) {
  const int dmax = argc > 1 ? std::atoi(argv[1]) : 10;
  // Silence the reference's device-copy diagnostics (no GPU here).
  std::FILE* devnull = std::fopen("/dev/null", "w");
  for (int d = 2; d <= dmax; ++d) {
    const int feval = 1 + 2 * d + 2 * d + 2 * d + 2 * d + 2 * d * (d - 1) + 4 * d * (d - 1) +
                      4 * d * (d - 1) * (d - 2) / 3 + (1 << d);
    quad::Rule<double> rule;
    Structures<double> cm;
    std::streambuf* saved = std::cout.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());
    rule.Init(d, feval, 0, 0, &cm);
    std::cout.rdbuf(saved);
    std::printf("%d feval %d\n", d, feval);
    std::printf("%d w", d);
    for (int i = 0; i < 45; ++i) std::printf(" %a", M(rule, CPURuleWt)[i]);
    std::printf("\n%d scale", d);
    for (int s = 0; s < 9; ++s)
      for (int r = 0; r < 5; ++r) std::printf(" %a", (r >= 1 && r <= 3) ? M(rule, CPUScale)[s * 5 + r] : 0.0);
    std::printf("\n%d norm", d);
    for (int s = 0; s < 9; ++s)
      for (int r = 0; r < 5; ++r) std::printf(" %a", (r >= 1 && r <= 3) ? M(rule, CPUNorm)[s * 5 + r] : 0.0);
    std::printf("\n%d gindex", d);
    for (int p = 0; p < feval; ++p) std::printf(" %d", M(rule, cpuGenPermGIndex)[p]);
    // Generator coordinates exactly as ActualCompute (Phases.cuh:157-189) builds them.
    std::printf("\n%d gen", d);
    std::vector<double> g(d);
    for (int p = 0; p < feval; ++p) {
      std::fill(g.begin(), g.end(), 0.0);
      const int start = M(rule, cpuGenPermVarStart)[p];
      const int cnt = M(rule, cpuGenPermVarStart)[p + 1] - start;
      const int gi = M(rule, cpuGenPermGIndex)[p];
      for (int k = 0; k < cnt; ++k) {
        const int pos = M(rule, genPtr)[start + k];
        const int ap = std::abs(pos);
        g[ap - 1] = (pos == ap) ? M(rule, cpuG)[gi * d + k] : -M(rule, cpuG)[gi * d + k];
      }
      for (int k = 0; k < d; ++k) std::printf(" %a", g[k]);
    }
    std::printf("\n");
  }
  std::fclose(devnull);
  return 0;
}
