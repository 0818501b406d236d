// Checks the C++ layer (include/pagani_gb300.cuh) with user functors against
// the library's own integrand families: a functor that spells out a family's
// operations must give bit-identical results through Workspace::integrate and
// through pg_integrate, on the unit cube and on a general box, in both kernel
// classes (ndim <= 8 and > 8), and per region through evaluate_regions; m-Cubes
// through cuda_mcubes::integrate and quad::mcubes to 1e-12.  Also
// runs a stateful functor (device table, copied through managed memory) and
// x*y on the unit square (test/cuda/pagani/do_integration_from_c.cu:21-37).
// Prints one line per case and exits non-zero on any mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pagani_gb300.cuh"

// The library's product-form families multiply their per-axis factors in two
// halves: f = L * R, L over axes 0..m-1 and R over m..d-1 (m = d / 2), each in
// axis order.
template <int ND, class H>
__device__ double split_product(const double* x, const H& h) {
  constexpr int m = ND / 2;
  double L = h(0, x[0]), R = h(m, x[m]);
  for (int k = 1; k < m; ++k) L = __dmul_rn(L, h(k, x[k]));
  for (int k = m + 1; k < ND; ++k) R = __dmul_rn(R, h(k, x[k]));
  return __dmul_rn(L, R);
}

// exp(-(a_k (x_k - u_k))^2) per axis (the GAUSSIAN family, c = 0).
template <int ND>
struct GaussProduct {
  double a[ND], u[ND];
  template <class... X>
  __device__ double operator()(X... xs) const {
    const double x[ND] = {static_cast<double>(xs)...};
    return split_product<ND>(x, [this](int k, double xk) {
      const double q = __dmul_rn(a[k], __dsub_rn(xk, u[k]));
      return exp(-__dmul_rn(q, q));
    });
  }
};

// 1 / (a_k^-2 + (x_k - u_k)^2) per axis (the PRODUCT_PEAK family).
template <int ND>
struct PeakProduct {
  double ia2[ND], u[ND];
  template <class... X>
  __device__ double operator()(X... xs) const {
    const double x[ND] = {static_cast<double>(xs)...};
    return split_product<ND>(x, [this](int k, double xk) {
      const double t = __dsub_rn(xk, u[k]);
      return __ddiv_rn(1.0, __fma_rn(t, t, ia2[k]));
    });
  }
};

// exp(-(a (x_k - u))^2) * c per axis (the GAUSSIAN family with c != 0), 3-D,
// non-template operator() so quad::mcubes can take its arity.
struct Gauss3c {
  double a, u, c;
  __device__ double operator()(double x, double y, double z) const {
    const double xs[3] = {x, y, z};
    return split_product<3>(xs, [this](int, double xk) {
      const double q = __dmul_rn(a, __dsub_rn(xk, u));
      return __dmul_rn(exp(-__dmul_rn(q, q)), c);
    });
  }
};

struct XY {
  __device__ double operator()(double x, double y) { return x * y; }  // non-const, as many reference functors
};

struct NanFn {
  __device__ double operator()(double, double, double) const { return nan(""); }
};

// Stateful functor: a piecewise-constant table on axis 0 times (y + z), the
// table in device memory owned by the functor (deep copy in its copy
// constructor, so the functor is not trivially copyable).
struct Tabulated {
  double* table = nullptr;
  int n = 0;
  Tabulated(int cells) : n(cells) {
    cudaMallocManaged(&table, sizeof(double) * n);
    for (int i = 0; i < n; ++i) table[i] = 1.0 + 0.5 * i;
  }
  Tabulated(const Tabulated& o) : n(o.n) {
    cudaMallocManaged(&table, sizeof(double) * n);
    cudaDeviceSynchronize();
    std::memcpy(table, o.table, sizeof(double) * n);
  }
  ~Tabulated() {
    if (table) cudaFree(table);
  }
  __device__ double operator()(double x, double y, double z) const {
    int i = (int)(x * n);
    i = i < 0 ? 0 : (i >= n ? n - 1 : i);
    return __dmul_rn(table[i], __dadd_rn(y, z));
  }
};

static int failures = 0;

// m-Cubes accumulates its per-bin sums with floating-point atomics (as the
// reference does, vegasT.cuh:306), so the adapted grid, and with it the
// estimate, varies in the last bits from run to run: compare at 1e-12.
static bool close(double a, double b, double rel) { return std::fabs(a - b) <= rel * std::fabs(b); }

static void report_mc(const char* name, const pagani::integration_result& u, const pg_result& f) {
  const bool ok = close(u.estimate, f.estimate, 1e-12) && close(u.errorest, f.errorest, 1e-9) &&
                  close(u.chi_sq, f.chi_sq, 1e-6) && u.iters == f.iters && u.status == f.status;
  std::printf("%s %s functor %.17g %.17g %.6g %zu %d family %.17g %.17g %.6g %llu %d\n", ok ? "PASS" : "FAIL", name,
              u.estimate, u.errorest, u.chi_sq, u.iters, u.status, f.estimate, f.errorest, f.chi_sq,
              (unsigned long long)f.iters, f.status);
  if (!ok) ++failures;
}

static bool same_bits(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }

static void report(const char* name, const pagani::integration_result& u, const pg_result& f) {
  const bool ok = (same_bits(u.estimate, f.estimate) || (std::isnan(u.estimate) && std::isnan(f.estimate))) &&
                  (same_bits(u.errorest, f.errorest) || (std::isnan(u.errorest) && std::isnan(f.errorest))) &&
                  u.nregions == f.nregions && u.iters == f.iters && u.status == f.status && u.neval == f.neval &&
                  u.nFinishedRegions == f.nfinished;
  std::printf("%s %s functor %.17g %.17g %zu %zu %d family %.17g %.17g %llu %llu %d\n", ok ? "PASS" : "FAIL", name,
              u.estimate, u.errorest, u.nregions, u.iters, u.status, f.estimate, f.errorest,
              (unsigned long long)f.nregions, (unsigned long long)f.iters, f.status);
  if (!ok) ++failures;
}

template <int ND>
static void gauss_case(pg_context* ctx, const char* name, double epsrel, bool box, unsigned seed) {
  GaussProduct<ND> g;
  pg_integrand fam;
  std::memset(&fam, 0, sizeof fam);
  fam.family = PG_FAMILY_GAUSSIAN;
  fam.ndim = ND;
  uint64_t s = seed;
  auto unif = [&s]() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  };
  double asum = 0;
  for (int k = 0; k < ND; ++k) {
    g.a[k] = unif();
    asum += g.a[k];
  }
  for (int k = 0; k < ND; ++k) {
    g.a[k] = g.a[k] * (12.0 / asum);
    g.u[k] = unif();
    fam.a[k] = g.a[k];
    fam.u[k] = g.u[k];
  }
  double lows[ND], highs[ND];
  for (int k = 0; k < ND; ++k) {
    lows[k] = box ? -0.25 * (k % 3) : 0.0;
    highs[k] = box ? 1.0 + 0.5 * (k % 2) : 1.0;
  }
  pagani::Volume<double, ND> vol(lows, highs);
  Workspace<double, ND> ws;
  const auto u = ws.integrate(g, epsrel, 0.0, vol);
  pg_result f;
  pg_integrate(ctx, &fam, epsrel, 0.0, lows, highs, nullptr, &f);
  report(name, u, f);
}

int main() {
  pg_context* ctx = nullptr;
  if (pg_context_create(0, &ctx) != PG_OK) {
    std::printf("FAIL no context\n");
    return 2;
  }
  // Gaussian, unit cube and box, both kernel classes.
  gauss_case<3>(ctx, "gauss3_unit", 1e-6, false, 11);
  gauss_case<5>(ctx, "gauss5_box", 1e-5, true, 12);
  gauss_case<8>(ctx, "gauss8_unit", 1e-4, false, 13);
  gauss_case<10>(ctx, "gauss10_unit", 1e-3, false, 14);

  // Product peak on a box, relerr classification off.
  {
    constexpr int ND = 6;
    PeakProduct<ND> p;
    pg_integrand fam;
    std::memset(&fam, 0, sizeof fam);
    fam.family = PG_FAMILY_PRODUCT_PEAK;
    fam.ndim = ND;
    double lows[ND], highs[ND];
    for (int k = 0; k < ND; ++k) {
      fam.a[k] = 1.5 + 0.25 * k;
      fam.u[k] = 0.3 + 0.05 * k;
      p.ia2[k] = 1.0 / (fam.a[k] * fam.a[k]);
      p.u[k] = fam.u[k];
      lows[k] = 0.1 * k;
      highs[k] = 1.0 + 0.1 * k;
    }
    Workspace<double, ND> ws;
    const auto u = ws.integrate(p, 1e-4, 0.0, quad::Volume<double, ND>(lows, highs), false);
    pg_options opt;
    pg_options_default(&opt);
    opt.relerr_classification = 0;
    pg_result f;
    pg_integrate(ctx, &fam, 1e-4, 0.0, lows, highs, &opt, &f);
    report("peak6_box_norelerr", u, f);
  }

  // x*y on the unit square at 1e-6: the C precedent's integrand.
  {
    Workspace<double, 2> ws;
    const auto u = ws.integrate(XY{}, 1e-6, 0.0, quad::Volume<double, 2>());
    pg_integrand fam;
    std::memset(&fam, 0, sizeof fam);
    fam.family = PG_FAMILY_PRODUCT;
    fam.ndim = 2;
    pg_result f;
    pg_integrate(ctx, &fam, 1e-6, 0.0, nullptr, nullptr, nullptr, &f);
    report("xy_unit", u, f);
    const bool ok = u.status == 0 && std::fabs(u.estimate - 0.25) <= 1e-6 * 0.25;
    std::printf("%s xy_value %.17g\n", ok ? "PASS" : "FAIL", u.estimate);
    if (!ok) ++failures;
  }

  // NaN integrand: same outcome as the NAN_VALUE family (test/cuda/pagani/NanIntegral.cu:25-37).
  {
    Workspace<double, 3> ws;
    const auto u = ws.integrate(NanFn{}, 1e-3, 0.0, quad::Volume<double, 3>());
    pg_integrand fam;
    std::memset(&fam, 0, sizeof fam);
    fam.family = PG_FAMILY_NAN_VALUE;
    fam.ndim = 3;
    pg_result f;
    pg_integrate(ctx, &fam, 1e-3, 0.0, nullptr, nullptr, nullptr, &f);
    report("nan3", u, f);
  }

  // Stateful functor through managed memory: integral of table(x) * (y + z)
  // over the unit cube = mean(table) * 1.
  {
    Tabulated t(16);
    double mean = 0;
    for (int i = 0; i < t.n; ++i) mean += t.table[i];
    mean /= t.n;
    Workspace<double, 3> ws;
    const auto u = ws.integrate(t, 1e-3, 0.0, quad::Volume<double, 3>());
    const bool ok = std::fabs(u.estimate - mean) <= 1e-3 * mean;
    std::printf("%s tabulated3 %.17g exact %.17g status %d nregions %zu\n", ok ? "PASS" : "FAIL", u.estimate, mean,
                u.status, u.nregions);
    if (!ok) ++failures;
  }

  // Per-region evaluation: functor vs family on the same regions.
  {
    constexpr int ND = 5;
    GaussProduct<ND> g;
    pg_integrand fam;
    std::memset(&fam, 0, sizeof fam);
    fam.family = PG_FAMILY_GAUSSIAN;
    fam.ndim = ND;
    for (int k = 0; k < ND; ++k) {
      g.a[k] = fam.a[k] = 2.0 + 0.5 * k;
      g.u[k] = fam.u[k] = 0.2 + 0.1 * k;
    }
    const size_t n = 4096;
    std::vector<double> left(ND * n), len(ND * n);
    for (size_t i = 0; i < n; ++i)
      for (int k = 0; k < ND; ++k) {
        const int depth = (int)((i * 7 + k * 3) % 6);
        const double h = std::ldexp(1.0, -depth);
        const size_t cells = (size_t)1 << depth;
        len[k * n + i] = h;
        left[k * n + i] = (double)((i * 13 + k * 5) % cells) * h;
      }
    std::vector<double> e1(n), r1(n), e2(n), r2(n);
    std::vector<int> b1(n), b2(n);
    Workspace<double, ND> ws;
    ws.evaluate_regions(g, quad::Volume<double, ND>(), n, left.data(), len.data(), e1.data(), r1.data(), b1.data());
    pg_evaluate_regions(ctx, &fam, nullptr, nullptr, n, left.data(), len.data(), e2.data(), r2.data(),
                        reinterpret_cast<int32_t*>(b2.data()), 0);
    size_t bad = 0;
    for (size_t i = 0; i < n; ++i)
      if (!same_bits(e1[i], e2[i]) || !same_bits(r1[i], r2[i]) || b1[i] != b2[i]) ++bad;
    std::printf("%s regions5 %zu of %zu differ\n", bad ? "FAIL" : "PASS", bad, n);
    if (bad) ++failures;
  }

  // Sub_regions overload (Workspace.cuh:148-158): a 5 x 5 first list, and
  // predict_split with its iteration-15 snapshot (Workspace.cuh:415-441).
  {
    PeakProduct<2> p;
    pg_integrand fam;
    std::memset(&fam, 0, sizeof fam);
    fam.family = PG_FAMILY_PRODUCT_PEAK;
    fam.ndim = 2;
    for (int k = 0; k < 2; ++k) {
      fam.a[k] = 30.0;
      fam.u[k] = k ? 0.61 : 0.37;
      p.ia2[k] = 1.0 / (fam.a[k] * fam.a[k]);
      p.u[k] = fam.u[k];
    }
    Workspace<double, 2> ws;
    Sub_regions<double, 2> five(5);
    const auto u = ws.integrate(p, five, 1e-6, 0.0, quad::Volume<double, 2>());
    five.refresh_host_device();
    pg_result f;
    pg_integrate_regions(ctx, &fam, five.LeftCoord, five.Length, five.size, 1e-6, 0.0, nullptr, nullptr, nullptr, &f);
    report("subregions5x5_peak2", u, f);

    Sub_regions<double, 2> four(4);
    const auto up = ws.integrate<PeakProduct<2>, true>(p, four, 1e-13, 0.0, quad::Volume<double, 2>());
    pg_options opt;
    pg_options_default(&opt);
    opt.predict_split = 1;
    pg_integrate(ctx, &fam, 1e-13, 0.0, nullptr, nullptr, &opt, &f);
    report("predict_split_peak2", up, f);
    int32_t sd = 0;
    uint64_t sn = 0;
    pg_last_snapshot(ctx, &sd, &sn, nullptr, nullptr, 0);
    std::vector<double> sl(sn * 2), sL(sn * 2), dl(four.snapshot_size * 2), dL(four.snapshot_size * 2);
    pg_last_snapshot(ctx, &sd, &sn, sl.data(), sL.data(), sn);
    cudaMemcpy(dl.data(), four.snapshot_dLeftCoord, dl.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(dL.data(), four.snapshot_dLength, dL.size() * 8, cudaMemcpyDeviceToHost);
    const bool ok = sn == (uint64_t)16 * 32768 && four.snapshot_size == sn && dl == sl && dL == sL;
    std::printf("%s predict_split_snapshot %llu %zu\n", ok ? "PASS" : "FAIL", (unsigned long long)sn,
                four.snapshot_size);
    if (!ok) ++failures;
  }

  // m-Cubes: functor vs family, same seed, same geometry (cuda/mcubes/vegasT.cuh:999-1030).
  {
    const double sigma = 0.1, c = 1.0 / (sigma * std::sqrt(2.0 * 3.14159265358979323846));
    Gauss3c g{1.0 / (sigma * std::sqrt(2.0)), 0.5, c};
    pg_integrand fam;
    std::memset(&fam, 0, sizeof fam);
    fam.family = PG_FAMILY_GAUSSIAN;
    fam.ndim = 3;
    fam.c = c;
    for (int k = 0; k < 3; ++k) {
      fam.a[k] = g.a;
      fam.u[k] = g.u;
    }
    quad::Volume<double, 3> vol;
    const auto u = cuda_mcubes::integrate<Gauss3c, 3>(g, 1e-3, 0.0, 1.0e6, &vol, 15, 10, 5);
    pg_mcubes_options opt;
    pg_mcubes_options_default(&opt);
    opt.ncall = 1.0e6;
    opt.titer = 15;
    opt.itmax = 10;
    opt.skip = 5;
    pg_result f;
    pg_mcubes_integrate(ctx, &fam, 1e-3, 0.0, nullptr, nullptr, &opt, &f);
    report_mc("mcubes_gauss3", u, f);
    // quad::mcubes (cuda/mcubes/mcubes.cuh:9-41): arity from operator(), epsabs before epsrel.
    quad::mcubes qm;
    const auto q = qm.integrate(g, 0.0, 1e-3, &vol);
    opt.ncall = (double)qm.maxcalls;
    opt.titer = qm.total_iters;
    opt.itmax = qm.adjust_iters;
    opt.skip = qm.skip_iters;
    pg_mcubes_integrate(ctx, &fam, 1e-3, 0.0, nullptr, nullptr, &opt, &f);
    report_mc("quad_mcubes_gauss3", q, f);
    const double exact = std::pow(std::erf(0.5 / (sigma * std::sqrt(2.0))), 3);
    const bool ok = std::fabs(u.estimate - exact) <= 5 * u.errorest;
    std::printf("%s mcubes_value %.17g exact %.17g err %.3g\n", ok ? "PASS" : "FAIL", u.estimate, exact, u.errorest);
    if (!ok) ++failures;
  }

  pg_context_destroy(ctx);
  std::printf("%s %d failures\n", failures ? "FAIL" : "DONE", failures);
  return failures ? 1 : 0;
}
