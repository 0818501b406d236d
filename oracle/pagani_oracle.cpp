// PAGANI CPU oracle -- TEST INFRASTRUCTURE ONLY.
//
// This file is the oracle of the GB300 library: a plain C++ restatement of the
// reference's PAGANI adaptive-cubature iteration.  Only tests/, the smoke check
// and bench.py's CPU-baseline leg may load it.  The product path never calls it.
//
// Every stage cites the reference file:line it restates (paths relative to the
// reference project root).  Floating-point contraction is written out explicitly
// with std::fma at the places where nvcc contracts the reference's expressions;
// the file is compiled with -ffp-contract=off so that nothing else is fused and
// the results are the same on x86-64 and aarch64 hosts.
//
// Global reductions follow the library's deterministic blocked Neumaier order
// (see canon_* below).  The reference uses thrust::reduce, whose order is
// unspecified, so any fixed order is a faithful restatement; using the same
// order as the GPU library makes GPU-vs-oracle comparisons bit-exact for
// integrands that use only IEEE-exact operations.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace orc {

constexpr int kNRules = 5;  // cuda/pagani/quad/quad.h:65
constexpr int kNSets = 9;   // cuda/pagani/quad/GPUquad/Rule.cuh:404-405
constexpr int kMaxDim = 16;

// ---------------------------------------------------------------------------
// Integrand families (same struct layout as pg_integrand in the C ABI).
// ---------------------------------------------------------------------------
enum Family : int32_t {
  FAM_CONSTANT = 0,
  FAM_OSCILLATORY = 1,
  FAM_PRODUCT_PEAK = 2,
  FAM_CORNER_PEAK = 3,
  FAM_GAUSSIAN = 4,
  FAM_C0 = 5,
  FAM_DISCONTINUOUS = 6,
  FAM_PRODUCT = 7,
  FAM_NAN = 8,
  FAM_BOX = 9,
  FAM_FUN6 = 10,
  FAM_GAUSSIAN_SUM = 11,
};

struct Integrand {
  int32_t family;
  int32_t ndim;
  double a[kMaxDim];
  double u[kMaxDim];
  double c;
};

// Parameters derived once on the host.  The GPU library derives the same values
// with the same operations (pg_prepare_integrand in the library).
struct Prepared {
  int family, ndim;
  double a[kMaxDim], u[kMaxDim], ia2[kMaxDim];
  double c, s0;
};

static Prepared prepare(const Integrand& f) {
  Prepared p{};
  p.family = f.family;
  p.ndim = f.ndim;
  for (int i = 0; i < kMaxDim; ++i) {
    p.a[i] = f.a[i];
    p.u[i] = f.u[i];
    p.ia2[i] = 1.0 / (f.a[i] * f.a[i]);
  }
  p.c = f.c;
  p.s0 = 2.0 * 3.14159265358979323846 * f.u[0];
  if (f.family == FAM_FUN6)
    p.c = 12.0 / (7.0 - 6.0 * std::log(2.0) * std::log(2.0) + std::log(64.0));
  if (f.family == FAM_GAUSSIAN_SUM) {  // c^d, d - 1 multiplies in axis order (1 when c is 0)
    p.s0 = 1.0;
    if (f.c != 0.0) {
      p.s0 = f.c;
      for (int k = 1; k < f.ndim; ++k) p.s0 = p.s0 * f.c;
    }
  }
  return p;
}

static inline double ipow(double s, int e) {
  // Binary exponentiation with a fixed multiplication order.
  double r = 1.0, b = s;
  while (e) {
    if (e & 1) r = r * b;
    e >>= 1;
    if (e) b = b * b;
  }
  return r;
}

// Per-axis factor of the product-form families.
static double factor(const Prepared& p, int k, double x) {
  switch (p.family) {
    case FAM_PRODUCT_PEAK: {
      const double t = x - p.u[k];
      return 1.0 / std::fma(t, t, p.ia2[k]);
    }
    case FAM_GAUSSIAN: {
      const double q = p.a[k] * (x - p.u[k]);
      const double v = std::exp(-(q * q));
      return p.c != 0.0 ? v * p.c : v;
    }
    case FAM_C0:
      return std::exp(-(p.a[k] * std::fabs(x - p.u[k])));
    case FAM_DISCONTINUOUS:
      return (x > p.u[k]) ? 0.0 : std::exp(p.a[k] * x);
  }
  return 1.0;
}

static double eval(const Prepared& p, const double* x) {
  const int d = p.ndim;
  switch (p.family) {
    case FAM_CONSTANT:
      return p.c;
    case FAM_OSCILLATORY: {
      double s = p.s0;
      for (int i = 0; i < d; ++i) s = std::fma(p.a[i], x[i], s);
      return std::cos(s);
    }
    case FAM_PRODUCT_PEAK:
    case FAM_GAUSSIAN:
    case FAM_C0:
    case FAM_DISCONTINUOUS: {
      // f = L * R: products of the per-axis factors of axes 0..m-1 and
      // m..d-1 (m = d / 2), each half in axis order.
      const int m = d / 2;
      double L = factor(p, 0, x[0]), R = factor(p, m, x[m]);
      for (int i = 1; i < m; ++i) L = L * factor(p, i, x[i]);
      for (int i = m + 1; i < d; ++i) R = R * factor(p, i, x[i]);
      return L * R;
    }
    case FAM_CORNER_PEAK: {
      double s = 1.0;
      for (int i = 0; i < d; ++i) s = std::fma(p.a[i], x[i], s);
      return 1.0 / ipow(s, d + 1);
    }
    case FAM_PRODUCT: {
      const int m = d / 2;
      double L = x[0], R = x[m];
      for (int i = 1; i < m; ++i) L = L * x[i];
      for (int i = m + 1; i < d; ++i) R = R * x[i];
      return L * R;
    }
    case FAM_NAN:
      return std::numeric_limits<double>::quiet_NaN();
    case FAM_BOX: {
      double s = 0.0;
      for (int i = 0; i < d; ++i) s = std::fma(x[i], x[i], s);
      return std::pow(s, 0.5 * p.c);
    }
    case FAM_GAUSSIAN_SUM: {
      // one exponential of the sum of squares (cuda/mcubes/demos/Gauss9D.cu:8-24)
      double s = 0.0;
      for (int i = 0; i < d; ++i) {
        const double q = p.a[i] * (x[i] - p.u[i]);
        s = std::fma(q, q, s);
      }
      return std::exp(-s) * p.s0;
    }
    case FAM_FUN6: {
      // test/cuda/pagani/accuracy_improves_with_epsrel.cu:267-275
      const double t = (std::pow(x[2], x[4]) * x[3]) * x[4];
      return p.c * ((x[0] * x[1] + t / (1.0 + x[0])) + x[5] * x[5]);
    }
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// Degree-9 cubature rule tables.
// Restates cuda/pagani/quad/GPUquad/Rule.cuh:24-270 (weights, generators,
// null-rule scale/norm) and :409-507 (point enumeration order).  The weight
// polynomials in NDIM are evaluated with the same grouping as the reference so
// that every table entry is the same double.
// ---------------------------------------------------------------------------
struct Rule {
  int ndim = 0, feval = 0;
  double w[kNSets * kNRules];
  double scale[kNSets * kNRules];
  double norm[kNSets * kNRules];
  double G[5];
  std::vector<int> set_of;     // [feval]
  std::vector<double> gen;     // [feval * ndim], point-major
};

int feval_count(int d) {
  // cuda/pagani/quad/quad.h:67-76
  return 1 + 8 * d + 2 * d * (d - 1) + 4 * d * (d - 1) + 4 * d * (d - 1) * (d - 2) / 3 + (1 << d);
}

static void rule9_weights(int ndim, double* w) {
  const double n = (double)ndim;
  // Constants of the degree-9 rule (Rule.cuh:36-147).
  const double c1 = -.002361170967785511788400941242259231309691;
  const double c2 = .1141539002385732526821323741697655347686;
  const double c3 = -.6383392007670238909386026193674701393074;
  const double c4 = .7484998850468520800423030047583803945205;
  const double d1 = -.001432401703339912514196154599769007103671;
  const double d2 = .05747150786448972594860897296200006759892;
  const double d3 = -.1422510457143424323449521620935950679394;
  const double d4 = -.06287502873828697998942424881040490136987;
  const double e1 = .2545911332489590890011611142429070613156;
  const double f1 = -1.207328566678236261002219995185143356737;
  const double f2 = .8956736576416067650809467826488567200939;
  const double g1 = -.3647935698604914666100134551377381205297;
  const double h1 = .003541756451678267682601411863388846964536;
  const double h2 = -.07260936739589367960492815865074633743652;
  const double h3 = .1055749162521899101218622863269817454540;
  const double i1 = .002148602555009868771294231899653510655506;
  const double i2 = -.03226856389295394999786630399875134318006;
  const double i3 = .01063678399023121748083624225818915724455;
  const double j1 = .01468910249614349017540783437728097691502;
  const double k1 = .5113470834646759143109387357149329909126;
  const double k2 = .4597644812080634464633352781605214342691;
  const double l1 = .1823967849302457333050067275688690602649;
  const double m1 = -.04508628929435784075980562738240804429658;
  const double m2 = .2141588352435279340097929526588394300172;
  const double n1 = -.02735154652654564472203690086290223507436;
  const double n2 = .05494106704871123410060080562462135546101;
  const double o1 = .1193759620257077529708962121565290178730;
  const double p1 = .6508951939192025059314756320878023215278;
  const double p2 = .1474493982943446016775696826942585013243;
  const double q1 = .01553241727660705326386197156586357005224;
  const double r1 = .003532809960709087023561817517751309380604;
  const double s1 = .09231719987444221619017126187763868745587;
  const double t1 = .2515001149531479199576969952416196054795;
  const double pow2 = (double)(1 << ndim);

  const double pc = n * (n * (n * c1 + c2) + c3) + c4;  // shared cubic
  const double pd = n * (n * (n * d1 + d2) + d3) - d4;
  const double ph = n * (n * h1 + h2) + h3;
  const double pi = n * (n * i1 + i2) + i3;
  const double pm = n * m1 + m2;
  const double pn = n * n1 + n2;

  double tab[kNSets * kNRules] = {
      // set 0: centre
      pc, pd, n * e1 - pd, ((n * (n * f1 + f2) - 1) + n * (n * (n * c1 + c2) + c3)) + c4, (n * g1 + 1) - pc,
      // set 1
      ph, pi, j1 - pi, ((n * k1 + k2) + n * (n * h1 + h2)) + h3, l1 - ph,
      // set 2
      pm, pn, o1 - pn, n * p1 + p2, -pm,
      // set 3
      .05769338449097348357291272840392627722165, .03499962660214358382244159694487155861542,
      -.05769338449097348357291272840392627722165, -1.386862771927828143599782668709014266770,
      -.05769338449097348357291272840392627722165,
      // set 4
      0, 0, -.2386668732575008878964134721962088068396, 0, 0,
      // set 5
      q1 - n * h1, r1 - n * i1, -(r1 - n * i1), (s1 + q1) - n * h1, -(q1 - n * h1),
      // set 6
      .02254314464717892037990281369120402214829, .01367577326327282236101845043145111753718,
      -.01367577326327282236101845043145111753718, -.3254475969596012529657378160439011607639,
      -.02254314464717892037990281369120402214829,
      // set 7
      .001770878225839133841300705931694423482268, .001074301277504934385647115949826755327753,
      -.001074301277504934385647115949826755327753, .001770878225839133841300705931694423482268,
      -.001770878225839133841300705931694423482268,
      // set 8
      t1 / pow2, d4 / pow2, -(d4 / pow2), t1 / pow2, -(t1 / pow2)};
  std::memcpy(w, tab, sizeof(tab));
}

static Rule make_rule(int ndim) {
  Rule R;
  R.ndim = ndim;
  R.feval = feval_count(ndim);
  rule9_weights(ndim, R.w);
  R.G[0] = .4779536579022695061928604197171830064732;
  R.G[1] = .2030285873691198677998034402373279133258;
  R.G[2] = .4476273546261781288207704806530998539285;
  R.G[3] = .125;
  R.G[4] = .3430378987808781457001426145164678603407;
  const int d = ndim;
  const int count[kNSets] = {1,         2 * d, 2 * d, 2 * d, 2 * d, 2 * d * (d - 1), 4 * d * (d - 1),
                             4 * d * (d - 1) * (d - 2) / 3, 1 << d};
  // Null-rule scale and normalisation (Rule.cuh:256-269).
  for (int i = 0; i < kNSets * kNRules; ++i) R.scale[i] = R.norm[i] = 0.0;
  for (int idx = 0; idx < kNSets; ++idx) {
    const double* sw = &R.w[idx * kNRules];
    for (int r = 1; r < kNRules - 1; ++r) {
      const double sc = (sw[r] == 0) ? 100 : -sw[r + 1] / sw[r];
      double sum = 0;
      for (int x = 0; x < kNSets; ++x) {
        const double* wx = &R.w[x * kNRules];
        sum += count[x] * std::fabs(wx[r + 1] + sc * wx[r]);
      }
      R.scale[idx * kNRules + r] = sc;
      R.norm[idx * kNRules + r] = 1 / sum;
    }
  }
  // Starting generator of each set (Rule.cuh:221-249).
  std::vector<double> g0(kNSets * d, 0.0);
  g0[d * 1] = R.G[0];
  g0[d * 2] = R.G[1];
  g0[d * 3] = R.G[2];
  g0[d * 4] = R.G[3];
  g0[d * 5] = R.G[0];
  g0[d * 5 + 1] = R.G[0];
  g0[d * 6] = R.G[0];
  g0[d * 6 + 1] = R.G[1];
  g0[d * 7] = R.G[0];
  if (d >= 2) g0[d * 7 + 1] = R.G[0];
  if (d >= 3) g0[d * 7 + 2] = R.G[0];
  for (int k = 0; k < d; ++k) g0[d * 8 + k] = R.G[4];

  // Enumerate the sign changes and permutations of every generator in the
  // reference's order (Rule.cuh:438-504): signs advance like a binary counter
  // from axis 0; when they wrap, the magnitudes step to the next permutation.
  R.set_of.clear();
  R.gen.clear();
  for (int s = 0; s < kNSets; ++s) {
    std::vector<double> g(g0.begin() + s * d, g0.begin() + (s + 1) * d);
    for (int m = 0; m < count[s]; ++m) {
      R.set_of.push_back(s);
      for (int k = 0; k < d; ++k) R.gen.push_back(g[k] == 0.0 ? 0.0 : g[k]);
      bool more_signs = false;
      for (int k = 0; k < d; ++k) {
        g[k] = -g[k];
        if (g[k] < -0.0000000000000001) {
          more_signs = true;
          break;
        }
      }
      if (more_signs) continue;
      for (int k = 1; k < d; ++k) {
        const double gk = g[k];
        if (g[k - 1] > gk) {
          size_t i, j = k, ix = k, dx = k - 1;
          for (i = 0; i < --j; ++i) {
            const double tmp = g[i];
            g[i] = g[j];
            g[j] = tmp;
            if (tmp <= gk) --dx;
            if (g[i] > gk) ix = i;
          }
          if (g[dx] <= gk) dx = ix;
          g[k] = g[dx];
          g[dx] = gk;
          break;
        }
      }
    }
  }
  return R;
}

// ---------------------------------------------------------------------------
// Deterministic blocked Neumaier reductions (the library's reduction order).
// Chunk = 2048 elements, 256 lanes x 8 items per lane (stride 256), lane
// partials merged by a shuffle-down tree per 32-lane warp, then the 8 warp
// partials by a tree with offsets 4,2,1.  Chunk partials are merged by one
// 256-lane pass (lane t takes chunks t, t+256, ...) and the same trees.
// ---------------------------------------------------------------------------
struct NS {
  double s, c;
};

static inline NS ns_merge(NS a, NS b) {
  const double t = a.s + b.s;
  const double e = (std::fabs(a.s) >= std::fabs(b.s)) ? ((a.s - t) + b.s) : ((b.s - t) + a.s);
  return NS{t, (a.c + b.c) + e};
}

static NS ns_block_tree(NS* lane) {
  // lane[0..255]; warp trees then warp-0 tree.
  NS warp[8];
  for (int w = 0; w < 8; ++w) {
    NS v[32];
    for (int l = 0; l < 32; ++l) v[l] = lane[w * 32 + l];
    for (int off = 16; off >= 1; off >>= 1)
      for (int l = 0; l < off; ++l) v[l] = ns_merge(v[l], v[l + off]);
    warp[w] = v[0];
  }
  for (int off = 4; off >= 1; off >>= 1)
    for (int l = 0; l < off; ++l) warp[l] = ns_merge(warp[l], warp[l + off]);
  return warp[0];
}

template <class Get>
static double canon_sum(size_t n, Get get) {
  const size_t nchunks = (n + 2047) / 2048;
  std::vector<NS> part(nchunks);
  for (size_t b = 0; b < nchunks; ++b) {
    NS lane[256];
    for (int t = 0; t < 256; ++t) {
      NS acc{0.0, 0.0};
      for (int k = 0; k < 8; ++k) {
        const size_t i = b * 2048 + (size_t)k * 256 + t;
        if (i < n) acc = ns_merge(acc, NS{get(i), 0.0});
      }
      lane[t] = acc;
    }
    part[b] = ns_block_tree(lane);
  }
  NS lane[256];
  for (int t = 0; t < 256; ++t) {
    NS acc{0.0, 0.0};
    for (size_t b = t; b < nchunks; b += 256) acc = ns_merge(acc, part[b]);
    lane[t] = acc;
  }
  const NS r = ns_block_tree(lane);
  return r.s + r.c;
}

// ---------------------------------------------------------------------------
// Region evaluation.  Restates INIT_REGION_POOL (Phases.cuh:301-363) and
// SampleRegionBlock / computePermutation (Sample.cuh:103-290) for one region,
// including the reduction order of the 64-thread block: thread t accumulates
// points t, t+64, ... with a fused multiply-add, the two 32-lane warps reduce
// with shuffle-down offsets 16..1 and the block sum is (warp0 + 0) + warp1
// (Sample.cuh:49-83).
// ---------------------------------------------------------------------------
struct EvalOut {
  double est, err;
  int bisect;
};

static EvalOut eval_region(const Rule& R, const Prepared& P, const double* lows, const double* highs,
                           const double* lower, const double* length) {
  const int d = R.ndim;
  double lo[kMaxDim], hi[kMaxDim], glo[kMaxDim], range[kMaxDim];
  double jac = 1.0, vol = 1.0, maxRange = 0.0;
  int maxDim = 0;
  for (int k = 0; k < d; ++k) {
    lo[k] = lower[k];
    hi[k] = lo[k] + length[k];
    vol *= hi[k] - lo[k];
    glo[k] = lows[k];
    range[k] = highs[k] - lows[k];
    const double r = hi[k] - lo[k];
    jac = jac * range[k];
    if (r > maxRange) {
      maxDim = k;
      maxRange = r;
    }
  }
  double lane_sum[64][kNRules];
  std::memset(lane_sum, 0, sizeof(lane_sum));
  double f64[64];
  double x[kMaxDim];
  for (int p = 0; p < R.feval; ++p) {
    const double* g = &R.gen[(size_t)p * d];
    for (int k = 0; k < d; ++k) {
      const double A = .5 + g[k], B = .5 - g[k];
      const double t = std::fma(A, lo[k], B * hi[k]);
      x[k] = std::fma(t, range[k], glo[k]);
    }
    const double fun = eval(P, x) * jac;
    if (p < 64) f64[p] = fun;
    const double* w = &R.w[R.set_of[p] * kNRules];
    double* acc = lane_sum[p & 63];
    for (int r = 0; r < kNRules; ++r) acc[r] = std::fma(fun, w[r], acc[r]);
  }
  // Fourth differences and split axis (Sample.cuh:194-218).
  int bisect = maxDim;
  {
    // base + ratio*(fp+fm) - (fp2+fm2), with the multiply that the
    // reference's compiled code fuses: base's for d <= 4, ratio's for d >= 5.
    const double q = R.G[1] / R.G[0];
    const double ratio = q * q;
    const double f02 = f64[0] * 2, omr = 1 - ratio;
    const double base = f02 * omr;
    double maxdiff = 0;
    for (int k = 0; k < d; ++k) {
      const double fp = f64[1 + 2 * k], fm = f64[2 + 2 * k];
      const double fp2 = f64[1 + 2 * k + 2 * d], fm2 = f64[2 + 2 * k + 2 * d];
      const double X = fp + fm;
      const double s = (d <= 4) ? std::fma(f02, omr, ratio * X) : std::fma(ratio, X, base);
      const double fd = std::fabs(s - (fp2 + fm2));
      if (fd > maxdiff) {
        maxdiff = fd;
        bisect = k;
      }
    }
  }
  double sum[kNRules];
  for (int r = 0; r < kNRules; ++r) {
    double v[64];
    for (int l = 0; l < 64; ++l) v[l] = lane_sum[l][r];
    double warp_tot[2];
    for (int w = 0; w < 2; ++w) {
      double a[32];
      for (int l = 0; l < 32; ++l) a[l] = v[w * 32 + l];
      for (int off = 16; off >= 1; off >>= 1)
        for (int l = 0; l < off; ++l) a[l] = a[l] + a[l + off];
      warp_tot[w] = a[0];
    }
    sum[r] = (warp_tot[0] + 0.0) + warp_tot[1];
  }
  // Null-rule error (Sample.cuh:261-289).
  for (int r = 1; r < kNRules - 1; ++r) {
    double maxerr = 0.;
    for (int s = 0; s < kNSets; ++s)
      maxerr = std::fmax(maxerr, std::fabs(std::fma(R.scale[s * kNRules + r], sum[r], sum[r + 1])) *
                                     R.norm[s * kNRules + r]);
    sum[r] = maxerr;
  }
  EvalOut o;
  o.est = vol * sum[0];
  o.err = vol * ((5. * sum[1] <= sum[2] && 5. * sum[2] <= sum[3])
                     ? 1. * sum[1]
                     : 5. * std::fmax(std::fmax(sum[1], sum[2]), sum[3]));
  o.bisect = bisect;
  return o;
}

// ---------------------------------------------------------------------------
// Region evaluation by generator-set sums (the library's PG_EVAL_SET_SUMS
// mode) for integrands that are products of per-axis factors.  Each rule sum
// is sum_s w[s][r] * S_s with S_s the sum of f over generator set s
// (Sample.cuh:145-148 accumulates f * w[set(p)][r] point by point); for
// f = prod_k h_k(x_k) the nine S_s follow from a recurrence over the axes on
// the 11 factor values h_k(centre), h_k(+-G_t).  The 4d+1 point values of the
// fourth differences (Sample.cuh:190-215) are formed exactly as eval() forms
// them (two half products in axis order), so the split axis is the
// point-by-point evaluation's.  Operation for operation the library's
// setsum_kernel.
// ---------------------------------------------------------------------------
static bool product_form(int family) {
  return family == FAM_PRODUCT_PEAK || family == FAM_GAUSSIAN || family == FAM_C0 || family == FAM_DISCONTINUOUS ||
         family == FAM_PRODUCT;
}

// The recurrence takes the axes other than `defer` in axis order, then
// `defer` (the library evaluates two siblings together and defers the axis
// they differ on; a region evaluated alone defers its last axis, which is the
// plain axis order).
static EvalOut eval_region_setsums(const Rule& R, const Prepared& P, const double* lows, const double* highs,
                                   const double* lower, const double* length, int defer) {
  const int d = R.ndim;
  double jac = 1.0;
  for (int k = 0; k < d; ++k) jac = jac * (highs[k] - lows[k]);
  double A[11], B[11];
  A[0] = .5 + 0.0;
  B[0] = .5 - 0.0;
  for (int t = 0; t < 5; ++t) {
    A[1 + t] = .5 + R.G[t];
    B[1 + t] = .5 - R.G[t];
    A[6 + t] = .5 + -R.G[t];
    B[6 + t] = .5 - -R.G[t];
  }
  double e0 = 1.0, a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0, b = 0.0, g = 0.0, t3 = 0.0, z = 1.0;
  double vol = 1.0, widest = 0.0;
  int maxdim = 0;
  double fv[kMaxDim][5];  // centre, +G0, -G0, +G1, -G1
  double pd[6] = {0, 0, 0, 0, 0, 0};  // c, p0..p4 of the deferred axis
  for (int kk = 0; kk <= d; ++kk) {
    // kk < d: axis kk (the deferred one only stores its terms); kk == d: the deferred axis enters
    const int k = kk == d ? defer : kk;
    if (kk == d) {
      const double c = pd[0], p0 = pd[1], p1 = pd[2], p2 = pd[3], p3 = pd[4], p4 = pd[5];
      t3 = std::fma(b, p0, t3 * c);
      g = std::fma(a1, p0, std::fma(a0, p1, g * c));
      b = std::fma(a0, p0, b * c);
      a0 = std::fma(e0, p0, a0 * c);
      a1 = std::fma(e0, p1, a1 * c);
      a2 = std::fma(e0, p2, a2 * c);
      a3 = std::fma(e0, p3, a3 * c);
      e0 = e0 * c;
      z = z * p4;
      break;
    }
    const double lo = lower[k], up = lo + length[k];
    const double side = up - lo;
    if (side > widest) {
      widest = side;
      maxdim = k;
    }
    vol = (k == 0) ? side : vol * side;
    const double glo = lows[k], range = highs[k] - lows[k];
    double h[11];
    for (int c = 0; c < 11; ++c) {
      const double t = std::fma(A[c], lo, B[c] * up);
      const double x = std::fma(t, range, glo);
      h[c] = (P.family == FAM_PRODUCT) ? x : factor(P, k, x);
    }
    fv[k][0] = h[0];
    fv[k][1] = h[1];
    fv[k][2] = h[6];
    fv[k][3] = h[2];
    fv[k][4] = h[7];
    const double c = h[0];
    const double p0 = h[1] + h[6], p1 = h[2] + h[7], p2 = h[3] + h[8], p3 = h[4] + h[9], p4 = h[5] + h[10];
    if (k == defer) {
      pd[0] = c, pd[1] = p0, pd[2] = p1, pd[3] = p2, pd[4] = p3, pd[5] = p4;
      continue;
    }
    t3 = std::fma(b, p0, t3 * c);
    g = std::fma(a1, p0, std::fma(a0, p1, g * c));
    b = std::fma(a0, p0, b * c);
    a0 = std::fma(e0, p0, a0 * c);
    a1 = std::fma(e0, p1, a1 * c);
    a2 = std::fma(e0, p2, a2 * c);
    a3 = std::fma(e0, p3, a3 * c);
    e0 = e0 * c;
    z = z * p4;
  }
  const bool scale_jac = jac != 1.0;
  const double S[kNSets] = {e0, a0, a1, a2, a3, b, g, t3, z};
  double s5[kNRules];
  for (int q = 0; q < kNRules; ++q) {
    double v = R.w[q] * S[0];
    for (int st = 1; st < kNSets; ++st) v = std::fma(R.w[st * kNRules + q], S[st], v);
    s5[q] = scale_jac ? v * jac : v;
  }
  // Fourth differences from the exact point values.
  const int m = d / 2;
  double Lc = fv[0][0], Rc = fv[m][0];
  for (int k = 1; k < m; ++k) Lc = Lc * fv[k][0];
  for (int k = m + 1; k < d; ++k) Rc = Rc * fv[k][0];
  double f0 = Lc * Rc;
  if (scale_jac) f0 = f0 * jac;
  const double f02 = f0 + f0;
  const double q = R.G[1] / R.G[0];
  const double ratio = q * q, omr = 1 - ratio;
  double maxdiff = 0;
  int bisect = maxdim;
  double pre = 1.0;
  for (int k = 0; k < d; ++k) {
    const bool lhalf = k < m;
    const int hbeg = lhalf ? 0 : m, hend = lhalf ? m : d;
    double f[4];
    for (int v = 0; v < 4; ++v) {
      double Pv = (k == hbeg) ? fv[k][1 + v] : pre * fv[k][1 + v];
      for (int j = k + 1; j < hend; ++j) Pv = Pv * fv[j][0];
      const double fp = lhalf ? Pv * Rc : Lc * Pv;
      f[v] = scale_jac ? fp * jac : fp;
    }
    pre = (k == hbeg) ? fv[k][0] : pre * fv[k][0];
    if (k + 1 == m) pre = 1.0;
    const double X = f[0] + f[1], Y = f[2] + f[3];
    const double s = (d <= 4) ? std::fma(f02, omr, ratio * X) : std::fma(ratio, X, f02 * omr);
    const double fd = std::fabs(s - Y);
    if (fd > maxdiff) {
      maxdiff = fd;
      bisect = k;
    }
  }
  // Null-rule error (Sample.cuh:261-289).
  double e[3];
  for (int r = 1; r < kNRules - 1; ++r) {
    double maxerr = 0.;
    for (int st = 0; st < kNSets; ++st)
      maxerr = std::fmax(maxerr, std::fabs(std::fma(R.scale[st * kNRules + r], s5[r], s5[r + 1])) *
                                     R.norm[st * kNRules + r]);
    e[r - 1] = maxerr;
  }
  EvalOut o;
  o.est = vol * s5[0];
  o.err = vol * ((5. * e[0] <= e[1] && 5. * e[1] <= e[2]) ? e[0] : 5. * std::fmax(std::fmax(e[0], e[1]), e[2]));
  o.bisect = bisect;
  return o;
}

// Evaluation mode of the oracle's evaluate_all: 0 point by point (the
// reference's order), 1 generator-set sums for the product-form families.
static int g_eval_mode = 0;
// Iterations of the last integration in which fix_error_budget_overflow fired.
static int g_budget_fixes = 0;

static void parallel_for(size_t n, int nthreads, const std::function<void(size_t, size_t)>& body) {
  if (nthreads <= 1 || n < 64) {
    body(0, n);
    return;
  }
  std::vector<std::thread> th;
  const size_t per = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    const size_t b = t * per, e = std::min(n, b + per);
    if (b >= e) break;
    th.emplace_back([&, b, e] { body(b, e); });
  }
  for (auto& t : th) t.join();
}

// With `siblings`, regions i and i + n/2 (n even) are the two children of one
// region (the list layout after a split): the set-sum evaluation defers the
// axis they differ on, as the library does when it evaluates them together.
static void evaluate_all(const Rule& R, const Prepared& P, const double* lows, const double* highs, size_t n,
                         const double* left, const double* len, double* est, double* err, int32_t* bis,
                         int nthreads, bool siblings = false) {
  const int d = R.ndim;
  const bool pairs = siblings && n % 2 == 0 && n > 0;
  parallel_for(n, nthreads, [&](size_t b, size_t e) {
    double lo[kMaxDim], ln[kMaxDim];
    for (size_t i = b; i < e; ++i) {
      for (int k = 0; k < d; ++k) {
        lo[k] = left[(size_t)k * n + i];
        ln[k] = len[(size_t)k * n + i];
      }
      int defer = d - 1;
      if (pairs) {
        const size_t j = i < n / 2 ? i + n / 2 : i - n / 2;
        for (int k = d - 1; k >= 0; --k)
          if (left[(size_t)k * n + i] != left[(size_t)k * n + j]) defer = k;
      }
      const EvalOut o = (g_eval_mode == 1 && product_form(P.family))
                            ? eval_region_setsums(R, P, lows, highs, lo, ln, defer)
                            : eval_region(R, P, lows, highs, lo, ln);
      est[i] = o.est;
      err[i] = o.err;
      bis[i] = o.bisect;
    }
  });
}

// ---------------------------------------------------------------------------
// Two-level error and relative-error classification.
// Restates RefineError (Phases.cuh:219-268) as launched by
// two_level_errorest_and_relerr_classify (hybrid.cuh:11-45).
// ---------------------------------------------------------------------------
static void two_level(size_t n, const double* est, const double* err, const double* parent_est, double* new_err,
                      uint8_t* active, double epsrel, bool relerr_classification) {
  for (size_t tid = 0; tid < n; ++tid) {
    double selfErr = err[tid];
    const double selfRes = est[tid];
    const size_t inRight = (2 * tid >= n);
    const size_t sib = inRight ? tid - n / 2 : tid + n / 2;
    const size_t par = tid - inRight * (n / 2);
    const double siblErr = err[sib], siblRes = est[sib];
    const double parRes = parent_est[par];
    double diff = siblRes + selfRes - parRes;
    diff = std::fabs(.25 * diff);
    const double e2 = selfErr + siblErr;
    if (e2 > 0.0) {
      const double c = 1 + 2 * diff / e2;
      selfErr *= c;
    }
    selfErr += diff;
    new_err[tid] = selfErr;
    const bool pass = relerr_classification && selfErr < std::fmax(epsrel * std::fabs(selfRes), 1e-200);
    active[tid] = pass ? 0 : 1;
  }
}

// ---------------------------------------------------------------------------
// Heuristic memory-pressure classifier.
// Restates cuda/pagani/quad/GPUquad/heuristic_classifier.cuh:89-452 and
// Workspace::heuristic_classify (Workspace.cuh:74-118).  The device memory is
// a parameter; the reference hard-codes 16e9 bytes (heuristic_classifier.cuh:89-94).
// ---------------------------------------------------------------------------
struct Classifier {
  double epsrel = 0, epsabs = 0;
  int required_digits = 0;
  double last[3] = {0, 0, 0};  // uninitialised in the reference; zero here
  size_t iters_collected = 0;
  double max_percent_error_budget = .25;
  double max_active_regions_percentage = .5;
  int ndim = 0;
  double total_mem = 16e9;

  size_t mem_required(size_t n) const {
    const size_t doubles = n + n + 2 * n + 2 * n + 2 * n * ndim + 2 * n * ndim + n * ndim * 2 + n * ndim * 2 + n +
                           n + n * ndim + n * ndim;
    const size_t ints = n + 2 * n + n;
    return 8 * doubles + 4 * ints;
  }
  size_t free_mem(size_t n) const {
    const size_t total = (size_t)total_mem;
    const size_t occ = mem_required(n);
    return total > occ ? total - occ : 1;
  }
  static std::string fixed15(double v) {
    std::ostringstream out;
    out.precision(15);
    out << std::fixed << v;
    return out.str();
  }
  bool sig_digits_same() const {
    double third = std::fabs(last[0]), second = std::fabs(last[1]), first = std::fabs(last[2]);
    while (first != 0. && first < 1.) first *= 10;
    while (second != 0. && second < 1.) second *= 10;
    while (third != 0. && third < 1.) third *= 10;
    const std::string a = fixed15(third), b = fixed15(second), c = fixed15(first);
    bool verdict = true;
    int sig = 0;
    for (int i = 0; i < required_digits + 1 && sig < required_digits && verdict; ++i) {
      const char ci = i < (int)c.size() ? c[i] : '\0';
      const char bi = i < (int)b.size() ? b[i] : '\0';
      const char ai = i < (int)a.size() ? a[i] : '\0';
      verdict = (ci == bi && bi == ai);
      sig += (verdict && ci != '.') ? 1 : 0;
    }
    return verdict;
  }
  bool estimate_converged() const { return !(iters_collected - 1 < 1 || !sig_digits_same()); }
  void store(double e) {
    last[0] = last[1];
    last[1] = last[2];
    last[2] = e;
    iters_collected++;
  }
  bool criteria_met(size_t n) const {
    const double ratio = (double)mem_required(n) / (double)free_mem(n);
    if (ratio > 1.) return true;
    if (ratio > .1 && estimate_converged()) return true;
    return false;
  }
};

struct ClassRes {
  bool pass_mem = false, pass_budget = false;
  double threshold = 0, low = 0, high = 0;
  size_t num_active = 0;
  double finished_errorest = 0;
  std::vector<uint8_t> flags;
};

static void apply_threshold(const Classifier& C, ClassRes& r, const double* err, size_t n) {
  r.flags.resize(n);
  for (size_t i = 0; i < n; ++i) r.flags[i] = err[i] > r.threshold ? 1 : 0;
  r.num_active = (size_t)canon_sum(n, [&](size_t i) { return (double)r.flags[i]; });
  const double pct = (double)(int)r.num_active / (double)(int)n;
  r.pass_mem = pct <= C.max_active_regions_percentage;
}

static ClassRes classify(Classifier& C, const double* err, size_t n, double iter_err, double iter_fin_err,
                         double total_fin_err) {
  ClassRes r;
  double mn = err[0], mx = err[0];
  for (size_t i = 1; i < n; ++i) {
    if (err[i] < mn) mn = err[i];
    if (err[i] > mx) mx = err[i];
  }
  r.low = mn;
  r.high = mx;
  r.threshold = iter_err / n;
  const double target = std::fabs(C.last[2]) * C.epsrel;
  size_t inc = 0, dec = 0;
  auto larger = [&]() {
    r.pass_mem = false;
    for (size_t cnt = 0; !r.pass_mem && cnt < 20; ++cnt) {
      apply_threshold(C, r, err, n);
      if (!r.pass_mem) {
        r.low = r.threshold;
        r.threshold += std::fabs(r.high - r.threshold) * .5;
      }
    }
  };
  do {
    if (!r.pass_mem && inc <= 20) {
      larger();
      inc++;
    }
    if (r.pass_mem) {
      const double dot = canon_sum(n, [&](size_t i) { return err[i] * (double)r.flags[i]; });
      const double extra = iter_err - dot - iter_fin_err;
      const double budget = target - total_fin_err;
      r.pass_budget = extra <= C.max_percent_error_budget * budget;
      r.finished_errorest = extra;
      if (!r.pass_budget && dec <= 20) {
        r.high = r.threshold;
        r.threshold -= std::fabs(r.low - r.threshold) * .5;
        r.pass_mem = false;
        dec++;
      }
    }
    const bool exhausted = dec >= 20 || inc >= 20;
    if (exhausted && C.max_percent_error_budget < .7) {
      C.max_percent_error_budget += 0.1;
      dec = inc = 0;
      r.low = mn;
      r.high = mx;
      r.threshold = iter_err / n;
    } else if (exhausted && C.max_percent_error_budget >= .7 && C.max_active_regions_percentage <= .7) {
      C.max_active_regions_percentage += .1;
    } else if (exhausted) {
      break;
    }
  } while (!r.pass_mem || !r.pass_budget);
  C.max_active_regions_percentage = .5;
  C.max_percent_error_budget = .25;
  return r;
}

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface used by the Python test harness.
// ---------------------------------------------------------------------------
extern "C" {

typedef struct {
  double estimate, errorest, chi_sq;
  uint64_t neval, nregions, nfinished, iters;
  int32_t status, last_phase;
} orc_result;

int orc_feval(int ndim) { return orc::feval_count(ndim); }

// Region-evaluation mode of every later evaluation and integration call:
// 0 point by point, 1 generator-set sums for the product-form families.
int orc_budget_fixes(void) { return orc::g_budget_fixes; }

int orc_set_eval_mode(int mode) {
  if (mode != 0 && mode != 1) return -1;
  orc::g_eval_mode = mode;
  return 0;
}

// Rule tables: w/scale/norm [45], set_of [feval], gen [feval*ndim] (point-major).
int orc_rule_tables(int ndim, double* w, double* scale, double* norm, int32_t* set_of, double* gen) {
  if (ndim < 2 || ndim > 15) return -1;
  const orc::Rule R = orc::make_rule(ndim);
  std::memcpy(w, R.w, sizeof(R.w));
  std::memcpy(scale, R.scale, sizeof(R.scale));
  std::memcpy(norm, R.norm, sizeof(R.norm));
  for (int p = 0; p < R.feval; ++p) set_of[p] = R.set_of[p];
  std::memcpy(gen, R.gen.data(), sizeof(double) * R.gen.size());
  return R.feval;
}

double orc_eval_point(const orc::Integrand* f, const double* x) {
  const orc::Prepared P = orc::prepare(*f);
  return orc::eval(P, x);
}

int orc_evaluate_regions(const orc::Integrand* f, const double* lows, const double* highs, uint64_t n,
                         const double* left, const double* length, double* est, double* err, int32_t* bisect,
                         int nthreads) {
  const int d = f->ndim;
  if (d < 2 || d > 15) return -1;
  const orc::Rule R = orc::make_rule(d);
  const orc::Prepared P = orc::prepare(*f);
  orc::evaluate_all(R, P, lows, highs, n, left, length, est, err, bisect, nthreads);
  return 0;
}

int orc_two_level(uint64_t n, const double* est, const double* err, const double* parent_est, double* new_err,
                  uint8_t* active, double epsrel, int relerr_classification) {
  orc::two_level(n, est, err, parent_est, new_err, active, epsrel, relerr_classification != 0);
  return 0;
}

double orc_canon_sum(const double* x, uint64_t n) {
  return orc::canon_sum(n, [&](size_t i) { return x[i]; });
}

// Uniform initial split (Sub_regions.cuh:11-36,253-274; partition rule Workspace.cuh:379-387).
uint64_t orc_uniform_split(int ndim, int parts, double* left, double* length) {
  size_t n = 1;
  for (int k = 0; k < ndim; ++k) n *= parts;
  if (!left) return n;
  const double len = 1. / (double)parts;
  for (size_t r = 0; r < n; ++r) {
    size_t q = r;
    for (int k = 0; k < ndim; ++k) {
      const size_t id = q % parts;
      q /= parts;
      left[(size_t)k * n + r] = (double)id * len;
      length[(size_t)k * n + r] = len;
    }
  }
  return n;
}

// Filter (Sub_region_filter.cuh:8-139) + split (Sub_region_splitter.cuh:8-88):
// compacts active regions in order and bisects each along its split axis.
// Output holds 2*A regions: child 0 at k, child 1 at A+k.  Returns A.
uint64_t orc_filter_split(int ndim, uint64_t n, const double* left, const double* length, const uint8_t* active,
                          const int32_t* bisect, const double* est, const double* err, double* out_left,
                          double* out_length, double* parent_est, double* parent_err) {
  size_t A = 0;
  for (size_t i = 0; i < n; ++i) A += active[i] ? 1 : 0;
  size_t k = 0;
  for (size_t i = 0; i < n; ++i) {
    if (!active[i]) continue;
    if (parent_est) parent_est[k] = est[i];
    if (parent_err) parent_err[k] = err[i];
    const int bd = bisect[i];
    for (int dd = 0; dd < ndim; ++dd) {
      const double l = left[(size_t)dd * n + i], h = length[(size_t)dd * n + i];
      if (dd == bd) {
        const double half = h / 2;
        out_left[(size_t)dd * 2 * A + k] = l + 0 * half;
        out_left[(size_t)dd * 2 * A + A + k] = l + 1 * half;
        out_length[(size_t)dd * 2 * A + k] = half;
        out_length[(size_t)dd * 2 * A + A + k] = half;
      } else {
        out_left[(size_t)dd * 2 * A + k] = l;
        out_left[(size_t)dd * 2 * A + A + k] = l;
        out_length[(size_t)dd * 2 * A + k] = h;
        out_length[(size_t)dd * 2 * A + A + k] = h;
      }
    }
    ++k;
  }
  return A;
}

// Full PAGANI iteration: Workspace::integrate, self-splitting overload
// (Workspace.cuh:361-494), with fix_error_budget_overflow (:121-146) and
// heuristic_classify (:74-118).  trace (optional) receives, per iteration,
// [N, A_after_classification, iter_est, iter_err, cumm_est, cumm_err].
// Workspace::integrate (Workspace.cuh:148-358,361-494): from the uniform
// split (init_n == 0) or from a caller-given first list (the Sub_regions
// overload); with predict_split, rel-err classification is off while the list
// has <= 15e6 regions, in the first 15 iterations and before anything finished
// (Workspace.cuh:415-420), and the list of iteration 15 is copied out
// (Workspace.cuh:437-441) when snap_cap allows.
int orc_integrate_regions(const orc::Integrand* f, double epsrel, double epsabs, const double* lows,
                          const double* highs, int relerr_classification, double total_device_mem, int max_iters,
                          int nthreads, const double* init_left, const double* init_len, uint64_t init_n,
                          int predict_split, double* snap_left, double* snap_len, uint64_t snap_cap,
                          uint64_t* snap_n, orc_result* out, double* trace, int trace_cap) {
  using namespace orc;
  const int d = f->ndim;
  if (d < 2 || d > 15 || !out) return -1;
  g_budget_fixes = 0;
  const Rule R = make_rule(d);
  const Prepared P = prepare(*f);
  const int parts = d < 5 ? 4 : (d <= 10 ? 2 : 1);
  size_t n;
  std::vector<double> left, len;
  if (init_n) {
    n = init_n;
    left.assign(init_left, init_left + n * d);
    len.assign(init_len, init_len + n * d);
  } else {
    n = orc_uniform_split(d, parts, nullptr, nullptr);
    left.resize(n * d);
    len.resize(n * d);
    orc_uniform_split(d, parts, left.data(), len.data());
  }
  if (snap_n) *snap_n = 0;
  std::vector<double> parent_est, parent_err;
  bool have_parent = false;
  Classifier C;
  C.epsrel = epsrel;
  C.epsabs = epsabs;
  C.required_digits = (int)std::ceil(std::log10(1 / epsrel));
  C.ndim = d;
  C.total_mem = total_device_mem > 0 ? total_device_mem : 16e9;
  orc_result cum{};
  cum.status = 1;
  cum.last_phase = -1;
  const uint64_t fev = (uint64_t)R.feval;
  std::vector<double> est, err, nerr;
  std::vector<int32_t> bis;
  std::vector<uint8_t> act;
  int ntrace = 0;
  for (int it = 0; it < max_iters && n > 0; ++it) {
    est.assign(n, 0);
    err.assign(n, 0);
    bis.assign(n, 0);
    act.assign(n, 1);
    evaluate_all(R, P, lows, highs, n, left.data(), len.data(), est.data(), err.data(), bis.data(), nthreads,
                 have_parent);
    cum.neval += n * fev;
    const double iter_est = canon_sum(n, [&](size_t i) { return est[i]; });
    const bool relerr =
        predict_split ? !(n <= 15000000 && it < 15 && cum.nregions == 0) : relerr_classification != 0;
    if (have_parent) {
      nerr.assign(n, 0);
      two_level(n, est.data(), err.data(), parent_est.data(), nerr.data(), act.data(), epsrel, relerr);
      err.swap(nerr);
    }
    const double iter_err = canon_sum(n, [&](size_t i) { return err[i]; });
    if (predict_split && cum.nregions == 0 && it == 15 && snap_n) {
      *snap_n = n;
      if (snap_left && snap_len && snap_cap >= n) {
        std::copy(left.begin(), left.begin() + n * d, snap_left);
        std::copy(len.begin(), len.begin() + n * d, snap_len);
      }
    }
    double* tr = (trace && ntrace < trace_cap) ? trace + 6 * ntrace : nullptr;
    if (tr) {
      tr[0] = (double)n;
      tr[2] = iter_est;
      tr[3] = iter_err;
      ++ntrace;
    }
    const double cest = std::fabs(cum.estimate + iter_est), cerr = cum.errorest + iter_err;
    if (cerr / cest <= epsrel || cerr <= epsabs) {
      cum.estimate += iter_est;
      cum.errorest += iter_err;
      cum.status = 0;
      cum.nregions += n;
      if (tr) {
        tr[1] = 0;
        tr[4] = cum.estimate;
        tr[5] = cum.errorest;
      }
      *out = cum;
      return ntrace;
    }
    C.store(cum.estimate + iter_est);
    double fin_est = iter_est - canon_sum(n, [&](size_t i) { return (double)act[i] * est[i]; });
    double fin_err = iter_err - canon_sum(n, [&](size_t i) { return (double)act[i] * err[i]; });
    // fix_error_budget_overflow
    {
      const double leaves_est = cum.estimate + iter_est;
      const double leaves_fin_err = cum.errorest + fin_err;
      if (leaves_fin_err > std::fabs(leaves_est) * epsrel) {
        ++g_budget_fixes;
        std::fill(act.begin(), act.end(), 1);
        fin_err = 0.;
        fin_est = 0.;
      }
    }
    // heuristic_classify
    bool must_terminate;
    {
      const double ratio = (double)C.mem_required(n) / (double)C.free_mem(n);
      const bool necessary = ratio > 1.;
      if (!C.criteria_met(n)) {
        must_terminate = necessary;
      } else {
        ClassRes hs = classify(C, err.data(), n, iter_err, fin_err, cum.errorest);
        const bool ok = hs.pass_mem && hs.pass_budget;
        if (ok) {
          act = hs.flags;
          fin_est = iter_est - canon_sum(n, [&](size_t i) { return (double)act[i] * est[i]; });
          fin_err = hs.finished_errorest;
        }
        must_terminate = (!ok && necessary) || hs.num_active == 0;
      }
    }
    if (must_terminate) {
      cum.estimate += iter_est;
      cum.errorest += iter_err;
      cum.nregions += n;
      if (tr) {
        tr[1] = -1;
        tr[4] = cum.estimate;
        tr[5] = cum.errorest;
      }
      *out = cum;
      return ntrace;
    }
    cum.estimate += fin_est;
    cum.errorest += fin_err;
    // filter
    size_t A = 0;
    for (size_t i = 0; i < n; ++i) A += act[i];
    if (tr) {
      tr[1] = (double)A;
      tr[4] = cum.estimate;
      tr[5] = cum.errorest;
    }
    cum.nregions += n - A;
    cum.nfinished += n - A;
    if (A == 0) {
      n = 0;
      cum.iters++;
      break;
    }
    std::vector<double> nl(2 * A * d), nln(2 * A * d);
    parent_est.assign(A, 0);
    parent_err.assign(A, 0);
    orc_filter_split(d, n, left.data(), len.data(), act.data(), bis.data(), est.data(), err.data(), nl.data(),
                     nln.data(), parent_est.data(), parent_err.data());
    have_parent = true;
    left.swap(nl);
    len.swap(nln);
    n = 2 * A;
    cum.iters++;
  }
  cum.nregions += n;
  *out = cum;
  return ntrace;
}

int orc_integrate(const orc::Integrand* f, double epsrel, double epsabs, const double* lows, const double* highs,
                  int relerr_classification, double total_device_mem, int max_iters, int nthreads, orc_result* out,
                  double* trace, int trace_cap) {
  return orc_integrate_regions(f, epsrel, epsabs, lows, highs, relerr_classification, total_device_mem, max_iters,
                               nthreads, nullptr, nullptr, 0, 0, nullptr, nullptr, 0, nullptr, out, trace, trace_cap);
}

}  // extern "C"

// ===========================================================================
// m-Cubes oracle.  Restates cuda_mcubes::vegas (cuda/mcubes/vegasT.cuh:643-997)
// and its sampling kernel (vegasT.cuh:136-485) with the library's random
// stream (Philox4x32-10, counter = cube, sample, axis pair, iteration), its
// work split (1024 x 256 threads, contiguous cube runs, per-thread sums,
// 32-lane shuffle-down trees then 8 warp sums in order) and its order of the
// f^2 bin sums, so the GPU's results differ from the oracle's only by the
// last bits of exp/pow/log (CUDA's against glibc's).
// ===========================================================================
namespace orc {

static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  // Philox4x32-10, Salmon, Moraes, Dror, Shaw, SC'11.
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

static double unit53(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)(m + 1) * 1.1102230246251565404236316680908203125e-16;
}

static void mc_rebin(double rc, int nd, const double* r, double* xin, double* xi) {
  int k = 0;
  double dr = 0.0, xn = 0.0, xo = 0.0;
  for (int i = 1; i < nd; i++) {
    while (rc > dr) dr += r[++k];
    if (k > 1) xo = xi[k - 1];
    xn = xi[k];
    dr -= rc;
    xin[i] = xn - (xn - xo) * dr / r[k];
  }
  for (int i = 1; i < nd; i++) xi[i] = xin[i];
  xi[nd] = 1.0;
}

}  // namespace orc

extern "C" {

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  orc::philox(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = c[i];
}

int orc_mcubes_integrate(const orc::Integrand* f, double epsrel, double epsabs, const double* lows,
                         const double* highs, double ncall, int titer, int itmax, int skip, int nbins, uint64_t seed,
                         double alpha, orc_result* out, double* trace, int trace_cap) {
  using namespace orc;
  const int d = f->ndim;
  const Prepared P = prepare(*f);
  const int nd = nbins > 1 ? nbins : 500;
  const int nb1 = nd + 1;
  const uint64_t ng = (uint64_t)std::pow(ncall / 2.0 + 0.25, 1.0 / d);
  if (ng < 1) return -1;
  double k = 1;
  for (int i = 1; i < d; ++i) k *= (double)ng;
  k *= (double)ng;
  const uint64_t ncubes = (uint64_t)k;
  const int npg = (int)std::max(ncall / k, 2.0);
  const double calls = (double)npg * k;
  double dxg = 1.0 / (double)ng, dv2g = 1;
  for (int i = 1; i <= d; ++i) dv2g *= dxg;
  dv2g = (calls * dv2g * calls * dv2g) / npg / npg / (npg - 1.0);
  const double xnd = nd;
  dxg *= xnd;
  double xjac = 1.0 / calls;
  std::vector<double> regn(d), dx(d);
  for (int j = 0; j < d; ++j) {
    regn[j] = lows ? lows[j] : 0.0;
    dx[j] = (highs ? highs[j] : 1.0) - regn[j];
    xjac *= dx[j];
  }
  std::vector<double> xi((size_t)d * nb1, 0.0), r(nb1, 1.0), xin(nb1, 0.0), dbin((size_t)d * nb1), dt(d);
  for (int j = 0; j < d; ++j) {
    xi[(size_t)j * nb1 + 1] = 1.0;
    mc_rebin(1.0 / xnd, nd, r.data(), xin.data(), &xi[(size_t)j * nb1]);
  }
  const int NB = 1024, NT = 256;
  const uint64_t nthreads = (uint64_t)NB * NT, per = (ncubes + nthreads - 1) / nthreads;
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  std::vector<double> part(2 * NB);
  const int nworkers = std::max(1u, std::thread::hardware_concurrency());
  // Per-block histograms, each formed in the library's order: rounds of one
  // sample per thread; per round, axis by axis, batches of 32 threads in which
  // the samples of one bin are summed in thread order before joining the bin.
  std::vector<double> part_hist((size_t)NB * d * nb1);
  auto iteration = [&](int it, bool adapt) {
    std::fill(dbin.begin(), dbin.end(), 0.0);
    std::vector<std::thread> th;
    for (int w = 0; w < nworkers; ++w) {
      th.emplace_back([&, w] {
        std::vector<double> hist((size_t)d * nb1);
        std::vector<double> rf2(NT);
        std::vector<int> rbin((size_t)d * NT);
        struct Lane {
          uint64_t c0, mine;
          double fb, f2b, fbg, f2bg;
          int kg[kMaxDim];
        };
        std::vector<Lane> L(NT);
        for (int b = w; b < NB; b += nworkers) {
          std::fill(hist.begin(), hist.end(), 0.0);
          for (int t = 0; t < NT; ++t) {
            const uint64_t tid = (uint64_t)b * NT + t;
            const uint64_t c0 = tid * per, c1 = std::min(ncubes, c0 + per);
            L[t] = Lane{c0, (c1 > c0 ? c1 - c0 : 0) * (uint64_t)npg, 0.0, 0.0, 0.0, 0.0, {}};
          }
          const uint64_t rounds = per * (uint64_t)npg;
          for (uint64_t round = 0; round < rounds; ++round) {
            for (int t = 0; t < NT; ++t) {
              Lane& S = L[t];
              rf2[t] = 0.0;
              for (int j = 0; j < d; ++j) rbin[(size_t)j * NT + t] = 0;
              if (round >= S.mine) continue;
              const uint64_t cube = S.c0 + round / (uint64_t)npg;
              const int s = 1 + (int)(round % (uint64_t)npg);
              if (s == 1) {
                uint64_t q = cube;
                for (int j = d - 1; j >= 0; --j) {
                  S.kg[j] = 1 + (int)(q % ng);
                  q /= ng;
                }
              }
              double wgt = xjac, x[kMaxDim];
              uint32_t rnd[4] = {0, 0, 0, 0};
              for (int j = 0; j < d; ++j) {
                if ((j & 1) == 0) {
                  rnd[0] = (uint32_t)cube;
                  rnd[1] = (uint32_t)s | ((uint32_t)(cube >> 32) << 16);
                  rnd[2] = (uint32_t)(j >> 1);
                  rnd[3] = (uint32_t)it;
                  philox(rnd, k0, k1);
                }
                const double ran = (j & 1) ? unit53(rnd[2], rnd[3]) : unit53(rnd[0], rnd[1]);
                const double xn = std::fma((double)S.kg[j] - ran, dxg, 1.0);
                const int bb = std::max(std::min((int)xn, nd), 1);
                const double* xij = &xi[(size_t)j * nb1];
                double xo, rc;
                if (bb > 1) {
                  xo = xij[bb] - xij[bb - 1];
                  rc = std::fma(xn - (double)bb, xo, xij[bb - 1]);
                } else {
                  xo = xij[bb];
                  rc = (xn - (double)bb) * xo;
                }
                x[j] = std::fma(rc, dx[j], regn[j]);
                wgt = wgt * (xo * xnd);
                rbin[(size_t)j * NT + t] = bb;
              }
              const double fv = wgt * eval(P, x);
              const double f2 = fv * fv;
              rf2[t] = f2;
              S.fb = S.fb + fv;
              S.f2b = S.f2b + f2;
              if (s == npg) {
                double v = std::sqrt(S.f2b * (double)npg);
                v = (v - S.fb) * (v + S.fb);
                if (v <= 0.0) v = 1.0e-30;
                S.fbg = S.fbg + S.fb;
                S.f2bg = S.f2bg + v;
                S.fb = S.f2b = 0.0;
              }
            }
            if (!adapt) continue;
            for (int j = 0; j < d; ++j)
              for (int i = 0; i < NT / 32; ++i)
                for (int l = 0; l < 32; ++l) {
                  const int bb = rbin[(size_t)j * NT + i * 32 + l];
                  bool lead = bb != 0;
                  for (int l2 = 0; l2 < l && lead; ++l2) lead = rbin[(size_t)j * NT + i * 32 + l2] != bb;
                  if (!lead) continue;
                  double sum = 0.0;
                  for (int l2 = l; l2 < 32; ++l2)
                    if (rbin[(size_t)j * NT + i * 32 + l2] == bb) sum = sum + rf2[i * 32 + l2];
                  hist[(size_t)j * nb1 + bb] = hist[(size_t)j * nb1 + bb] + sum;
                }
          }
          double w0[8], w1[8];
          for (int w8 = 0; w8 < 8; ++w8) {
            double a[32], c[32];
            for (int l = 0; l < 32; ++l) {
              a[l] = L[w8 * 32 + l].fbg;
              c[l] = L[w8 * 32 + l].f2bg;
            }
            for (int off = 16; off >= 1; off >>= 1)
              for (int l = 0; l < off; ++l) {
                a[l] = a[l] + a[l + off];
                c[l] = c[l] + c[l + off];
              }
            w0[w8] = a[0];
            w1[w8] = c[0];
          }
          double s0 = 0.0, s1 = 0.0;
          for (int w8 = 0; w8 < 8; ++w8) {
            s0 = s0 + w0[w8];
            s1 = s1 + w1[w8];
          }
          part[2 * b] = s0;
          part[2 * b + 1] = s1;
          if (adapt) std::copy(hist.begin(), hist.end(), part_hist.begin() + (size_t)b * d * nb1);
        }
      });
    }
    for (auto& t : th) t.join();
    if (adapt)
      for (size_t i = 0; i < dbin.size(); ++i) {
        double sum = 0.0;
        for (int b = 0; b < NB; ++b) sum = sum + part_hist[(size_t)b * dbin.size() + i];
        dbin[i] = sum;
      }
    double ti = 0, tsi = 0;
    for (int b = 0; b < NB; ++b) {
      ti += part[2 * b];
      tsi += part[2 * b + 1];
    }
    return std::make_pair(ti, tsi * dv2g);
  };
  double si = 0, swgt = 0, schi = 0, tgral = 0, sd = 0, chi2a = 0;
  int status = 1, ntr = 0;
  uint64_t iters = 0;
  auto record = [&](int it, double ti, double tsi) {
    if (trace && ntr < trace_cap) {
      double* t = trace + 4 * ntr++;
      t[0] = it;
      t[1] = ti;
      t[2] = tsi;
      t[3] = tgral;
    }
  };
  for (int it = 1; it <= itmax && status == 1; ++iters, ++it) {
    auto [ti, tsi] = iteration(it, true);
    if (it > skip) {
      const double wgt = 1.0 / tsi;
      si += wgt * ti;
      schi += wgt * ti * ti;
      swgt += wgt;
      tgral = si / swgt;
      chi2a = (schi - si * tgral) / (static_cast<double>(it) - 0.9999);
      if (chi2a < 0.0) chi2a = 0.0;
      sd = std::sqrt(1.0 / swgt);
      const bool ok = std::fabs(sd / tgral) <= epsrel || sd <= epsabs;
      status = (ok && it >= 5) ? 0 : 1;
    }
    record(it, ti, tsi);
    for (int j = 0; j < d; ++j) {
      double* dj = &dbin[(size_t)j * nb1];
      double xo = dj[1], xn = dj[2];
      dj[1] = (xo + xn) / 2.0;
      dt[j] = dj[1];
      for (int i = 2; i < nd; ++i) {
        const double rcv = xo + xn;
        xo = xn;
        xn = dj[i + 1];
        dj[i] = (rcv + xn) / 3.0;
        dt[j] += dj[i];
      }
      dj[nd] = (xo + xn) / 2.0;
      dt[j] += dj[nd];
    }
    for (int j = 0; j < d; ++j) {
      if (dt[j] > 0.0) {
        const double* dj = &dbin[(size_t)j * nb1];
        double rsum = 0.0;
        for (int i = 1; i <= nd; ++i) {
          r[i] = std::pow((1.0 - dj[i] / dt[j]) / (std::log(dt[j]) - std::log(dj[i])), alpha);
          rsum += r[i];
        }
        mc_rebin(rsum / xnd, nd, r.data(), xin.data(), &xi[(size_t)j * nb1]);
      }
    }
  }
  for (int it = itmax + 1; it <= titer && status; ++iters, ++it) {
    auto [ti, tsi] = iteration(it, false);
    const double wgt = 1.0 / tsi;
    si += wgt * ti;
    schi += wgt * ti * ti;
    swgt += wgt;
    tgral = si / swgt;
    chi2a = (schi - si * tgral) / (it - 0.9999);
    if (chi2a < 0.0) chi2a = 0.0;
    sd = std::sqrt(1.0 / swgt);
    const bool ok = std::fabs(sd / tgral) <= epsrel || sd <= epsabs;
    status = (ok && it >= 5) ? 0 : 1;
    record(it, ti, tsi);
  }
  orc_result R{};
  R.estimate = tgral;
  R.errorest = sd;
  R.chi_sq = chi2a;
  R.neval = (uint64_t)calls * iters;
  R.nregions = ncubes;
  R.iters = iters;
  R.status = status;
  R.last_phase = -1;
  *out = R;
  return ntr;
}

}  // extern "C"
