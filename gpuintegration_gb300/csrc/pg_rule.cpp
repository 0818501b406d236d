// Degree-9 rule tables (library side).  Compiled with -ffp-contract=off so the
// weight polynomials round exactly as the reference's host code does on x86-64.
#include <map>
#include "pg_rule.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace pg {

int feval_count(int d) {
  // Points of the degree-9 rule: cuda/pagani/quad/quad.h:67-76.
  return 1 + 2 * d + 2 * d + 2 * d + 2 * d + 2 * d * (d - 1) + 4 * d * (d - 1) + 4 * d * (d - 1) * (d - 2) / 3 +
         (1 << d);
}

namespace {

// Weights of the basic rule (column 0) and the four null rules (columns 1..4)
// for each generator set, as polynomials in the dimension n.  The constants
// and the grouping of every expression follow Rule.cuh:36-147; the grouping
// matters because each entry must round to the reference's double.
void weights(int ndim, double* W) {
  const double n = ndim;
  auto cubicC = [n] {
    return n * (n * (n * -.002361170967785511788400941242259231309691 + .1141539002385732526821323741697655347686) +
                -.6383392007670238909386026193674701393074) +
           .7484998850468520800423030047583803945205;
  };
  auto cubicD = [n] {
    return n * (n * (n * -.001432401703339912514196154599769007103671 + .05747150786448972594860897296200006759892) +
                -.1422510457143424323449521620935950679394) -
           -.06287502873828697998942424881040490136987;
  };
  auto quadH = [n] {
    return n * (n * .003541756451678267682601411863388846964536 + -.07260936739589367960492815865074633743652) +
           .1055749162521899101218622863269817454540;
  };
  auto quadI = [n] {
    return n * (n * .002148602555009868771294231899653510655506 + -.03226856389295394999786630399875134318006) +
           .01063678399023121748083624225818915724455;
  };
  auto linM = [n] { return n * -.04508628929435784075980562738240804429658 + .2141588352435279340097929526588394300172; };
  auto linN = [n] { return n * -.02735154652654564472203690086290223507436 + .05494106704871123410060080562462135546101; };
  const double p2 = (double)(1 << ndim);
  const double e8a = .2515001149531479199576969952416196054795, e8b = -.06287502873828697998942424881040490136987;
  const double lin5h = .01553241727660705326386197156586357005224, lin5i = .003532809960709087023561817517751309380604;
  double* w = W;
  // set 0 (centre point)
  w[0] = cubicC();
  w[1] = cubicD();
  w[2] = n * .2545911332489590890011611142429070613156 - cubicD();
  w[3] = ((n * (n * -1.207328566678236261002219995185143356737 + .8956736576416067650809467826488567200939) - 1) +
          n * (n * (n * -.002361170967785511788400941242259231309691 + .1141539002385732526821323741697655347686) +
               -.6383392007670238909386026193674701393074)) +
         .7484998850468520800423030047583803945205;
  w[4] = (n * -.3647935698604914666100134551377381205297 + 1) - cubicC();
  // set 1 (+-G0 on one axis)
  w[5] = quadH();
  w[6] = quadI();
  w[7] = .01468910249614349017540783437728097691502 - quadI();
  w[8] = ((n * .5113470834646759143109387357149329909126 + .4597644812080634464633352781605214342691) +
          n * (n * .003541756451678267682601411863388846964536 + -.07260936739589367960492815865074633743652)) +
         .1055749162521899101218622863269817454540;
  w[9] = .1823967849302457333050067275688690602649 - quadH();
  // set 2 (+-G1 on one axis)
  w[10] = linM();
  w[11] = linN();
  w[12] = .1193759620257077529708962121565290178730 - linN();
  w[13] = n * .6508951939192025059314756320878023215278 + .1474493982943446016775696826942585013243;
  w[14] = -linM();
  // set 3 (+-G2 on one axis)
  const double s3[5] = {.05769338449097348357291272840392627722165, .03499962660214358382244159694487155861542,
                        -.05769338449097348357291272840392627722165, -1.386862771927828143599782668709014266770,
                        -.05769338449097348357291272840392627722165};
  // set 4 (+-G3 on one axis)
  const double s4[5] = {0, 0, -.2386668732575008878964134721962088068396, 0, 0};
  std::memcpy(w + 15, s3, sizeof s3);
  std::memcpy(w + 20, s4, sizeof s4);
  // set 5 (+-G0 on two axes)
  w[25] = lin5h - n * .003541756451678267682601411863388846964536;
  w[26] = lin5i - n * .002148602555009868771294231899653510655506;
  w[27] = -(lin5i - n * .002148602555009868771294231899653510655506);
  w[28] = (.09231719987444221619017126187763868745587 + lin5h) - n * .003541756451678267682601411863388846964536;
  w[29] = -(lin5h - n * .003541756451678267682601411863388846964536);
  // set 6 (+-G0, +-G1 on two axes)
  const double s6[5] = {.02254314464717892037990281369120402214829, .01367577326327282236101845043145111753718,
                        -.01367577326327282236101845043145111753718, -.3254475969596012529657378160439011607639,
                        -.02254314464717892037990281369120402214829};
  // set 7 (+-G0 on three axes)
  const double s7[5] = {.001770878225839133841300705931694423482268, .001074301277504934385647115949826755327753,
                        -.001074301277504934385647115949826755327753, .001770878225839133841300705931694423482268,
                        -.001770878225839133841300705931694423482268};
  std::memcpy(w + 30, s6, sizeof s6);
  std::memcpy(w + 35, s7, sizeof s7);
  // set 8 (+-G4 on every axis)
  w[40] = e8a / p2;
  w[41] = e8b / p2;
  w[42] = -(e8b / p2);
  w[43] = e8a / p2;
  w[44] = -(e8a / p2);
}

// Advances g to the next point of its generator set in the reference's order
// (Rule.cuh:473-503): signs count like a binary number from axis 0; when every
// sign has wrapped the magnitudes step to the next permutation.
void next_point(std::vector<double>& g) {
  const int d = (int)g.size();
  for (int k = 0; k < d; ++k) {
    g[k] = -g[k];
    if (g[k] < -0.0000000000000001) return;
  }
  for (int k = 1; k < d; ++k) {
    const double pivot = g[k];
    if (!(g[k - 1] > pivot)) continue;
    size_t lo = 0, hi = k, ix = k, dx = k - 1;
    for (; lo < --hi; ++lo) {
      std::swap(g[lo], g[hi]);
      if (g[hi] <= pivot) --dx;
      if (g[lo] > pivot) ix = lo;
    }
    if (g[dx] <= pivot) dx = ix;
    g[k] = g[dx];
    g[dx] = pivot;
    return;
  }
}

}  // namespace

RuleTable make_rule(int d) {
  RuleTable r;
  r.ndim = d;
  r.feval = feval_count(d);
  weights(d, r.w);
  const double G[5] = {.4779536579022695061928604197171830064732, .2030285873691198677998034402373279133258,
                       .4476273546261781288207704806530998539285, .125,
                       .3430378987808781457001426145164678603407};
  std::memcpy(r.G, G, sizeof G);
  const int npts[kNSets] = {1,
                            2 * d,
                            2 * d,
                            2 * d,
                            2 * d,
                            2 * d * (d - 1),
                            4 * d * (d - 1),
                            4 * d * (d - 1) * (d - 2) / 3,
                            1 << d};
  // Null-rule scale/norm (Rule.cuh:256-269).
  std::fill(r.scale, r.scale + kNSets * kNRules, 0.0);
  std::fill(r.norm, r.norm + kNSets * kNRules, 0.0);
  for (int s = 0; s < kNSets; ++s) {
    for (int q = 1; q < kNRules - 1; ++q) {
      const double* ws = r.w + s * kNRules;
      const double f = (ws[q] == 0) ? 100 : -ws[q + 1] / ws[q];
      double tot = 0;
      for (int x = 0; x < kNSets; ++x) {
        const double* wx = r.w + x * kNRules;
        tot += npts[x] * std::fabs(wx[q + 1] + f * wx[q]);
      }
      r.scale[s * kNRules + q] = f;
      r.norm[s * kNRules + q] = 1 / tot;
    }
  }
  // Leading generator of each set (Rule.cuh:221-249).
  std::vector<std::vector<double>> lead(kNSets, std::vector<double>(d, 0.0));
  lead[1][0] = G[0];
  lead[2][0] = G[1];
  lead[3][0] = G[2];
  lead[4][0] = G[3];
  lead[5][0] = lead[5][1] = G[0];
  lead[6][0] = G[0];
  lead[6][1] = G[1];
  for (int k = 0; k < std::min(3, d); ++k) lead[7][k] = G[0];
  for (int k = 0; k < d; ++k) lead[8][k] = G[4];
  r.set_of.reserve(r.feval);
  r.gen.reserve((size_t)r.feval * d);
  r.code.reserve(r.feval);
  for (int s = 0; s < kNSets; ++s) {
    std::vector<double> g = lead[s];
    for (int m = 0; m < npts[s]; ++m) {
      uint64_t code = (uint64_t)s << 60;
      for (int k = 0; k < d; ++k) {
        const double v = (g[k] == 0.0) ? 0.0 : g[k];
        r.gen.push_back(v);
        int c = 0;
        for (int j = 0; j < 5; ++j) {
          if (v == G[j]) c = 1 + j;
          if (v == -G[j]) c = 6 + j;
        }
        code |= (uint64_t)c << (4 * k);
      }
      r.set_of.push_back(s);
      r.code.push_back(code);
      next_point(g);
    }
  }
  return r;
}

// Distinct code prefixes of the axes [a, a + m) in order of first appearance
// over the points; returns per point its node index at depth m and appends
// the entries of depths 2..m to levels[k].
static std::vector<int> half_trie(const RuleTable& r, int a, int m, std::vector<std::vector<uint16_t>>* levels) {
  const int np = r.feval;
  std::vector<int> node(np);
  for (int p = 0; p < np; ++p) node[p] = (int)((r.code[p] >> (4 * a)) & 15u);  // depth 1: the code
  for (int k = 2; k <= m; ++k) {
    std::map<std::pair<int, int>, int> index;  // (parent, code) -> node at depth k
    for (int p = 0; p < np; ++p) {
      const int c = (int)((r.code[p] >> (4 * (a + k - 1))) & 15u);
      const auto key = std::make_pair(node[p], c);
      auto it = index.find(key);
      int id;
      if (it == index.end()) {
        id = (int)index.size();
        index.emplace(key, id);
        (*levels)[k].push_back((uint16_t)(node[p] | (c << 12)));
      } else {
        id = it->second;
      }
      node[p] = id;
    }
  }
  return node;
}

void split_trie(const RuleTable& r, std::vector<uint16_t>* inner, std::vector<uint32_t>* leaf) {
  const int d = r.ndim, m = d / 2;
  std::vector<std::vector<uint16_t>> lv(d + 1), rv(d + 1);
  const std::vector<int> ln = half_trie(r, 0, m, &lv);
  const std::vector<int> rn = half_trie(r, m, d - m, &rv);
  inner->clear();
  for (int k = 2; k <= std::max(m, d - m); ++k) {
    if (k <= m) inner->insert(inner->end(), lv[k].begin(), lv[k].end());
    if (k <= d - m) inner->insert(inner->end(), rv[k].begin(), rv[k].end());
  }
  leaf->resize(r.feval);
  for (int p = 0; p < r.feval; ++p)
    (*leaf)[p] = (uint32_t)ln[p] | ((uint32_t)rn[p] << 12) | ((uint32_t)(r.code[p] >> 60) << 24);
}

void code_coefficients(const RuleTable& r, double* A, double* B) {
  A[0] = .5 + 0.0;
  B[0] = .5 - 0.0;
  for (int j = 0; j < 5; ++j) {
    A[1 + j] = .5 + r.G[j];
    B[1 + j] = .5 - r.G[j];
    A[6 + j] = .5 + -r.G[j];
    B[6 + j] = .5 - -r.G[j];
  }
}

}  // namespace pg
