// Degree-9 cubature rule of PAGANI (host side).
//
// The rule, its four null rules and the order of its evaluation points are the
// reference's (cuda/pagani/quad/GPUquad/Rule.cuh:24-270 and :370-510).  The
// library generates the tables itself; tests pin them bit for bit against the
// reference's own tables.
#pragma once

#include <stdint.h>

#include <vector>

#include "pg_common.cuh"

namespace pg {

struct RuleTable {
  int ndim = 0;
  int feval = 0;
  double w[kNSets * kNRules];      // weights [set * 5 + rule]
  double scale[kNSets * kNRules];  // null-rule combination factors (rules 1..3)
  double norm[kNSets * kNRules];   // null-rule normalisation (rules 1..3)
  double G[5];                     // generator magnitudes
  std::vector<int> set_of;         // [feval] generator set of each point
  std::vector<double> gen;         // [feval * ndim] point-major coordinates in [-.5, .5]
  // Packed point description for the kernels: 4 bits per axis give the index of
  // the coordinate in the per-region value table (0 = centre, 1..5 = +G[0..4],
  // 6..10 = -G[0..4]); bits 60..63 hold the generator set.
  std::vector<uint64_t> code;
};

int feval_count(int ndim);
RuleTable make_rule(int ndim);

// Prefix tries of the two halves of the points' per-axis codes, for
// integrands f = L * R with L the product of the factors of axes 0..m-1 and R
// that of axes m..d-1 (m = d / 2), each half in axis order.  In a half
// starting at axis a, a depth-k node is a distinct code prefix
// (c_a..c_{a+k-1}); its value is its parent's value times the factor of axis
// a+k-1 at code c_{a+k-1}, so each half product is formed with exactly the
// roundings of the definition, once per distinct prefix.  Depth-1 node i is
// code i.  `inner` lists, for depth k = 2, 3, ...: the left half's depth-k
// entries (while k <= m), then the right half's (while k <= d - m); entry =
// parent index (12 bits) | code << 12.  `leaf` gives per point, in rule
// order: left node index at depth m | right node index at depth d - m << 12 |
// generator set << 24.  A half of k axes has feval_count(k) nodes at depth k
// (feval_count(1) = 11).
void split_trie(const RuleTable& r, std::vector<uint16_t>* inner, std::vector<uint32_t>* leaf);

// A = .5 + g and B = .5 - g for the 11 coordinate codes, as the reference
// computes them per point (Sample.cuh:126-130).
void code_coefficients(const RuleTable& r, double* A, double* B);

}  // namespace pg
