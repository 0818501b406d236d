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

// Prefix trie of the points' per-axis codes, for integrands that are a
// left-to-right product of per-axis factors: a depth-k node is a distinct
// prefix (c_0..c_{k-1}); its value is its parent's value times the factor of
// axis k-1 at code c_{k-1}, so every point's product is formed with exactly
// the roundings of v = f_0 * f_1 * ... * f_{d-1}, sharing common prefixes.
// Depth-1 node i is code i.  Entries for depths 2..d follow each other; entry
// = parent index (12 bits) | code << 12; depth d lists the points in rule
// order.  Depth k has feval_count(k) nodes (feval_count(1) = 11).
std::vector<uint16_t> prefix_trie(const RuleTable& r);

// A = .5 + g and B = .5 - g for the 11 coordinate codes, as the reference
// computes them per point (Sample.cuh:126-130).
void code_coefficients(const RuleTable& r, double* A, double* B);

}  // namespace pg
