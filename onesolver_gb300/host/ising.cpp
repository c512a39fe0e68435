// ising.cpp -- Ising -> QUBO conversion of COO text files.
//
// Replaces benchmarks/annealing/scripts/convert_qbsolv_to_coo.py, which reads
// an Ising model in COO form with dimod (BQM.from_coo(..., vartype="SPIN"):
// lines "i j bias", 1-based variables, i == j a linear bias), changes it to
// binary variables, relabels the variables to 0-based (:24-25) and writes
// "p qubo 0 N N C" followed by "i j coef" for every (i, j) of to_qubo() in
// sorted order (:27-36). With s = 2 x - 1, the published change of variables
// gives
//   Q_ii = 2 h_i - 2 sum_j J_ij,   Q_ij = 4 J_ij (i < j),
//   offset = sum_{i<j} J_ij - sum_i h_i,
// so that E_ising(s) = E_qubo(x) + offset; the offset is returned apart (the
// qbsolv format has none, and the reference's plots drop it, plot.py:32).
// Coefficients are written as the shortest decimal that reads back to the
// same double, as Python's float formatting does.
#include <charconv>
#include <cmath>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "errors.hpp"
#include "onesolver.h"

namespace {

std::string shortest(double v) {
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof buf, v);
  std::string s(buf, r.ptr);
  // Python prints integral floats with a trailing ".0"
  if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
  return s;
}

struct Converted {
  int n = 0;
  std::map<std::pair<int, int>, double> q;  // (i, j), i <= j, 0-based
  double offset = 0.0;
};

Converted convert(const char *text, size_t len) {
  std::map<int, double> h;
  std::map<std::pair<int, int>, double> J;
  int maxv = 0;
  std::istringstream in(std::string(text, len));
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    size_t p = line.find_first_not_of(" \t\r");
    if (p == std::string::npos || line[p] == '#' || line[p] == 'c') continue;
    std::istringstream ls(line);
    long long i = 0, j = 0;
    double v = 0.0;
    std::string rest;
    if (!(ls >> i >> j >> v) || (ls >> rest))
      throw std::invalid_argument("line " + std::to_string(lineno) + ": expected \"i j bias\"");
    if (i < 1 || j < 1 || i > (1 << 24) || j > (1 << 24))
      throw std::invalid_argument("line " + std::to_string(lineno) + ": variables are numbered from 1");
    if (!std::isfinite(v)) throw std::invalid_argument("line " + std::to_string(lineno) + ": bias is not finite");
    maxv = std::max(maxv, (int)std::max(i, j));
    if (i == j) {
      h[(int)i] += v;
    } else {
      const int a = (int)std::min(i, j), b = (int)std::max(i, j);
      J[{a, b}] += v;
    }
  }
  // Variables: every index that appears (dimod keeps only those), relabelled
  // i -> i - 1 as the reference script does.
  std::map<int, int> present;
  for (auto &kv : h) present[kv.first] = 1;
  for (auto &kv : J) present[kv.first.first] = present[kv.first.second] = 1;
  if (maxv == 0) throw std::invalid_argument("no variables");
  Converted c;
  c.n = (int)present.size();
  std::map<int, double> lin;
  for (auto &kv : present) lin[kv.first] = 2.0 * (h.count(kv.first) ? h[kv.first] : 0.0);
  double sum_h = 0.0, sum_j = 0.0;
  for (auto &kv : h) sum_h += kv.second;
  for (auto &kv : J) {
    lin[kv.first.first] -= 2.0 * kv.second;
    lin[kv.first.second] -= 2.0 * kv.second;
    sum_j += kv.second;
    c.q[{kv.first.first - 1, kv.first.second - 1}] = 4.0 * kv.second;
  }
  for (auto &kv : lin) c.q[{kv.first - 1, kv.first - 1}] = kv.second;
  c.offset = sum_j - sum_h;
  return c;
}

}  // namespace

extern "C" {

os_status os_ising_to_qubo_text(const char *ising_text, size_t len, char *out, size_t cap, size_t *len_out,
                                double *offset) {
  return os::guard([&] {
    OS_REQUIRE(ising_text && len_out, "null argument");
    const Converted c = convert(ising_text, len);
    size_t couplers = 0;
    for (auto &kv : c.q) couplers += kv.first.first != kv.first.second;
    std::string s = "p qubo 0 " + std::to_string(c.n) + " " + std::to_string(c.n) + " " +
                    std::to_string(couplers) + "\n";
    for (auto &kv : c.q)
      s += std::to_string(kv.first.first) + " " + std::to_string(kv.first.second) + " " + shortest(kv.second) +
           "\n";
    *len_out = s.size();
    if (offset) *offset = c.offset;
    if (out) {
      OS_REQUIRE(cap >= s.size(), "output buffer holds %zu bytes, %zu needed", cap, s.size());
      std::memcpy(out, s.data(), s.size());
    }
  });
}

}  // extern "C"
