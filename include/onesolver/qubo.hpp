// qubo.hpp -- the QUBO model class and .qubo reader of oneSolver, without
// Boost.
//
// Mirrors include/model/qubo.hpp of quantumz-io/oneSolver: the same class
// (qubo::QUBOModel<NodeType, CoefType>), the same coefficient stores
// (std::unordered_map keyed by node / node pair with helpers::hash_pair), the
// same builder validation (QUBOBuilder, qubo.hpp:282-379) and the same file
// grammar (parse_qubo, qubo.hpp:392-417). The reference parses with
// Boost.Spirit; this header hand-writes a recursive-descent reader that
// accepts and rejects the same inputs:
//
//   file        := comment* header? (comment | coefficient)*
//   comment     := 'c' printable* (eol | eoi)
//   header      := "p qubo" uint uint(max_nodes) uint(num_linear)
//                  uint(num_quadratic) (eol | eoi)
//   coefficient := index index real (eol | eoi)
//   index       := uint ' '          (one literal space right after digits)
//
// with blanks (space, tab) skipped before every token, eol = "\r\n" | "\n" |
// "\r", and the whole input consumed. A failure anywhere throws
// std::invalid_argument("Parsing failed. Incorrect file format."), a
// lower-triangle entry throws from the builder as the reference does.
// Decimal values are converted with strtod (correctly rounded).
#ifndef ONESOLVER_QUBO_HPP_
#define ONESOLVER_QUBO_HPP_

#include <cctype>
#include <charconv>
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <istream>
#include <iterator>
#include <ostream>
#include <set>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>

namespace helpers {

// helpers::hash_pair, include/helpers/hash.hpp:19-35, the hash of the
// coupler map. The reference xors the element hashes; with std::hash<int>
// the identity, every coupler (i, j) of a Chimera cell or any banded pattern
// then falls into a few buckets and the map degrades to linear chains (15 ms
// to parse a 2,048-spin file). Here the two hashes are mixed (a multiply by
// the 64-bit golden ratio and a boost-style combine); only the hash values
// and the map's iteration order differ, not the API.
struct hash_pair {
  template <class T1, class T2>
  size_t operator()(const std::pair<T1, T2> &p) const {
    const uint64_t a = (uint64_t)std::hash<T1>{}(p.first) * 0x9E3779B97F4A7C15ull;
    const uint64_t b = (uint64_t)std::hash<T2>{}(p.second);
    return (size_t)(a ^ (b + 0x9E3779B97F4A7C15ull + (a << 6) + (a >> 2)));
  }
};

// helpers::insert_model, include/helpers/insert.hpp:27-38: insert or
// overwrite.
template <class Key, class CoefType, class Hash>
void insert_model(std::unordered_map<Key, CoefType, Hash> &um, const Key &key,
                  const CoefType &val) {
  um[key] = val;
}

}  // namespace helpers

namespace qubo {

template <class NodeType, class CoefType>
using LinearCoef = std::unordered_map<NodeType, CoefType>;

template <class NodeType, class CoefType>
using QuadraticCoef =
    std::unordered_map<std::pair<NodeType, NodeType>, CoefType, helpers::hash_pair>;

// qubo::QUBOModel, include/model/qubo.hpp:53-163.
template <class NodeType, class CoefType> class QUBOModel {
protected:
  LinearCoef<NodeType, CoefType> linear;
  QuadraticCoef<NodeType, CoefType> quadratic;
  unsigned long num_nodes = 0;

public:
  QUBOModel(LinearCoef<NodeType, CoefType> &c_linear,
            QuadraticCoef<NodeType, CoefType> &c_quadratic)
      : linear(c_linear), quadratic(c_quadratic) {}

  // "QUBO model" followed by " i--i:v " per linear term and "i--j:v" per
  // quadratic term, values through std::to_string (qubo.hpp:182-202).
  std::string str() const {
    std::string s("QUBO model");
    for (auto &qii : linear) {
      s.append(" " + std::to_string(qii.first) + "--" + std::to_string(qii.first) +
               ":" + std::to_string(qii.second) + " ");
    }
    for (auto &qij : quadratic) {
      s.append(std::to_string(qij.first.first) + "--" +
               std::to_string(qij.first.second) + ":" + std::to_string(qij.second));
    }
    return s;
  }

  void add_variable(const NodeType &vi, const CoefType &hi) {
    helpers::insert_model(linear, vi, hi);
  }

  void add_connection(const std::pair<NodeType, NodeType> &connection,
                      const CoefType &Ji) {
    helpers::insert_model(quadratic, connection, Ji);
  }

  // A missing key reads as 0 (qubo.hpp:216-240).
  const CoefType get_variable(const NodeType &vi) const {
    auto it = linear.find(vi);
    return it == linear.end() ? CoefType(0) : it->second;
  }

  const CoefType get_connection(const std::pair<NodeType, NodeType> &connection) const {
    auto it = quadratic.find(connection);
    return it == quadratic.end() ? CoefType(0) : it->second;
  }

  void set_nodes(int number) { num_nodes = number; }
  unsigned long get_nodes() const { return num_nodes; }

  const LinearCoef<NodeType, CoefType> &linear_terms() const { return linear; }
  const QuadraticCoef<NodeType, CoefType> &quadratic_terms() const { return quadratic; }

  static QUBOModel<int, double> load(std::istream &stream);
};

template <class NodeType, class CoefType>
std::ostream &operator<<(std::ostream &os, const QUBOModel<NodeType, CoefType> &q) {
  os << q.str();
  return os;
}

// QUBOBuilder, include/model/qubo.hpp:282-379: collects coefficients and
// validates the header counts.
struct QUBOBuilder {
private:
  LinearCoef<int, double> linear_c{};
  QuadraticCoef<int, double> quadratic_c{};
  long num_quadratic = -1;
  long num_linear = -1;
  long max_nodes = -1;
  std::set<int> used_nodes;

public:
  // The first occurrence of a key wins (unordered_map::insert), i > j throws.
  void add_element(int i, int j, double coef) {
    if (i == j) {
      linear_c.insert({i, coef});
    } else if (i < j) {
      quadratic_c.insert({{i, j}, coef});
    } else {
      throw std::invalid_argument("Incorrect file, encountered coefficient "
                                  "from lower triangle of QUBO matrix.");
    }
    used_nodes.insert(i);
    used_nodes.insert(j);
  }

  void set_num_quadratic(long value) { num_quadratic = value; }
  void set_num_linear(long value) { num_linear = value; }
  void set_max_nodes(long value) { max_nodes = value; }

  QUBOModel<int, double> build_qubo() {
    if (linear_c.size() == 0 && quadratic_c.size() == 0) {
      throw std::invalid_argument("An empty input, no coefficients defined.");
    }
    if (num_quadratic == -1 || num_linear == -1 || max_nodes == -1) {
      throw std::invalid_argument("No header line or header line misformatted.");
    }
    if (num_linear > max_nodes) {
      throw std::invalid_argument("Number of linear terms is greater than num nodes.");
    }
    if ((long)quadratic_c.size() != num_quadratic) {
      throw std::invalid_argument(
          "Number of quadratic terms is not equal to the declared one.");
    }
    if ((long)linear_c.size() != num_linear) {
      throw std::invalid_argument(
          "Number of linear terms is not equal to the declared one.");
    }
    QUBOModel<int, double> q(linear_c, quadratic_c);
    q.set_nodes(*used_nodes.rbegin() + 1);
    return q;
  }
};

namespace detail {

// Cursor over the input with the reference grammar's token rules.
class QuboReader {
public:
  QuboReader(const char *b, const char *e) : p_(b), end_(e) {}

  bool at_end() const { return p_ == end_; }
  const char *pos() const { return p_; }
  void reset(const char *p) { p_ = p; }

  void skip_blanks() {
    while (p_ != end_ && (*p_ == ' ' || *p_ == '\t')) ++p_;
  }

  // eol | eoi, after skipping blanks.
  bool line_end() {
    skip_blanks();
    if (p_ == end_) return true;
    if (*p_ == '\r') {
      ++p_;
      if (p_ != end_ && *p_ == '\n') ++p_;
      return true;
    }
    if (*p_ == '\n') {
      ++p_;
      return true;
    }
    return false;
  }

  // Unsigned decimal (no sign), failing on overflow of 32 bits.
  bool uint_token(unsigned long &out) {
    skip_blanks();
    const char *q = p_;
    unsigned long long v = 0;
    while (q != end_ && *q >= '0' && *q <= '9') {
      v = v * 10 + (unsigned)(*q - '0');
      if (v > 0xFFFFFFFFull) return false;
      ++q;
    }
    if (q == p_) return false;
    out = (unsigned long)v;
    p_ = q;
    return true;
  }

  // index := uint followed immediately by one space.
  bool index_token(long &out) {
    const char *save = p_;
    unsigned long v;
    if (!uint_token(v) || p_ == end_ || *p_ != ' ' || v > (unsigned long)INT_MAX) {
      p_ = save;
      return false;
    }
    ++p_;
    out = (long)v;
    return true;
  }

  // real := sign? (digits ('.' digits?)? | '.' digits) exponent?
  //         | sign? ("nan" | "inf" | "infinity"), case-insensitive.
  bool real_token(double &out) {
    skip_blanks();
    const char *q = p_;
    if (q != end_ && (*q == '+' || *q == '-')) ++q;
    const char *mant = q;
    auto ieq = [&](const char *word) {
      const char *r = q;
      for (const char *w = word; *w; ++w, ++r)
        if (r == end_ || std::tolower((unsigned char)*r) != *w) return (const char *)nullptr;
      return r;
    };
    const char *special = nullptr;
    if ((special = ieq("infinity")) || (special = ieq("inf")) || (special = ieq("nan"))) {
      std::string tok(p_, special);
      out = std::strtod(tok.c_str(), nullptr);
      p_ = special;
      return true;
    }
    bool digits = false;
    while (q != end_ && std::isdigit((unsigned char)*q)) { ++q; digits = true; }
    if (q != end_ && *q == '.') {
      ++q;
      while (q != end_ && std::isdigit((unsigned char)*q)) { ++q; digits = true; }
    }
    if (!digits) return false;
    if (q != end_ && (*q == 'e' || *q == 'E')) {
      const char *r = q + 1;
      if (r != end_ && (*r == '+' || *r == '-')) ++r;
      const char *ed = r;
      while (r != end_ && std::isdigit((unsigned char)*r)) ++r;
      if (r != ed) q = r;  // an exponent without digits is not consumed
    }
    (void)mant;
    // from_chars is correctly rounded like strtod and reads the buffer in
    // place; it takes no leading '+', which strtod handles.
    const auto r = std::from_chars(*p_ == '+' ? p_ + 1 : p_, q, out);
    if (*p_ == '+' || r.ec != std::errc() || r.ptr != q) {
      std::string tok(p_, q);
      out = std::strtod(tok.c_str(), nullptr);
    }
    p_ = q;
    return true;
  }

  // comment := 'c' printable* (eol | eoi)
  bool comment() {
    const char *save = p_;
    skip_blanks();
    if (p_ == end_ || *p_ != 'c') { p_ = save; return false; }
    ++p_;
    while (p_ != end_ && (std::isprint((unsigned char)*p_) || *p_ == '\t')) ++p_;
    if (!line_end()) { p_ = save; return false; }
    return true;
  }

  // header := "p qubo" uint uint uint uint (eol | eoi)
  bool header(QUBOBuilder &b) {
    const char *save = p_;
    skip_blanks();
    static const char lit[] = "p qubo";
    for (const char *l = lit; *l; ++l, ++p_) {
      if (p_ == end_ || *p_ != *l) { p_ = save; return false; }
    }
    unsigned long target, max_nodes, num_linear, num_quadratic;
    if (!uint_token(target)) { p_ = save; return false; }
    if (!uint_token(max_nodes)) { p_ = save; return false; }
    b.set_max_nodes((long)(int)max_nodes);
    if (!uint_token(num_linear)) { p_ = save; return false; }
    b.set_num_linear((long)(int)num_linear);
    if (!uint_token(num_quadratic)) { p_ = save; return false; }
    b.set_num_quadratic((long)(int)num_quadratic);
    if (!line_end()) { p_ = save; return false; }
    return true;
  }

  // coefficient := index index real (eol | eoi); the builder sees the triple
  // before the line end is checked, as the semantic action does.
  bool coefficient(QUBOBuilder &b) {
    const char *save = p_;
    long i, j;
    double v;
    if (!index_token(i)) { p_ = save; return false; }
    if (!index_token(j)) { p_ = save; return false; }
    if (!real_token(v)) { p_ = save; return false; }
    b.add_element((int)i, (int)j, v);
    if (!line_end()) { p_ = save; return false; }
    return true;
  }

private:
  const char *p_;
  const char *end_;
};

}  // namespace detail

// parse_qubo, include/model/qubo.hpp:392-417.
inline QUBOModel<int, double> parse_qubo(const char *first, const char *last) {
  QUBOBuilder builder;
  detail::QuboReader r(first, last);
  while (!r.at_end() && r.comment()) {
  }
  if (!r.at_end()) r.header(builder);
  while (!r.at_end()) {
    if (r.comment()) continue;
    if (r.coefficient(builder)) continue;
    break;
  }
  if (!r.at_end()) {
    throw std::invalid_argument("Parsing failed. Incorrect file format.");
  }
  return builder.build_qubo();
}

// QUBOModel::load, include/model/qubo.hpp:425-430.
template <class NodeType, class CoefType>
QUBOModel<int, double> QUBOModel<NodeType, CoefType>::load(std::istream &stream) {
  std::string text((std::istreambuf_iterator<char>(stream)),
                   std::istreambuf_iterator<char>());
  return parse_qubo(text.data(), text.data() + text.size());
}

}  // namespace qubo

#endif  // ONESOLVER_QUBO_HPP_
