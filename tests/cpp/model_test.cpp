// C++ port of the reference's model unit tests (tests/qubo_test.cpp,
// tests/qubo_helpers_test.cpp, tests/io_test.cpp) against the header-only
// mirror in include/onesolver/. Prints one line per failed check and exits
// non-zero on failure.
#include <cstdio>
#include <sstream>
#include <string>
#include <vector>

#include "onesolver/qubo.hpp"
#include "onesolver/qubo_helpers.hpp"
#include "onesolver/solution.hpp"

static int failures = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                 \
    }                                                             \
  } while (0)

int main() {
  {  // qubo_test.cpp:14-29: add_variable overwrites
    qubo::LinearCoef<int, double> lin{{1, -0.4}, {2, 1.1}, {3, -1.0}, {4, -1.2}};
    qubo::QuadraticCoef<int, double> quad{{{1, 2}, 1.0}, {{1, 3}, 7.2}, {{1, 4}, 1.0},
                                          {{2, 3}, 2.0}, {{2, 4}, 1.9}, {{3, 4}, 3.0}};
    qubo::QUBOModel<int, double> q(lin, quad);
    q.add_variable(1, 20);
    CHECK(q.get_variable(1) == 20);
  }
  {  // qubo_test.cpp:31-40: add_connection
    qubo::LinearCoef<int, double> lin{};
    qubo::QuadraticCoef<int, double> quad{};
    qubo::QUBOModel<int, double> q(lin, quad);
    q.add_connection(std::make_pair(1, 2), 20);
    CHECK(q.get_connection(std::make_pair(1, 2)) == 20);
    CHECK(q.get_connection(std::make_pair(2, 1)) == 0);
  }
  {  // qubo_test.cpp:42-55: str()
    qubo::LinearCoef<int, int> lin{};
    qubo::QuadraticCoef<int, int> quad{};
    qubo::QUBOModel<int, int> q(lin, quad);
    q.add_variable(1, 10);
    q.add_connection(std::make_pair(1, 2), 20);
    CHECK(q.str() == "QUBO model 1--1:10 1--2:20");
  }
  {  // qubo_helpers_test.cpp:12-30: flatten layout
    qubo::LinearCoef<int, double> lin{{0, 0.5}, {1, -2.0}, {2, 1.0}, {4, -1.5}};
    qubo::QuadraticCoef<int, double> quad{{{0, 1}, 1.0}, {{0, 3}, 7.2},  {{1, 4}, -1.0},
                                          {{2, 3}, 2.0}, {{2, 4}, -1.5}, {{3, 4}, -3.5}};
    qubo::QUBOModel<int, double> inst(lin, quad);
    inst.set_nodes(5);
    std::vector<double> expected{0.5, 1.0,  0.0, 7.2, 0.0, 1.0, -2.0, 0.0, 0.0,  -1.0, 0.0,  0.0, 1.0,
                                 2.0, -1.5, 7.2, 0.0, 2.0, 0.0, -3.5, 0.0, -1.0, -1.5, -3.5, -1.5};
    CHECK(helpers::flatten_qubo(inst) == expected);
  }
  {  // io_test.cpp:41-68 via QUBOModel::load on a stream
    std::stringstream ss("c qubo Target MaxNodes NumNodes NumLinks\np qubo 0 100 2 2\nc comment\n"
                         "0 0 -0.5\n0 1 2.0\n1 2 4\n2 2 -0.7\n");
    ss.unsetf(std::ios::skipws);
    auto m = qubo::QUBOModel<int, double>::load(ss);
    CHECK(m.get_nodes() == 3);
    CHECK(m.get_variable(0) == -0.5);
    CHECK(m.get_variable(2) == -0.7);
    CHECK(m.get_connection(std::pair(0, 1)) == 2.0);
    CHECK(m.get_connection(std::pair(1, 2)) == 4.0);
  }
  {  // io_test.cpp:70-83: lower triangle throws std::invalid_argument
    std::stringstream ss("p qubo 0 100 2 2\n0 0 -0.5\n1 0 2.0\n1 2 4\n2 2 -0.7\n");
    bool threw = false;
    try {
      qubo::QUBOModel<int, double>::load(ss);
    } catch (const std::invalid_argument &) {
      threw = true;
    }
    CHECK(threw);
  }
  {  // io_test.cpp:108-118: Solution::save bytes
    char state[] = {0, 1, 1, 0, 1};
    qubo::Solution s(state, state + 5, -12.5);
    std::stringstream out;
    s.save(out);
    CHECK(out.str() == "0,1,2,3,4,energy\n0,1,1,0,1,-12.5\n");
  }
  if (failures == 0) std::printf("ok\n");
  return failures ? 1 : 0;
}
