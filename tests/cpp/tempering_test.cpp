// Host-side pieces of include/onesolver/tempering.hpp (no GPU): the model ->
// CSR conversion that pt::temper and pa::anneal hand to the C ABI, and the
// geometric ladder. Prints "ok" or one line per failed check.
#include <cmath>
#include <cstdio>

#include "onesolver/tempering.hpp"

static int failures = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                                 \
    }                                                             \
  } while (0)

int main() {
  // Linear terms on the diagonal; couplings (i < j) in both triangles, columns
  // ascending; zero couplings and keys with i >= j dropped, as the flatten of
  // the reference keeps only i < j keys (qubo_helpers.hpp:26-44).
  qubo::LinearCoef<int, double> lin{{0, -1.5}, {3, 2.0}};
  qubo::QuadraticCoef<int, double> quad{{{0, 2}, 4.0}, {{0, 1}, -1.0}, {{1, 3}, 0.5},
                                        {{2, 1}, 9.0}, {{1, 2}, 0.0}};
  qubo::QUBOModel<int, double> m(lin, quad);
  m.set_nodes(4);
  const pt::Csr c = pt::to_csr(m);
  CHECK(c.n == 4);
  CHECK((c.row_ptr == std::vector<int32_t>{0, 2, 4, 5, 6}));
  CHECK((c.col == std::vector<int32_t>{1, 2, 0, 3, 0, 1}));
  CHECK((c.val == std::vector<double>{-1.0, 4.0, -1.0, 0.5, 4.0, 0.5}));
  CHECK((c.diag == std::vector<double>{-1.5, 0.0, 0.0, 2.0}));

  const std::vector<double> b = pt::geometric_ladder(0.1, 6.4, 7);
  CHECK(b.size() == 7 && b[0] == 0.1);
  for (int k = 1; k < 7; ++k) CHECK(std::fabs(b[k] / b[k - 1] - 2.0) < 1e-12);
  CHECK(pt::geometric_ladder(0.5, 3.0, 1) == std::vector<double>{0.5});

  if (failures == 0) std::printf("ok\n");
  return failures ? 1 : 0;
}
