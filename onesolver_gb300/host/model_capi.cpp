// model_capi.cpp -- C ABI of the model and file IO (host only, no GPU).
//
// Exposes the C++ mirror of qubo::QUBOModel (include/onesolver/qubo.hpp),
// helpers::flatten_qubo and qubo::Solution::save through os_model_* and
// os_solution_csv, so that non-C++ callers (and the test suite) run the same
// parser and writers the CLIs use.
#include <cstring>
#include <fstream>
#include <sstream>

#include "errors.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/qubo_helpers.hpp"
#include "onesolver/solution.hpp"

struct os_model {
  qubo::QUBOModel<int, double> model;
  explicit os_model(qubo::QUBOModel<int, double> &&m) : model(std::move(m)) {}
};

namespace {

os_status parse_into(const char *b, const char *e, os_model **out) {
  return os::guard([&] {
    OS_REQUIRE(out != nullptr, "null output");
    try {
      *out = new os_model(qubo::parse_qubo(b, e));
    } catch (const std::invalid_argument &ex) {
      os::throw_error(OS_PARSE_ERROR, "%s", ex.what());
    }
  });
}

void copy_out(const std::string &s, char *out, size_t cap, size_t *len_out) {
  if (len_out) *len_out = s.size();
  OS_REQUIRE(out != nullptr && cap > s.size(), "output buffer too small (%zu bytes needed)",
             s.size() + 1);
  std::memcpy(out, s.c_str(), s.size() + 1);
}

}  // namespace

extern "C" {

os_status os_model_parse(const char *text, size_t len, os_model **out) {
  if (!text && len) return os::fail(OS_INVALID_ARG, "null text");
  const char *b = text ? text : "";
  return parse_into(b, b + len, out);
}

os_status os_model_load_file(const char *path, os_model **out) {
  if (!path) return os::fail(OS_INVALID_ARG, "null path");
  std::ifstream f(path, std::ios::binary);
  if (!f) return os::fail(OS_INVALID_ARG, "can not open input file: %s", path);
  std::stringstream ss;
  ss << f.rdbuf();
  std::string text = ss.str();
  return parse_into(text.data(), text.data() + text.size(), out);
}

void os_model_free(os_model *model) { delete model; }

int64_t os_model_nodes(const os_model *m) { return m ? (int64_t)m->model.get_nodes() : -1; }

int64_t os_model_num_linear(const os_model *m) {
  return m ? (int64_t)m->model.linear_terms().size() : -1;
}

int64_t os_model_num_quadratic(const os_model *m) {
  return m ? (int64_t)m->model.quadratic_terms().size() : -1;
}

double os_model_get_variable(const os_model *m, int32_t i) {
  return m ? m->model.get_variable(i) : 0.0;
}

double os_model_get_connection(const os_model *m, int32_t i, int32_t j) {
  return m ? m->model.get_connection(std::make_pair((int)i, (int)j)) : 0.0;
}

os_status os_model_flatten(const os_model *m, double *out, size_t cap) {
  return os::guard([&] {
    OS_REQUIRE(m && out, "null argument");
    const size_t n = m->model.get_nodes();
    OS_REQUIRE(cap >= n * n, "output holds %zu values, %zu needed", cap, n * n);
    helpers::flatten_qubo_into(m->model, out);
  });
}

os_status os_model_str(const os_model *m, char *out, size_t cap, size_t *len_out) {
  return os::guard([&] {
    OS_REQUIRE(m != nullptr, "null model");
    copy_out(m->model.str(), out, cap, len_out);
  });
}

os_status os_solution_csv(const char *state, int32_t n, double energy, char *out, size_t cap,
                          size_t *len_out) {
  return os::guard([&] {
    OS_REQUIRE((state || n == 0) && n >= 0, "bad state");
    qubo::Solution sol(state, state + n, energy);
    std::ostringstream ss;
    sol.save(ss);
    copy_out(ss.str(), out, cap, len_out);
  });
}

}  // extern "C"
