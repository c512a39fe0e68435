// cli_options.hpp -- a small option reader with the conventions the
// reference's Boost.program_options CLIs accept: "--name value" and
// "--name=value", "--help", defaults shown as "(=value)".
#ifndef ONESOLVER_CLI_OPTIONS_HPP_
#define ONESOLVER_CLI_OPTIONS_HPP_

#include <cstdio>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace cli {

struct Option {
  std::string name, help, def;
  bool has_default = false, flag = false;
};

class Options {
public:
  void add(const std::string &name, const std::string &help) { opts_.push_back({name, help, "", false, false}); }
  void add(const std::string &name, const std::string &def, const std::string &help) {
    opts_.push_back({name, help, def, true, false});
  }
  void add_flag(const std::string &name, const std::string &help) { opts_.push_back({name, help, "", false, true}); }

  // Throws std::invalid_argument on an unknown option or a missing value.
  void parse(int argc, char **argv) {
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i];
      if (a.rfind("--", 0) != 0) throw std::invalid_argument("unexpected argument '" + a + "'");
      std::string name = a.substr(2), value;
      bool inline_value = false;
      auto eq = name.find('=');
      if (eq != std::string::npos) {
        value = name.substr(eq + 1);
        name = name.substr(0, eq);
        inline_value = true;
      }
      const Option *o = find(name);
      if (!o) throw std::invalid_argument("unrecognised option '--" + name + "'");
      if (o->flag) {
        values_[name] = "1";
        continue;
      }
      if (!inline_value) {
        if (i + 1 >= argc) throw std::invalid_argument("the required argument for option '--" + name + "' is missing");
        value = argv[++i];
      }
      values_[name] = value;
    }
  }

  bool count(const std::string &name) const { return values_.count(name) != 0; }

  std::string get(const std::string &name) const {
    auto it = values_.find(name);
    if (it != values_.end()) return it->second;
    const Option *o = find(name);
    return o && o->has_default ? o->def : std::string();
  }

  double get_double(const std::string &name) const {
    const std::string v = get(name);
    size_t pos = 0;
    double d = std::stod(v, &pos);
    if (pos != v.size()) throw std::invalid_argument("the argument ('" + v + "') for option '--" + name + "' is invalid");
    return d;
  }

  unsigned long get_uint(const std::string &name) const {
    const std::string v = get(name);
    if (v.empty() || v[0] == '-') throw std::invalid_argument("the argument ('" + v + "') for option '--" + name + "' is invalid");
    size_t pos = 0;
    unsigned long u = std::stoul(v, &pos);
    if (pos != v.size()) throw std::invalid_argument("the argument ('" + v + "') for option '--" + name + "' is invalid");
    return u;
  }

  void print(std::ostream &os, const std::string &title) const {
    os << title << ":\n";
    for (auto &o : opts_) {
      std::string head = "  --" + o.name;
      if (!o.flag) head += o.has_default ? " arg (=" + o.def + ")" : " arg";
      os << head;
      for (size_t k = head.size(); k < 40; ++k) os << ' ';
      os << (head.size() >= 40 ? " " : "") << o.help << "\n";
    }
  }

private:
  const Option *find(const std::string &name) const {
    for (auto &o : opts_)
      if (o.name == name) return &o;
    return nullptr;
  }
  std::vector<Option> opts_;
  std::map<std::string, std::string> values_;
};

}  // namespace cli

#endif  // ONESOLVER_CLI_OPTIONS_HPP_
