// one-solver-exhaustive -- exhaustive search CLI on the GPU.
//
// Same flags, messages and exit codes as the reference's
// app/one-solver-exhaustive.cpp (options :31-37, validation :48-61, run and
// save :74-100), with --device-type gpu (the default here) and an additive
// --all-minimisers FILE that writes every degenerate minimiser, one CSV row
// each in the Solution::save format.
#include <fstream>
#include <iostream>

#include "../apps/cli_options.hpp"
#include "onesolver/devices.hpp"
#include "onesolver/exhaustive.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/solution.hpp"

int main(int argc, char *argv[]) {
  try {
    cli::Options options;
    options.add_flag("help", "produce help message");
    options.add("input", "input file");
    options.add("output", "output file");
    options.add("device-type", "gpu", "device type to use (gpu; cpu and host are not built)");
    options.add("all-minimisers", "also write every degenerate minimiser to this file");
    options.parse(argc, argv);
    if (options.count("help")) {
      options.print(std::cout, "Allowed options");
      std::cout << std::endl;
      return 0;
    }
    if (!options.count("input")) {
      std::cerr << "No input file provided." << std::endl;
      return -1;
    }
    if (!options.count("output")) {
      std::cerr << "No output file provided." << std::endl;
      return -1;
    }
    const std::string input_file = options.get("input"), output_file = options.get("output");
    const std::string device_type = options.get("device-type");
    if (device_type != "cpu" && device_type != "gpu" && device_type != "host") {
      std::cerr << "Unknown device type: " << device_type << std::endl;
      return -1;
    }
    std::cout << "Reading input from: " << input_file << std::endl;
    std::cout << "Output will be saved to: " << output_file << std::endl;
    std::ifstream qubo_file(input_file);
    if (!qubo_file) {
      std::cerr << "can not open input file: " << input_file << std::endl;
      return -1;
    }
    qubo_file.unsetf(std::ios::skipws);
    auto instance = qubo::QUBOModel<int, double>::load(qubo_file);

    std::unique_ptr<os::Queue> q_ptr;
    try {
      auto selector = devices::construct_device_selector(device_type);
      q_ptr.reset(new os::Queue(selector->device));
    } catch (std::runtime_error &) {
      std::cerr << "No devices of given type could be initialized." << std::endl;
      return 1;
    }
    std::cout << "Using device: " << q_ptr->device_name() << std::endl;

    auto solution = exhaustive::solve(*q_ptr, instance);
    std::ofstream results_file(output_file);
    solution.save(results_file);
    results_file.close();

    if (options.count("all-minimisers")) {
      auto all = exhaustive::solve_all(*q_ptr, instance);
      std::ofstream f(options.get("all-minimisers"));
      const unsigned n = (unsigned)instance.get_nodes();
      for (unsigned i = 0; i < n; ++i) f << i << ',';
      f << "energy" << std::endl;
      for (auto s : all.states) {
        for (unsigned i = 0; i < n; ++i) f << ((s >> i) & 1ull) << ',';
        f << all.energy << std::endl;
      }
    }
  } catch (std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  } catch (...) {
    std::cerr << "Exception of unknown type!\n";
    return 1;
  }
  return 0;
}
