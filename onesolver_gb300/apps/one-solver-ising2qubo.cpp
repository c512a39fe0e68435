// one-solver-ising2qubo -- Ising COO file -> QUBO file.
//
// Replaces benchmarks/annealing/scripts/convert_qbsolv_to_coo.py (dimod
// BQM.from_coo -> change_vartype("BINARY") -> relabel to 0-based -> "p qubo"
// text) so that droplet instances and generated Ising models need no Python
// dependency; the conversion itself is os_ising_to_qubo_text. The constant
// offset (E_ising = E_qubo + offset) is printed, not written.
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include "../apps/cli_options.hpp"
#include "onesolver.h"

int main(int argc, char *argv[]) {
  try {
    cli::Options options;
    options.add_flag("help", "produce help message");
    options.add("input", "Ising model in COO form (\"i j bias\", variables from 1)");
    options.add("output", "QUBO file to write");
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
    std::ifstream in(options.get("input"), std::ios::binary);
    if (!in) {
      std::cerr << "can not open input file: " << options.get("input") << std::endl;
      return -1;
    }
    const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    size_t len = 0;
    double offset = 0.0;
    if (os_ising_to_qubo_text(text.data(), text.size(), nullptr, 0, &len, &offset) != OS_OK) {
      std::cerr << "error: " << os_last_error() << std::endl;
      return 1;
    }
    std::vector<char> out(len);
    if (os_ising_to_qubo_text(text.data(), text.size(), out.data(), out.size(), &len, &offset) != OS_OK) {
      std::cerr << "error: " << os_last_error() << std::endl;
      return 1;
    }
    std::ofstream of(options.get("output"), std::ios::binary);
    of.write(out.data(), (std::streamsize)len);
    std::cout.precision(17);
    std::cout << "offset " << offset << std::endl;
  } catch (std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
