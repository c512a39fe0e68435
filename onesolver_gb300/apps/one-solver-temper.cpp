// one-solver-temper -- parallel tempering and population annealing CLI on the
// GPU (--method pt | pa).
//
// No counterpart in the reference, whose annealing benchmark names parallel
// tempering and population annealing as the next solvers
// (benchmarks/annealing/performance.md:52-59).
// Input, output, device selection, messages and the result CSV follow
// app/one-solver-anneal.cpp so that the two tools are interchangeable in a
// pipeline; the schedule options become a geometric ladder of inverse
// temperatures (pt) or a linear annealing schedule of num-temps steps (pa).
#include <fstream>
#include <iostream>

#include "../apps/cli_options.hpp"
#include "onesolver/devices.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/solution.hpp"
#include "onesolver/tempering.hpp"

int main(int argc, char *argv[]) {
  try {
    cli::Options options;
    options.add_flag("help", "produce help message");
    options.add("input", "input file");
    options.add("output", "output file");
    options.add("method", "pt", "pt (parallel tempering) or pa (population annealing)");
    options.add("num-temps", "24", "number of temperatures (pt: replicas per chain; pa: schedule steps)");
    options.add("population", "16384", "pa: number of replicas");
    options.add("num-chains", "32", "number of independent replica chains");
    options.add("num-rounds", "1000", "number of exchange rounds");
    options.add("sweeps-per-round", "5", "sweeps of every replica between exchange rounds (pa: per step)");
    options.add("beta-min", "0.05", "smallest inverse temperature (pt: geometric ladder; pa: linear schedule)");
    options.add("beta-max", "3", "largest inverse temperature (pt: geometric ladder; pa: linear schedule)");
    options.add("device-type", "gpu", "device type to use (gpu; cpu and host are not built)");
    options.add("seed", "1234", "random seed");
    options.add("resync-every", "100", "rounds between FP64 local-field resyncs (0 = end only)");
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
    const double beta_min = options.get_double("beta-min"), beta_max = options.get_double("beta-max");
    const int num_temps = (int)options.get_uint("num-temps");
    if (device_type != "cpu" && device_type != "gpu" && device_type != "host") {
      std::cerr << "Unknown device type: " << device_type << std::endl;
      return -1;
    }
    if (beta_max <= 0 || beta_min <= 0) {
      std::cerr << "Invalid ladder, both ends of beta range need to be positive" << std::endl;
      return -1;
    }
    if (beta_min > beta_max) {
      std::cerr << "Invalid ladder, beta-min is greater than beta-max" << std::endl;
      return -1;
    }
    if (num_temps < 1) {
      std::cerr << "Invalid ladder, num-temps must be positive" << std::endl;
      return -1;
    }
    const std::string method = options.get("method");
    if (method != "pt" && method != "pa") {
      std::cerr << "Unknown method: " << method << std::endl;
      return -1;
    }
    pt::Options opt;
    opt.num_chains = (unsigned)options.get_uint("num-chains");
    opt.num_rounds = (int)options.get_uint("num-rounds");
    opt.sweeps_per_round = (int)options.get_uint("sweeps-per-round");
    opt.seed = std::stoull(options.get("seed"));
    opt.resync_every = (int)options.get_uint("resync-every");

    std::cout << "Reading input from: " << input_file << std::endl;
    std::cout << "Output will be saved to: " << output_file << std::endl;
    if (method == "pt") {
      std::cout << "Beta ladder: " << num_temps << " geometric values in [" << beta_min << ", " << beta_max << "]"
                << std::endl;
      std::cout << "Chains: " << opt.num_chains << ", rounds: " << opt.num_rounds
                << ", sweeps per round: " << opt.sweeps_per_round << std::endl;
    } else {
      std::cout << "Beta schedule: " << num_temps << " linear steps in [" << beta_min << ", " << beta_max << "]"
                << std::endl;
      std::cout << "Population: " << options.get_uint("population") << ", sweeps per step: " << opt.sweeps_per_round
                << std::endl;
    }

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

    qubo::Solution solution = [&] {
      if (method == "pt") return pt::temper(instance, *q_ptr, pt::geometric_ladder(beta_min, beta_max, num_temps), opt);
      pa::Options po;
      po.population = (unsigned)options.get_uint("population");
      po.sweeps_per_beta = opt.sweeps_per_round;
      po.seed = opt.seed;
      po.resync_every = opt.resync_every;
      std::vector<double> schedule(num_temps);
      for (int k = 0; k < num_temps; ++k)
        schedule[k] = num_temps == 1 ? beta_max : beta_min + (beta_max - beta_min) * k / (double)(num_temps - 1);
      return pa::anneal(instance, *q_ptr, schedule, po);
    }();
    std::ofstream results_file(output_file);
    solution.save(results_file);
    results_file.close();
  } catch (std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  } catch (...) {
    std::cerr << "Exception of unknown type!\n";
    return 1;
  }
  return 0;
}
