// one-solver-anneal -- simulated annealing CLI on the GPU.
//
// Same flags, defaults, messages and exit codes as the reference's
// app/one-solver-anneal.cpp (options :55-72, validation :83-115, echo
// :117-127, schedules :153-161, run and save :163-170, errors :171-176),
// with --device-type gpu (the default here: this library has no host/cpu
// backend) and additive options for the new solver features.
#include <fstream>
#include <iostream>

#include "../apps/cli_options.hpp"
#include "onesolver/annealing.hpp"
#include "onesolver/devices.hpp"
#include "onesolver/qubo.hpp"
#include "onesolver/solution.hpp"

int main(int argc, char *argv[]) {
  try {
    cli::Options options;
    options.add_flag("help", "produce help message");
    options.add("input", "input file");
    options.add("output", "output file");
    options.add("num-iter", "100", "number of iterations of the algorithm");
    options.add("num-tries", "100", "number of trajectories to try");
    options.add("schedule-type", "geometric", "type of beta schedule tu use, either linear or geometric");
    options.add("beta-min", "0.1", "minimum value of beta in the annealing schedule (default 0.1)");
    options.add("beta-max", "1", "maximum value of beta in the annealing schedule (default 1.0)");
    options.add("device-type", "gpu", "device type to use (gpu; cpu and host are not built)");
    options.add("sweeps-per-beta", "1", "steps per beta value");
    options.add("site-order", "random", "random (one random site per step) or sequential (one sweep per step)");
    options.add("acceptance", "reference", "reference (exp((E-E')/beta) > u) or physical (exp(-beta dE) > u)");
    options.add("seed", "1234", "random seed");
    options.add("resync-every", "0", "steps between FP64 local-field resyncs (0 = end only)");
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
    const std::string schedule_type = options.get("schedule-type"), device_type = options.get("device-type");
    const unsigned num_iter = (unsigned)options.get_uint("num-iter");
    const unsigned num_tries = (unsigned)options.get_uint("num-tries");
    const double beta_min = options.get_double("beta-min"), beta_max = options.get_double("beta-max");

    if (device_type != "cpu" && device_type != "gpu" && device_type != "host") {
      std::cerr << "Unknown device type: " << device_type << std::endl;
      return -1;
    }
    if (schedule_type != "linear" && schedule_type != "geometric") {
      std::cerr << "Unknown beta schedule: " << schedule_type << std::endl;
      return -1;
    }
    if (beta_max < 0 || beta_min < 0) {
      std::cerr << "Invalid schedule, both ends of beta range need to be positive" << std::endl;
      return -1;
    }
    if (beta_min >= beta_max) {
      std::cerr << "Invalid schedule, initial beta is not lesser than final beta" << std::endl;
      return -1;
    }
    sa::Options opt;
    const std::string order = options.get("site-order"), acc = options.get("acceptance");
    if (order != "random" && order != "sequential") {
      std::cerr << "Unknown site order: " << order << std::endl;
      return -1;
    }
    if (acc != "reference" && acc != "physical") {
      std::cerr << "Unknown acceptance rule: " << acc << std::endl;
      return -1;
    }
    opt.site_order = order == "random" ? OS_SITES_RANDOM : OS_SITES_SEQUENTIAL;
    opt.acceptance = acc == "reference" ? OS_ACCEPT_REFERENCE : OS_ACCEPT_PHYSICAL;
    opt.seed = std::stoull(options.get("seed"));
    opt.resync_every = (int)options.get_uint("resync-every");
    const int sweeps_per_beta = (int)options.get_uint("sweeps-per-beta");

    std::cout << "Reading input from: " << input_file << std::endl;
    std::cout << "Output will be saved to: " << output_file << std::endl;
    std::cout << "Schedule type: " << schedule_type << std::endl;
    std::cout << "Beta range: [" << beta_min << ", " << beta_max << "]" << std::endl;
    std::cout << "Number of iterations: " << num_iter << std::endl;
    std::cout << "Number of tries: " << num_tries << std::endl;

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

    std::vector<double> beta_schedule(num_iter);
    if (schedule_type == "linear")
      sa::construct_linear_beta_schedule(beta_schedule, beta_min, beta_max, num_iter);
    else
      sa::construct_geometric_beta_schedule(beta_schedule, beta_min, beta_max, num_iter);

    auto solution = sa::anneal(instance, *q_ptr, beta_schedule, (int)num_iter, num_tries, sweeps_per_beta, opt);
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
