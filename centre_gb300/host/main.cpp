// main.cpp -- centre_gpu: the reference's centre_OMP driver (src/main_smp.cpp)
// with the three stages running on the GPU library.
//
//   centre_gpu -i input.cfg [-O] [--device N] [--print-inputs]
//              [--learned-neighbours K]
//
// Same input file and output files as the reference.  Errors end the run
// with a non-zero exit status (the reference exits with status 0 after
// printing an error).  -O overwrites existing output files, as in the
// reference; without it an existing output file is an error.
#include <sys/stat.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "inputs.hpp"
#include "stages.hpp"

using namespace centre_host;

namespace {

const char *arg_value(int argc, char **argv, const char *opt) {
  for (int i = 1; i + 1 < argc; ++i)
    if (std::strcmp(argv[i], opt) == 0) return argv[i + 1];
  return nullptr;
}

bool has_flag(int argc, char **argv, const char *opt) {
  for (int i = 1; i < argc; ++i)
    if (std::strcmp(argv[i], opt) == 0) return true;
  return false;
}

void usage() {
  std::cout << "usage: centre_gpu -i <input.cfg> [-O] [--device N] [--print-inputs]\n"
               "  -i             input file ([control] [discretization] [histogram]\n"
               "                 [vonmiseskde] [entropy] sections, as for centre_OMP)\n"
               "  -O             overwrite existing output files\n"
               "  --device N     CUDA device (default 0)\n"
               "  --print-inputs parse and print the inputs, then stop\n"
               "  --learned-neighbours K\n"
               "                 choose K partners per DOF with the learned pair screen\n"
               "                 (after discretisation) instead of a neighbor file; the\n"
               "                 lists are written to outfilepath/neigh_learned.txt\n";
}

bool exists(const std::string &p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

int main(int argc, char **argv) {
  if (has_flag(argc, argv, "-h") || has_flag(argc, argv, "--help")) {
    usage();
    return 0;
  }
  const char *cfg = arg_value(argc, argv, "-i");
  if (!cfg) {
    std::cerr << "-i inputfile is a required option" << std::endl;
    return 2;
  }
  const bool overwrite = has_flag(argc, argv, "-O");
  const char *dev = arg_value(argc, argv, "--device");
  Inputs in;
  std::string err;
  if (!in.init(cfg, &err)) {
    std::cerr << "input error: " << err << std::endl;
    return 2;
  }
  if (has_flag(argc, argv, "--print-inputs")) {
    std::cout << in.describe();
    return 0;
  }
  bool bad = false;
  for (const std::string &f : in.required_files)
    if (!exists(f)) {
      std::cerr << "Error:: required-file (" << f << ") doesn't exist." << std::endl;
      bad = true;
    }
  for (const std::string &f : in.unwanted_files)
    if (exists(f)) {
      if (!overwrite) {
        std::cerr << "Error:: file-to-write (" << f << ") already exists." << std::endl;
        bad = true;
      } else if (std::remove(f.c_str()) != 0) {
        std::cerr << "Error removing file (" << f << ")" << std::endl;
        return 3;
      }
    }
  if (bad) {
    std::cerr << "To force overwriting existing files use -O option with program" << std::endl;
    return 3;
  }
  Gpu gpu(dev ? std::atoi(dev) : 0);
  if (!gpu.ok()) {
    std::cerr << gpu.create_error() << std::endl;
    return 4;
  }
  std::ofstream info(out_path(in, in.control.infofile).c_str());
  info << "pid " << getpid() << "\n";
  const auto t0 = std::chrono::steady_clock::now();
  auto stage = [&](const char *name, auto &&fn) {
    const auto ts = std::chrono::steady_clock::now();
    std::string e;
    if (!fn(&e)) {
      std::cerr << name << " failed: " << e << std::endl;
      info << name << " FAILED: " << e << std::endl;
      return false;
    }
    const double dt = seconds_since(ts);
    std::printf("TIME: %s: %.4f seconds.\n", name, dt);
    info << name << " COMPLETED " << dt << " s" << std::endl;
    return true;
  };
  Discretizer discretizer(in, gpu);
  if (!stage("Discretization", [&](std::string *e) { return discretizer.run(e); })) return 5;
  if (const char *k = arg_value(argc, argv, "--learned-neighbours")) {
    const std::string path = out_path(in, "neigh_learned.txt");
    if (!stage("Pair screen", [&](std::string *e) {
          return learn_neighbours(in, gpu, (uint32_t)std::atoi(k), path, e);
        }))
      return 5;
  }
  EntropyCalculator calculator(in, gpu);
  if (!stage("Entropy calculation", [&](std::string *e) { return calculator.run(e); })) return 5;
  EntropyScorer scorer(in, gpu);
  if (!stage("Entropy scoring", [&](std::string *e) { return scorer.run(e); })) return 5;
  std::printf("TIME: Total execution: %.4f seconds.\n", seconds_since(t0));
  std::cout << "Execution completed successfully..." << std::endl;
  return 0;
}
