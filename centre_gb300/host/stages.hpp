// stages.hpp -- the reference's three pipeline stages over the GPU library.
//
// Same call surface as the reference: each stage is built from the parsed
// inputs and has run() (src/Discretizer.h:36-60, src/EntropyCalculator.h:
// 72-125, src/EntropyScorer.h:14-21); the stages talk only through the files
// in the output path, with the reference's names and layouts:
//   bin_{bonds,angles,torsions}.nc      (src/Netcdf_TrjInt.cpp:542-755)
//   entcontri_{bnd,ang,tor}-1d.nc, entcontri_{bnd,ang,tor,ba,bd,ad}-2d.nc
//                                       (src/Netcdf_EntContri.cpp:577-769)
//   MIE-/MIST-<est>_convergence_b-<nb>.<ext>, Tree-MIST-<est>_b-<nb>_s-<k>.<ext>
//                                       (src/EntropyScorer.cpp:571-866)
// All arithmetic runs in libcentre_gpu through the C ABI of centre_gpu.h;
// these classes read and write files and arrange the calls.
#pragma once

#include <string>

#include "centre_gpu.h"
#include "inputs.hpp"

namespace centre_host {

// A library context on one device, released on destruction.
class Gpu {
 public:
  explicit Gpu(int device);
  ~Gpu();
  Gpu(const Gpu &) = delete;
  Gpu &operator=(const Gpu &) = delete;
  bool ok() const { return ctx_ != nullptr; }
  centre_ctx *ctx() const { return ctx_; }
  // "what: status text: detail" for a failed call
  std::string error(int rc, const std::string &what) const;
  const std::string &create_error() const { return create_error_; }

 private:
  centre_ctx *ctx_ = nullptr;
  std::string create_error_;
};

class Discretizer {
 public:
  Discretizer(const Inputs &inputs, Gpu &gpu) : in_(inputs), gpu_(gpu) {}
  bool run(std::string *err);

 private:
  bool run_type(int bat_type, std::string *err);
  const Inputs &in_;
  Gpu &gpu_;
};

class EntropyCalculator {
 public:
  EntropyCalculator(const Inputs &inputs, Gpu &gpu) : in_(inputs), gpu_(gpu) {}
  bool run(std::string *err);

 private:
  const Inputs &in_;
  Gpu &gpu_;
};

class EntropyScorer {
 public:
  EntropyScorer(const Inputs &inputs, Gpu &gpu) : in_(inputs), gpu_(gpu) {}
  bool run(std::string *err);

 private:
  const Inputs &in_;
  Gpu &gpu_;
};

// Neighbour lists chosen from the data by the learned pair screen
// (centre_gpu_screen) instead of a neighbor file: reads the bin files, keeps
// `nneigh` partners per DOF, replaces `inputs.neighbours` and writes the
// lists to `path` in the reference's neighbour-file grammar
// (src/Centre.cpp:459-593) so the reference can score the same pairs.
bool learn_neighbours(Inputs &inputs, Gpu &gpu, uint32_t nneigh, const std::string &path,
                      std::string *err);

// File helpers shared with the command-line tool.
std::string out_path(const Inputs &in, const std::string &name);

}  // namespace centre_host
