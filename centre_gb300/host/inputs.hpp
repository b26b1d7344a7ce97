// inputs.hpp -- the reference's INI input file and the DOF/pair sets it
// selects.
//
// Keys, defaults and derived values follow Inputs::Inputs / Inputs::Init
// (src/Inputs.cpp:12-1060) and the file tokenisation of
// Utils::parseConfiguration (src/Utils.cpp:198-270): "[section]" headers,
// "key = v1, v2  # comment" lines, '#' comment lines, a quoted value taken
// whole.  DOF subsets and neighbour lists follow SubsetData and Neighbors
// (src/Centre.cpp:161-593).
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace centre_host {

// Work-set bits (src/Centre.h:96-110).
enum BatSet : uint32_t {
  kNothing = 0, kB1D = 1, kA1D = 2, kD1D = 4, kX1D = 7, kBB2D = 8, kAA2D = 16, kDD2D = 32,
  kXX2D = 63, kBA2D = 64, kBD2D = 128, kAD2D = 256, kXY2D = 511,
};

enum class PdfMethod { kHistogram, kVonMisesKDE };
enum class Method { kMIE, kAMIE, kMIST, kAMIST };
// Estimator codes as the C ABI takes them (CENTRE_ML ... CENTRE_JS).
enum Estimator : uint8_t { kML = 0, kMM = 1, kCS = 2, kJS = 3 };

const char *estimator_name(uint8_t e);

using Config = std::map<std::string, std::vector<std::string>>;

// "section.key" -> values, tokenised as the reference does.
Config parse_config(const std::string &path, bool *ok);

struct ControlParams {
  std::string infilepath, outfilepath, infofile = "progress.info";
  int nsteps = 20;
  bool discretize = true, calcentropy = true, genconvgdata = true;
  unsigned cachedscrtdimspercpu = 5, cacheentcdimspercpu = 10, dscrinfofreq = 25,
           entcinfofreq = 500;
};

struct BatParams {
  std::vector<std::string> fnames;
  std::vector<uint64_t> nframes;
  unsigned nbond = 0, nangle = 0, ndihed = 0;
  uint64_t randseed = 0;
  bool shuffleframes = false, shuffledofs = false, optimizedih = true;
  PdfMethod pdfmethod = PdfMethod::kHistogram;
};

struct VmkdeParams {
  int nmaxconf = 5;
  bool writefreq = false;
  uint32_t writeset = kNothing;
  int writestepstart = 255, writestepstride = 1;
  double kappa = 1.0;
  unsigned sdosteps = 5, sdoiterations = 1000;
  double sdoconvlimit = 0.0001;
};

struct HistParams {
  int nbinref = 0;
  std::vector<uint8_t> bin_schemes;
  bool writefreq = false;
  uint32_t writeset = kNothing;
  int writestepstart = 255, writestepstride = 1;
};

struct EntropyParams {
  uint32_t workset = kXY2D;
  bool shuffleblocks = false;
  int shuffleblocktimes = 1;
  bool usesubset = false, useneighbor = false, jacobian = true;
  std::string subsetfile, neighborfile;
  uint64_t startframe = 0, strideframe = 1, nframe = 0, nframes_eff = 0;
  std::string reportfileext = "csv";
};

// DOF ids taking part per type (0-based ids within the type).
struct Subset {
  std::vector<uint32_t> bonds, angles, torsions;
  uint32_t total_bonds = 0, total_angles = 0, total_torsions = 0;
};

// Pair lists: key id -> partner ids, per block (std::map keeps keys sorted,
// as the reference's maps do).
struct Neighbours {
  std::map<uint32_t, std::vector<uint32_t>> bb, aa, dd, ba, bd, ad;
};

class Inputs {
 public:
  // Parse, fill defaults, read BAT headers for counts and frames, build the
  // subset and neighbour lists.  Returns false with *err on a bad input.
  bool init(const std::string &path, std::string *err);

  ControlParams control;
  BatParams bats;
  VmkdeParams vmkde;
  HistParams hist;
  EntropyParams entropy;
  Method method = Method::kMIST;
  std::vector<uint8_t> estimators;
  Subset subset;
  Neighbours neighbours;
  std::vector<std::string> required_files, unwanted_files;

  uint64_t total_frames() const;   // sum over BAT files
  std::string describe() const;     // the parsed inputs, one key per line

 private:
  bool apply(const Config &cfg, std::string *err);
  bool derive(std::string *err);
};

// Subset / neighbour file readers (src/Centre.cpp:206-268, :459-593).
bool read_subset(const std::string &path, uint32_t workset, Subset &out, std::string *err);
bool read_neighbours(const std::string &path, uint32_t workset, Neighbours &out,
                     std::string *err);
// Every pair of the subset, as Neighbors(SubsetData) builds them.
void all_pairs(const Subset &s, uint32_t workset, Neighbours &out);

}  // namespace centre_host
