// inputs.cpp -- input file, subsets and neighbour lists (see inputs.hpp).
#include "inputs.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "ncfile.hpp"

namespace centre_host {
namespace {

std::string trim(const std::string &s, const char *chars = " \t") {
  const size_t b = s.find_first_not_of(chars);
  if (b == std::string::npos) return {};
  const size_t e = s.find_last_not_of(chars);
  return s.substr(b, e - b + 1);
}

// Utils::string2bool: "true"/"false" in any case; anything else is false.
bool to_bool(std::string s) {
  std::transform(s.begin(), s.end(), s.begin(), ::tolower);
  return s == "true";
}

int to_int(const std::string &s) { return std::atoi(s.c_str()); }

bool is_dir(const std::string &p) {
  struct stat st;
  return !p.empty() && stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

bool file_exists(const std::string &p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}

std::string join(const std::string &dir, const std::string &f) {
  if (dir.empty()) return f;
  return dir.back() == '/' ? dir + f : dir + "/" + f;
}

uint32_t parse_set(const std::vector<std::string> &v) {
  static const std::map<std::string, uint32_t> names = {
      {"B1D", kB1D}, {"A1D", kA1D}, {"D1D", kD1D}, {"1D", kX1D}, {"BB2D", kBB2D},
      {"AA2D", kAA2D}, {"DD2D", kDD2D}, {"XX2D", kXX2D}, {"BA2D", kBA2D}, {"BD2D", kBD2D},
      {"AD2D", kAD2D}, {"2D", kXY2D}};
  uint32_t set = kNothing;
  for (const std::string &t : v) {
    if (t == "NONE") return kNothing;
    auto it = names.find(t);
    if (it != names.end()) set |= it->second;
  }
  return set;
}

// Number of DOFs of each type and frames of a CENTRE BAT file.
bool bat_header(const std::string &path, unsigned &nb, unsigned &na, unsigned &nd,
                uint64_t &nframes, std::string *err) {
  NcFile f;
  if (!f.open(path, err)) return false;
  const NcAtt *conv = f.att("convention");
  if (!conv || conv->as_text() != "CENTRE") {
    if (err) *err = path + ": not a CENTRE BAT trajectory (convention attribute)";
    return false;
  }
  auto len = [&](const char *d) -> uint64_t {
    const int id = f.dim_id(d);
    return id < 0 ? 0 : f.dim_len(id);
  };
  nb = (unsigned)len("bond");
  na = (unsigned)len("angle");
  nd = (unsigned)len("dihedral");
  nframes = len("frame");
  return true;
}

}  // namespace

const char *estimator_name(uint8_t e) {
  switch (e) {
    case kML: return "ML";
    case kMM: return "MM";
    case kCS: return "CS";
    case kJS: return "JS";
    default: return "??";
  }
}

Config parse_config(const std::string &path, bool *ok) {
  Config ans;
  std::ifstream in(path.c_str());
  if (ok) *ok = (bool)in;
  std::string line, section;
  while (std::getline(in, line, '\n')) {
    line = trim(line);
    if (line.empty() || line[0] == '#') continue;
    if (line.size() > 2 && line.front() == '[' && line.back() == ']') {
      section = line.substr(1, line.size() - 2);
      continue;
    }
    const size_t eq = line.find('=');
    std::string key = trim(line.substr(0, eq));
    if (!section.empty()) key = section + "." + key;
    std::string value = eq == std::string::npos ? std::string() : trim(line.substr(eq + 1));
    std::vector<std::string> values;
    const size_t q1 = value.find_first_of('"'), q2 = value.find_last_of('"');
    if (q1 != std::string::npos && q2 != std::string::npos && q2 > q1) {
      values.push_back(value.substr(q1 + 1, q2 - q1 - 1));
    } else {
      std::istringstream words(value);
      std::string tok;
      while (words >> tok) {
        if (tok[0] == '#') break;
        values.push_back(trim(tok, ","));
      }
    }
    ans[key] = values;
  }
  return ans;
}

bool Inputs::apply(const Config &cfg, std::string *err) {
  for (const auto &kv : cfg) {
    const std::string &k = kv.first;
    const std::vector<std::string> &v = kv.second;
    if (v.empty()) continue;
    const std::string &s = v[0];
    if (k == "control.nsteps") control.nsteps = (uint8_t)to_int(s);
    else if (k == "control.discretize") control.discretize = to_bool(s);
    else if (k == "control.calcentropy") control.calcentropy = to_bool(s);
    else if (k == "control.genconvgdata") control.genconvgdata = to_bool(s);
    else if (k == "control.dscrinfofreq") control.dscrinfofreq = (unsigned)to_int(s);
    else if (k == "control.entcinfofreq") control.entcinfofreq = (unsigned)to_int(s);
    else if (k == "control.cachedscrtdimspercpu") control.cachedscrtdimspercpu = (unsigned)to_int(s);
    else if (k == "control.cacheentcdimspercpu") control.cacheentcdimspercpu = (unsigned)to_int(s);
    else if (k == "control.outfilepath") control.outfilepath = s;
    else if (k == "control.infilepath") control.infilepath = s;
    else if (k == "control.infofile") control.infofile = s;
    else if (k == "discretization.nbond") bats.nbond = (unsigned)to_int(s);
    else if (k == "discretization.nangle") bats.nangle = (unsigned)to_int(s);
    else if (k == "discretization.ndihed") bats.ndihed = (unsigned)to_int(s);
    else if (k == "discretization.fname") bats.fnames = v;   // every listed file, in order
    else if (k == "discretization.nframe") {
      bats.nframes.clear();
      for (const std::string &t : v) bats.nframes.push_back((uint64_t)std::atoll(t.c_str()));
    } else if (k == "discretization.randseed") bats.randseed = (uint64_t)to_int(s);
    else if (k == "discretization.shuffleframes") bats.shuffleframes = to_bool(s);
    else if (k == "discretization.shuffledofs") bats.shuffledofs = to_bool(s);
    else if (k == "discretization.optimizedih") bats.optimizedih = to_bool(s);
    else if (k == "discretization.pdfmethod") {
      std::string m = s;
      std::transform(m.begin(), m.end(), m.begin(), ::tolower);
      if (m == "histogram") bats.pdfmethod = PdfMethod::kHistogram;
      else if (m == "vonmiseskde") bats.pdfmethod = PdfMethod::kVonMisesKDE;
    } else if (k == "vonmiseskde.nmaxconf") vmkde.nmaxconf = (uint8_t)to_int(s);
    else if (k == "vonmiseskde.writefreq") vmkde.writefreq = to_bool(s);
    else if (k == "vonmiseskde.writeset") vmkde.writeset = parse_set(v);
    else if (k == "vonmiseskde.writestepstart") vmkde.writestepstart = (uint8_t)to_int(s);
    else if (k == "vonmiseskde.writestepstride") vmkde.writestepstride = (uint8_t)to_int(s);
    else if (k == "vonmiseskde.kappa") vmkde.kappa = std::atof(s.c_str());
    else if (k == "vonmiseskde.sdosteps") vmkde.sdosteps = (unsigned)to_int(s);
    else if (k == "vonmiseskde.sdoiterations") vmkde.sdoiterations = (unsigned)to_int(s);
    else if (k == "vonmiseskde.sdoconvlimit") vmkde.sdoconvlimit = std::atof(s.c_str());
    else if (k == "histogram.referencenbins") hist.nbinref = (uint8_t)to_int(s);
    else if (k == "histogram.nbins") {
      hist.bin_schemes.clear();
      for (const std::string &t : v) hist.bin_schemes.push_back((uint8_t)to_int(t));
    } else if (k == "histogram.writefreq") hist.writefreq = to_bool(s);
    else if (k == "histogram.writeset") hist.writeset = parse_set(v);
    else if (k == "histogram.writestepstart") hist.writestepstart = (uint8_t)to_int(s);
    else if (k == "histogram.writestepstride") hist.writestepstride = (uint8_t)to_int(s);
    else if (k == "entropy.workset") entropy.workset = parse_set(v);
    else if (k == "entropy.shuffleblocks") entropy.shuffleblocks = to_bool(s);
    else if (k == "entropy.shuffleblocktimes") entropy.shuffleblocktimes = to_int(s);
    else if (k == "entropy.usesubset") entropy.usesubset = to_bool(s);
    else if (k == "entropy.useneighbor") entropy.useneighbor = to_bool(s);
    else if (k == "entropy.jacobian") entropy.jacobian = to_bool(s);
    else if (k == "entropy.subsetfile") entropy.subsetfile = s;
    else if (k == "entropy.neighborfile") entropy.neighborfile = s;
    else if (k == "entropy.startframe") entropy.startframe = (uint64_t)to_int(s);
    else if (k == "entropy.strideframe") entropy.strideframe = (uint64_t)to_int(s);
    else if (k == "entropy.nframe") entropy.nframe = (uint64_t)to_int(s);
    else if (k == "entropy.scoringmethod") {
      if (s == "MIE") method = Method::kMIE;
      else if (s == "AMIE") method = Method::kAMIE;
      else if (s == "MIST") method = Method::kMIST;
      else if (s == "AMIST") method = Method::kAMIST;
    } else if (k == "entropy.estimator") {
      for (const std::string &t : v) {
        if (t == "ML") estimators.push_back(kML);
        else if (t == "MM") estimators.push_back(kMM);
        else if (t == "CS") estimators.push_back(kCS);
        else if (t == "JS") estimators.push_back(kJS);
      }
    } else if (k == "entropy.reportfileext") entropy.reportfileext = s;
  }
  if (control.nsteps <= 0) {
    if (err) *err = "[control] nsteps must be at least 1";
    return false;
  }
  if (entropy.strideframe == 0) entropy.strideframe = 1;
  return true;
}

uint64_t Inputs::total_frames() const {
  uint64_t n = 0;
  for (uint64_t v : bats.nframes) n += v;
  return n;
}

bool Inputs::derive(std::string *err) {
  // DOF counts and frames from the BAT headers (Inputs.cpp:555-625); when
  // the BAT file is absent and discretisation is off, from the bin files
  if (bats.nframes.size() != bats.fnames.size()) {
    bats.nframes.resize(bats.fnames.size(), 0);
    for (size_t i = 0; i < bats.fnames.size(); ++i) {
      const std::string p = join(control.infilepath, bats.fnames[i]);
      unsigned nb = 0, na = 0, nd = 0;
      uint64_t nf = 0;
      std::string e2;
      if (!bat_header(p, nb, na, nd, nf, &e2)) {
        if (control.discretize) {
          if (err) *err = e2;
          return false;
        }
        // counts from the bin files the discretiser wrote
        const char *files[3] = {"bin_bonds.nc", "bin_angles.nc", "bin_torsions.nc"};
        unsigned *cnt[3] = {&nb, &na, &nd};
        for (int t = 0; t < 3; ++t) {
          NcFile f;
          std::string e3;
          if (!f.open(join(control.outfilepath, files[t]), &e3)) continue;
          const int di = f.dim_id("dims"), fi = f.dim_id("frames");
          *cnt[t] = (unsigned)f.dim_len(di);
          nf = f.dim_len(fi);
        }
        if (nf == 0) {
          if (err) *err = e2 + " (and no bin files in the output path)";
          return false;
        }
      }
      auto check = [&](unsigned &have, unsigned got, const char *what) {
        if (have == 0) have = got;
        else if (have != got) {
          if (err) *err = std::string("earlier ") + what + " count differs in " + p;
          return false;
        }
        return true;
      };
      if (!check(bats.nbond, nb, "bond") || !check(bats.nangle, na, "angle") ||
          !check(bats.ndihed, nd, "dihedral"))
        return false;
      if (nf == 0) {
        if (err) *err = "file '" + p + "' must have more than 0 frames";
        return false;
      }
      bats.nframes[i] = nf;
    }
  }
  const uint64_t numfrm = total_frames();
  if (entropy.nframe > numfrm || entropy.nframe == 0) entropy.nframe = numfrm;
  if (entropy.nframe > 0 && (entropy.startframe > 0 || entropy.strideframe > 1))
    entropy.nframes_eff =
        (entropy.nframe - entropy.startframe + entropy.strideframe - 1) / entropy.strideframe;
  else
    entropy.nframes_eff = entropy.nframe;
  if (!is_dir(control.infilepath)) {
    if (err) *err = "infilepath (" + control.infilepath + ") is not a directory";
    return false;
  }
  if (!is_dir(control.outfilepath)) {
    if (err) *err = "outfilepath (" + control.outfilepath + ") is not a directory";
    return false;
  }
  // von Mises KDE: one scheme of nmaxconf conformers, torsions only
  // (Inputs.cpp:720-750)
  if (bats.pdfmethod == PdfMethod::kVonMisesKDE) {
    hist.nbinref = vmkde.nmaxconf;
    hist.bin_schemes.assign(1, (uint8_t)vmkde.nmaxconf);
    hist.writefreq = vmkde.writefreq;
    hist.writeset = vmkde.writeset;
    if (control.discretize) {
      const uint32_t ws = entropy.workset;
      if (ws & kD1D) entropy.workset = kD1D;
      if (ws & kDD2D) entropy.workset = kD1D | kDD2D;
    }
  }
  if (hist.bin_schemes.empty()) {
    if (err) *err = "[histogram] nbins is required";
    return false;
  }
  if (hist.nbinref == 0) hist.nbinref = hist.bin_schemes[0];
  if (estimators.empty()) estimators.push_back(kMM);
  // DOF subset and pair lists
  const uint32_t ws = entropy.workset;
  if (entropy.usesubset) {
    const std::string sp = join(control.infilepath, entropy.subsetfile);
    if (!file_exists(sp)) {
      if (err) *err = "subset file (" + entropy.subsetfile + ") does not exist";
      return false;
    }
    if (!read_subset(sp, ws, subset, err)) return false;
    if (entropy.useneighbor) {
      const std::string np = join(control.infilepath, entropy.neighborfile);
      if (!file_exists(np)) {
        if (err) *err = "neighbor file (" + entropy.neighborfile + ") does not exist";
        return false;
      }
      if (!read_neighbours(np, ws, neighbours, err)) return false;
    } else {
      all_pairs(subset, ws, neighbours);
    }
  } else {
    subset = Subset();
    if (ws & kB1D)
      for (uint32_t i = 0; i < bats.nbond; ++i) subset.bonds.push_back(i);
    if (ws & kA1D)
      for (uint32_t i = 0; i < bats.nangle; ++i) subset.angles.push_back(i);
    if (ws & kD1D)
      for (uint32_t i = 0; i < bats.ndihed; ++i) subset.torsions.push_back(i);
    subset.total_bonds = bats.nbond;
    subset.total_angles = bats.nangle;
    subset.total_torsions = bats.ndihed;
    all_pairs(subset, ws, neighbours);
  }
  if (hist.writefreq && hist.writestepstart == 255) hist.writestepstart = control.nsteps - 1;
  if (vmkde.writefreq && vmkde.writestepstart == 255) vmkde.writestepstart = control.nsteps - 1;
  // files a run needs and files it would overwrite (main_smp.cpp:80-110)
  required_files.clear();
  unwanted_files.clear();
  const bool need_b = ws & (kB1D | kBB2D | kBA2D | kBD2D);
  const bool need_a = ws & (kA1D | kAA2D | kBA2D | kAD2D);
  const bool need_d = ws & (kD1D | kDD2D | kBD2D | kAD2D);
  if (control.discretize) {
    for (const std::string &f : bats.fnames) required_files.push_back(join(control.infilepath, f));
    if (need_b) unwanted_files.push_back(join(control.outfilepath, "bin_bonds.nc"));
    if (need_a) unwanted_files.push_back(join(control.outfilepath, "bin_angles.nc"));
    if (need_d) unwanted_files.push_back(join(control.outfilepath, "bin_torsions.nc"));
  } else if (control.calcentropy) {
    if (need_b) required_files.push_back(join(control.outfilepath, "bin_bonds.nc"));
    if (need_a) required_files.push_back(join(control.outfilepath, "bin_angles.nc"));
    if (need_d) required_files.push_back(join(control.outfilepath, "bin_torsions.nc"));
  }
  if (control.calcentropy) {
    const std::pair<uint32_t, const char *> files[] = {
        {kB1D | kBB2D, "entcontri_bnd-1d.nc"}, {kA1D | kAA2D, "entcontri_ang-1d.nc"},
        {kD1D | kDD2D, "entcontri_tor-1d.nc"}, {kBB2D, "entcontri_bnd-2d.nc"},
        {kAA2D, "entcontri_ang-2d.nc"}, {kDD2D, "entcontri_tor-2d.nc"},
        {kBA2D, "entcontri_ba-2d.nc"}, {kBD2D, "entcontri_bd-2d.nc"},
        {kAD2D, "entcontri_ad-2d.nc"}};
    for (const auto &f : files)
      if (ws & f.first) unwanted_files.push_back(join(control.outfilepath, f.second));
    // histogram dumps (Inputs.cpp:826-872: the bond-bond file is listed by
    // the write set alone)
    if (hist.writefreq) {
      const uint32_t hs = hist.writeset;
      const std::pair<uint32_t, const char *> hfiles[] = {
          {hs & ws & kB1D, "hist_bnd-1d.nc"}, {hs & ws & kA1D, "hist_ang-1d.nc"},
          {hs & ws & kD1D, "hist_tor-1d.nc"}, {hs & kBB2D, "hist_bnd-2d.nc"},
          {hs & ws & kAA2D, "hist_ang-2d.nc"}, {hs & ws & kDD2D, "hist_tor-2d.nc"},
          {hs & ws & kBA2D, "hist_ba-2d.nc"}, {hs & ws & kBD2D, "hist_bd-2d.nc"},
          {hs & ws & kAD2D, "hist_ad-2d.nc"}};
      for (const auto &f : hfiles)
        if (f.first) unwanted_files.push_back(join(control.outfilepath, f.second));
    }
  }
  return true;
}

bool Inputs::init(const std::string &path, std::string *err) {
  bool ok = false;
  Config cfg = parse_config(path, &ok);
  if (!ok) {
    if (err) *err = "cannot read input file " + path;
    return false;
  }
  return apply(cfg, err) && derive(err);
}

std::string Inputs::describe() const {
  std::ostringstream o;
  o << "control.infilepath = " << control.infilepath << "\n"
    << "control.outfilepath = " << control.outfilepath << "\n"
    << "control.nsteps = " << control.nsteps << "\n"
    << "control.discretize = " << control.discretize << "\n"
    << "control.calcentropy = " << control.calcentropy << "\n"
    << "control.genconvgdata = " << control.genconvgdata << "\n"
    << "discretization.fname =";
  for (const std::string &f : bats.fnames) o << " " << f;
  o << "\ndiscretization.nframe =";
  for (uint64_t n : bats.nframes) o << " " << n;
  o << "\ndiscretization.nbond = " << bats.nbond << "\n"
    << "discretization.nangle = " << bats.nangle << "\n"
    << "discretization.ndihed = " << bats.ndihed << "\n"
    << "discretization.optimizedih = " << bats.optimizedih << "\n"
    << "discretization.pdfmethod = "
    << (bats.pdfmethod == PdfMethod::kHistogram ? "histogram" : "vonmiseskde") << "\n"
    << "vonmiseskde.nmaxconf = " << vmkde.nmaxconf << "\n"
    << "vonmiseskde.kappa = " << vmkde.kappa << "\n"
    << "vonmiseskde.sdosteps = " << vmkde.sdosteps << "\n"
    << "vonmiseskde.sdoiterations = " << vmkde.sdoiterations << "\n"
    << "vonmiseskde.sdoconvlimit = " << vmkde.sdoconvlimit << "\n"
    << "histogram.referencenbins = " << hist.nbinref << "\n"
    << "histogram.nbins =";
  for (uint8_t b : hist.bin_schemes) o << " " << (int)b;
  o << "\nentropy.workset = " << entropy.workset << "\n"
    << "entropy.jacobian = " << entropy.jacobian << "\n"
    << "entropy.usesubset = " << entropy.usesubset << "\n"
    << "entropy.useneighbor = " << entropy.useneighbor << "\n"
    << "entropy.startframe = " << entropy.startframe << "\n"
    << "entropy.strideframe = " << entropy.strideframe << "\n"
    << "entropy.nframe = " << entropy.nframe << "\n"
    << "entropy.nframes_eff = " << entropy.nframes_eff << "\n"
    << "entropy.scoringmethod = "
    << (method == Method::kMIE ? "MIE" : method == Method::kAMIE ? "AMIE"
        : method == Method::kMIST ? "MIST" : "AMIST") << "\n"
    << "entropy.estimator =";
  for (uint8_t e : estimators) o << " " << estimator_name(e);
  o << "\nentropy.reportfileext = " << entropy.reportfileext << "\n"
    << "subset.sizes = " << subset.bonds.size() << " " << subset.angles.size() << " "
    << subset.torsions.size() << "\n";
  auto count = [](const std::map<uint32_t, std::vector<uint32_t>> &m) {
    size_t n = 0;
    for (const auto &kv : m) n += kv.second.size();
    return n;
  };
  o << "neighbours.pairs = " << count(neighbours.bb) << " " << count(neighbours.aa) << " "
    << count(neighbours.dd) << " " << count(neighbours.ba) << " " << count(neighbours.bd) << " "
    << count(neighbours.ad) << "\n";
  return o.str();
}

bool read_subset(const std::string &path, uint32_t workset, Subset &out, std::string *err) {
  out = Subset();
  std::ifstream file(path.c_str());
  std::string chunk;
  while (std::getline(file, chunk, ';')) {
    if (!chunk.empty() && chunk[0] == '#') {
      file >> std::ws;
      continue;
    }
    std::istringstream s(chunk);
    std::string kind;
    uint32_t total = 0, n = 0;
    s >> kind >> total >> n;
    if (kind.empty()) {
      file >> std::ws;
      continue;
    }
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < n; ++i) {
      uint32_t v;
      if (!(s >> v)) {
        if (err) *err = "subset file: expected " + std::to_string(n) + " " + kind + " values";
        return false;
      }
      ids.push_back(v);
    }
    if (kind == "bond" && (workset & kB1D)) {
      out.total_bonds = total;
      out.bonds = ids;
    } else if (kind == "angle" && (workset & kA1D)) {
      out.total_angles = total;
      out.angles = ids;
    } else if (kind == "torsion" && (workset & kD1D)) {
      out.total_torsions = total;
      out.torsions = ids;
    }
    file >> std::ws;
  }
  return true;
}

bool read_neighbours(const std::string &path, uint32_t workset, Neighbours &out,
                     std::string *err) {
  out = Neighbours();
  std::ifstream file(path.c_str());
  std::string chunk;
  while (std::getline(file, chunk, ';')) {
    if (!chunk.empty() && chunk[0] == '#') {
      file >> std::ws;
      continue;
    }
    std::istringstream s(chunk);
    std::string kind;
    uint32_t key = 0, n = 0;
    s >> kind >> key >> n;
    if (kind.empty() || n == 0) {
      file >> std::ws;
      continue;
    }
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < n; ++i) {
      uint32_t v;
      if (!(s >> v)) {
        if (err) *err = "neighbor file: expected " + std::to_string(n) + " values for " + kind;
        return false;
      }
      ids.push_back(v);
    }
    std::map<uint32_t, std::vector<uint32_t>> *m = nullptr;
    if (kind == "bond" && (workset & kBB2D)) m = &out.bb;
    else if (kind == "angle" && (workset & kAA2D)) m = &out.aa;
    else if (kind == "torsion" && (workset & kDD2D)) m = &out.dd;
    else if (kind == "bacross" && (workset & kBA2D)) m = &out.ba;
    else if (kind == "bdcross" && (workset & kBD2D)) m = &out.bd;
    else if (kind == "adcross" && (workset & kAD2D)) m = &out.ad;
    if (m) m->insert({key, ids});   // the first entry of a key wins, as in the reference
    file >> std::ws;
  }
  return true;
}

void all_pairs(const Subset &s, uint32_t ws, Neighbours &out) {
  out = Neighbours();
  auto upper = [](const std::vector<uint32_t> &v, std::map<uint32_t, std::vector<uint32_t>> &m) {
    for (size_t i = 0; i + 1 < v.size(); ++i)
      m[v[i]] = std::vector<uint32_t>(v.begin() + i + 1, v.end());
  };
  auto cross = [](const std::vector<uint32_t> &x, const std::vector<uint32_t> &y,
                  std::map<uint32_t, std::vector<uint32_t>> &m) {
    for (uint32_t k : x) m[k] = y;
  };
  if (ws & kB1D) {
    if (ws & kBB2D) upper(s.bonds, out.bb);
    if (ws & kBA2D) cross(s.bonds, s.angles, out.ba);
    if (ws & kBD2D) cross(s.bonds, s.torsions, out.bd);
  }
  if (ws & kA1D) {
    if (ws & kAA2D) upper(s.angles, out.aa);
    if (ws & kAD2D) cross(s.angles, s.torsions, out.ad);
  }
  if ((ws & kD1D) && (ws & kDD2D)) upper(s.torsions, out.dd);
}

}  // namespace centre_host
