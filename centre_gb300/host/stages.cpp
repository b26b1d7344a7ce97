// stages.cpp -- Discretizer, EntropyCalculator, EntropyScorer over the GPU
// library (see stages.hpp).
#include "stages.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <unordered_map>
#include <vector>

#include "ncfile.hpp"

namespace centre_host {
namespace {

// Value the reference stores for extremes it does not compute
// (Constants::DEFAULT_BAT_VALUE, used for KDE-binned DOFs).
constexpr double kDefaultBatValue = 1000.0;

std::string join(const std::string &dir, const std::string &f) {
  if (dir.empty()) return f;
  return dir.back() == '/' ? dir + f : dir + "/" + f;
}

const char *bin_file(int t) {
  return t == 1 ? "bin_bonds.nc" : t == 2 ? "bin_angles.nc" : "bin_torsions.nc";
}

const char *bat_var(int t) { return t == 1 ? "bond" : t == 2 ? "angle" : "dihedral"; }

bool fail(std::string *err, const std::string &m) {
  if (err) *err = m;
  return false;
}

centre_entropy_params make_params(const Inputs &in) {
  centre_entropy_params p;
  memset(&p, 0, sizeof(p));
  p.nframes = in.entropy.nframes_eff;
  p.nsteps = (uint8_t)in.control.nsteps;
  p.nschemes = (uint8_t)in.hist.bin_schemes.size();
  p.nestimators = (uint8_t)in.estimators.size();
  p.jacobian = in.entropy.jacobian ? 1 : 0;
  p.kde = in.bats.pdfmethod == PdfMethod::kVonMisesKDE ? 1 : 0;
  p.counts_form = CENTRE_COUNTS_AUTO;
  for (size_t s = 0; s < in.hist.bin_schemes.size() && s < 16; ++s)
    p.bin_schemes[s] = in.hist.bin_schemes[s];
  for (size_t e = 0; e < in.estimators.size() && e < 4; ++e) p.estimators[e] = in.estimators[e];
  return p;
}

// bin_<type>.nc with the reference's dimensions, attributes and variables
// (Netcdf_TrjInt::NC_create / writeRecords).
bool write_bins(const std::string &path, const char *content, uint32_t ndof,
                const std::vector<uint8_t> &schemes, uint64_t nframes,
                const std::vector<double> &ext, const std::vector<uint8_t> &coord,
                std::string *err) {
  NcOut o;
  o.version = 5;
  o.dims = {{"dims", 0}, {"extremes", 4}, {"bin_scheme_count", schemes.size()},
            {"frames", nframes}};
  o.atts = {NcAtt::text("title", std::string(content) + " Integer Vectors"),
            NcAtt::text("application", "CENTRE"), NcAtt::text("program", "Real2Int"),
            NcAtt::text("programVersion", "1.0.0"), NcAtt::text("convention", "CENTRE_Real"),
            NcAtt::text("conventionVersion", "1.0"), NcAtt::text("content", content),
            NcAtt::values<uint32_t>("ncoordims", kNcUInt, {ndof}),
            NcAtt::values<uint8_t>("nbinSchemes", kNcUByte, {(uint8_t)schemes.size()}),
            NcAtt::values<uint8_t>("binSchemes", kNcUByte, schemes)};
  std::vector<uint32_t> ids(ndof);
  for (uint32_t i = 0; i < ndof; ++i) ids[i] = i;
  o.vars = {{"dimid", {0}, {}, kNcUInt, ids.data()},
            {"extreme", {0, 1}, {}, kNcDouble, ext.data()},
            {"coord", {0, 2, 3}, {}, kNcUByte, coord.data()}};
  o.numrecs = ndof;
  return nc_write(path, o, err);
}

// entcontri_*.nc: records of DOF ids and contri_S [rec][est][scheme][step]
// (Netcdf_EntContri::NC_create, src/Netcdf_EntContri.cpp:577-769).  The
// reference's header writes a ubyte "title" (its diagonal flag) over the
// text title, and an 11-character "convention"; both are kept.
bool write_entcontri(const std::string &path, const std::string &content, int order,
                     const std::vector<uint64_t> &dim_lens, int nsteps,
                     const std::vector<uint8_t> &schemes, int nest,
                     const std::vector<uint32_t> &ids, const std::vector<double> &contri,
                     std::string *err) {
  const uint8_t full = order == 1;
  NcOut o;
  o.version = 5;
  o.dims = {{"records", 0}, {"estimators", (uint64_t)nest}, {"nbin_schemes", schemes.size()},
            {"nsteps", (uint64_t)nsteps}, {"ids", (uint64_t)order}};
  o.atts = {NcAtt::values<uint8_t>("title", kNcUByte, {(uint8_t)(full ? 0 : 1)}),
            NcAtt::text("application", "CENTRE"), NcAtt::text("program", "Real2Int"),
            NcAtt::text("programVersion", "1.0.0"),
            NcAtt::text("convention", std::string("EntropyContibution").substr(0, 11)),
            NcAtt::text("conventionVersion", "1.0"), NcAtt::text("content", content),
            NcAtt::values<uint8_t>("order", kNcUByte, {(uint8_t)order}),
            NcAtt::values<uint8_t>("nsteps", kNcUByte, {(uint8_t)nsteps}),
            NcAtt::values<uint8_t>("storagetype", kNcUByte, {(uint8_t)(full ? 0 : 3)}),
            NcAtt::values<uint8_t>("ndims", kNcUByte, {(uint8_t)order}),
            NcAtt::values<uint64_t>("dimLengths", kNcUInt64, dim_lens),
            NcAtt::values<uint8_t>("nbinSchemes", kNcUByte, {(uint8_t)schemes.size()}),
            NcAtt::values<uint8_t>("binSchemes", kNcUByte, schemes)};
  o.vars = {{"id", {0, 4}, {}, kNcUInt, ids.data()},
            {"contri_S", {0, 1, 2, 3}, {}, kNcDouble, contri.data()}};
  o.numrecs = ids.size() / (size_t)order;
  return nc_write(path, o, err);
}

// hist_*.nc: the counts behind the entropies, written when [histogram]
// writefreq is on (Netcdf_HistUtil, src/Netcdf_HistUtils.cpp:217-270 for the
// sizes and :804-1029 for the header; records as EntropyCalculator::run1d /
// run2d_xx / run2d_xy fill them, src/EntropyCalculator.cpp:176-186,
// :575-586).  As in the reference, the ubyte diagonal flag is written under
// the attribute name "title" (over the text title) and the application
// attribute is spelled "appication".  Records: id [ndims], extrema
// [ndims][4], bin mids [ndims * sum nb], cumulative counts of the written
// steps [nsteps_eff][sum nb^ndims].
struct HistSteps {
  int first, stride, neff;
};

HistSteps hist_steps(const Inputs &in, int nsteps) {
  // Netcdf_HistUtil's clamping (src/Netcdf_HistUtils.cpp:227-232)
  HistSteps h;
  const int ns = nsteps < 1 ? 1 : nsteps;
  const int first = in.hist.writestepstart;
  h.first = (first < 0 || first >= ns) ? ns - 1 : first;
  const int st = in.hist.writestepstride;
  h.stride = st < 1 ? 1 : (st > ns ? ns : st);
  h.neff = (ns - h.first + h.stride - 1) / h.stride;
  return h;
}

// bin mids of one DOF for every scheme: binData1D's running offset
// (src/Estimators.cpp:67-77)
void append_mids(double mn, double mx, const std::vector<uint8_t> &schemes,
                 std::vector<double> &out) {
  for (uint8_t nb : schemes) {
    const double w = (mx - mn) / nb, half = w / 2.0;
    double off = mn;
    for (int i = 0; i < nb; ++i) {
      out.push_back(off + half);
      off += w;
    }
  }
}

bool write_hist(const std::string &path, const std::string &content, int ndims,
                const HistSteps &hs, int nsteps, const std::vector<uint64_t> &dim_lens,
                uint8_t storage, const std::vector<uint8_t> &schemes,
                const std::vector<uint32_t> &ids, const std::vector<double> &extrema,
                const std::vector<double> &mids, const std::vector<uint64_t> &freq,
                std::string *err) {
  uint64_t sum = 0, pow_sum = 0;
  for (uint8_t nb : schemes) {
    sum += nb;
    pow_sum += ndims == 1 ? nb : (uint64_t)nb * nb;
  }
  NcOut o;
  o.version = 5;
  o.dims = {{"records", 0}, {"dimsXbin_sum", sum * ndims}, {"bin_pow_dims_sum", pow_sum},
            {"nsteps_eff", (uint64_t)hs.neff}, {"ids", (uint64_t)ndims}, {"extremes", 4}};
  o.atts = {NcAtt::values<uint8_t>("title", kNcUByte, {(uint8_t)(storage != 0 ? 1 : 0)}),
            NcAtt::text("appication", "CENTRE"), NcAtt::text("program", "Real2Int"),
            NcAtt::text("programVersion", "1.0.0"), NcAtt::text("convention", "CENTRE_HIST"),
            NcAtt::text("conventionVersion", "1.0"), NcAtt::text("content", content),
            NcAtt::values<uint8_t>("order", kNcUByte, {(uint8_t)ndims}),
            NcAtt::values<uint8_t>("firstStep", kNcUByte, {(uint8_t)hs.first}),
            NcAtt::values<uint8_t>("nsteps", kNcUByte, {(uint8_t)(nsteps < 1 ? 1 : nsteps)}),
            NcAtt::values<uint8_t>("stepStride", kNcUByte, {(uint8_t)hs.stride}),
            NcAtt::values<uint8_t>("storagetype", kNcUByte, {storage}),
            NcAtt::values<uint8_t>("ndims", kNcUByte, {(uint8_t)ndims}),
            NcAtt::values<uint64_t>("dimLengths", kNcUInt64, dim_lens),
            NcAtt::values<uint8_t>("nbinSchemes", kNcUByte, {(uint8_t)schemes.size()}),
            NcAtt::values<uint8_t>("binSchemes", kNcUByte, schemes)};
  o.vars = {{"id", {0, 4}, {}, kNcUInt, ids.data()},
            {"extrema", {0, 4, 5}, {}, kNcDouble, extrema.data()},
            {"mid", {0, 1}, {}, kNcDouble, mids.data()},
            {"freq", {0, 3, 2}, {}, kNcUInt64, freq.data()}};
  o.numrecs = ids.size() / (size_t)ndims;
  return nc_write(path, o, err);
}

struct EntFile {
  std::vector<uint32_t> ids;       // [rec][order]
  std::vector<double> contri;      // [rec][G]
  uint64_t nrec = 0;
};

bool read_entcontri(const std::string &path, int order, uint64_t G, EntFile &out,
                    std::string *err) {
  NcFile f;
  if (!f.open(path, err)) return false;
  const NcVar *id = f.var("id"), *cs = f.var("contri_S");
  if (!id || !cs) return fail(err, path + ": missing id / contri_S");
  if (!f.read_all(*id, out.ids, err) || !f.read_all(*cs, out.contri, err)) return false;
  out.nrec = f.numrecs;
  if (out.ids.size() != out.nrec * (uint64_t)order || out.contri.size() != out.nrec * G)
    return fail(err, path + ": record sizes do not match the inputs (order, estimators, schemes, steps)");
  return true;
}

// The bins of the DOFs of one type, as the entropy stage reads them
// (Netcdf_TrjInt::readCoords with start/stride frame selection).
struct TypeBins {
  std::vector<uint32_t> ids;       // DOF ids loaded, in array order
  std::vector<uint8_t> bins;       // [dof][scheme][frames_eff]
  std::vector<double> ext;         // [dof][4]
};

bool load_type(const Inputs &in, int t, const std::vector<uint32_t> &ids, TypeBins &out,
               std::string *err) {
  out.ids = ids;
  if (ids.empty()) return true;
  const std::string path = out_path(in, bin_file(t));
  NcFile f;
  if (!f.open(path, err)) return false;
  const NcVar *dimid = f.var("dimid"), *ext = f.var("extreme"), *coord = f.var("coord");
  if (!dimid || !ext || !coord) return fail(err, path + ": not a bin file");
  const std::vector<uint64_t> shp = f.shape(*coord);
  const uint64_t nsch = shp[1], nfr = shp[2];
  const size_t S = in.hist.bin_schemes.size();
  if (nsch != S) return fail(err, path + ": bin scheme count differs from [histogram] nbins");
  const uint64_t n_eff = in.entropy.nframes_eff, st = in.entropy.startframe,
                 sd = in.entropy.strideframe;
  if (n_eff == 0 || st + (n_eff - 1) * sd >= nfr)
    return fail(err, path + ": frame selection outside the file");
  std::vector<uint32_t> file_ids;
  std::vector<double> file_ext;
  if (!f.read_all(*dimid, file_ids, err) || !f.read_all(*ext, file_ext, err)) return false;
  std::unordered_map<uint32_t, uint64_t> rec_of;
  for (uint64_t r = 0; r < file_ids.size(); ++r) rec_of[file_ids[r]] = r;
  out.bins.resize(ids.size() * S * n_eff);
  out.ext.resize(ids.size() * 4);
  std::vector<uint8_t> row(S * nfr);
  for (size_t k = 0; k < ids.size(); ++k) {
    auto it = rec_of.find(ids[k]);
    if (it == rec_of.end()) return fail(err, path + ": no record for DOF id " + std::to_string(ids[k]));
    if (!f.read_rows(*coord, it->second, 1, row.data(), err)) return false;
    for (size_t s = 0; s < S; ++s) {
      uint8_t *dst = &out.bins[(k * S + s) * n_eff];
      const uint8_t *src = &row[s * nfr];
      if (sd == 1) memcpy(dst, src + st, n_eff);
      else
        for (uint64_t i = 0; i < n_eff; ++i) dst[i] = src[st + i * sd];
    }
    memcpy(&out.ext[k * 4], &file_ext[it->second * 4], 4 * sizeof(double));
  }
  return true;
}

void ids_in_pairs(const std::map<uint32_t, std::vector<uint32_t>> &m, bool keys, bool parts,
                  std::vector<uint32_t> &ids) {
  for (const auto &kv : m) {
    if (keys) ids.push_back(kv.first);
    if (parts) ids.insert(ids.end(), kv.second.begin(), kv.second.end());
  }
}

// subset ids in order, then any other id a pair list names (ascending)
std::vector<uint32_t> dof_order(const std::vector<uint32_t> &subset,
                                const std::vector<uint32_t> &extra_ids) {
  std::vector<uint32_t> out = subset;
  std::vector<uint32_t> extra = extra_ids;
  std::sort(extra.begin(), extra.end());
  extra.erase(std::unique(extra.begin(), extra.end()), extra.end());
  std::vector<uint32_t> have = subset;
  std::sort(have.begin(), have.end());
  for (uint32_t v : extra)
    if (!std::binary_search(have.begin(), have.end(), v)) out.push_back(v);
  return out;
}

std::string fixed4(double v, int width) {
  std::ostringstream o;
  o << std::setw(width) << std::fixed << std::left << std::setprecision(4) << v;
  return o.str();
}

}  // namespace

std::string out_path(const Inputs &in, const std::string &name) {
  return join(in.control.outfilepath, name);
}

Gpu::Gpu(int device) {
  const int rc = centre_gpu_create(&ctx_, device);
  if (rc != CENTRE_OK) {
    create_error_ = std::string("centre_gpu_create: ") + centre_gpu_strerror(rc);
    ctx_ = nullptr;
  }
}

Gpu::~Gpu() {
  if (ctx_) centre_gpu_destroy(ctx_);
}

std::string Gpu::error(int rc, const std::string &what) const {
  std::string s = what + ": " + centre_gpu_strerror(rc);
  if (ctx_) {
    const char *d = centre_gpu_last_error(ctx_);
    if (d && *d) s += std::string(": ") + d;
  }
  return s;
}

// ------------------------------------------------------------ Discretizer --
bool Discretizer::run(std::string *err) {
  if (!in_.control.discretize) return true;
  const uint32_t ws = in_.entropy.workset;
  if ((ws & (kB1D | kBB2D | kBA2D | kBD2D)) && !run_type(1, err)) return false;
  if ((ws & (kA1D | kBA2D | kAA2D | kAD2D)) && !run_type(2, err)) return false;
  if ((ws & (kD1D | kBD2D | kAD2D | kDD2D)) && !run_type(3, err)) return false;
  return true;
}

bool Discretizer::run_type(int t, std::string *err) {
  const uint32_t n = t == 1 ? in_.bats.nbond : t == 2 ? in_.bats.nangle : in_.bats.ndihed;
  const uint64_t frames = in_.total_frames();
  const std::vector<uint8_t> &schemes = in_.hist.bin_schemes;
  const size_t S = schemes.size();
  const bool kde = in_.bats.pdfmethod == PdfMethod::kVonMisesKDE;
  std::vector<uint8_t> coord((size_t)n * S * frames);
  std::vector<double> ext((size_t)n * 4, 0.0);
  std::vector<double> minima;
  std::vector<uint8_t> nfound;
  if (kde) {
    minima.assign((size_t)n * in_.vmkde.nmaxconf, 0.0);
    nfound.assign(n, 0);
  }
  // DOF blocks of at most ~1 GB of float32 frames; frames of every BAT file
  // are concatenated in the order the files are listed
  const uint64_t blk = std::max<uint64_t>(1, std::min<uint64_t>(n, (1ull << 28) / std::max<uint64_t>(frames, 1)));
  std::vector<float> data;
  for (uint32_t d0 = 0; d0 < n; d0 += (uint32_t)blk) {
    const uint32_t k = (uint32_t)std::min<uint64_t>(blk, n - d0);
    data.assign((size_t)k * frames, 0.f);
    uint64_t foff = 0;
    for (size_t fi = 0; fi < in_.bats.fnames.size(); ++fi) {
      NcFile f;
      const std::string path = join(in_.control.infilepath, in_.bats.fnames[fi]);
      if (!f.open(path, err)) return false;
      const NcVar *v = f.var(bat_var(t));
      if (!v) return fail(err, path + ": no variable " + bat_var(t));
      const std::vector<uint64_t> shp = f.shape(*v);
      const uint64_t nf = in_.bats.nframes[fi];
      if (shp.size() != 2 || shp[1] != n || shp[0] < nf)
        return fail(err, path + ": " + bat_var(t) + " has an unexpected shape");
      const uint64_t chunk = std::max<uint64_t>(1, (64ull << 20) / (n * 4ull));
      std::vector<float> rows;
      for (uint64_t r = 0; r < nf; r += chunk) {
        const uint64_t m = std::min(chunk, nf - r);
        rows.resize(m * n);
        if (!f.read_rows(*v, r, m, rows.data(), err)) return false;
        for (uint64_t i = 0; i < m; ++i)
          for (uint32_t d = 0; d < k; ++d) data[(size_t)d * frames + foff + r + i] = rows[i * n + d0 + d];
      }
      foff += nf;
    }
    int rc;
    if (!kde) {
      rc = centre_gpu_discretize(gpu_.ctx(), t, data.data(), k, frames, schemes.data(),
                                 (uint32_t)S, (uint8_t)in_.hist.nbinref,
                                 in_.bats.optimizedih ? 1 : 0, &coord[(size_t)d0 * S * frames],
                                 &ext[(size_t)d0 * 4]);
    } else {
      rc = centre_gpu_discretize_vmkde(gpu_.ctx(), data.data(), k, frames,
                                       (uint8_t)in_.vmkde.nmaxconf, in_.vmkde.kappa,
                                       in_.vmkde.sdosteps, in_.vmkde.sdoconvlimit,
                                       in_.vmkde.sdoiterations, &coord[(size_t)d0 * frames],
                                       &minima[(size_t)d0 * in_.vmkde.nmaxconf], &nfound[d0]);
      for (uint32_t d = 0; d < k; ++d)
        for (int q = 0; q < 4; ++q)
          ext[(size_t)(d0 + d) * 4 + q] = (q == 3 && t != 3) ? 0.0 : kDefaultBatValue;
    }
    if (rc != CENTRE_OK) return fail(err, gpu_.error(rc, std::string("discretising ") + bat_var(t)));
  }
  const char *content = t == 1 ? "B" : t == 2 ? "A" : "T";
  if (!write_bins(out_path(in_, bin_file(t)), content, n, schemes, frames, ext, coord, err))
    return false;
  if (kde && t == 3) {
    // src/Discretizer.cpp:247-259
    std::ofstream log(out_path(in_, "vmkde_torsions_minimas.out").c_str());
    for (uint32_t d = 0; d < n; ++d) {
      log << "torsion " << std::setw(6) << std::right << d << " " << (int)nfound[d];
      for (int m = 0; m < nfound[d]; ++m)
        log << " " << std::fixed << std::setprecision(8) << minima[(size_t)d * in_.vmkde.nmaxconf + m];
      log << ";" << std::endl;
    }
  }
  return true;
}

// ------------------------------------------------------- EntropyCalculator --
bool EntropyCalculator::run(std::string *err) {
  if (!in_.control.calcentropy) return true;
  const uint32_t ws = in_.entropy.workset;
  const Neighbours &nb = in_.neighbours;
  const Subset &ss = in_.subset;
  // DOFs of each type: the subset, plus any id a pair list names
  std::vector<uint32_t> xb, xa, xd;
  ids_in_pairs(nb.bb, true, true, xb);
  ids_in_pairs(nb.ba, true, false, xb);
  ids_in_pairs(nb.bd, true, false, xb);
  ids_in_pairs(nb.aa, true, true, xa);
  ids_in_pairs(nb.ba, false, true, xa);
  ids_in_pairs(nb.ad, true, false, xa);
  ids_in_pairs(nb.dd, true, true, xd);
  ids_in_pairs(nb.bd, false, true, xd);
  ids_in_pairs(nb.ad, false, true, xd);
  const bool want_b = ws & (kB1D | kBB2D | kBA2D | kBD2D);
  const bool want_a = ws & (kA1D | kAA2D | kBA2D | kAD2D);
  const bool want_d = ws & (kD1D | kDD2D | kBD2D | kAD2D);
  TypeBins tb[3];
  if (want_b && !load_type(in_, 1, dof_order(ss.bonds, xb), tb[0], err)) return false;
  if (want_a && !load_type(in_, 2, dof_order(ss.angles, xa), tb[1], err)) return false;
  if (want_d && !load_type(in_, 3, dof_order(ss.torsions, xd), tb[2], err)) return false;
  const size_t S = in_.hist.bin_schemes.size();
  const uint64_t nfr = in_.entropy.nframes_eff;
  // one array of every DOF: bonds, angles, torsions
  std::vector<uint8_t> types, bins;
  std::vector<double> ext;
  std::unordered_map<uint32_t, uint32_t> index_of[3];
  uint32_t ndof = 0;
  for (int t = 0; t < 3; ++t) {
    for (size_t k = 0; k < tb[t].ids.size(); ++k) {
      index_of[t][tb[t].ids[k]] = ndof++;
      types.push_back((uint8_t)(t + 1));
    }
    bins.insert(bins.end(), tb[t].bins.begin(), tb[t].bins.end());
    ext.insert(ext.end(), tb[t].ext.begin(), tb[t].ext.end());
  }
  if (ndof == 0) return true;
  centre_entropy_params p = make_params(in_);
  const uint64_t G = (uint64_t)p.nestimators * p.nschemes * p.nsteps;
  std::vector<double> s1((size_t)ndof * G);
  const bool dump = in_.hist.writefreq;
  const uint32_t dumpset = in_.hist.writeset;
  const HistSteps hs = hist_steps(in_, p.nsteps);
  uint64_t nbsum = 0, nb2sum = 0;
  for (uint8_t nb : in_.hist.bin_schemes) {
    nbsum += nb;
    nb2sum += (uint64_t)nb * nb;
  }
  std::vector<uint64_t> freq1;
  if (dump) freq1.resize((size_t)ndof * p.nsteps * nbsum);
  int rc = centre_gpu_entropy1d(gpu_.ctx(), &p, ndof, types.data(), bins.data(), ext.data(),
                                s1.data(), dump ? freq1.data() : nullptr);
  if (rc != CENTRE_OK) return fail(err, gpu_.error(rc, "1-D entropies"));
  // 1-D files: records in subset order (EntropyCalculator::run1d)
  struct OneD {
    uint32_t set;
    int t;
    const std::vector<uint32_t> *ids;
    const char *file, *content, *hfile;
    uint32_t hset;
  } oned[3] = {{kB1D | kBB2D, 0, &ss.bonds, "entcontri_bnd-1d.nc", "B", "hist_bnd-1d.nc", kB1D},
               {kA1D | kAA2D, 1, &ss.angles, "entcontri_ang-1d.nc", "A", "hist_ang-1d.nc", kA1D},
               {kD1D | kDD2D, 2, &ss.torsions, "entcontri_tor-1d.nc", "D", "hist_tor-1d.nc",
                kD1D}};
  for (const OneD &o : oned) {
    if (!(ws & o.set)) continue;
    std::vector<uint32_t> ids = *o.ids;
    std::vector<double> contri;
    contri.reserve(ids.size() * G);
    for (uint32_t id : ids) {
      const uint32_t i = index_of[o.t][id];
      contri.insert(contri.end(), &s1[(size_t)i * G], &s1[(size_t)i * G] + G);
    }
    if (!write_entcontri(out_path(in_, o.file), o.content, 1, {(uint64_t)ids.size()},
                         p.nsteps, in_.hist.bin_schemes, p.nestimators, ids, contri, err))
      return false;
    if (dump && (dumpset & ws & o.hset)) {
      std::vector<double> extrema, mids;
      std::vector<uint64_t> freq;
      for (uint32_t id : ids) {
        const uint32_t i = index_of[o.t][id];
        extrema.insert(extrema.end(), &ext[(size_t)i * 4], &ext[(size_t)i * 4] + 4);
        append_mids(ext[(size_t)i * 4], ext[(size_t)i * 4 + 1], in_.hist.bin_schemes, mids);
        for (int k = 0; k < hs.neff; ++k) {
          const uint64_t *row =
              &freq1[((size_t)i * p.nsteps + hs.first + (size_t)k * hs.stride) * nbsum];
          freq.insert(freq.end(), row, row + nbsum);
        }
      }
      if (!write_hist(out_path(in_, o.hfile), o.content, 1, hs, p.nsteps,
                      {(uint64_t)ids.size()}, 0, in_.hist.bin_schemes, ids, extrema, mids, freq,
                      err))
        return false;
    }
  }
  // 2-D: every pair list, one GPU call
  struct TwoD {
    uint32_t set;
    int tx, ty;
    const std::map<uint32_t, std::vector<uint32_t>> *m;
    const char *file, *content, *hfile;
  } twod[6] = {{kBB2D, 0, 0, &nb.bb, "entcontri_bnd-2d.nc", "B/B", "hist_bnd-2d.nc"},
               {kAA2D, 1, 1, &nb.aa, "entcontri_ang-2d.nc", "A/A", "hist_ang-2d.nc"},
               {kDD2D, 2, 2, &nb.dd, "entcontri_tor-2d.nc", "D/D", "hist_tor-2d.nc"},
               {kBA2D, 0, 1, &nb.ba, "entcontri_ba-2d.nc", "B/A", "hist_ba-2d.nc"},
               {kBD2D, 0, 2, &nb.bd, "entcontri_bd-2d.nc", "B/D", "hist_bd-2d.nc"},
               {kAD2D, 1, 2, &nb.ad, "entcontri_ad-2d.nc", "A/D", "hist_ad-2d.nc"}};
  std::vector<uint32_t> pairs;                 // [npairs][2] array indices
  std::vector<size_t> block_start(7, 0);
  bool ordered = true;
  for (int b = 0; b < 6; ++b) {
    block_start[b] = pairs.size() / 2;
    if (!(ws & twod[b].set)) continue;
    for (const auto &kv : *twod[b].m)
      for (uint32_t partner : kv.second) {
        const uint32_t i = index_of[twod[b].tx][kv.first], j = index_of[twod[b].ty][partner];
        if (i >= j) ordered = false;
        pairs.push_back(i);
        pairs.push_back(j);
      }
  }
  block_start[6] = pairs.size() / 2;
  const uint64_t npairs = pairs.size() / 2;
  if (npairs == 0) return true;
  std::vector<double> s2;
  const uint64_t all = (uint64_t)ndof * (ndof - 1) / 2;
  if (ordered && npairs == all) {
    // every pair i<j is asked for: the all-pairs kernels, then pick records
    std::vector<double> s2all(all * G);
    rc = centre_gpu_entropy2d(gpu_.ctx(), &p, ndof, types.data(), bins.data(), ext.data(), all,
                              nullptr, s2all.data());
    if (rc != CENTRE_OK) return fail(err, gpu_.error(rc, "2-D entropies"));
    s2.resize(npairs * G);
    for (uint64_t q = 0; q < npairs; ++q) {
      const uint64_t i = pairs[2 * q], j = pairs[2 * q + 1];
      const uint64_t r = i * ndof - i * (i + 1) / 2 + (j - i - 1);
      memcpy(&s2[q * G], &s2all[r * G], G * sizeof(double));
    }
  } else {
    s2.resize(npairs * G);
    rc = centre_gpu_entropy2d(gpu_.ctx(), &p, ndof, types.data(), bins.data(), ext.data(), npairs,
                              pairs.data(), s2.data());
    if (rc != CENTRE_OK) return fail(err, gpu_.error(rc, "2-D entropies"));
  }
  for (int b = 0; b < 6; ++b) {
    if (!(ws & twod[b].set)) continue;
    std::vector<uint32_t> ids;
    for (const auto &kv : *twod[b].m)
      for (uint32_t partner : kv.second) {
        ids.push_back(kv.first);
        ids.push_back(partner);
      }
    const size_t q0 = block_start[b], q1 = block_start[b + 1];
    std::vector<double> contri(s2.begin() + q0 * G, s2.begin() + q1 * G);
    const uint64_t nx = twod[b].tx == 0 ? ss.bonds.size() : twod[b].tx == 1 ? ss.angles.size() : ss.torsions.size();
    const uint64_t ny = twod[b].ty == 0 ? ss.bonds.size() : twod[b].ty == 1 ? ss.angles.size() : ss.torsions.size();
    if (!write_entcontri(out_path(in_, twod[b].file), twod[b].content, 2, {nx, ny}, p.nsteps,
                         in_.hist.bin_schemes, p.nestimators, ids, contri, err))
      return false;
    if (dump && (dumpset & ws & twod[b].set) && q1 > q0) {
      // joint counts of the block's pairs, a bounded number of pairs per call
      const uint64_t per_pair = (uint64_t)p.nsteps * nb2sum;
      const uint64_t chunk = std::max<uint64_t>(1, (uint64_t(1) << 27) / per_pair);
      std::vector<uint64_t> cnt, freq;
      std::vector<double> extrema, mids;
      freq.reserve((q1 - q0) * (size_t)hs.neff * nb2sum);
      for (uint64_t c0 = q0; c0 < q1; c0 += chunk) {
        const uint64_t nc = std::min<uint64_t>(chunk, q1 - c0);
        cnt.resize(nc * per_pair);
        rc = centre_gpu_counts2d(gpu_.ctx(), &p, ndof, bins.data(), nc, &pairs[2 * c0],
                                 cnt.data());
        if (rc != CENTRE_OK) return fail(err, gpu_.error(rc, "2-D histograms"));
        for (uint64_t q = 0; q < nc; ++q)
          for (int k = 0; k < hs.neff; ++k) {
            const uint64_t *row =
                &cnt[(q * p.nsteps + hs.first + (size_t)k * hs.stride) * nb2sum];
            freq.insert(freq.end(), row, row + nb2sum);
          }
      }
      for (uint64_t q = q0; q < q1; ++q) {
        const uint32_t i = pairs[2 * q], j = pairs[2 * q + 1];
        extrema.insert(extrema.end(), &ext[(size_t)i * 4], &ext[(size_t)i * 4] + 4);
        extrema.insert(extrema.end(), &ext[(size_t)j * 4], &ext[(size_t)j * 4] + 4);
        // per scheme: the first DOF's mids, then the second's (binData2D)
        for (uint8_t nbk : in_.hist.bin_schemes) {
          const std::vector<uint8_t> one(1, nbk);
          append_mids(ext[(size_t)i * 4], ext[(size_t)i * 4 + 1], one, mids);
          append_mids(ext[(size_t)j * 4], ext[(size_t)j * 4 + 1], one, mids);
        }
      }
      const uint8_t storage = twod[b].tx == twod[b].ty ? 0 : 3;   // FULL / UPPER
      if (!write_hist(out_path(in_, twod[b].hfile), twod[b].content, 2, hs, p.nsteps, {nx, ny},
                      storage, in_.hist.bin_schemes, ids, extrema, mids, freq, err))
        return false;
    }
  }
  (void)S;
  (void)nfr;
  return true;
}

// ------------------------------------------------------ learned neighbours --
bool learn_neighbours(Inputs &in, Gpu &gpu, uint32_t nneigh, const std::string &path,
                      std::string *err) {
  const uint32_t ws = in.entropy.workset;
  const Subset &ss = in.subset;
  TypeBins tb[3];
  if (!load_type(in, 1, ss.bonds, tb[0], err) || !load_type(in, 2, ss.angles, tb[1], err) ||
      !load_type(in, 3, ss.torsions, tb[2], err))
    return false;
  std::vector<uint8_t> types, bins;
  std::vector<double> ext;
  std::vector<std::pair<int, uint32_t>> who;   // (type index, DOF id) per array slot
  for (int t = 0; t < 3; ++t) {
    for (uint32_t id : tb[t].ids) {
      types.push_back((uint8_t)(t + 1));
      who.push_back({t, id});
    }
    bins.insert(bins.end(), tb[t].bins.begin(), tb[t].bins.end());
    ext.insert(ext.end(), tb[t].ext.begin(), tb[t].ext.end());
  }
  const uint32_t ndof = (uint32_t)types.size();
  if (ndof < 3) return fail(err, "learned neighbours need at least 3 DOFs");
  centre_entropy_params p = make_params(in);
  centre_screen_params sp;
  memset(&sp, 0, sizeof(sp));
  sp.feat_div = 5;
  const uint64_t all = (uint64_t)ndof * (ndof - 1) / 2;
  sp.ntrain = (uint32_t)std::min<uint64_t>(200000, std::max<uint64_t>(4096, all));
  sp.batch = std::min<uint32_t>(4096, sp.ntrain);
  sp.nneigh = std::min<uint32_t>(nneigh, ndof - 1);
  sp.nprefilter = std::min<uint32_t>(std::max<uint32_t>(4 * sp.nneigh, 64), 1024);
  sp.nprefilter = std::max(sp.nprefilter, sp.nneigh);
  sp.epochs = 3;
  sp.lr = 2e-3f;
  sp.train = 1;
  sp.init_weights = 1;
  sp.seed = in.bats.randseed ? in.bats.randseed : 17;
  std::vector<float> w(CENTRE_SCREEN_NPARAMS);
  const uint64_t cap = (uint64_t)ndof * sp.nneigh;
  std::vector<uint32_t> pairs(2 * cap);
  uint64_t npairs = 0;
  const int rc = centre_gpu_screen(gpu.ctx(), &p, &sp, ndof, types.data(), bins.data(),
                                   ext.data(), w.data(), nullptr, cap, pairs.data(), &npairs);
  if (rc != CENTRE_OK) return fail(err, gpu.error(rc, "pair screen"));
  // array order is bonds, angles, torsions: i < j puts the lower type first
  Neighbours nb;
  std::map<uint32_t, std::vector<uint32_t>> *block[3][3] = {
      {&nb.bb, &nb.ba, &nb.bd}, {nullptr, &nb.aa, &nb.ad}, {nullptr, nullptr, &nb.dd}};
  const uint32_t need[3][3] = {{kBB2D, kBA2D, kBD2D}, {0, kAA2D, kAD2D}, {0, 0, kDD2D}};
  for (uint64_t q = 0; q < npairs; ++q) {
    const auto a = who[pairs[2 * q]], b = who[pairs[2 * q + 1]];
    if (!(ws & need[a.first][b.first])) continue;
    (*block[a.first][b.first])[a.second].push_back(b.second);
  }
  std::ofstream o(path.c_str());
  const char *kind[6] = {"bond", "angle", "torsion", "bacross", "bdcross", "adcross"};
  const std::map<uint32_t, std::vector<uint32_t>> *maps[6] = {&nb.bb, &nb.aa, &nb.dd,
                                                               &nb.ba, &nb.bd, &nb.ad};
  for (int k = 0; k < 6; ++k)
    for (const auto &kv : *maps[k]) {
      o << kind[k] << " " << kv.first << " " << kv.second.size();
      for (uint32_t v : kv.second) o << " " << v;
      o << ";\n";
    }
  if (!o) return fail(err, "cannot write " + path);
  in.neighbours = nb;
  in.entropy.useneighbor = true;
  return true;
}

// ----------------------------------------------------------- EntropyScorer --
bool EntropyScorer::run(std::string *err) {
  if (!in_.control.genconvgdata) return true;
  const uint32_t ws = in_.entropy.workset;
  centre_entropy_params p = make_params(in_);
  const uint64_t G = (uint64_t)p.nestimators * p.nschemes * p.nsteps;
  // 1-D contributions of each type present in the work set
  const char *files1[3] = {"entcontri_bnd-1d.nc", "entcontri_ang-1d.nc", "entcontri_tor-1d.nc"};
  const uint32_t sets1[3] = {kB1D | kBB2D | kBA2D | kBD2D, kA1D | kAA2D | kBA2D | kAD2D,
                             kD1D | kDD2D | kBD2D | kAD2D};
  std::vector<uint8_t> types;
  std::vector<double> s1;
  std::vector<uint32_t> dof_id;
  std::unordered_map<uint32_t, uint32_t> index_of[3];
  for (int t = 0; t < 3; ++t) {
    if (!(ws & sets1[t])) continue;
    EntFile f;
    if (!read_entcontri(out_path(in_, files1[t]), 1, G, f, err)) return false;
    for (uint64_t r = 0; r < f.nrec; ++r) {
      index_of[t][f.ids[r]] = (uint32_t)types.size();
      types.push_back((uint8_t)(t + 1));
      dof_id.push_back(f.ids[r]);
    }
    s1.insert(s1.end(), f.contri.begin(), f.contri.end());
  }
  const uint32_t ndof = (uint32_t)types.size();
  if (ndof == 0) return fail(err, "no 1-D entropy contributions to score");
  // 2-D contributions in the order the reference adds graph edges:
  // B/B, B/A, B/D, A/A, A/D, D/D (EntropyScorer.cpp:640-735)
  struct Blk {
    uint32_t set;
    int tx, ty;
    const char *file;
  } blks[6] = {{kBB2D, 0, 0, "entcontri_bnd-2d.nc"}, {kBA2D, 0, 1, "entcontri_ba-2d.nc"},
               {kBD2D, 0, 2, "entcontri_bd-2d.nc"}, {kAA2D, 1, 1, "entcontri_ang-2d.nc"},
               {kAD2D, 1, 2, "entcontri_ad-2d.nc"}, {kDD2D, 2, 2, "entcontri_tor-2d.nc"}};
  std::vector<uint32_t> pairs;
  std::vector<double> s2;
  for (const Blk &b : blks) {
    if (!(ws & b.set)) continue;
    EntFile f;
    if (!read_entcontri(out_path(in_, b.file), 2, G, f, err)) return false;
    for (uint64_t r = 0; r < f.nrec; ++r) {
      auto ix = index_of[b.tx].find(f.ids[2 * r]), iy = index_of[b.ty].find(f.ids[2 * r + 1]);
      if (ix == index_of[b.tx].end() || iy == index_of[b.ty].end())
        return fail(err, std::string(b.file) + ": pair names a DOF without 1-D contribution");
      pairs.push_back(ix->second);
      pairs.push_back(iy->second);
    }
    s2.insert(s2.end(), f.contri.begin(), f.contri.end());
  }
  const uint64_t npairs = pairs.size() / 2;
  const bool tree = in_.method == Method::kMIST;
  std::vector<double> mie(G * CENTRE_SUMS_COLS), mist(G * CENTRE_SUMS_COLS);
  const uint32_t cap = ndof > 0 ? ndof - 1 : 0;
  std::vector<uint32_t> tr(G * std::max<uint32_t>(cap, 1)), ntree(G);
  const int rc = centre_gpu_score(gpu_.ctx(), &p, ndof, types.data(), s1.data(), npairs,
                                  npairs ? pairs.data() : nullptr, s2.data(), tree ? 1 : 0,
                                  nullptr, mie.data(), mist.data(), tr.data(), ntree.data());
  if (rc != CENTRE_OK) return fail(err, gpu_.error(rc, "scoring"));
  // MI of the pairs, for the tree files
  std::vector<double> mi;
  if (tree) {
    mi.resize(npairs * G);
    for (uint64_t q = 0; q < npairs; ++q)
      for (uint64_t g = 0; g < G; ++g)
        mi[q * G + g] = s1[(size_t)pairs[2 * q] * G + g] + s1[(size_t)pairs[2 * q + 1] * G + g] -
                        s2[q * G + g];
  }
  const uint64_t step_size = in_.entropy.nframes_eff / (uint64_t)p.nsteps;
  const char type_c[5] = "-BAT";
  const int fw = 13;
  const char *header[CENTRE_SUMS_COLS] = {"BOND-S1", "ANGLE-S1", "DIHED-S1", "B/B-S2", "B/B-I2",
                                          "A/A-S2", "A/A-I2", "D/D-S2", "D/D-I2", "B/A-S2",
                                          "B/A-I2", "B/D-S2", "B/D-I2", "A/D-S2", "A/D-I2",
                                          "S1", "S2"};
  auto write_sums = [&](const std::string &path, const std::vector<double> &rows, uint64_t g0) {
    std::ofstream o(path.c_str());
    o << std::setw(fw) << std::left << "TIME";
    for (const char *h : header) o << ", " << std::setw(fw) << std::left << h;
    o << std::endl;
    for (int st = 0; st < p.nsteps; ++st) {
      std::ostringstream t;
      t << std::setw(fw) << std::left << step_size * (uint64_t)(st + 1);
      o << t.str();
      for (int c = 0; c < CENTRE_SUMS_COLS; ++c)
        o << ", " << fixed4(rows[(g0 + st) * CENTRE_SUMS_COLS + c], fw);
      o << std::endl;
    }
    return (bool)o;
  };
  const std::string ext = in_.entropy.reportfileext;
  for (int e = 0; e < p.nestimators; ++e)
    for (int s = 0; s < p.nschemes; ++s) {
      const uint64_t g0 = ((uint64_t)e * p.nschemes + s) * p.nsteps;
      const std::string tag = std::string(estimator_name(p.estimators[e])) + "_convergence_b-" +
                              std::to_string((int)p.bin_schemes[s]) + "." + ext;
      if (!write_sums(out_path(in_, "MIE-" + tag), mie, g0))
        return fail(err, "cannot write MIE-" + tag);
      if (!tree) continue;
      if (!write_sums(out_path(in_, "MIST-" + tag), mist, g0))
        return fail(err, "cannot write MIST-" + tag);
      for (int st = 0; st < p.nsteps; ++st) {
        const uint64_t g = g0 + st;
        const std::string name = "Tree-MIST-" + std::string(estimator_name(p.estimators[e])) +
                                 "_b-" + std::to_string((int)p.bin_schemes[s]) + "_s-" +
                                 std::to_string(st) + "." + ext;
        std::ofstream o(out_path(in_, name).c_str());
        o << "TD1, TD2, IndexDim1, IndexDim2, MI" << std::endl;
        for (uint32_t k = 0; k < ntree[g]; ++k) {
          const uint64_t q = tr[g * cap + k];
          const uint32_t a = pairs[2 * q], b = pairs[2 * q + 1];
          o << std::setw(3) << std::left << type_c[types[a]] << ", " << std::setw(3) << std::left
            << type_c[types[b]] << ", " << std::setw(9) << std::left << dof_id[a] << ", "
            << std::setw(9) << std::left << dof_id[b] << ", " << std::setw(3) << std::left
            << std::setprecision(6) << std::fixed << mi[q * G + g] << std::endl;
        }
        if (!o) return fail(err, "cannot write " + name);
      }
    }
  return true;
}

}  // namespace centre_host
