// ref_shim.cpp -- C entry points over the reference's own numeric code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the unmodified reference sources (src/Estimators.cpp, src/Real2Int.cpp,
// src/Centre.cpp, src/Utils.cpp, src/Convergance.cpp of shaileshp51/centre,
// read where they lie) into oracle/_ref/libcentre_ref.so.  Tests use it to
// pin the C restatement in oracle/centre_oracle.c and to generate the golden
// fixtures under tests/golden/.  Nothing here is shipped or measured.
#include <cstdint>
#include <cstring>
#include <vector>

#include "Centre.h"
#include "Estimators.h"
#include "Real2Int.h"
#include "Utils.h"

extern "C" {

// Real2Int::bndReal2Int / angReal2Int / dihReal2Int (src/Real2Int.cpp:27,131,244)
int ref_real2int(int type, const float *x, uint64_t n, const uint8_t *schemes,
                 int nschemes, uint8_t bins_ref, int optimize, double *ext,
                 uint8_t *out) {
  std::vector<hbin_t> bs(schemes, schemes + nschemes);
  std::vector<data_t> data(x, x + n);
  std::vector<hbin_t> bins(n * nschemes, 0);
  double mn = 0, mx = 0, av = 0, ph = 0;
  int rc;
  if (type == 1)
    rc = Real2Int::bndReal2Int(0, bs, data, &mn, &mx, &av, bins);
  else if (type == 2)
    rc = Real2Int::angReal2Int(0, bs, data, &mn, &mx, &av, bins);
  else
    rc = Real2Int::dihReal2Int(0, bs, bins_ref, optimize != 0, data, &mn, &mx,
                               &av, &ph, bins);
  ext[0] = mn;
  ext[1] = mx;
  ext[2] = av;
  ext[3] = (type == 3) ? ph : 0.0;
  std::memcpy(out, bins.data(), bins.size());
  return rc;
}

// Real2Int::getMinimaPositions (src/Real2Int.cpp:481)
int ref_vmkde(const float *x, uint64_t n, uint8_t nconf, double kappa,
              uint32_t step_sdo, double conv, uint32_t max_iter,
              double *minima, uint8_t *found, uint8_t *out) {
  std::vector<data_t> data(x, x + n);
  std::vector<double> mins(nconf, 0.0);
  std::vector<hbin_t> bins(n, 0);
  hbin_t fm = 0;
  int rc = Real2Int::getMinimaPositions(0, false, nconf, kappa, step_sdo, conv,
                                        max_iter, data, mins, fm, bins);
  for (int i = 0; i < nconf; ++i) minima[i] = mins[i];
  *found = fm;
  std::memcpy(out, bins.data(), n);
  return rc;
}

double ref_bessel_i(int n, double x) { return Utils::modifiedBesselI(n, x); }

// binData1D + entropy1D (src/Estimators.cpp:56, :217)
int ref_entropy1d(int type, const uint8_t *bins, uint64_t nframes,
                  uint8_t nsteps, const uint8_t *schemes, int nschemes,
                  double mn, double mx, const uint8_t *ests, int nests,
                  int jacobian, int kde, uint64_t *freq, double *entropy) {
  std::vector<hbin_t> bs(schemes, schemes + nschemes);
  size_t nsum = 0;
  for (int i = 0; i < nschemes; ++i) nsum += schemes[i];
  std::vector<ull_int> fr(nsteps * nsum, 0);
  std::vector<double> mids(nsum, 0.0);
  std::vector<EntropyEstimators> es;
  for (int i = 0; i < nests; ++i) es.push_back((EntropyEstimators)ests[i]);
  std::vector<double> ent(nests * nsteps * nschemes, 0.0);
  int rc = binData1D(nsteps, bs, nframes, mn, mx,
                     const_cast<hbin_t *>(bins), fr, mids);
  if (rc) return rc;
  rc = entropy1D((BAT_t)type, 0, es, nsteps, nframes / nsteps, mn, mx,
                 jacobian != 0, kde != 0, bs, fr, ent);
  if (freq) std::memcpy(freq, fr.data(), fr.size() * sizeof(uint64_t));
  std::memcpy(entropy, ent.data(), ent.size() * sizeof(double));
  return rc;
}

// binData2D + entropy2D (src/Estimators.cpp:130, :391)
int ref_entropy2d(int type1, int type2, const uint8_t *b1, const uint8_t *b2,
                  uint64_t nframes, uint8_t nsteps, const uint8_t *schemes,
                  int nschemes, double mn1, double mx1, double mn2, double mx2,
                  const uint8_t *ests, int nests, int jacobian, int kde,
                  uint64_t *freq, double *entropy) {
  std::vector<hbin_t> bs(schemes, schemes + nschemes);
  size_t nsq = 0, nsum = 0;
  for (int i = 0; i < nschemes; ++i) {
    nsq += schemes[i] * schemes[i];
    nsum += schemes[i];
  }
  std::vector<ull_int> fr(nsteps * nsq, 0);
  std::vector<double> mids(2 * nsum, 0.0);
  std::vector<EntropyEstimators> es;
  for (int i = 0; i < nests; ++i) es.push_back((EntropyEstimators)ests[i]);
  std::vector<double> ent(nests * nsteps * nschemes, 0.0);
  int rc = binData2D(nsteps, bs, nframes, mn1, mx1, mn2, mx2,
                     const_cast<hbin_t *>(b1), const_cast<hbin_t *>(b2), fr,
                     mids);
  if (rc) return rc;
  rc = entropy2D((BAT_t)type1, (BAT_t)type2, 0, 1, es, nsteps,
                 nframes / nsteps, mn1, mx1, mn2, mx2, jacobian != 0, kde != 0,
                 bs, fr, ent);
  if (freq) std::memcpy(freq, fr.data(), fr.size() * sizeof(uint64_t));
  std::memcpy(entropy, ent.data(), ent.size() * sizeof(double));
  return rc;
}

// boruvkaMST (src/Centre.cpp:5); returns tree edges as (src, dst, weight)
int64_t ref_mst(uint32_t nv, uint64_t ne, const uint32_t *src,
                const uint32_t *dst, const double *w, uint32_t *tsrc,
                uint32_t *tdst, double *tw) {
  Graph g;
  for (uint32_t v = 0; v < nv; ++v) g.nodes.push_back(Node(BAT_t::DIHEDRAL, v));
  for (uint64_t e = 0; e < ne; ++e)
    g.edges.push_back(Edge((int)src[e], (int)dst[e], w[e]));
  std::vector<Edge> t = boruvkaMST(g);
  for (size_t i = 0; i < t.size(); ++i) {
    tsrc[i] = (uint32_t)t[i].source;
    tdst[i] = (uint32_t)t[i].dest;
    tw[i] = t[i].weight;
  }
  return (int64_t)t.size();
}

}  // extern "C"
