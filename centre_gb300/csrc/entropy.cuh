// entropy.cuh -- parameter blocks and helpers shared by the count/entropy
// kernels.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace centre {

// Entropy-stage parameters as the kernels see them.
struct EntParams {
  uint64_t nframes;
  uint64_t step_size;   // nframes / nsteps (src/EntropyScorer.cpp:22)
  int nsteps;
  int nschemes;
  int nests;
  int jacobian;
  int kde;
  int nbins_sum;        // sum of the schemes' bin counts
  uint8_t schemes[kMaxSchemes];
  int scheme_off[kMaxSchemes];
  uint8_t ests[4];
};

// A tile of pairs handled by one CTA of the atomic count kernel.
struct PairTask {
  uint32_t rows[4];
  uint32_t cols[16];
  uint64_t out[16];     // output pair index per (row, col); ~0 = skip
  uint8_t nr, nc;
};

struct PairParams {
  const uint8_t *bins;
  uint64_t nframes;
  uint64_t step_size;
  uint64_t ntile;       // tiles per side (all-pairs mode)
  uint32_t ndof;
  int nschemes;
  int scheme;
  int nb;
  int nsteps;
  int all_pairs;
  int tile;             // DOFs per tile side (all-pairs mode)
};

constexpr int kTabSmem = 1024;      // c ln c entries kept in shared memory
constexpr int kTabGlobal = 1 << 16; // entries in the global table

// round(c ln c * 2^32); exact integer sums of these give the joint-entropy
// cell sum independent of summation order.
__device__ __forceinline__ unsigned long long clnc_fixed(unsigned c) {
  if (c < 2) return 0ull;
  const double v = (double)c * log((double)c) * kClncScale;
  return __double2ull_rn(v);
}

int init_clnc_table(centre_ctx *ctx, unsigned long long *tab);
int launch_entropy1d(centre_ctx *ctx, const EntParams &P, uint32_t ndof, const uint8_t *d_types,
                     const uint8_t *d_bins, const double *d_ext, double *d_s1,
                     unsigned long long *d_freq, double *d_lsum);
int pair_tile_for(int nb);
int launch_pairs_atomic(centre_ctx *ctx, const PairParams &P, const PairTask *d_tasks,
                        uint64_t ntasks, const unsigned long long *d_tab,
                        unsigned long long *d_sclnc, unsigned *d_nnz, unsigned *d_counts);
int launch_finalize2d(centre_ctx *ctx, const EntParams &P, int scheme, const uint32_t *d_pairs,
                      int all_pairs, uint32_t ndof, const double *d_ext, const double *d_lsum,
                      const unsigned long long *d_sclnc, const unsigned *d_nnz, uint64_t npairs,
                      double *d_s2);
int launch_entropy2d_counts(centre_ctx *ctx, const EntParams &P, int scheme,
                            const uint32_t *d_pairs, const uint8_t *d_types, const double *d_ext,
                            const unsigned *d_counts, uint64_t p0, uint64_t np, uint64_t npairs,
                            double *d_s2);

// discretize.cu
int launch_discretize(centre_ctx *ctx, int bat_type, const float *d_data, uint32_t ndof,
                      uint64_t nframes, const uint8_t *schemes, uint32_t nschemes,
                      uint8_t bins_ref, int optimize, uint8_t *d_bins, double *d_ext);

// pairs_tc.cu
bool tc_supported(centre_ctx *ctx, int nb, uint64_t nframes);
int launch_pairs_tc(centre_ctx *ctx, const PairParams &P, const unsigned long long *d_tab,
                    unsigned long long *d_sclnc, unsigned *d_nnz);

// score.cu
struct ScoreParams {
  uint32_t ndof;
  uint64_t npairs;
  int G;                // nests * nschemes * nsteps
  int all_pairs;
  int sorted_types;     // DOF types non-decreasing (bonds, angles, torsions)
  uint32_t type_start[4];
  uint32_t type_count[4];
};
int launch_score(centre_ctx *ctx, const ScoreParams &S, const uint8_t *d_types,
                 const uint32_t *d_pairs, const double *d_s1, const double *d_s2, double *d_mi,
                 double *h_mie, int build_tree, double *h_mist, uint32_t *h_tree,
                 uint32_t *h_ntree);

}  // namespace centre
