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
  int fix_scale;        // moment scale s of the joint counts (moment_scale())
  double fix_inv;       // 2^-s
};

// A tile of pairs handled by one CTA of the atomic count kernel.
struct PairTask {
  uint32_t rows[4];
  uint32_t cols[16];
  uint64_t out[16];     // output pair index per (row, col); ~0 = skip
  uint8_t nr, nc;
};

// One trajectory of a batch (device copy; see batch.cu).
struct BatchSys {
  const uint8_t *bins;
  uint64_t nframes;
  uint64_t step_size;
  uint64_t ntile;        // tiles per side of the all-pairs grid
  uint64_t stripe;       // tile columns per stripe of the tile order
  uint64_t item_begin;   // first work item of this trajectory
  uint32_t ndof;
  unsigned long long *sclnc;
  unsigned *nnz;
};

struct BatchCommon {
  uint64_t item0;        // first item to process (autotuning samples)
  int nsteps;
  int nschemes;
  int scheme;
  int nb;
  int fix_scale;         // moment scale s (counts beyond the table)
};

struct PairParams {
  const uint8_t *bins;
  uint64_t nframes;
  uint64_t step_size;
  uint64_t ntile;       // tiles per side (all-pairs mode)
  uint64_t stripe;      // tile columns per stripe of the tile order (all-pairs
                        // mode; set by launch_pairs_atomic)
  uint32_t ndof;
  int nschemes;
  int scheme;
  int nb;
  int nsteps;
  int all_pairs;
  int tile;             // DOFs per tile side (all-pairs mode)
  int fix_scale;        // moment scale s (counts beyond the table)
  int want_nnz;         // non-empty cell counts needed (Miller-Madow); the
                        // 4 x 4 histogram kernel skips them otherwise
};

constexpr int kTabGlobal = 1 << 16; // entries of a fixed-point c ln c table

// c*log(c) in double precision, the per-cell term of the joint entropy.
// Every count form evaluates it through this one expression (or reads it
// from the table the same expression filled), so all forms see identical
// doubles.
__device__ __forceinline__ double clnc_value(unsigned c) {
  return (c < 2) ? 0.0 : (double)c * log((double)c);
}

// The joint-count moments.  Per pair and step the count kernels produce
//     X = sum over cells of F(c),   F(c) = round(c ln c * 2^s),
// an unsigned 64-bit integer, and the number of non-empty cells.  The scale s
// is fixed per call from the frames used, n (moment_scale): the largest s <= 52
// with n ln n * 2^s <= 2^63, so no sum of cells (at most n ln n plus half a
// unit per cell) can overflow.  Every count form reads F from the same table
// (or evaluates the same expression beyond it), and integer sums do not
// depend on their order, so all forms give the same X to the last bit.  The
// rounding of F is at most 2^-(s+1) per cell, so X * 2^-s differs from the
// double sum of c ln c by at most cells * 2^-(s+1): with 2^-s <= 2 n ln n /
// 2^63 that moves an entropy (X/n) by less than cells * ln n / 2^63, about
// 1e-13 at 255 bins and 2^27 frames.
__device__ __forceinline__ unsigned long long clnc_fix(unsigned c, int s) {
  return __double2ull_rn(clnc_value(c) * ldexp(1.0, s));
}

// Row-major upper-triangular pair (i, j), i < j, of index p among all pairs
// of n items: a single-precision estimate of the row, corrected exactly with
// integer arithmetic (no FP64 on the per-element path).
// (Conversions go through 32-bit integers: 64-bit integer <-> float
// conversions run on the FP64 pipe, which is scarce on this part.)
__device__ __forceinline__ void tri_pair(uint64_t p, uint64_t n, uint32_t &i, uint32_t &j) {
  const float nn = (float)(uint32_t)n;
  const float pf = __fmaf_rn((float)(uint32_t)(p >> 32), 4294967296.f, (float)(uint32_t)p);
  const float disc = (2.f * nn - 1.f) * (2.f * nn - 1.f) - 8.f * pf;
  long long r = (int)((2.f * nn - 1.f - sqrtf(fmaxf(disc, 0.f))) * 0.5f);
  if (r < 0) r = 0;
  if (r > (long long)n - 2) r = (long long)n - 2;
  auto start = [n](long long rr) { return (uint64_t)rr * n - (uint64_t)rr * (uint64_t)(rr + 1) / 2; };
  while (r > 0 && start(r) > p) --r;
  while (r + 1 < (long long)n - 1 && start(r + 1) <= p) ++r;
  i = (uint32_t)r;
  j = (uint32_t)(p - start(r) + (uint64_t)r + 1);
}

// Tile columns per stripe of the all-pairs tile order (decode_all_pairs_tile)
// for tiles of `tile` DOFs per side and nframes bytes per DOF row.
uint64_t all_pairs_stripe(int tile, uint64_t nframes, uint64_t ntile);
// Moment scale for n frames used (see clnc_fix).
int moment_scale(uint64_t n);
// Fills tab[c] = F(c) for c < kTabGlobal at scale s (one kernel launch on
// the context's stream; no allocation).
int fill_fix_table(centre_ctx *ctx, unsigned long long *tab, int s);
// The context's table for scale s, built on first use (cudaMalloc: call it
// before any stream capture).
const unsigned long long *fix_table(centre_ctx *ctx, int s, int *status);
int launch_entropy1d(centre_ctx *ctx, const EntParams &P, uint32_t ndof, const uint8_t *d_types,
                     const uint8_t *d_bins, const double *d_ext, double *d_s1,
                     unsigned long long *d_freq, double *d_lsum);
int pair_tile_for(int nb);
int launch_pairs_atomic(centre_ctx *ctx, const PairParams &P, const PairTask *d_tasks,
                        uint64_t ntasks, const unsigned long long *d_fix,
                        unsigned long long *d_sclnc, unsigned *d_nnz, unsigned *d_counts);
int prepare_pairs_hist_batch(centre_ctx *ctx, int tile, int nb);
size_t pairs_hist_batch_smem(int tile, int nb);
int pairs_hist_batch_occupancy(centre_ctx *ctx, int tile, int threads, int nb, int *per_sm);
int launch_pairs_hist_batch(centre_ctx *ctx, const BatchSys *d_sys, int nsys, uint64_t nitems,
                            const BatchCommon &B, int tile, int threads, int grid,
                            const unsigned long long *d_fix);
int launch_pairs_global(centre_ctx *ctx, const PairParams &P, const uint32_t *d_pairs,
                        uint64_t p0, uint64_t np, const unsigned long long *d_fix,
                        unsigned long long *d_sclnc, unsigned *d_nnz, unsigned *d_counts);
int launch_finalize2d(centre_ctx *ctx, const EntParams &P, int scheme, const uint32_t *d_pairs,
                      int all_pairs, uint32_t ndof, const double *d_ext, const double *d_lsum,
                      const unsigned long long *d_sclnc, const unsigned *d_nnz, uint64_t npairs,
                      double *d_s2);
int launch_finalize2d_into(centre_ctx *ctx, const EntParams &P, int scheme, uint32_t ndof,
                           const double *d_ext, const double *d_lsum,
                           const unsigned long long *d_sclnc, const unsigned *d_nnz,
                           uint64_t npairs, double *d_logw, double *d_s2);
int launch_entropy2d_counts(centre_ctx *ctx, const EntParams &P, int scheme,
                            const uint32_t *d_pairs, const uint8_t *d_types, const double *d_ext,
                            const unsigned *d_counts, uint64_t p0, uint64_t np, uint64_t npairs,
                            double *d_s2);

// discretize.cu
int launch_discretize(centre_ctx *ctx, int bat_type, const float *d_data, uint32_t ndof,
                      uint64_t nframes, const uint8_t *schemes, uint32_t nschemes,
                      uint8_t bins_ref, int optimize, uint8_t *d_bins, double *d_ext,
                      bool reset_flag = true);

// vmkde.cu
int launch_vmkde(centre_ctx *ctx, const float *d_data, uint32_t ndof, uint64_t nframes,
                 uint8_t nmaxconf, double kappa, uint32_t sdo_nstep, double sdo_conv,
                 uint32_t sdo_niter, uint8_t *d_bins, double *d_minima, uint8_t *d_nfound,
                 double *d_work);
size_t vmkde_work_doubles(uint32_t ndof);

// gridkde.cu
int launch_gridkde(centre_ctx *ctx, int bat_type, const float *d_data, uint32_t ndof,
                   uint64_t nframes, int ngrid, double kappa, uint8_t *d_bins, double *d_minima,
                   uint8_t *d_nmin, uint8_t *d_nbins, void *d_work);
size_t gridkde_work_bytes(uint32_t ndof);
int launch_df_exp_eval(centre_ctx *ctx, const double *d_y, uint64_t n, double *d_out);

// gemm_tc.cu: the driver's cuTensorMapEncodeTiled (null when unavailable)
void *tensor_map_encoder();
// gemm_tc.cu: R = X X^T (X bf16 n x K, leading dimension ldx, a multiple of
// 8; R fp32 n x n, leading dimension ldr, a multiple of 4)
int launch_corr_gemm(centre_ctx *ctx, const void *X, uint32_t n, uint32_t K, uint32_t ldx,
                     float *R, uint32_t ldr);

// pairs_tc.cu
bool tc_supported(centre_ctx *ctx, int nb, uint64_t nframes);
// largest bin count at which AUTO prefers the tensor-core contraction over
// a shared-memory histogram that fits (none: the two are within 2 % at 16 bins,
// 120.2 vs 118.7 ms for the 2994-DOF chain, and the histogram is faster above
// it); AUTO takes the contraction only where the histograms do not fit shared
// memory
constexpr int kTcAutoMaxBins = 0;
int launch_pairs_tc(centre_ctx *ctx, const PairParams &P, const unsigned long long *d_fix,
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
size_t score_scratch_bytes(const ScoreParams &S, bool tree);
int launch_score_async(centre_ctx *ctx, const ScoreParams &S, const uint8_t *d_types,
                       const uint32_t *d_pairs, const double *d_s1, const double *d_s2,
                       double *d_mi, double *d_mie, double *d_mist, void *d_scratch);
int launch_score(centre_ctx *ctx, const ScoreParams &S, const uint8_t *d_types,
                 const uint32_t *d_pairs, const double *d_s1, const double *d_s2, double *d_mi,
                 double *h_mie, int build_tree, double *h_mist, uint32_t *h_tree,
                 uint32_t *h_ntree);

}  // namespace centre
