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

// Unsigned 128-bit accumulator for the per-cell c ln c terms.
struct __align__(16) U128 {
  unsigned long long lo, hi;
};

// One trajectory of a batch (device copy; see batch.cu).
struct BatchSys {
  const uint8_t *bins;
  uint64_t nframes;
  uint64_t step_size;
  uint64_t ntile;        // tiles per side of the all-pairs grid
  uint64_t item_begin;   // first work item of this trajectory
  uint32_t ndof;
  U128 *sclnc;
  unsigned *nnz;
};

struct BatchCommon {
  uint64_t item0;        // first item to process (autotuning samples)
  int nsteps;
  int nschemes;
  int scheme;
  int nb;
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

__device__ __forceinline__ U128 u128_add(U128 a, U128 b) {
  U128 r;
  asm("add.cc.u64 %0, %2, %4;\n\taddc.u64 %1, %3, %5;"
      : "=l"(r.lo), "=l"(r.hi)
      : "l"(a.lo), "l"(a.hi), "l"(b.lo), "l"(b.hi));
  return r;
}

__device__ __forceinline__ U128 u128_shfl_xor(U128 v, int o) {
  v.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
  v.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
  return v;
}

// c*log(c) in double precision, the per-cell term of the joint entropy.
// Every count form evaluates it through this one expression (or reads it
// from the table the same expression filled), so all forms see identical
// doubles.
__device__ __forceinline__ double clnc_value(unsigned c) {
  return (c < 2) ? 0.0 : (double)c * log((double)c);
}

// A non-negative double v (0 or >= 1) represented exactly as an integer
// multiple of 2^-52: its 53-bit significand shifted by its exponent (a double
// >= 1 is a multiple of its ulp >= 2^-52, so the shift is a left shift and
// nothing is rounded).  Integer sums of these are the exact sums of the
// per-cell doubles, so the cell sum is independent of how cells are spread
// over threads, tiles or count kernels.  c ln c < 2^12 (counts below 630)
// fits in the low word alone.
constexpr int kFixShift = 52;   // fixed point: value * 2^52
__device__ __forceinline__ U128 u128_from_double(double v) {
  U128 r;
  r.lo = 0ull;
  r.hi = 0ull;
  // integer test for +-0 (no FP64 instruction: FP64 issue is scarce on this part)
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  if ((bits << 1) == 0ull) return r;
  // value * 2^52 = m * 2^(e - 1023), e the biased exponent
  const int s = (int)((bits >> 52) & 0x7ff) - 1023 + (kFixShift - 52);
  const unsigned long long m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  if (s >= 64) {
    r.hi = m << (s - 64);
  } else {
    r.lo = m << s;
    r.hi = s ? (m >> (64 - s)) : 0ull;
  }
  return r;
}

__device__ __forceinline__ U128 clnc_fixed(unsigned c) { return u128_from_double(clnc_value(c)); }

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

__host__ __device__ __forceinline__ double u128_value(U128 x) {
  return (double)x.hi * 0x1p12 + (double)x.lo * 0x1p-52;
}

int init_clnc_table(centre_ctx *ctx, double *tab);
int launch_entropy1d(centre_ctx *ctx, const EntParams &P, uint32_t ndof, const uint8_t *d_types,
                     const uint8_t *d_bins, const double *d_ext, double *d_s1,
                     unsigned long long *d_freq, double *d_lsum);
int pair_tile_for(int nb);
int launch_pairs_atomic(centre_ctx *ctx, const PairParams &P, const PairTask *d_tasks,
                        uint64_t ntasks, const double *d_tab, U128 *d_sclnc, unsigned *d_nnz,
                        unsigned *d_counts);
int prepare_pairs_hist_batch(centre_ctx *ctx, int tile, int nb);
size_t pairs_hist_batch_smem(int tile, int nb);
int pairs_hist_batch_occupancy(centre_ctx *ctx, int tile, int threads, int nb, int *per_sm);
int launch_pairs_hist_batch(centre_ctx *ctx, const BatchSys *d_sys, int nsys, uint64_t nitems,
                            const BatchCommon &B, int tile, int threads, int grid,
                            const double *d_tab);
int launch_pairs_global(centre_ctx *ctx, const PairParams &P, const uint32_t *d_pairs,
                        uint64_t p0, uint64_t np, const double *d_tab, U128 *d_sclnc,
                        unsigned *d_nnz, unsigned *d_counts);
int launch_finalize2d(centre_ctx *ctx, const EntParams &P, int scheme, const uint32_t *d_pairs,
                      int all_pairs, uint32_t ndof, const double *d_ext, const double *d_lsum,
                      const U128 *d_sclnc, const unsigned *d_nnz, uint64_t npairs,
                      double *d_s2);
int launch_finalize2d_into(centre_ctx *ctx, const EntParams &P, int scheme, uint32_t ndof,
                           const double *d_ext, const double *d_lsum, const U128 *d_sclnc,
                           const unsigned *d_nnz, uint64_t npairs, double *d_logw,
                           double *d_s2);
int launch_entropy2d_counts(centre_ctx *ctx, const EntParams &P, int scheme,
                            const uint32_t *d_pairs, const uint8_t *d_types, const double *d_ext,
                            const unsigned *d_counts, uint64_t p0, uint64_t np, uint64_t npairs,
                            double *d_s2);

// discretize.cu
int launch_discretize(centre_ctx *ctx, int bat_type, const float *d_data, uint32_t ndof,
                      uint64_t nframes, const uint8_t *schemes, uint32_t nschemes,
                      uint8_t bins_ref, int optimize, uint8_t *d_bins, double *d_ext);

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

// pairs_tc.cu
bool tc_supported(centre_ctx *ctx, int nb, uint64_t nframes);
// largest bin count at which AUTO prefers the tensor-core contraction over
// a shared-memory histogram that fits (none: with interleaved histograms the
// histogram form is faster at every bin count it covers, e.g. 134 vs 159 ms
// at 16 bins for the 2994-DOF chain); AUTO takes the contraction only where
// the histograms do not fit shared memory
constexpr int kTcAutoMaxBins = 0;
int launch_pairs_tc(centre_ctx *ctx, const PairParams &P, const double *d_tab, U128 *d_sclnc,
                    unsigned *d_nnz);

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
