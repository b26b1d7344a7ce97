/*
 * centre_gpu.h -- C ABI of the GB300 (sm_103a) CENTRE entropy hot path.
 *
 * The reference (shaileshp51/centre) has no plugin or FFI layer: its hot path
 * is three C++ stage classes (Discretizer, EntropyCalculator, EntropyScorer)
 * over free numeric functions.  Each entry point below replaces one of those
 * functions or stage loops; the reference file:line it stands in for is given
 * beside it.  Signatures use plain pointers and sizes only.
 *
 * Conventions
 *  - Every call returns a centre_status (0 = success, < 0 = error) and never
 *    exits the process; centre_gpu_strerror() names the code and
 *    centre_gpu_last_error() gives a message for the last failing call.
 *  - Functions without a suffix take HOST pointers and block until their
 *    results are back in host memory.  The *_dev variants take DEVICE pointers
 *    and are enqueued on the context's stream (centre_gpu_set_stream) without
 *    synchronising.
 *  - One context per host thread; a context is not thread-safe.
 *  - Layouts are the reference's:
 *      BAT input   [ndof][nframes] float32, DOF-major (Netcdf_BAT.cpp:236-330
 *                  transposes the file's [frame][dof] into this)
 *      bins        [ndof][nschemes][nframes] uint8 (Netcdf_TrjInt coord var)
 *      extremes    [ndof][4] float64: min, max, avg, phase
 *      entropies   [ndof or npairs][nestimators][nschemes][nsteps] float64
 *                  (Netcdf_EntContri contri_S, Estimators.cpp:239-243)
 *      pairs       [npairs][2] uint32 DOF indices into the bins array
 */
#ifndef CENTRE_GPU_H
#define CENTRE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CENTRE_GPU_ABI_VERSION 1

typedef struct centre_ctx centre_ctx;

typedef enum centre_status {
  CENTRE_OK = 0,
  CENTRE_E_ARG = -1,          /* invalid argument                           */
  CENTRE_E_CUDA = -2,         /* CUDA runtime error                         */
  CENTRE_E_NOMEM = -3,        /* device allocation failed                   */
  CENTRE_E_BINRANGE = -4,     /* a bin index >= its scheme's bin count      */
  CENTRE_E_TIMEOUT = -5,      /* a device-side wait ran out its limit       */
  CENTRE_E_UNSUPPORTED = -6,  /* combination not supported on this path     */
  CENTRE_E_NODEVICE = -7      /* no usable sm_103 device                    */
} centre_status;

/* BAT_t, src/Centre.h:42-47 */
enum { CENTRE_NONE = 0, CENTRE_BOND = 1, CENTRE_ANGLE = 2, CENTRE_DIHEDRAL = 3 };
/* EntropyEstimators, src/Centre.h:89-94 */
enum { CENTRE_ML = 0, CENTRE_MM = 1, CENTRE_CS = 2, CENTRE_JS = 3 };
/* How the 2-D joint counts are formed. */
enum {
  CENTRE_COUNTS_AUTO = 0,   /* histogram form where it fits, else TC      */
  CENTRE_COUNTS_ATOMIC = 1, /* shared-memory atomic histograms            */
  CENTRE_COUNTS_TC = 2      /* FP8 one-hot O^T O on tcgen05 tensor cores
                             * (16-255 bins, at most 2^22 frames)        */
};

/* Entropy-stage parameters ([entropy]/[control]/[histogram] keys of the
 * reference input file, src/Inputs.cpp:100-553). */
typedef struct centre_entropy_params {
  uint64_t nframes;           /* frames per DOF in the bins array           */
  uint8_t nsteps;             /* [control] nsteps                           */
  uint8_t nschemes;           /* number of bin schemes                      */
  uint8_t nestimators;        /* number of estimators                       */
  uint8_t jacobian;           /* [entropy] jacobian                         */
  uint8_t kde;                /* pdfmethod == vonmiseskde                   */
  uint8_t counts_form;        /* CENTRE_COUNTS_*                            */
  uint8_t bin_schemes[16];    /* [histogram] nbins (first nschemes used)    */
  uint8_t estimators[4];      /* [entropy] estimator (first nestimators)    */
} centre_entropy_params;

/* ------------------------------------------------------------ context ---- */
int centre_gpu_create(centre_ctx **ctx, int device);
void centre_gpu_destroy(centre_ctx *ctx);
const char *centre_gpu_strerror(int status);
const char *centre_gpu_last_error(const centre_ctx *ctx);
int centre_gpu_set_stream(centre_ctx *ctx, void *cuda_stream);
int centre_gpu_synchronize(centre_ctx *ctx);
/* Number of kernels this library has launched on the context so far. */
uint64_t centre_gpu_launch_count(const centre_ctx *ctx);

/* Device time of the library's hot kernels, measured with CUDA events on the
 * context's stream while timing is enabled (no reference counterpart: the
 * reference's ProgState timers, src/main_common.h:52-163, time whole
 * stages on the host).  centre_gpu_timer synchronises the stream and
 * returns the milliseconds and launch count accumulated since timing was
 * enabled for one class. */
enum {
  CENTRE_TIMER_DISCRETIZE = 0, /* histogram discretisation kernel      */
  CENTRE_TIMER_COUNTS1D = 1,   /* 1-D counts / entropies kernel        */
  CENTRE_TIMER_PAIRS = 2,      /* 2-D joint count kernel (either form) */
  CENTRE_TIMER_SCORE = 3,      /* MI, sums and spanning-tree kernels   */
  CENTRE_TIMER_CLASSES = 4
};
int centre_gpu_enable_timing(centre_ctx *ctx, int enable);
int centre_gpu_timer(centre_ctx *ctx, int which, double *ms, uint64_t *launches);

/* ----------------------------------------------------- discretisation ---- */
/* Histogram binning of one DOF-type block: Real2Int::bndReal2Int
 * (src/Real2Int.cpp:27), ::angReal2Int (:131), ::dihReal2Int (:244), driven
 * per DOF as in Discretizer::run_dtype (src/Discretizer.cpp:138-207).
 * bins_ref and optimize_dih are [histogram] referencenbins and
 * [discretization] optimizedih.  Bin indices and min/max/phase are
 * bit-identical to the reference; avg agrees to rounding. */
int centre_gpu_discretize(centre_ctx *ctx, int bat_type, const float *data,
                          uint32_t ndof, uint64_t nframes,
                          const uint8_t *bin_schemes, uint32_t nschemes,
                          uint8_t bins_ref, int optimize_dih, uint8_t *bins,
                          double *extremes);
int centre_gpu_discretize_dev(centre_ctx *ctx, int bat_type, const float *data,
                              uint32_t ndof, uint64_t nframes,
                              const uint8_t *bin_schemes, uint32_t nschemes,
                              uint8_t bins_ref, int optimize_dih,
                              uint8_t *bins, double *extremes);

/* von Mises KDE conformer assignment of torsions: Real2Int::getMinimaPositions
 * (src/Real2Int.cpp:481) with analyticGrad=false as Discretizer.cpp:177 calls
 * it.  minima [ndof][nmaxconf] radians (unused slots 0), nfound [ndof];
 * bins [ndof][nframes].  The reference records min/max/avg/phase as 1000.0
 * for KDE-binned DOFs (Discretizer.cpp:139-142).  The grid sums run in FP64
 * in a different order from the reference, so minima agree to rounding and
 * a frame lying within rounding of a minimum can take the other label. */
int centre_gpu_discretize_vmkde(centre_ctx *ctx, const float *data,
                                uint32_t ndof, uint64_t nframes,
                                uint8_t nmaxconf, double kappa,
                                uint32_t sdo_nstep, double sdo_conv,
                                uint32_t sdo_niter, uint8_t *bins,
                                double *minima, uint8_t *nfound);

/* Grid-KDE conformer binning of one DOF-type block (bat_type 1 bonds, 2
 * angles, 3 torsions), a KDE variant with no reference counterpart beside
 * centre_gpu_discretize_vmkde (which follows Real2Int::getMinimaPositions,
 * src/Real2Int.cpp:481, for torsions only).  Torsions: von Mises kernel
 * exp(kappa (cos(g - a) - 1)) on ngrid points g_j = 2 pi j / ngrid.  Bonds and
 * angles: Gaussian kernel with h = 1.06 sigma N^(-1/5) on ngrid points
 * lo + (j + 1/2)(hi - lo)/ngrid (kappa unused).  Grid minima
 * (d_j < d_{j-1}, d_j <= d_{j+1}, cyclic for torsions) bound the conformer
 * intervals; bins [ndof][nframes] = interval index (linear: #minima <= x;
 * torsions: (#{minima <= a} + M - 1) mod M).  minima [ndof][ngrid] (first
 * nmin[d] used), nbins [ndof] = bins used by the DOF.  ngrid 3..128.  Grid
 * sums are FP64; non-finite inputs give CENTRE_E_ARG.  Entropies of these
 * bins take the KDE form (bin width 1), as for the reference's KDE. */
int centre_gpu_discretize_gridkde(centre_ctx *ctx, int bat_type, const float *data,
                                  uint32_t ndof, uint64_t nframes, uint32_t ngrid,
                                  double kappa, uint8_t *bins, double *minima,
                                  uint8_t *nmin, uint8_t *nbins);
int centre_gpu_discretize_gridkde_dev(centre_ctx *ctx, int bat_type, const float *data,
                                      uint32_t ndof, uint64_t nframes, uint32_t ngrid,
                                      double kappa, uint8_t *bins, double *minima,
                                      uint8_t *nmin, uint8_t *nbins);

/* Diagnostics: the double-float e^y (y <= 0; ~48-bit, table-driven, on the
 * FP32 pipe) that the grid KDE's torsion sums use, evaluated for host
 * doubles y into host doubles out, so tests can bound its error against
 * FP64.  No reference counterpart. */
int centre_gpu_df_exp_eval(centre_ctx *ctx, const double *y, uint64_t n, double *out);

/* ------------------------------------------------------------ entropy ---- */
/* 1-D counts and entropies: binData1D (src/Estimators.cpp:56) + entropy1D
 * (:217) for every DOF, as EntropyCalculator::run1d (EntropyCalculator.cpp:
 * 156-199).  s1 [ndof][nest][nsch][nsteps]; freq (optional, may be NULL)
 * [ndof][nsteps][sum nb] cumulative counts. */
int centre_gpu_entropy1d(centre_ctx *ctx, const centre_entropy_params *p,
                         uint32_t ndof, const uint8_t *types,
                         const uint8_t *bins, const double *extremes,
                         double *s1, uint64_t *freq);
int centre_gpu_entropy1d_dev(centre_ctx *ctx, const centre_entropy_params *p,
                             uint32_t ndof, const uint8_t *types,
                             const uint8_t *bins, const double *extremes,
                             double *s1, uint64_t *freq);

/* 2-D joint entropies of a pair list: binData2D (src/Estimators.cpp:130) +
 * entropy2D (:391) per pair, as EntropyCalculator::run2d_xx/run2d_xy
 * (EntropyCalculator.cpp:281, :674).  pairs == NULL means every pair i<j of
 * the ndof DOFs in row-major order.  s2 [npairs][nest][nsch][nsteps]. */
int centre_gpu_entropy2d(centre_ctx *ctx, const centre_entropy_params *p,
                         uint32_t ndof, const uint8_t *types,
                         const uint8_t *bins, const double *extremes,
                         uint64_t npairs, const uint32_t *pairs, double *s2);
int centre_gpu_entropy2d_dev(centre_ctx *ctx, const centre_entropy_params *p,
                             uint32_t ndof, const uint8_t *types,
                             const uint8_t *bins, const double *extremes,
                             uint64_t npairs, const uint32_t *pairs,
                             double *s2);

/* The all-pairs case of centre_gpu_entropy2d_dev without allocating any
 * memory: no context is needed, all scratch space comes from one fixed
 * device array of 16 MiB inside the library.  No counterpart in the
 * reference, which allocates host memory per pair.  It serves callers that
 * must not call cudaMalloc: plug-ins whose host application owns every byte
 * of device memory through its own pool and forbids foreign allocations, and
 * loops that must not stall on the device-wide synchronisation an
 * allocation can cause.
 *   - Device pointers, enqueued on `cuda_stream`; returns after the stream
 *     has finished the call (it reads back an error flag).
 *   - ML and Miller-Madow estimators, shared-memory histogram counts only
 *     (CENTRE_E_UNSUPPORTED otherwise).
 *   - Sizes whose scratch exceeds the array (about 1.3 million pair-steps,
 *     e.g. 500 DOFs with 10 steps) are rejected with CENTRE_E_ARG before anything
 *     runs; larger problems use centre_gpu_entropy2d_dev.
 *   - The first call on a device records the array's address and fills a
 *     table in it (refilled when a call's frame count needs another
 *     fixed-point scale); make that first call before any stream capture.
 *   - Every call on a device shares the array: calls that overlap on the GPU
 *     (other streams, other host threads) race and must be serialised. */
int centre_gpu_entropy2d_static(const centre_entropy_params *p, uint32_t ndof,
                                const uint8_t *types, const uint8_t *bins,
                                const double *extremes, double *s2,
                                void *cuda_stream);

/* Joint counts only, for parity checks of the count kernels: binData2D
 * (src/Estimators.cpp:130-205) per pair.  freq [npairs][nsteps][sum nb^2]
 * cumulative, cell a*nb+b. */
int centre_gpu_counts2d(centre_ctx *ctx, const centre_entropy_params *p,
                        uint32_t ndof, const uint8_t *bins, uint64_t npairs,
                        const uint32_t *pairs, uint64_t *freq);

/* The learned screen's correlation matrix on the tensor cores (no
 * counterpart in the reference, which reads neighbour lists from files,
 * src/Centre.cpp:459-593): R = X X^T for X, n rows of K bf16 values with
 * leading dimension ldx (a multiple of 8, 16-byte aligned), into R, n rows
 * of fp32 with leading dimension ldr (a multiple of 4).  Device pointers;
 * returns when the GEMM has finished. */
int centre_gpu_corr_gemm_dev(centre_ctx *ctx, const void *X, uint32_t n, uint32_t K,
                             uint32_t ldx, float *R, uint32_t ldr);

/* Integer moments of the joint counts of every pair i<j for one bin scheme,
 * as both count forms produce them (no reference counterpart: the
 * reference keeps the counts themselves, src/Estimators.cpp:130-205, and sums
 * p log p in entropy2D, :586-631).  Per pair and step: the sum over cells of
 * round(c*ln(c) * 2^s) as an unsigned 64-bit integer and the number of
 * non-empty cells; s (returned in *scale) is the largest s <= 52 with
 * n ln n * 2^s <= 2^63 for the n frames used, so no sum overflows.  Used to
 * check that the tensor-core and atomic forms count identically.
 *   clnc [npairs][nsteps] uint64, nnz [npairs][nsteps] uint32. */
int centre_gpu_pair_moments(centre_ctx *ctx, const centre_entropy_params *p,
                            uint32_t ndof, const uint8_t *bins, int scheme,
                            uint64_t *clnc, uint32_t *nnz, int *scale);

/* ------------------------------------------------------------ scoring ---- */
/* Number of doubles per (estimator, scheme, step) in the sums outputs: the
 * columns of the reference's MIE/MIST convergence CSV after TIME
 * (EntropyScorer.cpp:574-629): BOND-S1 ANGLE-S1 DIHED-S1, then S2 and I2 for
 * B/B A/A D/D B/A B/D A/D, then S1 and S2 totals. */
#define CENTRE_SUMS_COLS 17

/* EntropyScorer::run (src/EntropyScorer.cpp:287-866): MI = S_i + S_j - S_ij
 * (getMaxMI2D, src/Convergance.cpp:183-194), MIE sums, and when build_tree is
 * non-zero the MIST maximum spanning tree (boruvkaMST, src/Centre.cpp:5) over
 * the pair list in the given order (edge order breaks ties: the first edge
 * of largest MI wins, as in the reference).  DOF types give the B/A/D
 * blocks.
 *   mi        [npairs][nest][nsch][nsteps] (may be NULL)
 *   mie_sums  [nest][nsch][nsteps][CENTRE_SUMS_COLS]
 *   mist_sums [nest][nsch][nsteps][CENTRE_SUMS_COLS] (build_tree only)
 *   tree      [nest][nsch][nsteps][ndof-1] pair indices, sorted by MI desc
 *             then index (build_tree only); ntree [nest][nsch][nsteps]. */
int centre_gpu_score(centre_ctx *ctx, const centre_entropy_params *p,
                     uint32_t ndof, const uint8_t *types, const double *s1,
                     uint64_t npairs, const uint32_t *pairs, const double *s2,
                     int build_tree, double *mi, double *mie_sums,
                     double *mist_sums, uint32_t *tree, uint32_t *ntree);
int centre_gpu_score_dev(centre_ctx *ctx, const centre_entropy_params *p,
                         uint32_t ndof, const uint8_t *types, const double *s1,
                         uint64_t npairs, const uint32_t *pairs,
                         const double *s2, int build_tree, double *mi,
                         double *mie_sums, double *mist_sums, uint32_t *tree,
                         uint32_t *ntree);

/* -------------------------------------------------------------- batch ---- */
/* One trajectory of a batch: device arrays in the single-trajectory layouts
 * above (types [ndof], bins [ndof][nschemes][nframes], extremes [ndof][4],
 * s1 [ndof][est][sch][steps], s2 [ndof*(ndof-1)/2][est][sch][steps] over all
 * pairs i<j, mi like s2 or NULL) and host rows for the sums
 * (mie_sums, mist_sums [est][sch][steps][CENTRE_SUMS_COLS]; mist_sums may be
 * NULL to skip the spanning tree).  Each trajectory has its own frame count;
 * the convergence steps are prefixes of it (src/Estimators.cpp:162-188). */
typedef struct centre_system {
  uint32_t ndof;
  uint64_t nframes;
  const uint8_t *types;
  const uint8_t *bins;
  const double *extremes;
  double *s1;
  double *s2;
  double *mi;
  double *mie_sums;
  double *mist_sums;
} centre_system;

/* EntropyCalculator::run (src/EntropyCalculator.cpp:1090) followed by
 * EntropyScorer::run (src/EntropyScorer.cpp:7) for nsys trajectories at
 * once: 1-D entropies, all-pairs joint entropies (one persistent count
 * kernel over every trajectory's pair tiles), MI, MIE sums and, where asked,
 * the MIST tree sums.  The work is captured into one CUDA graph, cached by
 * the call's arguments and replayed when the same batch comes back; the
 * count kernel's tile shape and block size are tuned on the first call for
 * each (bins, steps, schemes).  ML and MM estimators; p->nframes is ignored
 * (each trajectory's nframes is used).  Returns after the sums are on the
 * host. */
int centre_gpu_entropy_batch_dev(centre_ctx *ctx, const centre_entropy_params *p,
                                 uint32_t nsys, const centre_system *sys);

/* -------------------------------------------------------- pair screen ---- */
/* Learned neighbour selection for A-MIE / A-MIST.  The reference takes the
 * pairs of its approximate methods from a neighbour file made outside the
 * program (useneighbor=true, Neighbors(fname), src/Centre.cpp:459-593);
 * this selects them from the data.  A BF16 MLP 12 -> 64 -> 64 -> 1 scores
 * the partners that pass a correlation prefilter from 12 per-pair features
 * (prefix marginal entropies, DOF types, index distance within the type,
 * the 2x2 correlation block of (cos, sin) or standardised bin columns, a
 * Gaussian MI proxy); the network is trained on exact MI of random pairs at
 * the first of feat_div convergence steps.  No reference counterpart. */
#define CENTRE_SCREEN_NPARAMS 5057
typedef struct centre_screen_params {
  uint32_t feat_div;    /* features and labels use the first nframes/feat_div frames */
  uint32_t ntrain;      /* random training pairs                                 */
  uint32_t nprefilter;  /* partners per DOF kept by the correlation prefilter   */
  uint32_t nneigh;      /* partners per DOF kept by the network                 */
  uint32_t epochs;      /* training epochs                                       */
  uint32_t batch;       /* minibatch size                                        */
  float lr;             /* Adam learning rate                                    */
  uint8_t train;        /* 1: train the network here, 0: use weights as given   */
  uint8_t init_weights; /* with train: start from seeded random weights         */
  uint64_t seed;
} centre_screen_params;

/* Device inputs as centre_gpu_entropy1d_dev (DOF types in bonds, angles,
 * torsions order); weights [CENTRE_SCREEN_NPARAMS] host FP32 (in, and the
 * trained weights out when training), losses [epochs] host mean squared
 * error per epoch (may be NULL); pairs: device [capacity][2] out, every
 * selected pair i<j in row-major order, *npairs their number (capacity
 * ndof*nneigh always suffices). */
int centre_gpu_screen_dev(centre_ctx *ctx, const centre_entropy_params *p,
                          const centre_screen_params *sp, uint32_t ndof,
                          const uint8_t *types, const uint8_t *bins,
                          const double *extremes, float *weights, float *losses,
                          uint64_t capacity, uint32_t *pairs, uint64_t *npairs);

/* The same with host inputs and a host pair list [capacity][2]. */
int centre_gpu_screen(centre_ctx *ctx, const centre_entropy_params *p,
                      const centre_screen_params *sp, uint32_t ndof,
                      const uint8_t *types, const uint8_t *bins,
                      const double *extremes, float *weights, float *losses,
                      uint64_t capacity, uint32_t *pairs, uint64_t *npairs);

/* One forward and backward pass of the screen network over n samples
 * (host arrays): feats [n][12], targets [n]; pred [n] (may be NULL), grad
 * [CENTRE_SCREEN_NPARAMS] of the mean squared error, *loss that error.
 * Exposes the training kernels for gradient checks. */
int centre_gpu_screen_mlp_grad(centre_ctx *ctx, const float *weights, uint64_t n,
                               const float *feats, const float *targets, float *pred,
                               float *grad, double *loss);

#ifdef __cplusplus
}
#endif
#endif /* CENTRE_GPU_H */
