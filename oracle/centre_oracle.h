/*
 * centre_oracle.h -- CPU oracle for the CENTRE entropy hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (shaileshp51/centre, files cited per function) used as the
 * checker for the CUDA library and as the timed CPU baseline.  Nothing in the
 * product (the centre_gb300 package, its CUDA library or its C-ABI) links,
 * loads or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own
 * translation units compiled from source (oracle/_ref, built by
 * oracle/Makefile) on seeded inputs, and against the golden outputs shipped in
 * the reference's test_examples/example-1 (bin_*.nc, MIE/MIST CSVs, trees).
 *
 * Layouts follow the reference exactly:
 *   bins      [scheme][frame]                      (Netcdf_TrjInt coord)
 *   freq 1-D  [step][sum_s nb_s]                   (Estimators.cpp:87)
 *   freq 2-D  [step][sum_s nb_s^2], cell a*nb+b    (Estimators.cpp:171,178)
 *   entropy   [estimator][scheme][step]            (Estimators.cpp:239-243)
 */
#ifndef CENTRE_ORACLE_H
#define CENTRE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_NONE = 0, ORC_BOND = 1, ORC_ANGLE = 2, ORC_DIHEDRAL = 3 };
enum { ORC_ML = 0, ORC_MM = 1, ORC_CS = 2, ORC_JS = 3 };

/* Histogram discretisation (src/Real2Int.cpp:27-73, :131-184, :244-479). */
int orc_bnd_real2int(const float *x, uint64_t n, const uint8_t *schemes,
                     int nschemes, double *min_d, double *max_d,
                     double *avg_d, uint8_t *out);
int orc_ang_real2int(const float *x, uint64_t n, const uint8_t *schemes,
                     int nschemes, double *min_d, double *max_d,
                     double *avg_d, uint8_t *out);
int orc_dih_real2int(const float *x, uint64_t n, const uint8_t *schemes,
                     int nschemes, uint8_t bins_ref, int optimize,
                     double *min_d, double *max_d, double *avg_d,
                     double *phase_d, uint8_t *out);

/* Whole DOF block: [ndof][nframes] floats -> [ndof][nschemes][nframes] bins
 * and [ndof][4] extremes (min, max, avg, phase) as Discretizer.cpp:138-207. */
int orc_discretize_block(int bat_type, const float *x, uint32_t ndof,
                         uint64_t nframes, const uint8_t *schemes,
                         int nschemes, uint8_t bins_ref, int optimize,
                         uint8_t *bins, double *extremes, int nthreads);

/* von Mises KDE conformer assignment (src/Real2Int.cpp:481-716). */
double orc_bessel_i(int n, double x);
int orc_vmkde_minima(const float *x, uint64_t n, uint8_t n_conf_max,
                     double kappa, uint32_t step_sdo, double conv,
                     uint32_t max_iter, double *minima, uint8_t *found,
                     uint8_t *out);

/* Counts (src/Estimators.cpp:56-118, :130-205). */
int orc_bin1d(uint8_t nsteps, const uint8_t *schemes, int nschemes,
              uint64_t nframes, double min_d, double max_d,
              const uint8_t *data, uint64_t *freq, double *mids);
int orc_bin2d(uint8_t nsteps, const uint8_t *schemes, int nschemes,
              uint64_t nframes, double min1, double max1, double min2,
              double max2, const uint8_t *d1, const uint8_t *d2,
              uint64_t *freq, double *mids);

/* Plug-in entropies (src/Estimators.cpp:217-389, :391-651). */
int orc_entropy1d(int type, const uint8_t *ests, int nests, uint8_t nsteps,
                  uint64_t step_size, double min_d, double max_d,
                  int jacobian, int kde, const uint8_t *schemes, int nschemes,
                  const uint64_t *freq, double *entropy);
int orc_entropy2d(int type1, int type2, const uint8_t *ests, int nests,
                  uint8_t nsteps, uint64_t step_size, double min1,
                  double max1, double min2, double max2, int jacobian,
                  int kde, const uint8_t *schemes, int nschemes,
                  const uint64_t *freq, double *entropy);

/* Batched helpers used by tests and the CPU baseline (OpenMP when built with
 * -fopenmp).  dof bins are [ndof][nschemes][nframes]; extremes [ndof][4];
 * types [ndof]; outputs [ndof or npairs][nests][nschemes][nsteps]. */
int orc_entropy1d_block(uint32_t ndof, const uint8_t *types,
                        const uint8_t *bins, const double *extremes,
                        uint64_t nframes, uint8_t nsteps,
                        const uint8_t *schemes, int nschemes,
                        const uint8_t *ests, int nests, int jacobian, int kde,
                        double *s1, int nthreads);
int orc_entropy2d_pairs(uint64_t npairs, const uint32_t *pairs,
                        const uint8_t *types, const uint8_t *bins,
                        const double *extremes, uint64_t nframes,
                        uint8_t nsteps, const uint8_t *schemes, int nschemes,
                        const uint8_t *ests, int nests, int jacobian, int kde,
                        double *s2, int nthreads);

/* Boruvka maximum spanning tree (src/Centre.cpp:5-143).  Writes the indices
 * of tree edges in the order the reference pushes them; returns the count. */
int64_t orc_boruvka_mst(uint32_t nv, uint64_t ne, const uint32_t *src,
                        const uint32_t *dst, const double *w,
                        uint64_t *tree);

#ifdef __cplusplus
}
#endif
#endif
