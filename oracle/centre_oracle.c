/*
 * centre_oracle.c -- CPU oracle for the CENTRE entropy hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library and the timed
 * CPU baseline ("port").  The product never links or calls this file.
 *
 * Every function restates one reference routine of shaileshp51/centre in
 * plain C, keeping the reference's arithmetic (double precision, same
 * operation order, same integer casts) so that bin indices and counts are
 * bit-identical to the reference and entropies agree to rounding.  The
 * reference file:line each function follows is given in its comment.
 *
 * Parity pin: tests/test_oracle_ref.py compares this file against the
 * reference's own translation units compiled from source (oracle/_ref) on
 * seeded inputs; tests/test_oracle_golden.py compares it against fixtures
 * generated from the reference (tests/golden/) and against the example-1
 * outputs shipped with the reference.
 */
#include "centre_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/configcentre.h:22 and src/Constants.h:92-101 */
#define ORC_DX 5.0e-9
#define ORC_PI 3.141592653589793
#define ORC_SQRTPI 1.7724538509055159
#define ORC_TWOPI 6.283185307179586
#define ORC_DEGRAD 0.017453292519943295

/* (hbin_t) floor(v): the reference converts a double to unsigned char; on
 * the platforms it targets that is a truncating int conversion followed by
 * keeping the low byte. */
static inline uint8_t to_bin(double v) { return (uint8_t)(int32_t)floor(v); }

static void minmaxsum(const float *x, uint64_t n, double *mn, double *mx,
                      double *sum) {
  double lo = 1.0e100, hi = -1.0e100, s = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    s += x[i];
    if (lo > x[i]) lo = x[i];
    if (hi < x[i]) hi = x[i];
  }
  *mn = lo;
  *mx = hi;
  *sum = s;
}

static void bin_linear(const float *x, uint64_t n, const uint8_t *schemes,
                       int nschemes, double lo, double hi, uint8_t *out) {
  for (int b = 0; b < nschemes; ++b) {
    double width = (hi - lo) / (int)schemes[b];
    uint8_t *o = out + (uint64_t)b * n;
    for (uint64_t i = 0; i < n; ++i) {
      uint8_t t = to_bin((x[i] - lo) / width);
      o[i] = (t == schemes[b]) ? (uint8_t)(t - 1) : t;
    }
  }
}

/* src/Real2Int.cpp:27-73 */
int orc_bnd_real2int(const float *x, uint64_t n, const uint8_t *schemes,
                     int nschemes, double *min_d, double *max_d,
                     double *avg_d, uint8_t *out) {
  double lo, hi, sum;
  if (n == 0) return -1;
  minmaxsum(x, n, &lo, &hi, &sum);
  lo -= ORC_DX;
  if (lo < 0.0) lo = 0.0;
  hi += ORC_DX;
  if ((hi - lo) < 1.0e-4) hi += 0.05;
  bin_linear(x, n, schemes, nschemes, lo, hi, out);
  *min_d = lo;
  *max_d = hi;
  *avg_d = sum / n;
  return 0;
}

/* src/Real2Int.cpp:131-184 */
int orc_ang_real2int(const float *x, uint64_t n, const uint8_t *schemes,
                     int nschemes, double *min_d, double *max_d,
                     double *avg_d, uint8_t *out) {
  double lo, hi, sum;
  if (n == 0) return -1;
  minmaxsum(x, n, &lo, &hi, &sum);
  lo -= ORC_DX;
  if (lo < 0.0) lo = 0.0;
  hi += ORC_DX;
  if (hi > ORC_PI) hi = ORC_PI;
  if ((hi - lo) < 1.0e-4) hi += 0.05;
  bin_linear(x, n, schemes, nschemes, lo, hi, out);
  *min_d = lo;
  *max_d = hi;
  *avg_d = sum / n;
  return 0;
}

/* src/Real2Int.cpp:244-479.  The first bin-scheme slice of `out` doubles as
 * scratch for the coarse occupancy histogram, as in the reference. */
int orc_dih_real2int(const float *x, uint64_t n, const uint8_t *schemes,
                     int nschemes, uint8_t bins_ref, int optimize,
                     double *min_d, double *max_d, double *avg_d,
                     double *phase_d, uint8_t *out) {
  const double dx = ORC_DX;
  double lo = 1.0e100, hi = -1.0e100, avg;
  double lo1 = 6.5, hi1 = 0.0, lo2 = 6.5, hi2 = 0.0, lo3 = 1.0e100, hi3 = 0.0;
  double sum = 0.0, disp = 0.0;
  int dpind = 0;
  int nfit = (3 * (int)bins_ref > 180) ? 180 : 3 * (int)bins_ref;
  if (n == 0 || nfit == 0) return -1;

  if (optimize) {
    const double fit_lo = 0.0, fit_hi = ORC_TWOPI + dx;
    const double bs = (fit_hi - fit_lo) / nfit;
    uint64_t *prob = (uint64_t *)calloc((size_t)nfit, sizeof(uint64_t));
    unsigned char *empty = (unsigned char *)calloc((size_t)2 * nfit, 1);
    double *center = (double *)malloc(sizeof(double) * (size_t)nfit);
    unsigned nempty = 0, minidx = 0;
    for (uint64_t i = 0; i < n; ++i) {
      int t = (int)fabs(floor((x[i] - fit_lo) / bs));
      out[i] = (uint8_t)t;
    }
    for (uint64_t i = 0; i < n; ++i) {
      if (out[i] >= nfit) {
        free(prob); free(empty); free(center);
        return -2;
      }
      prob[out[i]]++;
    }
    for (int i = 0; i < nfit; ++i) {
      center[i] = fit_lo + (i + 0.5) * bs;
      if (prob[i] > 0) {
        empty[i] = 0;
      } else {
        empty[i] = 1;
        nempty++;
      }
      empty[nfit + i] = 0;
    }
    if (nempty == 0) {
      /* every coarse bin populated: cut at the least populated one */
      double rec = (double)prob[0];
      minidx = 0;
      for (int j = 1; j < nfit; ++j)
        if (prob[j] < rec) {
          rec = (double)prob[j];
          minidx = (unsigned)j;
        }
    } else {
      /* longest circular run of empty coarse bins */
      int j = 0;
      unsigned run = 0, best = 0;
      while (empty[j] == 0 && j < nfit) ++j;
      minidx = (unsigned)j;
      for (int k = 0; k < nfit; ++k) empty[k + nfit] = empty[k];
      for (int q = j; q < 2 * nfit; ++q) {
        if (empty[q]) {
          run++;
        } else {
          if (run > best) {
            minidx = (unsigned)(q - (int)run);
            best = run;
          }
          run = 0;
        }
      }
    }
    if ((int)minidx >= nfit) {
      free(prob); free(empty); free(center);
      return -3;
    }
    disp = ORC_TWOPI - center[minidx];
    free(prob);
    free(empty);
    free(center);
  }

  for (uint64_t i = 0; i < n; ++i) {
    sum += x[i];
    if (lo1 > x[i]) lo1 = x[i];
    if (hi1 < x[i]) hi1 = x[i];
    double s2 = fmod(x[i] + ORC_PI, ORC_TWOPI);
    if (s2 < lo2) lo2 = s2;
    if (s2 > hi2) hi2 = s2;
    if (optimize) {
      double s3 = fmod(x[i] + disp, ORC_TWOPI);
      if (s3 < lo3) lo3 = s3;
      if (s3 > hi3) hi3 = s3;
    }
  }

  if (!optimize) {
    if (fabs((hi1 - lo1) - (hi2 - lo2)) <= 1.0e-1) {
      lo = lo1; hi = hi1; dpind = 0;
    } else if ((hi1 - lo1) < (hi2 - lo2)) {
      lo = lo1; hi = hi1; dpind = 0;
    } else {
      lo = lo2; hi = hi2; dpind = 1;
    }
  } else {
    lo = lo3; hi = hi3; dpind = 2;
  }
  lo -= dx;
  if (lo < 0.0) lo = 0.0;
  hi += dx;
  if (hi > ORC_TWOPI) hi = ORC_TWOPI;
  if ((hi - lo) < 1.0e-4) hi += 0.05;
  avg = sum / n;
  if (dpind == 1) avg = fmod((sum / n) + ORC_PI, ORC_TWOPI);
  if (dpind == 2) avg = fmod((sum / n) + disp, ORC_TWOPI);
  *min_d = lo;
  *max_d = hi;
  *avg_d = avg;
  *phase_d = optimize ? disp : dpind * ORC_PI;

  for (int b = 0; b < nschemes; ++b) {
    uint8_t nb = schemes[b];
    double width = (hi - lo) / (int)nb;
    uint8_t *o = out + (uint64_t)b * n;
    for (uint64_t i = 0; i < n; ++i) {
      double v;
      if (dpind == 0)
        v = x[i];
      else if (dpind == 1)
        v = fmod(x[i] + ORC_PI, ORC_TWOPI);
      else
        v = fmod(x[i] + disp, ORC_TWOPI);
      uint8_t t = to_bin((v - lo) / width);
      o[i] = (t == nb) ? (uint8_t)(t - 1) : t;
    }
  }
  return 0;
}

/* Discretizer.cpp:138-207: per-DOF dispatch and the extremes record. */
int orc_discretize_block(int bat_type, const float *x, uint32_t ndof,
                         uint64_t nframes, const uint8_t *schemes,
                         int nschemes, uint8_t bins_ref, int optimize,
                         uint8_t *bins, double *extremes, int nthreads) {
  int err = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic) reduction(| : err)
#else
  (void)nthreads;
#endif
  for (int64_t d = 0; d < (int64_t)ndof; ++d) {
    const float *xd = x + (uint64_t)d * nframes;
    uint8_t *bd = bins + (uint64_t)d * nschemes * nframes;
    double *e = extremes + 4 * (uint64_t)d;
    double phase = 0.0;
    int rc;
    if (bat_type == ORC_BOND)
      rc = orc_bnd_real2int(xd, nframes, schemes, nschemes, &e[0], &e[1],
                            &e[2], bd);
    else if (bat_type == ORC_ANGLE)
      rc = orc_ang_real2int(xd, nframes, schemes, nschemes, &e[0], &e[1],
                            &e[2], bd);
    else
      rc = orc_dih_real2int(xd, nframes, schemes, nschemes, bins_ref,
                            optimize, &e[0], &e[1], &e[2], &phase, bd);
    e[3] = (bat_type == ORC_DIHEDRAL) ? phase : 0.0;
    if (rc) err |= 1;
  }
  return err ? -1 : 0;
}

/* ---------------------------------------------------------------- KDE ---- */

/* Abramowitz & Stegun 9.8.1-9.8.4 polynomial approximations of I0 and I1,
 * and Miller's downward recurrence for In (src/Utils.cpp:60-171). */
static double bessel_i0(double x) {
  static const double p[7] = {1.0, 3.5156229, 3.0899424, 1.2067429,
                              0.2659732, 0.360768e-1, 0.45813e-2};
  static const double q[9] = {0.39894228, 0.1328592e-1, 0.225319e-2,
                              -0.157565e-2, 0.916281e-2, -0.2057706e-1,
                              0.2635537e-1, -0.1647633e-1, 0.392377e-2};
  if (fabs(x) < 3.75) {
    double y = x / 3.75;
    y = y * y;
    double t = p[3] + y * (p[4] + y * (p[5] + y * p[6]));
    return p[0] + y * (p[1] + y * (p[2] + y * t));
  }
  double ax = fabs(x), y = 3.75 / ax, bx = exp(ax) / sqrt(ax);
  double t = q[5] + y * (q[6] + y * (q[7] + y * q[8]));
  double a = q[0] + y * (q[1] + y * (q[2] + y * (q[3] + y * (q[4] + y * t))));
  return a * bx;
}

static double bessel_i1(double x) {
  static const double p[7] = {0.5, 0.87890594, 0.51498869, 0.15084934,
                              0.2658733e-1, 0.301532e-2, 0.32411e-3};
  static const double q[9] = {0.39894228, -0.3988024e-1, -0.362018e-2,
                              0.163801e-2, -0.1031555e-1, 0.2282967e-1,
                              -0.2895312e-1, 0.1787654e-1, -0.420059e-2};
  if (fabs(x) < 3.75) {
    double y = x / 3.75;
    y = y * y;
    double t = p[3] + y * (p[4] + y * (p[5] + y * p[6]));
    return x * (p[0] + y * (p[1] + y * (p[2] + y * t)));
  }
  double ax = fabs(x), y = 3.75 / ax, bx = exp(ax) / sqrt(ax);
  double t = q[5] + y * (q[6] + y * (q[7] + y * q[8]));
  double a = q[0] + y * (q[1] + y * (q[2] + y * (q[3] + y * (q[4] + y * t))));
  return a * bx;
}

double orc_bessel_i(int n, double x) {
  if (n == 0) return bessel_i0(x);
  if (n == 1) return bessel_i1(x);
  if (fabs(x) < 1.e-10) return 0.0;
  double tox = 2.0 / x, t1, t2 = 1.0, t3 = 0.0, res = 0.0;
  int m = 2 * ((n + (int)(sqrt((float)(40 * n)))));
  for (int i = m; i >= 1; --i) {
    t1 = t3 + (double)(i * tox * t2);
    t3 = t2;
    t2 = t1;
    if (fabs(t2) > 1.e10) {
      t2 *= 1.e-10;
      t3 *= 1.e-10;
      res *= 1.e-10;
    }
    if (i == n) res = t3;
  }
  return res * bessel_i0(x) / t2;
}

/* src/Real2Int.cpp:659-698 (density is not used by the caller). */
static void vm_grid_point(double h, double xg, const float *a, uint64_t n,
                          double *grad, double *sec) {
  double g = 0.0, s = 0.0;
  for (uint64_t j = 0; j < n; ++j) {
    double d = xg - a[j];
    double c = cos(d), sn = sin(d);
    double e = exp(h * c);
    g = g - sn * e;
    s = s + (h * (sn * sn) - c) * e;
  }
  double denom = (ORC_TWOPI * n * orc_bessel_i(0, h));
  *grad = g * h / denom;
  *sec = s * h / denom;
}

/* src/Real2Int.cpp:481-657 with analyticGrad=false (Discretizer.cpp:177). */
int orc_vmkde_minima(const float *x, uint64_t n, uint8_t n_conf_max,
                     double kappa, uint32_t step_sdo, double conv,
                     uint32_t max_iter, double *minima, uint8_t *found,
                     uint8_t *out) {
  double cmax[9], smax[9] = {0};
  double grad[361], sec[361];
  int nmax = 0;
  double h = pow((3 * n * (kappa * kappa) * orc_bessel_i(2, 2 * kappa) /
                  (4 * ORC_SQRTPI * pow(orc_bessel_i(0, kappa), 2.0))),
                 (2.0 / 5.0));
  for (int i = 0; i <= 360; ++i) {
    vm_grid_point(h, i * ORC_DEGRAD, x, n, &grad[i], &sec[i]);
    if (i > 0 && (grad[i - 1] * grad[i]) <= 0.0 && sec[i] < -1.0e-4 &&
        nmax < 9) {
      cmax[nmax] = i / 2.0 + (i - 1) / 2.0;
      smax[nmax] = sec[i] / 2.0 + sec[i - 1] / 2.0;
      nmax++;
    }
  }
  for (int i = 0; i < nmax - 1; ++i)
    for (int j = i + 1; j < nmax; ++j)
      if (smax[i] > smax[j]) {
        double t = smax[i]; smax[i] = smax[j]; smax[j] = t;
        t = cmax[i]; cmax[i] = cmax[j]; cmax[j] = t;
      }
  int fm = (n_conf_max < nmax) ? n_conf_max : nmax;
  for (int i = 0; i < fm - 1; ++i)
    for (int j = i + 1; j < fm; ++j)
      if (cmax[i] > cmax[j]) {
        double t = cmax[i]; cmax[i] = cmax[j]; cmax[j] = t;
      }
  if (fm == 1) {
    minima[0] = cmax[0] - 180.0;
    if (minima[0] < 0.0) minima[0] += 360.0;
  } else {
    for (int i = 0; i < fm; ++i) {
      if (i == 0) {
        minima[i] = (cmax[i] + cmax[fm - 1] - 360.0) / 2.0;
        if (minima[i] < 0.0) minima[i] += 360;
      } else {
        minima[i] = (cmax[i] + cmax[i - 1]) / 2.0;
      }
    }
  }
  if (fm > 1) {
    for (int m = 0; m < fm; ++m) {
      int it = 0, done = 0;
      while (!done && it < (int)max_iter) {
        it++;
        int ii = (int)minima[m];
        double g = fabs(minima[m] - 1 - ii) * grad[ii] +
                   fabs(minima[m] - ii) * grad[1 + ii];
        if (fabs(g) < conv) {
          done = 1;
        } else {
          double st = step_sdo * g;
          if (fabs(st) > 5.0) st = (st / fabs(st)) * 5.0;
          minima[m] = minima[m] - st;
          if (minima[m] < 0.0) minima[m] += 360.0;
          if (minima[m] >= 360.0) minima[m] -= 360.0;
        }
      }
    }
  }
  for (int i = 0; i < fm - 1; ++i)
    for (int j = i + 1; j < fm; ++j)
      if (minima[i] > minima[j]) {
        double t = minima[i]; minima[i] = minima[j]; minima[j] = t;
      }
  for (int i = 0; i < fm; ++i) minima[i] *= ORC_DEGRAD;
  for (uint64_t k = 0; k < n; ++k) {
    if (fm == 1) {
      out[k] = 0;
    } else {
      for (int j = 0; j < fm; ++j) {
        if (j == 0) {
          if (x[k] < minima[j] || x[k] > minima[fm - 1]) out[k] = (uint8_t)j;
        } else if (x[k] < minima[j] && x[k] > minima[j - 1]) {
          out[k] = (uint8_t)j;
        }
      }
    }
  }
  *found = (uint8_t)fm;
  return 0;
}

/* ------------------------------------------------------------- counts ---- */

/* src/Estimators.cpp:56-118 */
int orc_bin1d(uint8_t nsteps, const uint8_t *schemes, int nschemes,
              uint64_t nframes, double min_d, double max_d,
              const uint8_t *data, uint64_t *freq, double *mids) {
  int nsum = 0;
  for (int s = 0; s < nschemes; ++s) nsum += schemes[s];
  if (mids) {
    int off = 0;
    for (int s = 0; s < nschemes; ++s) {
      int nb = schemes[s];
      double w = (max_d - min_d) / nb, hw = w / 2.0, at = min_d;
      for (int i = 0; i < nb; ++i) {
        mids[off + i] = at + hw;
        at += w;
      }
      off += nb;
    }
  }
  memset(freq, 0, sizeof(uint64_t) * (size_t)nsteps * nsum);
  uint64_t step = nframes / nsteps;
  int boff = 0;
  for (int s = 0; s < nschemes; ++s) {
    int nb = schemes[s];
    const uint8_t *d = data + (uint64_t)s * nframes;
    for (int i = 0; i < nsteps; ++i) {
      uint64_t *f = freq + (uint64_t)nsum * i + boff;
      const uint8_t *di = d + (uint64_t)i * step;
      for (uint64_t j = 0; j < step; ++j) {
        if (di[j] >= nb) return -2;
        f[di[j]] += 1;
      }
    }
    for (int i = 1; i < nsteps; ++i) {
      uint64_t *f = freq + (uint64_t)nsum * i + boff;
      for (int j = 0; j < nb; ++j) f[j] += f[j - nsum];
    }
    boff += nb;
  }
  return 0;
}

/* src/Estimators.cpp:130-205 (get2D21DIndex :120 is a*nb+b for 2-D) */
int orc_bin2d(uint8_t nsteps, const uint8_t *schemes, int nschemes,
              uint64_t nframes, double min1, double max1, double min2,
              double max2, const uint8_t *d1, const uint8_t *d2,
              uint64_t *freq, double *mids) {
  int nsq = 0;
  for (int s = 0; s < nschemes; ++s) nsq += schemes[s] * schemes[s];
  if (mids) {
    int off = 0;
    for (int s = 0; s < nschemes; ++s) {
      int nb = schemes[s];
      double w1 = (max1 - min1) / nb, h1 = w1 / 2, a1 = min1;
      double w2 = (max2 - min2) / nb, h2 = w2 / 2, a2 = min2;
      for (int i = 0; i < nb; ++i) {
        mids[off + i] = a1 + h1;
        a1 += w1;
        mids[off + nb + i] = a2 + h2;
        a2 += w2;
      }
      off += 2 * nb;
    }
  }
  memset(freq, 0, sizeof(uint64_t) * (size_t)nsteps * nsq);
  uint64_t step = nframes / nsteps;
  int boff = 0;
  for (int s = 0; s < nschemes; ++s) {
    int nb = schemes[s];
    const uint8_t *a = d1 + (uint64_t)s * nframes;
    const uint8_t *b = d2 + (uint64_t)s * nframes;
    for (int i = 0; i < nsteps; ++i) {
      uint64_t *f = freq + (uint64_t)nsq * i + boff;
      uint64_t o = (uint64_t)i * step;
      for (uint64_t j = 0; j < step; ++j) {
        if (a[o + j] >= nb || b[o + j] >= nb) return -2;
        f[(size_t)a[o + j] * nb + b[o + j]] += 1;
      }
    }
    for (int i = 1; i < nsteps; ++i) {
      uint64_t *f = freq + (uint64_t)nsq * i + boff;
      for (int j = 0; j < nb * nb; ++j) f[j] += f[j - nsq];
    }
    boff += nb * nb;
  }
  return 0;
}

/* ------------------------------------------------------------ entropy ---- */

static double jac(int type, double mid) {
  if (type == ORC_BOND) return pow(mid, 2);
  if (type == ORC_ANGLE) return sin(mid);
  return 1.0;
}

/* src/Estimators.cpp:217-389 */
int orc_entropy1d(int type, const uint8_t *ests, int nests, uint8_t nsteps,
                  uint64_t step_size, double min_d, double max_d,
                  int jacobian, int kde, const uint8_t *schemes, int nschemes,
                  const uint64_t *freq, double *entropy) {
  int nsum = 0;
  for (int s = 0; s < nschemes; ++s) nsum += schemes[s];
  int has_jac = (type == ORC_BOND || type == ORC_ANGLE);
  double f[256], mid[256];
  for (int e = 0; e < nests; ++e) {
    int est = ests[e];
    int foff = 0;
    for (int s = 0; s < nschemes; ++s) {
      int nb = schemes[s];
      double width = (max_d - min_d) / nb;
      double hw = width / 2;
      if (kde) width = 1.0;
      for (int j = 0; j < nb; ++j)
        mid[j] = has_jac ? (min_d + j * width + hw) : 0.0;
      for (int i = 0; i < nsteps; ++i) {
        const uint64_t *c = freq + (uint64_t)i * nsum + foff;
        double nd = (i + 1.0) * step_size;
        double acc = 0.0;
        uint8_t blank = 0, single = 0;
        for (int j = 0; j < nb; ++j) f[j] = c[j] / (nd);
        if (est == ORC_MM) {
          for (int j = 0; j < nb; ++j)
            if (c[j] == 0) ++blank;
        } else if (est == ORC_CS) {
          for (int j = 0; j < nb; ++j)
            if (c[j] == 1) ++single;
          for (int j = 0; j < nb; ++j)
            f[j] = (1 - (single / nd)) * (c[j] / nd);
        } else if (est == ORC_JS) {
          double tk = 1.0 / (double)nb, s2 = 0, t2 = 0;
          for (int j = 0; j < nb; ++j) {
            s2 += f[j] * f[j];
            t2 += ((tk - f[j]) * (tk - f[j]));
          }
          double lam = (1 - s2) / ((nd - 1) * t2);
          for (int j = 0; j < nb; ++j) f[j] = (lam * tk) + ((1 - lam) * f[j]);
        }
        for (int j = 0; j < nb; ++j) {
          double pd = f[j] / width;
          if (pd > 0.0) {
            double den = (est == ORC_CS) ? 1 - pow((1 - f[j]), nd) : 1.0;
            if (jacobian && has_jac) {
              double jf = jac(type, mid[j]);
              pd = pd / jf;
              acc += (est == ORC_CS) ? (jf * pd * log(pd) / den)
                                     : (jf * pd * log(pd));
            } else {
              acc += (est == ORC_CS) ? (pd * log(pd) / den) : (pd * log(pd));
            }
          }
        }
        acc *= -width;
        if (est == ORC_MM) acc += ((nb - blank) - 1) / (2.0 * nd);
        entropy[(uint64_t)e * nsteps * nschemes + (uint64_t)s * nsteps + i] =
            acc;
      }
      foff += nb;
    }
  }
  return 0;
}

/* src/Estimators.cpp:391-651, including the Chao-Shen branch's use of the
 * row bin centre for the second DOF's Jacobian (:555-566). */
int orc_entropy2d(int type1, int type2, const uint8_t *ests, int nests,
                  uint8_t nsteps, uint64_t step_size, double min1,
                  double max1, double min2, double max2, int jacobian,
                  int kde, const uint8_t *schemes, int nschemes,
                  const uint64_t *freq, double *entropy) {
  int nsq = 0;
  for (int s = 0; s < nschemes; ++s) nsq += schemes[s] * schemes[s];
  int hj1 = (type1 == ORC_BOND || type1 == ORC_ANGLE);
  int hj2 = (type2 == ORC_BOND || type2 == ORC_ANGLE);
  double *f = (double *)malloc(sizeof(double) * 256 * 256);
  double mid1[256], mid2[256];
  for (int e = 0; e < nests; ++e) {
    int est = ests[e];
    int foff = 0;
    for (int s = 0; s < nschemes; ++s) {
      int nb = schemes[s];
      unsigned nb2 = (unsigned)nb * nb;
      double w1 = (max1 - min1) / nb, hw1 = w1 / 2;
      double w2 = (max2 - min2) / nb, hw2 = w2 / 2;
      if (kde) {
        w1 = 1.0;
        w2 = 1.0;
      }
      for (int j = 0; j < nb; ++j) {
        mid1[j] = hj1 ? (min1 + (j * w1) + hw1) : 0.0;
        mid2[j] = hj2 ? (min2 + (j * w2) + hw2) : 0.0;
      }
      double area = w1 * w2;
      for (int i = 0; i < nsteps; ++i) {
        const uint64_t *c = freq + (uint64_t)i * nsq + foff;
        double nd = (i + 1.0) * step_size;
        double acc = 0.0, jf1 = 1.0, jf2 = 1.0;
        unsigned blank = 0, single = 0;
        for (unsigned q = 0; q < nb2; ++q) f[q] = c[q] / nd;
        if (est == ORC_MM) {
          for (unsigned q = 0; q < nb2; ++q)
            if (c[q] == 0) ++blank;
        } else if (est == ORC_CS) {
          for (unsigned q = 0; q < nb2; ++q)
            if (c[q] == 1) ++single;
          for (unsigned q = 0; q < nb2; ++q)
            f[q] = (1 - (single / nd)) * (c[q] / nd);
        } else if (est == ORC_JS) {
          double tk = 1.0 / (double)nb, s2 = 0, t2 = 0;
          for (int j = 0; j < nb; ++j)
            for (int k = 0; k < nb; ++k) {
              double v = f[j * nb + k];
              s2 += v * v;
              t2 += ((tk - v) * (tk - v));
            }
          double lam = (1 - s2) / ((nd - 1) * t2);
          for (unsigned q = 0; q < nb2; ++q)
            f[q] = (lam * tk) + ((1 - lam) * f[q]);
        }
        for (int j = 0; j < nb; ++j) {
          if (hj1) jf1 = jac(type1, mid1[j]);
          double row = 0.0;
          for (int k = 0; k < nb; ++k) {
            double fv = f[j * nb + k];
            double pd = fv / area;
            if (pd > 0.0) {
              if (est == ORC_CS) {
                double den = 1 - pow((1 - fv), nd);
                if (hj2) jf2 = jac(type2, mid2[j]);
                if (jacobian) {
                  double jf = (jf1 * jf2);
                  pd = pd / jf;
                  row += (jf * pd * log(pd) / den);
                } else {
                  row += (pd * log(pd) / den);
                }
              } else {
                if (hj2) jf2 = jac(type2, mid2[k]);
                if (jacobian) {
                  double jf = (jf1 * jf2);
                  pd = pd / jf;
                  row += (jf * pd * log(pd));
                } else {
                  row += (pd * log(pd));
                }
              }
            }
          }
          row *= -area;
          acc += row;
        }
        if (est == ORC_MM) acc += ((nb2 - blank) - 1) / (2.0 * nd);
        entropy[(uint64_t)e * nsteps * nschemes + (uint64_t)s * nsteps + i] =
            acc;
      }
      foff += (int)nb2;
    }
  }
  free(f);
  return 0;
}

/* EntropyCalculator.cpp:156-199 over a DOF block. */
int orc_entropy1d_block(uint32_t ndof, const uint8_t *types,
                        const uint8_t *bins, const double *extremes,
                        uint64_t nframes, uint8_t nsteps,
                        const uint8_t *schemes, int nschemes,
                        const uint8_t *ests, int nests, int jacobian, int kde,
                        double *s1, int nthreads) {
  int nsum = 0, err = 0;
  for (int s = 0; s < nschemes; ++s) nsum += schemes[s];
  uint64_t step = nframes / nsteps;
  uint64_t per = (uint64_t)nests * nschemes * nsteps;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic) reduction(| : err)
#else
  (void)nthreads;
#endif
  for (int64_t d = 0; d < (int64_t)ndof; ++d) {
    uint64_t *fr = (uint64_t *)malloc(sizeof(uint64_t) * nsteps * nsum);
    const double *e = extremes + 4 * d;
    if (orc_bin1d(nsteps, schemes, nschemes, nframes, e[0], e[1],
                  bins + (uint64_t)d * nschemes * nframes, fr, NULL))
      err |= 1;
    else
      orc_entropy1d(types[d], ests, nests, nsteps, step, e[0], e[1],
                    jacobian, kde, schemes, nschemes, fr, s1 + d * per);
    free(fr);
  }
  return err ? -1 : 0;
}

/* EntropyCalculator.cpp:530-590 over an explicit pair list. */
int orc_entropy2d_pairs(uint64_t npairs, const uint32_t *pairs,
                        const uint8_t *types, const uint8_t *bins,
                        const double *extremes, uint64_t nframes,
                        uint8_t nsteps, const uint8_t *schemes, int nschemes,
                        const uint8_t *ests, int nests, int jacobian, int kde,
                        double *s2, int nthreads) {
  int nsq = 0, err = 0;
  for (int s = 0; s < nschemes; ++s) nsq += schemes[s] * schemes[s];
  uint64_t step = nframes / nsteps;
  uint64_t per = (uint64_t)nests * nschemes * nsteps;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(| : err)
#endif
  {
    uint64_t *fr = (uint64_t *)malloc(sizeof(uint64_t) * nsteps * nsq);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int64_t p = 0; p < (int64_t)npairs; ++p) {
      uint32_t a = pairs[2 * p], b = pairs[2 * p + 1];
      const double *ea = extremes + 4 * (uint64_t)a;
      const double *eb = extremes + 4 * (uint64_t)b;
      if (orc_bin2d(nsteps, schemes, nschemes, nframes, ea[0], ea[1], eb[0],
                    eb[1], bins + (uint64_t)a * nschemes * nframes,
                    bins + (uint64_t)b * nschemes * nframes, fr, NULL))
        err |= 1;
      else
        orc_entropy2d(types[a], types[b], ests, nests, nsteps, step, ea[0],
                      ea[1], eb[0], eb[1], jacobian, kde, schemes, nschemes,
                      fr, s2 + p * per);
    }
    free(fr);
  }
  (void)nthreads;
  return err ? -1 : 0;
}

/* ---------------------------------------------------------------- MST ---- */

static uint32_t uf_find(uint32_t *parent, uint32_t i) {
  uint32_t r = i;
  while (parent[r] != r) r = parent[r];
  while (parent[i] != r) { /* path compression, as the recursive original */
    uint32_t nx = parent[i];
    parent[i] = r;
    i = nx;
  }
  return r;
}

/* src/Centre.cpp:126-143 */
static void uf_union(uint32_t *parent, uint32_t *rank, uint32_t x,
                     uint32_t y) {
  uint32_t xr = uf_find(parent, x), yr = uf_find(parent, y);
  if (rank[xr] < rank[yr])
    parent[xr] = yr;
  else if (rank[xr] > rank[yr])
    parent[yr] = xr;
  else {
    parent[yr] = xr;
    rank[xr]++;
  }
}

/* src/Centre.cpp:5-115.  A component keeps the first edge (lowest index) of
 * strictly largest weight; picked edges are merged in component order. */
int64_t orc_boruvka_mst(uint32_t nv, uint64_t ne, const uint32_t *src,
                        const uint32_t *dst, const double *w,
                        uint64_t *tree) {
  uint32_t *parent = (uint32_t *)malloc(sizeof(uint32_t) * (nv ? nv : 1));
  uint32_t *rank = (uint32_t *)calloc(nv ? nv : 1, sizeof(uint32_t));
  int64_t *best = (int64_t *)malloc(sizeof(int64_t) * (nv ? nv : 1));
  int64_t nt = 0;
  uint32_t ntrees = nv;
  for (uint32_t v = 0; v < nv; ++v) {
    parent[v] = v;
    best[v] = -1;
  }
  while (ntrees > 1) {
    uint64_t upd = 0;
    for (uint64_t i = 0; i < ne; ++i) {
      uint32_t s1 = uf_find(parent, src[i]), s2 = uf_find(parent, dst[i]);
      if (s1 != s2) {
        if (best[s1] == -1 || w[best[s1]] < w[i]) {
          best[s1] = (int64_t)i;
          upd++;
        }
        if (best[s2] == -1 || w[best[s2]] < w[i]) {
          best[s2] = (int64_t)i;
          upd++;
        }
      }
    }
    if (upd == 0) {
      for (uint64_t i = 0; i < ne; ++i) {
        uint32_t s1 = uf_find(parent, src[i]), s2 = uf_find(parent, dst[i]);
        if (s1 != s2) {
          if (best[s1] == -1 || w[best[s1]] <= w[i]) {
            best[s1] = (int64_t)i;
            upd++;
            break;
          }
          if (best[s2] == -1 || w[best[s2]] <= w[i]) {
            best[s2] = (int64_t)i;
            upd++;
            break;
          }
        }
      }
    }
    if (upd == 0) break;
    for (uint32_t v = 0; v < nv; ++v) {
      if (best[v] != -1) {
        uint64_t e = (uint64_t)best[v];
        uint32_t s1 = uf_find(parent, src[e]), s2 = uf_find(parent, dst[e]);
        if (s1 != s2) {
          tree[nt++] = e;
          uf_union(parent, rank, s1, s2);
          ntrees--;
        }
      }
    }
    for (uint32_t v = 0; v < nv; ++v) best[v] = -1;
  }
  free(parent);
  free(rank);
  free(best);
  return nt;
}
