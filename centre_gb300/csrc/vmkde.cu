// vmkde.cu -- von Mises kernel-density conformer assignment of torsions.
//
// Reference: Real2Int::getMinimaPositions (src/Real2Int.cpp:481-657) with
// analyticGrad = false as Discretizer::run_dtype calls it
// (src/Discretizer.cpp:177), Real2Int::vonMises (:659-698) and the modified
// Bessel functions of src/Utils.cpp:60-171.
//
// Per torsion the reference evaluates, on the 361-point 1-degree grid, the
// density's gradient and second derivative as sums over all frames of
// exp(h cos(x - a_j)) (h = bandwidth from kappa and the frame count), detects
// maxima where the gradient changes sign with a negative curvature, keeps the
// sharpest nmaxconf, guesses a minimum between neighbouring maxima, refines
// each by steepest descent on the linearly interpolated grid gradient, and
// labels each frame with the interval between minima it falls in.
//
// GB300 mapping
//  * vmkde_grid_kernel: one CTA per torsion, one thread per grid point; the
//    frames are staged in shared memory as (cos a, sin a) so each (grid
//    point, frame) term needs only FMAs and one FP64 exp:
//    cos(x - a) = cos x cos a + sin x sin a, sin(x - a) = sin x cos a -
//    cos x sin a.  Sums are FP64 like the reference's; their order differs,
//    so grid values agree to rounding, not bit for bit.
//  * vmkde_minima_kernel: one thread per torsion runs the reference's serial
//    maximum detection, sorting, minimum guess and descent unchanged.
//  * vmkde_assign_kernel: one thread per frame applies the interval tests.
//  The bandwidth is computed on the host with the reference's Bessel
//  approximations (host code is compiled without FMA contraction), so it is
//  the reference's value to the last bit.
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "dfloat.cuh"

namespace centre {
namespace {

constexpr double kDegRad = 0.017453292519943295;   // src/Constants.h:100
constexpr double kSqrtPi = 1.7724538509055159;     // src/Constants.h:93
constexpr double kTwoPiV = 6.283185307179586;      // src/Constants.h:94
constexpr int kGrid = 361;
constexpr int kMaxConf = 9;
constexpr int kStageFrames = 2048;

// Abramowitz & Stegun 9.8.1-9.8.4 polynomial approximations and Miller's
// downward recurrence, as src/Utils.cpp:60-171 evaluates them.
double host_bessel_i0(double x) {
  static const double p[7] = {1.0, 3.5156229, 3.0899424, 1.2067429,
                              0.2659732, 0.360768e-1, 0.45813e-2};
  static const double q[9] = {0.39894228, 0.1328592e-1, 0.225319e-2,
                              -0.157565e-2, 0.916281e-2, -0.2057706e-1,
                              0.2635537e-1, -0.1647633e-1, 0.392377e-2};
  if (fabs(x) < 3.75) {
    double y = x / 3.75;
    y = y * y;
    const double t = p[3] + y * (p[4] + y * (p[5] + y * p[6]));
    return p[0] + y * (p[1] + y * (p[2] + y * t));
  }
  const double ax = fabs(x), y = 3.75 / ax, bx = exp(ax) / sqrt(ax);
  const double t = q[5] + y * (q[6] + y * (q[7] + y * q[8]));
  return (q[0] + y * (q[1] + y * (q[2] + y * (q[3] + y * (q[4] + y * t))))) * bx;
}

double host_bessel_i1(double x) {
  static const double p[7] = {0.5, 0.87890594, 0.51498869, 0.15084934,
                              0.2658733e-1, 0.301532e-2, 0.32411e-3};
  static const double q[9] = {0.39894228, -0.3988024e-1, -0.362018e-2,
                              0.163801e-2, -0.1031555e-1, 0.2282967e-1,
                              -0.2895312e-1, 0.1787654e-1, -0.420059e-2};
  if (fabs(x) < 3.75) {
    double y = x / 3.75;
    y = y * y;
    const double t = p[3] + y * (p[4] + y * (p[5] + y * p[6]));
    return x * (p[0] + y * (p[1] + y * (p[2] + y * t)));
  }
  const double ax = fabs(x), y = 3.75 / ax, bx = exp(ax) / sqrt(ax);
  const double t = q[5] + y * (q[6] + y * (q[7] + y * q[8]));
  return (q[0] + y * (q[1] + y * (q[2] + y * (q[3] + y * (q[4] + y * t))))) * bx;
}

double host_bessel_in(int n, double x) {
  if (n == 0) return host_bessel_i0(x);
  if (n == 1) return host_bessel_i1(x);
  if (fabs(x) < 1.e-10) return 0.0;
  const double tox = 2.0 / x;
  double t1, t2 = 1.0, t3 = 0.0, res = 0.0;
  const int m = 2 * ((n + (int)(sqrt((float)(40 * n)))));
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
  return res * host_bessel_i0(x) / t2;
}

// Grid sums of one torsion: grad[g] and sec[g] as vonMises() returns them.
// With a bandwidth h <= 700 the terms run in double-float arithmetic on the
// FP32 pipe (dfloat.cuh): e^(h c) = e^h e^(h (c - 1)), the second factor by
// the table-driven double-float exp (it is at most 1, so it stays in FP32
// range), sums in double-float, and e^h applied once in FP64 at the end;
// terms agree with FP64 to ~1e-12 relative.  A grid point whose scaled
// weight sum is below kDfFloor (terms beyond the FP32 range could matter
// there) is summed again in FP64, as is every grid point when h > 700.
constexpr double kDfFloor = 1e-10;

__global__ void __launch_bounds__(384)
vmkde_grid_kernel(const float *__restrict__ data, uint64_t n, double h, double denom,
                  double *__restrict__ grad, double *__restrict__ sec) {
  __shared__ float4 fr[kStageFrames];       // cos a, sin a as double-floats
  __shared__ float dftab[2 * kDfExpTable];
  const uint64_t d = blockIdx.x;
  const float *x = data + d * n;
  const int g = threadIdx.x;
  const double xg = g * kDegRad;
  const double cg = cos(xg), sg = sin(xg);
  const bool use_df = h <= 700.0;
  if (g < kDfExpTable) {
    const double t = exp2((double)g / kDfExpTable);
    const float hi = __double2float_rn(t);
    dftab[2 * g] = hi;
    dftab[2 * g + 1] = __double2float_rn(t - (double)hi);
  }
  double G = 0.0, Sc = 0.0;
  bool need = g < kGrid;
  if (use_df) {
    const dfl cgd = df_from_double(cg), sgd = df_from_double(sg);
    const dfl hd = df_from_double(h);
    dfl Gd = df_make(0.0f, 0.0f), Sd = df_make(0.0f, 0.0f), Wd = df_make(0.0f, 0.0f);
    for (uint64_t f0 = 0; f0 < n; f0 += kStageFrames) {
      const int cnt = (int)((n - f0) < (uint64_t)kStageFrames ? (n - f0) : (uint64_t)kStageFrames);
      __syncthreads();
      for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
        double sa, ca;
        sincos((double)x[f0 + j], &sa, &ca);
        const dfl c2 = df_from_double(ca), s2 = df_from_double(sa);
        fr[j] = make_float4(c2.hi, c2.lo, s2.hi, s2.lo);
      }
      __syncthreads();
      if (g < kGrid) {
        for (int j = 0; j < cnt; ++j) {
          const float4 q = fr[j];
          const dfl ca = df_make(q.x, q.y), sa = df_make(q.z, q.w);
          const dfl c = df_add(df_mul(cgd, ca), df_mul(sgd, sa));                  // cos(xg - a)
          const dfl sn = df_add(df_mul(sgd, ca), df_mul(cgd, df_make(-sa.hi, -sa.lo)));  // sin
          const dfl e = df_exp_neg(df_mul(hd, df_add(c, df_make(-1.0f, 0.0f))), dftab);
          Gd = df_add(Gd, df_mul(df_make(-sn.hi, -sn.lo), e));
          const dfl w = df_add(df_mul(hd, df_mul(sn, sn)), df_make(-c.hi, -c.lo));
          Sd = df_add(Sd, df_mul(w, e));
          Wd = df_add(Wd, e);
        }
      }
    }
    if (g < kGrid) {
      const double eh = exp(h);
      G = df_value(Gd.hi, Gd.lo) * eh;
      Sc = df_value(Sd.hi, Sd.lo) * eh;
      need = df_value(Wd.hi, Wd.lo) < kDfFloor;
    }
  }
  __syncthreads();
  if (__syncthreads_or(need)) {
    // FP64 sums, frames staged as (cos a, sin a) doubles in the same buffer
    double *cs = reinterpret_cast<double *>(fr);
    double *sn = cs + kStageFrames;
    double G2 = 0.0, S2 = 0.0;
    for (uint64_t f0 = 0; f0 < n; f0 += kStageFrames) {
      const int cnt = (int)((n - f0) < (uint64_t)kStageFrames ? (n - f0) : (uint64_t)kStageFrames);
      __syncthreads();
      for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
        double s, c;
        sincos((double)x[f0 + j], &s, &c);
        cs[j] = c;
        sn[j] = s;
      }
      __syncthreads();
      if (need) {
        for (int j = 0; j < cnt; ++j) {
          const double ca = cs[j], sa = sn[j];
          const double c = cg * ca + sg * sa;   // cos(xg - a)
          const double s = sg * ca - cg * sa;   // sin(xg - a)
          const double e = exp(h * c);
          G2 = G2 - s * e;
          S2 = S2 + (h * (s * s) - c) * e;
        }
      }
    }
    if (need) {
      G = G2;
      Sc = S2;
    }
  }
  if (g < kGrid) {
    grad[d * kGrid + g] = G * h / denom;
    sec[d * kGrid + g] = Sc * h / denom;
  }
}

// The reference's serial part (src/Real2Int.cpp:517-634), one thread per
// torsion: maxima, sort by curvature, keep nconf, minima guess, descent.
__global__ void vmkde_minima_kernel(uint32_t ndof, const double *__restrict__ grad,
                                    const double *__restrict__ sec, int nconf, uint32_t step_sdo,
                                    double conv, uint32_t max_iter, double *__restrict__ minima,
                                    uint8_t *__restrict__ nfound) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= ndof) return;
  const double *gr = grad + (uint64_t)d * kGrid;
  const double *se = sec + (uint64_t)d * kGrid;
  double cmax[kMaxConf], smax[kMaxConf], mins[kMaxConf];
  int nmax = 0;
  for (int i = 1; i <= 360; ++i) {
    if ((gr[i - 1] * gr[i]) <= 0.0 && se[i] < -1.0e-4 && nmax < kMaxConf) {
      cmax[nmax] = i / 2.0 + (i - 1) / 2.0;
      smax[nmax] = se[i] / 2.0 + se[i - 1] / 2.0;
      nmax++;
    }
  }
  for (int i = 0; i < nmax - 1; ++i)
    for (int j = i + 1; j < nmax; ++j)
      if (smax[i] > smax[j]) {
        double t = smax[i]; smax[i] = smax[j]; smax[j] = t;
        t = cmax[i]; cmax[i] = cmax[j]; cmax[j] = t;
      }
  const int fm = (nconf < nmax) ? nconf : nmax;
  for (int i = 0; i < fm - 1; ++i)
    for (int j = i + 1; j < fm; ++j)
      if (cmax[i] > cmax[j]) {
        double t = cmax[i]; cmax[i] = cmax[j]; cmax[j] = t;
      }
  if (fm == 1) {
    mins[0] = cmax[0] - 180.0;
    if (mins[0] < 0.0) mins[0] += 360.0;
  } else {
    for (int i = 0; i < fm; ++i) {
      if (i == 0) {
        mins[i] = (cmax[i] + cmax[fm - 1] - 360.0) / 2.0;
        if (mins[i] < 0.0) mins[i] += 360;
      } else {
        mins[i] = (cmax[i] + cmax[i - 1]) / 2.0;
      }
    }
  }
  if (fm > 1) {
    for (int m = 0; m < fm; ++m) {
      uint32_t it = 0;
      bool done = false;
      while (!done && it < max_iter) {
        it++;
        const int ii = (int)mins[m];
        const double g = __dadd_rn(__dmul_rn(fabs(mins[m] - 1 - ii), gr[ii]),
                                   __dmul_rn(fabs(mins[m] - ii), gr[1 + ii]));
        if (fabs(g) < conv) {
          done = true;
        } else {
          double st = __dmul_rn((double)step_sdo, g);
          if (fabs(st) > 5.0) st = (st / fabs(st)) * 5.0;
          mins[m] = mins[m] - st;
          if (mins[m] < 0.0) mins[m] += 360.0;
          if (mins[m] >= 360.0) mins[m] -= 360.0;
        }
      }
    }
  }
  for (int i = 0; i < fm - 1; ++i)
    for (int j = i + 1; j < fm; ++j)
      if (mins[i] > mins[j]) {
        double t = mins[i]; mins[i] = mins[j]; mins[j] = t;
      }
  for (int i = 0; i < fm; ++i) minima[(uint64_t)d * nconf + i] = mins[i] * kDegRad;
  for (int i = fm; i < nconf; ++i) minima[(uint64_t)d * nconf + i] = 0.0;
  nfound[d] = (uint8_t)fm;
}

// Conformer index of every frame (src/Real2Int.cpp:636-653); frames in no
// interval keep 0 like the reference's zero-initialised vector.
__global__ void vmkde_assign_kernel(const float *__restrict__ data, uint32_t ndof, uint64_t n,
                                    const double *__restrict__ minima,
                                    const uint8_t *__restrict__ nfound, int nconf,
                                    uint8_t *__restrict__ bins) {
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)ndof * n) return;
  const uint64_t d = idx / n;
  const int fm = nfound[d];
  const double *mn = minima + d * nconf;
  const double x = (double)data[idx];
  uint8_t out = 0;
  if (fm > 1) {
    for (int j = 0; j < fm; ++j) {
      if (j == 0) {
        if (x < mn[0] || x > mn[fm - 1]) out = (uint8_t)j;
      } else if (x < mn[j] && x > mn[j - 1]) {
        out = (uint8_t)j;
      }
    }
  }
  bins[idx] = out;
}

}  // namespace

int launch_vmkde(centre_ctx *ctx, const float *d_data, uint32_t ndof, uint64_t nframes,
                 uint8_t nmaxconf, double kappa, uint32_t sdo_nstep, double sdo_conv,
                 uint32_t sdo_niter, uint8_t *d_bins, double *d_minima, uint8_t *d_nfound,
                 double *d_work) {
  if (nmaxconf == 0 || nmaxconf > kMaxConf)
    return set_error(ctx, CENTRE_E_ARG, "nmaxconf must be 1..9");
  if (ndof == 0 || nframes == 0) return CENTRE_OK;
  // bandwidth and normalisation exactly as src/Real2Int.cpp:509-514, :692-693
  const double h = pow((3 * nframes * (kappa * kappa) * host_bessel_in(2, 2 * kappa) /
                        (4 * kSqrtPi * pow(host_bessel_in(0, kappa), 2.0))),
                       (2.0 / 5.0));
  const double denom = (kTwoPiV * nframes * host_bessel_in(0, h));
  double *d_grad = d_work;
  double *d_sec = d_work + (uint64_t)ndof * kGrid;
  {
    KernelTimer kt(ctx, CENTRE_TIMER_DISCRETIZE);
    vmkde_grid_kernel<<<ndof, 384, 0, ctx->stream>>>(d_data, nframes, h, denom, d_grad, d_sec);
    vmkde_minima_kernel<<<(ndof + 127) / 128, 128, 0, ctx->stream>>>(
        ndof, d_grad, d_sec, nmaxconf, sdo_nstep, sdo_conv, sdo_niter, d_minima, d_nfound);
    const uint64_t tot = (uint64_t)ndof * nframes;
    vmkde_assign_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(
        d_data, ndof, nframes, d_minima, d_nfound, nmaxconf, d_bins);
  }
  ctx->launches += 3;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

size_t vmkde_work_doubles(uint32_t ndof) { return (size_t)2 * ndof * kGrid; }

}  // namespace centre
