// gridkde.cu -- grid kernel-density conformer binning of bonds, angles and
// torsions.
//
// A KDE variant for every DOF type, next to the reference's torsion-only von
// Mises KDE (vmkde.cu, Real2Int::getMinimaPositions, src/Real2Int.cpp:481):
//  * torsions: von Mises kernel exp(kappa (cos(g - a) - 1)) with a fixed
//    concentration kappa, on G evenly spaced points g_j = 2 pi j / G of the
//    circle;
//  * bonds and angles: Gaussian kernel exp(-(g - x)^2 / (2 h^2)) with
//    Silverman's bandwidth h = 1.06 sigma N^(-1/5) (sigma the population
//    standard deviation of the DOF's frames), on G points
//    g_j = lo + (j + 1/2)(hi - lo) / G over the DOF's range [lo, hi].
// The density's grid minima (d_j < d_{j-1} and d_j <= d_{j+1}; cyclic for
// torsions) split the DOF's range into conformer intervals, like the
// reference's minima split the circle, and every frame gets the index of its
// interval: linear DOFs bin(x) = #{minima <= x} (M minima, M + 1 bins);
// torsions bin(a) = (#{minima <= a} + M - 1) mod M, the interval that wraps
// through 0 taking index M - 1 (M bins; one bin without minima).
// The reference has no such mode, so its results are pinned only by the CPU
// restatement in the oracle, which follows the same definitions.
//
// GB300 mapping: one CTA of 4 warps per DOF.
//  * torsions: lane l owns grid points l, l + 32, ...; each warp takes a
//    quarter of the frames 32 at a time, every lane loading one frame
//    (coalesced) and preparing its half-angle sine and cosine, then the 32
//    frames are broadcast by warp shuffles and each lane adds its grid
//    points' terms.  The terms run in double-float arithmetic on the FP32
//    pipe (dfloat.cuh): kappa (cos t - 1) = -2 kappa sin^2(t/2) with
//    sin((g - a)/2) from the half-angle products (no cancellation near
//    t = 0), e^y by a table-driven double-float exp, double-float sums; the
//    terms agree with FP64 to ~1e-12 relative.  A grid point whose
//    double-float density is below kDfFloor is summed again in FP64: terms
//    under the FP32 range (below e^-87, dropped) or with a subnormal low word
//    (below e^-70) could otherwise matter there, so empty regions of the
//    circle keep FP64 values (above the floor the dropped mass, at most
//    N e^-70, stays below 4e-13 of the density for N up to 10^8).
//  * bonds/angles: every thread takes its own frames and walks the grid
//    outwards from the frame's nearest grid point with the Gaussian's
//    multiplicative recurrence (z_{j+1} = z_j + s, s = step / h):
//    e_{j+1} = e_j r_j, r_{j+1} = r_j exp(-s^2), so a frame costs three exps
//    and two FP64 multiplies per grid point instead of one exp per point; its
//    terms go to the thread's own column of a shared-memory accumulator.
//    Terms agree with the direct exp to ~1e-14 relative (50 recurrence
//    steps).
// The partial sums are combined in a fixed order, one thread finds the minima
// and the CTA labels the DOF's frames.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dfloat.cuh"

namespace centre {
namespace {

constexpr double kTwoPiG = 6.283185307179586;   // src/Constants.h:94
constexpr int kGkThreads = 128;
constexpr int kGkWarps = kGkThreads / 32;
constexpr int kMaxGrid = 128;
constexpr int kPerLane = kMaxGrid / 32;
constexpr double kDfFloor = 1e-10;   // double-float densities below: FP64 again

// Per-DOF Gaussian grid of a bond/angle DOF: lo, grid step, 1/h; degenerate
// (zero range or zero spread) DOFs get step 0 and a single bin.
struct LinGrid {
  double lo, step, inv_h;
};

__device__ __forceinline__ double block_sum(double v, double *red) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < kGkWarps; ++w) s += red[w];   // same order in every thread
  return s;
}

// min, max, mean and population standard deviation of one bond/angle DOF
// (two passes, fixed reduction order), then its grid and bandwidth.
__global__ void __launch_bounds__(kGkThreads)
gridkde_stats_kernel(const float *__restrict__ data, uint64_t n, int ngrid,
                     LinGrid *__restrict__ grids, int *__restrict__ flag) {
  const uint64_t d = blockIdx.x;
  const float *x = data + d * n;
  const int tid = threadIdx.x;
  __shared__ double red[kGkWarps];
  __shared__ float fmn[kGkWarps], fmx[kGkWarps];
  float mn = INFINITY, mx = -INFINITY;
  double s = 0.0;
  bool bad = false;
  for (uint64_t i = tid; i < n; i += kGkThreads) {
    const float v = x[i];
    bad |= !isfinite(v);
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
    s += (double)v;
  }
  if (bad) atomicOr(flag, kFlagDomain);
  for (int o = 16; o; o >>= 1) {
    mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  if ((tid & 31) == 0) {
    fmn[tid >> 5] = mn;
    fmx[tid >> 5] = mx;
  }
  const double mean = block_sum(s, red) / (double)n;
  for (int w = 0; w < kGkWarps; ++w) {
    mn = fminf(mn, fmn[w]);
    mx = fmaxf(mx, fmx[w]);
  }
  double q = 0.0;
  for (uint64_t i = tid; i < n; i += kGkThreads) {
    const double e = (double)x[i] - mean;
    q += e * e;
  }
  const double var = block_sum(q, red) / (double)n;
  if (tid == 0) {
    const double sigma = sqrt(var);
    const double h = 1.06 * sigma * pow((double)n, -0.2);
    LinGrid g;
    g.lo = (double)mn;
    g.step = ((double)mx - (double)mn) / ngrid;
    g.inv_h = (h > 0.0) ? 1.0 / h : 0.0;
    if (!(g.step > 0.0) || !(h > 0.0)) g.step = 0.0;
    grids[d] = g;
  }
}

// Grid sums, minima and frame labels of one DOF per CTA.
template <bool kTorsion>
__global__ void __launch_bounds__(kGkThreads)
gridkde_kernel(const float *__restrict__ data, uint64_t n, int ngrid, double kappa,
               const LinGrid *__restrict__ grids, uint8_t *__restrict__ bins,
               double *__restrict__ minima, uint8_t *__restrict__ nmin_out,
               uint8_t *__restrict__ nbins_out, int *__restrict__ flag) {
  const uint64_t d = blockIdx.x;
  const float *x = data + d * n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ double part[kGkWarps][kMaxGrid];
  extern __shared__ double gacc[];   // bonds/angles: [ngrid][kGkThreads]
  __shared__ double dens[kMaxGrid];
  __shared__ double mpos[kMaxGrid];
  __shared__ int nm_s;
  LinGrid lg;
  lg.lo = 0.0;
  lg.step = 0.0;
  lg.inv_h = 0.0;
  if (!kTorsion) lg = grids[d];
  const bool flat = !kTorsion && lg.step == 0.0;

  // this lane's grid points
  double ga[kPerLane], gb[kPerLane], acc[kPerLane];
#pragma unroll
  for (int k = 0; k < kPerLane; ++k) {
    const int j = lane + 32 * k;
    acc[k] = 0.0;
    if (kTorsion) {
      const double g = kTwoPiG * j / ngrid;
      ga[k] = cos(g);
      gb[k] = sin(g);
    } else {
      ga[k] = lg.lo + (j + 0.5) * lg.step;
      gb[k] = 0.0;
    }
  }
  if (kTorsion) {
    __shared__ float dftab[2 * kDfExpTable];
    if (tid < kDfExpTable) {
      const double t = exp2((double)tid / kDfExpTable);
      const float hi = __double2float_rn(t);
      dftab[2 * tid] = hi;
      dftab[2 * tid + 1] = __double2float_rn(t - (double)hi);
    }
    __syncthreads();
    dfl sgh[kPerLane], cgh[kPerLane], dacc[kPerLane];
#pragma unroll
    for (int k = 0; k < kPerLane; ++k) {
      const double h = 0.5 * kTwoPiG * (lane + 32 * k) / ngrid;   // half the grid angle
      sgh[k] = df_from_double(sin(h));
      cgh[k] = df_from_double(cos(h));
      dacc[k] = df_make(0.0f, 0.0f);
    }
    const dfl m2k = df_from_double(-2.0 * kappa);
    const uint64_t per = (n + kGkWarps - 1) / kGkWarps;
    const uint64_t f0 = (uint64_t)warp * per, f1 = min(n, f0 + per);
    bool bad = false;
    for (uint64_t b = f0; b < f1; b += 32) {
      const uint64_t i = b + lane;
      const int cnt = (int)min((uint64_t)32, f1 - b);
      dfl sa = df_make(0.0f, 0.0f), ca = df_make(1.0f, 0.0f);
      if (i < f1) {
        const float v = x[i];
        bad |= !isfinite(v);
        double sh, ch;
        sincos(0.5 * (double)v, &sh, &ch);
        sa = df_from_double(sh);
        ca = df_from_double(ch);
      }
      for (int f = 0; f < cnt; ++f) {
        const dfl saf = df_make(__shfl_sync(0xffffffffu, sa.hi, f), __shfl_sync(0xffffffffu, sa.lo, f));
        const dfl caf = df_make(__shfl_sync(0xffffffffu, ca.hi, f), __shfl_sync(0xffffffffu, ca.lo, f));
#pragma unroll
        for (int k = 0; k < kPerLane; ++k) {
          if (lane + 32 * k < ngrid) {
            // sin((g - a)/2), then kappa (cos(g - a) - 1) = -2 kappa sin^2
            const dfl sd = df_add(df_mul(sgh[k], caf), df_mul(cgh[k], df_make(-saf.hi, -saf.lo)));
            const dfl y = df_mul(df_mul(sd, sd), m2k);
            dacc[k] = df_add(dacc[k], df_exp_neg(y, dftab));
          }
        }
      }
    }
    if (bad) atomicOr(flag, kFlagDomain);
#pragma unroll
    for (int k = 0; k < kPerLane; ++k)
      if (lane + 32 * k < ngrid) part[warp][lane + 32 * k] = df_value(dacc[k].hi, dacc[k].lo);
    __syncthreads();
    // grid points below the double-float range: FP64 sums (lanes own grid
    // points as above; the other lanes idle through the frames)
    bool tiny = false;
#pragma unroll
    for (int k = 0; k < kPerLane; ++k) {
      const int j = lane + 32 * k;
      if (j < ngrid) {
        double t = 0.0;
        for (int w = 0; w < kGkWarps; ++w) t += part[w][j];
        tiny |= t < kDfFloor;
      }
    }
    if (__syncthreads_or(tiny)) {
#pragma unroll
      for (int k = 0; k < kPerLane; ++k) acc[k] = 0.0;
      bool need[kPerLane];
#pragma unroll
      for (int k = 0; k < kPerLane; ++k) {
        const int j = lane + 32 * k;
        double t = 0.0;
        if (j < ngrid)
          for (int w = 0; w < kGkWarps; ++w) t += part[w][j];
        need[k] = j < ngrid && t < kDfFloor;
      }
      __syncthreads();
      for (uint64_t b = f0; b < f1; b += 32) {
        const uint64_t i = b + lane;
        const int cnt = (int)min((uint64_t)32, f1 - b);
        double p = 0.0, q = 0.0;
        if (i < f1) sincos((double)x[i], &q, &p);   // p = cos a, q = sin a
        for (int f = 0; f < cnt; ++f) {
          const double pf = __shfl_sync(0xffffffffu, p, f);
          const double qf = __shfl_sync(0xffffffffu, q, f);
#pragma unroll
          for (int k = 0; k < kPerLane; ++k)
            if (need[k]) acc[k] += exp(kappa * (ga[k] * pf + gb[k] * qf - 1.0));
        }
      }
#pragma unroll
      for (int k = 0; k < kPerLane; ++k)
        if (need[k]) part[warp][lane + 32 * k] = acc[k];
    }
  } else {
    for (int j = 0; j < ngrid; ++j) gacc[j * kGkThreads + tid] = 0.0;
    if (!flat) {
      const double sg = lg.step * lg.inv_h;
      const double qg = exp(-sg * sg);
      for (uint64_t i = tid; i < n; i += kGkThreads) {
        const double v = (double)x[i];
        int j0 = (int)floor((v - lg.lo) / lg.step);
        j0 = max(0, min(ngrid - 1, j0));
        const double z0 = (lg.lo + (j0 + 0.5) * lg.step - v) * lg.inv_h;
        const double e0 = exp(-0.5 * z0 * z0);
        gacc[j0 * kGkThreads + tid] += e0;
        double ef = e0, eb = e0;
        double r = exp(-z0 * sg - 0.5 * sg * sg);    // e_{j0+1} / e_{j0}
        double u = exp(z0 * sg - 0.5 * sg * sg);     // e_{j0-1} / e_{j0}
        int jf = j0 + 1, jb = j0 - 1;
        for (int t = 0; t < ngrid - 1; ++t) {
          const bool fw = jf < ngrid;
          double e = fw ? ef : eb;
          double m = fw ? r : u;
          e *= m;
          m *= qg;
          if (fw) {
            ef = e;
            r = m;
          } else {
            eb = e;
            u = m;
          }
          gacc[(fw ? jf : jb) * kGkThreads + tid] += e;
          jf += fw ? 1 : 0;
          jb -= fw ? 0 : 1;
        }
      }
    }
    __syncthreads();
    for (int j = tid; j < ngrid; j += kGkThreads) {
      double t = 0.0;
      for (int w = 0; w < kGkThreads; ++w) t += gacc[j * kGkThreads + w];
      part[0][j] = t;
      for (int w = 1; w < kGkWarps; ++w) part[w][j] = 0.0;
    }
  }
  __syncthreads();
  for (int j = tid; j < ngrid; j += kGkThreads) {
    double s = 0.0;
    for (int w = 0; w < kGkWarps; ++w) s += part[w][j];
    dens[j] = s;
  }
  __syncthreads();
  if (tid == 0) {
    int m = 0;
    if (!flat) {
      if (kTorsion) {
        for (int j = 0; j < ngrid; ++j) {
          const double l = dens[(j + ngrid - 1) % ngrid], r = dens[(j + 1) % ngrid];
          if (dens[j] < l && dens[j] <= r) mpos[m++] = kTwoPiG * j / ngrid;
        }
      } else {
        for (int j = 1; j + 1 < ngrid; ++j)
          if (dens[j] < dens[j - 1] && dens[j] <= dens[j + 1])
            mpos[m++] = lg.lo + (j + 0.5) * lg.step;
      }
    }
    nm_s = m;
    for (int j = 0; j < ngrid; ++j) minima[d * ngrid + j] = (j < m) ? mpos[j] : 0.0;
    nmin_out[d] = (uint8_t)m;
    nbins_out[d] = (uint8_t)(kTorsion ? (m > 0 ? m : 1) : m + 1);
  }
  __syncthreads();
  const int m = nm_s;
  uint8_t *out = bins + d * n;
  for (uint64_t i = tid; i < n; i += kGkThreads) {
    const double v = (double)x[i];
    int lo = 0, hi = m;   // number of minima <= v
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (mpos[mid] <= v) lo = mid + 1; else hi = mid;
    }
    int b = lo;
    if (kTorsion) b = (m > 0) ? (lo + m - 1) % m : 0;
    out[i] = (uint8_t)b;
  }
}

// e^y of the double-float exponential for given doubles y (its test hook)
__global__ void df_exp_eval_kernel(const double *__restrict__ y, uint64_t n,
                                   double *__restrict__ out) {
  __shared__ float tab[2 * kDfExpTable];
  if (threadIdx.x < kDfExpTable) {
    const double t = exp2((double)threadIdx.x / kDfExpTable);
    const float hi = __double2float_rn(t);
    tab[2 * threadIdx.x] = hi;
    tab[2 * threadIdx.x + 1] = __double2float_rn(t - (double)hi);
  }
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const dfl r = df_exp_neg(df_from_double(y[i]), tab);
    out[i] = df_value(r.hi, r.lo);
  }
}

}  // namespace

int launch_df_exp_eval(centre_ctx *ctx, const double *d_y, uint64_t n, double *d_out) {
  if (n == 0) return CENTRE_OK;
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 1024);
  df_exp_eval_kernel<<<grid, 256, 0, ctx->stream>>>(d_y, n, d_out);
  ctx->launches += 1;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

size_t gridkde_work_bytes(uint32_t ndof) { return sizeof(LinGrid) * (size_t)ndof; }

int launch_gridkde(centre_ctx *ctx, int bat_type, const float *d_data, uint32_t ndof,
                   uint64_t nframes, int ngrid, double kappa, uint8_t *d_bins, double *d_minima,
                   uint8_t *d_nmin, uint8_t *d_nbins, void *d_work) {
  if (bat_type < 1 || bat_type > 3) return set_error(ctx, CENTRE_E_ARG, "bat_type must be 1..3");
  if (ngrid < 3 || ngrid > kMaxGrid)
    return set_error(ctx, CENTRE_E_ARG, "ngrid must be 3..128");
  if (bat_type == 3 && !(kappa > 0.0 && std::isfinite(kappa)))
    return set_error(ctx, CENTRE_E_ARG, "kappa must be positive and finite");
  if (ndof == 0 || nframes == 0) return CENTRE_OK;
  LinGrid *d_grids = reinterpret_cast<LinGrid *>(d_work);
  CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  {
    KernelTimer kt(ctx, CENTRE_TIMER_DISCRETIZE);
    if (bat_type == 3) {
      gridkde_kernel<true><<<ndof, kGkThreads, 0, ctx->stream>>>(
          d_data, nframes, ngrid, kappa, d_grids, d_bins, d_minima, d_nmin, d_nbins, ctx->d_flag);
      ctx->launches += 1;
    } else {
      gridkde_stats_kernel<<<ndof, kGkThreads, 0, ctx->stream>>>(d_data, nframes, ngrid, d_grids,
                                                                  ctx->d_flag);
      const size_t smem = sizeof(double) * (size_t)ngrid * kGkThreads;
      CENTRE_CUDA(ctx, cudaFuncSetAttribute(gridkde_kernel<false>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
      gridkde_kernel<false><<<ndof, kGkThreads, smem, ctx->stream>>>(
          d_data, nframes, ngrid, kappa, d_grids, d_bins, d_minima, d_nmin, d_nbins, ctx->d_flag);
      ctx->launches += 2;
    }
  }
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

}  // namespace centre
