// discretize.cu -- histogram discretisation of BAT coordinates into uint8 bins.
//
// Follows Real2Int::bndReal2Int / angReal2Int / dihReal2Int
// (src/Real2Int.cpp:27-73, :131-184, :244-479) as driven by
// Discretizer::run_dtype (src/Discretizer.cpp:138-207).
//
// GB300 design
//  * One thread-block cluster per DOF.  Each CTA of the cluster stages its
//    slice of the DOF's frames in shared memory (one HBM read), reduces its
//    slice, and the CTAs combine their partial min/max/sum/occupancy through
//    distributed shared memory.
//  * The reference bins with one IEEE double division per element:
//    floor(RN(RN(v - lo) / w)).  FP64 throughput is a small fraction of FP32
//    on GB300, so instead every bin edge is turned into an exact float
//    threshold: the reference's quantiser is a non-decreasing function of the
//    float input x (RN is monotone, the fold v = x + c - 2pi is exact and
//    monotone within each side of the fold point), so bin(x) is the number of
//    thresholds <= x.  Thresholds are found once per DOF by bisection over
//    float bit patterns evaluating the reference expression in double; the
//    per-element work is then an FP32 guess plus one or two float compares.
//    The bins are bit-identical to the reference by construction.
//  * The min/max of the shifted torsion values RN(x + c) mod 2pi are exact:
//    RN(x + c) is monotone in x, so per side of the fold point it is reached
//    at the float min/max of x.  No per-element FP64 work remains except the
//    avg sum, which is kept in double-float (FP32 pairs) per thread.
#include <cooperative_groups.h>

#include <cfloat>
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace centre {
namespace {

constexpr double kPi = 3.141592653589793;      // src/Constants.h:92
constexpr double kTwoPi = 6.283185307179586;   // src/Constants.h:94
constexpr double kDx = 5.0e-9;                 // src/configcentre.h:22
#ifndef CENTRE_DISC_THREADS
#define CENTRE_DISC_THREADS 512
#endif
#ifndef CENTRE_DISC_MIN_BLOCKS
#define CENTRE_DISC_MIN_BLOCKS 3     // resident CTAs per SM (registers <= 40)
#endif
constexpr int kThreads = CENTRE_DISC_THREADS;
static_assert(kThreads >= 256 && kThreads <= 1024 && kThreads % 32 == 0,
              "the table build gives each thread at most one entry of 256");
constexpr int kMaxFit = 180;                   // src/Real2Int.cpp:269
// cluster size cap and shared-memory slice per CTA (build-time knobs; a DOF
// whose slice exceeds the budget at the largest cluster is read twice, the
// second time from L2, instead of staged).  Every CTA of a cluster repeats
// the per-DOF serial phases (cluster reduction, range, thresholds, table), so
// few CTAs per DOF and more resident CTAs per SM win: on 2994 DOFs x 100,000
// frames, clusters of 2 unstaged with 3 CTAs of 512 threads per SM took
// 1.17 ms against 2.63 ms for staged clusters of 4 at 2 CTAs per SM.
#ifndef CENTRE_DISC_MAX_CLUSTER
#define CENTRE_DISC_MAX_CLUSTER 2
#endif
#ifndef CENTRE_DISC_STAGE_KB
#define CENTRE_DISC_STAGE_KB 104
#endif
constexpr int kMaxCluster = CENTRE_DISC_MAX_CLUSTER;
constexpr size_t kStageBytes = CENTRE_DISC_STAGE_KB * 1024;
constexpr int kLut = 256;                      // binning lookup-table entries

struct DiscParams {
  int type;              // 1 bond, 2 angle, 3 torsion
  int optimize;
  int nschemes;
  uint64_t nframes;
  uint64_t slice;        // frames per CTA (multiple of 16)
  int staged;            // slice lives in shared memory
  int nfit;              // coarse occupancy bins (torsions, optimize)
  double fit_bs;         // coarse bin size
  float xpi;             // smallest float x with RN(x + pi) >= 2pi
  float xmax_ok;         // largest float accepted for this DOF type
  uint8_t schemes[kMaxSchemes];
  float tfit[kMaxFit + 1];   // tfit[k]: smallest x with coarse bin >= k
};

// Partial reductions a CTA publishes to its cluster.
struct Partial {
  float xmin, xmax;            // raw values
  float cmin[2], cmax[2];      // pi-shift sides: [0] unfolded, [1] folded
  float dmin[2], dmax[2];      // displacement-shift sides
  double sum;
  int bad;
  unsigned hist[kMaxFit];
};

// --- exact reference arithmetic (double, no contraction) -------------------

// Value the reference bins for input x: x, or fmod(x + c, 2pi).  With x in
// [0, 2pi) (checked) and c in (0, 2pi], a = RN(x + c) lies in [0, 4pi), and
// fmod(a, 2pi) is a when a < 2pi and exactly a - 2pi otherwise (fmod is
// exact, and so is the subtraction by Sterbenz's lemma since 2pi <= a <
// 2 * 2pi), so the conditional subtraction returns the same double.
__device__ __forceinline__ double shifted(float x, int dpind, double c) {
  if (dpind == 0) return (double)x;
  double a = __dadd_rn((double)x, c);
  return a >= kTwoPi ? __dsub_rn(a, kTwoPi) : a;
}

// floor((v - lo) / w) as the reference computes it, before the (t == nb)
// clamp (src/Real2Int.cpp:65, :462-473).
__device__ __forceinline__ int ref_bin(float x, int dpind, double c, double lo,
                                       double w) {
  double v = shifted(x, dpind, c);
  double q = __ddiv_rn(__dsub_rn(v, lo), w);
  return (int)floor(q);
}

// Smallest float x in [a, b] (non-negative, a <= b) with pred(x) true, given
// pred monotone (false...true) and pred(b) true.
template <class Pred>
__device__ float bisect_first(float a, float b, Pred pred) {
  if (a == 0.0f) a = 0.0f;   // -0 would order below every positive float's bits
  int lo = __float_as_int(a), hi = __float_as_int(b);
  if (pred(a)) return a;
  // invariant: pred(lo) false, pred(hi) true
  while (hi - lo > 1) {
    int mid = lo + ((hi - lo) >> 1);
    if (pred(__int_as_float(mid)))
      hi = mid;
    else
      lo = mid;
  }
  return __int_as_float(hi);
}

// Bracketed variant: tries [guess - 4, guess + 4] (floats) first, then
// [guess - 256, guess + 256], then the whole range.  The guess from the
// double expression is usually within a few floats of the threshold.
template <class Pred>
__device__ float bisect_guess(float a, float b, float guess, Pred pred) {
  if (a == 0.0f) a = 0.0f;
  int ga = __float_as_int(a), gb = __float_as_int(b);
  int g = __float_as_int(fminf(fmaxf(guess, a), b));
  for (int span = 4; span <= 256; span *= 64) {
    int l = max(ga, g - span), h = min(gb, g + span);
    float fl = __int_as_float(l), fh = __int_as_float(h);
    if (pred(fh) && (l == ga || !pred(fl))) return bisect_first(fl, fh, pred);
  }
  return bisect_first(a, b, pred);
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// --- block reductions -------------------------------------------------------
// One block-wide reduction of NM minima, NM maxima, a double sum and an OR
// flag (one barrier round instead of one per value); results valid in thread 0.
template <int NM>
__device__ void block_minmax(float (&mn)[NM], float (&mx)[NM], double &sum, int &flag,
                             float *red /*[2*NM][32]*/, double *redd /*[32]*/,
                             int *redb /*[32]*/) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NM; ++q)
    for (int o = 16; o; o >>= 1) {
      mn[q] = fminf(mn[q], __shfl_xor_sync(0xffffffffu, mn[q], o));
      mx[q] = fmaxf(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], o));
    }
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  flag = __any_sync(0xffffffffu, flag) ? 1 : 0;
  if (l == 0) {
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      red[q * 32 + w] = mn[q];
      red[(NM + q) * 32 + w] = mx[q];
    }
    redd[w] = sum;
    redb[w] = flag;
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      mn[q] = l < nw ? red[q * 32 + l] : FLT_MAX;
      mx[q] = l < nw ? red[(NM + q) * 32 + l] : -FLT_MAX;
      for (int o = 16; o; o >>= 1) {
        mn[q] = fminf(mn[q], __shfl_xor_sync(0xffffffffu, mn[q], o));
        mx[q] = fmaxf(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], o));
      }
    }
    sum = l < nw ? redd[l] : 0.0;
    for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    flag = __any_sync(0xffffffffu, l < nw ? redb[l] : 0) ? 1 : 0;
  }
}

struct DofState {
  int dpind;
  double c;          // shift constant (pi or displacement)
  float xfold;       // smallest x that folds (RN(x + c) >= 2pi)
  double lo, hi, avg, phase;
  float clsmin[2], clsmax[2];   // raw-x range of each side of the fold
  int has[2];
  int kmin[kMaxSchemes][2], kmax[kMaxSchemes][2];
  int bad;
};

__global__ void __launch_bounds__(kThreads, CENTRE_DISC_MIN_BLOCKS)
discretize_kernel(const float *__restrict__ data, uint8_t *__restrict__ bins,
                  double *__restrict__ extremes, const __grid_constant__ DiscParams P,
                  int *__restrict__ flag) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int csize = (int)cluster.num_blocks();
  const uint64_t dof = blockIdx.x / csize;
  const uint64_t n = P.nframes;
  const uint64_t f0 = (uint64_t)rank * P.slice;
  const uint64_t f1 = min(n, f0 + P.slice);
  const uint64_t cnt = f1 > f0 ? f1 - f0 : 0;
  const float *gsrc = data + dof * n + f0;

  extern __shared__ __align__(16) unsigned char dyn[];
  float *stage = reinterpret_cast<float *>(dyn);
  // thresholds after the staged slice: [scheme][side][k], k = 0..255
  float *thr = reinterpret_cast<float *>(dyn + (P.staged ? P.slice * 4 : 0));
  __shared__ Partial part[2];   // [0]: first reduction, [1]: displacement pass
  // one buffer for two phases: per-warp coarse occupancy counters while the
  // slice is scanned, the binning lookup table (per scheme) afterwards
  constexpr int kFitWords = (kMaxFit + 1) / 2;   // two 16-bit counters a word
  __shared__ uint32_t phase_buf[(kThreads / 32) * kFitWords > 2 * kLut
                                    ? (kThreads / 32) * kFitWords : 2 * kLut];
  uint32_t *lut_code = phase_buf;
  float *lut_t = reinterpret_cast<float *>(phase_buf + kLut);
  __shared__ double redd[32];
  __shared__ DofState st;

  const int tid = threadIdx.x;
  // fit thresholds in shared memory: the lanes of a warp index them by
  // their own coarse bin, which would serialise on the constant bank
  __shared__ float tfit_s[kMaxFit + 1];
  // coarse occupancy: a private histogram per warp (16-bit counters, two to
  // a word; a warp sees at most 32 x slice/blockDim frames of a slice) so
  // the same-bin atomics of clustered torsions stay inside one warp
  uint32_t *warp_fit = phase_buf + (threadIdx.x >> 5) * kFitWords;
  // a warp counts at most 32 * ceil(slice / blockDim) + 256 frames of its
  // slice; beyond 16 bits the CTA-wide 32-bit counters are used directly
  const bool small_fit = 32ull * ((P.slice + kThreads - 1) / kThreads) + 256 < 65536ull;
  for (int i = tid; i < kMaxFit; i += blockDim.x) part[0].hist[i] = 0;
  for (int i = tid; i < (kThreads / 32) * kFitWords; i += blockDim.x) phase_buf[i] = 0;
  if (P.type == 3 && P.optimize)
    for (int i = tid; i <= P.nfit; i += blockDim.x) tfit_s[i] = P.tfit[i];
  __syncthreads();

  // ---- pass 1: stage, min/max/sum, pi-shift sides, coarse occupancy ------
  const bool is_tor = (P.type == 3);
  float xmin = FLT_MAX, xmax = -FLT_MAX;
  float cmin0 = FLT_MAX, cmax0 = -FLT_MAX, cmin1 = FLT_MAX, cmax1 = -FLT_MAX;
  float s_hi = 0.f, s_lo = 0.f;
  int bad = 0;
  auto visit = [&](float x) {
    xmin = fminf(xmin, x);
    xmax = fmaxf(xmax, x);
    float s, e;
    two_sum(s_hi, x, s, e);
    s_hi = s;
    s_lo = __fadd_rn(s_lo, e);
    // domain: bonds >= 0, angles in [0, pi], torsions in [0, 2pi), finite;
    // xmax_ok is the exact float image of the double bound
    if (!(x >= 0.f && x <= P.xmax_ok)) bad = 1;
    if (is_tor) {
      if (x >= P.xpi) {
        cmin1 = fminf(cmin1, x);
        cmax1 = fmaxf(cmax1, x);
      } else {
        cmin0 = fminf(cmin0, x);
        cmax0 = fmaxf(cmax0, x);
      }
      if (P.optimize) {
        // coarse bin = number of fit thresholds <= x (exact, thresholds are
        // evaluated with the reference expression); guess then correct
        int k = (int)(x * (float)(1.0 / P.fit_bs));
        k = min(max(k, 0), P.nfit - 1);
        while (k > 0 && x < tfit_s[k]) --k;
        while (k < P.nfit - 1 && x >= tfit_s[k + 1]) ++k;
        if (small_fit) atomicAdd(&warp_fit[k >> 1], (k & 1) ? 0x10000u : 1u);
        else atomicAdd(&part[0].hist[k], 1u);
      }
    }
  };
  const bool vec = ((n & 3) == 0) && ((f0 & 3) == 0);
  if (vec) {
    const float4 *g4 = reinterpret_cast<const float4 *>(gsrc);
    float4 *s4 = reinterpret_cast<float4 *>(stage);
    uint64_t n4 = cnt >> 2;
    // four independent 16-byte loads in flight per thread before any use:
    // the slice streams at HBM rate instead of one load latency per step
    const uint64_t T = blockDim.x;
    uint64_t i = tid;
    for (; i + 3 * T < n4; i += 4 * T) {
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = __ldg(g4 + i + u * T);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (P.staged) s4[i + u * T] = v[u];
        visit(v[u].x); visit(v[u].y); visit(v[u].z); visit(v[u].w);
      }
    }
    for (; i < n4; i += T) {
      float4 v = __ldg(g4 + i);
      if (P.staged) s4[i] = v;
      visit(v.x); visit(v.y); visit(v.z); visit(v.w);
    }
    for (uint64_t i = (n4 << 2) + tid; i < cnt; i += blockDim.x) {
      float v = __ldg(gsrc + i);
      if (P.staged) stage[i] = v;
      visit(v);
    }
  } else {
    for (uint64_t i = tid; i < cnt; i += blockDim.x) {
      float v = __ldg(gsrc + i);
      if (P.staged) stage[i] = v;
      visit(v);
    }
  }
  const float *src = P.staged ? stage : gsrc;

  __shared__ float redm[6][32];
  __shared__ int redb[32];
  {
    float mn[3] = {xmin, cmin0, cmin1}, mx[3] = {xmax, cmax0, cmax1};
    double ds = (double)s_hi + (double)s_lo;
    int anybad = bad;
    block_minmax<3>(mn, mx, ds, anybad, &redm[0][0], redd, redb);
    if (tid == 0) {
      part[0].xmin = mn[0];
      part[0].xmax = mx[0];
      part[0].cmin[0] = mn[1];
      part[0].cmax[0] = mx[1];
      part[0].cmin[1] = mn[2];
      part[0].cmax[1] = mx[2];
      part[0].sum = ds;
      part[0].bad = anybad;
    }
    if (is_tor && P.optimize) {
      // sum the per-warp counters into the CTA's occupancy
      __syncthreads();
      if (small_fit)
        for (int k = tid; k < P.nfit; k += blockDim.x) {
          unsigned c = 0;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            c += (phase_buf[w * kFitWords + (k >> 1)] >> ((k & 1) * 16)) & 0xFFFFu;
          part[0].hist[k] = c;
        }
    }
  }
  cluster.sync();

  // ---- combine the cluster's partials (every CTA, same order) ------------
  if (tid == 0) {
    float gxmin = FLT_MAX, gxmax = -FLT_MAX, c0n = FLT_MAX, c0x = -FLT_MAX,
          c1n = FLT_MAX, c1x = -FLT_MAX;
    double sum = 0.0;
    int gbad = 0;
    for (int q = 0; q < csize; ++q) {
      const Partial *pp = cluster.map_shared_rank(&part[0], q);
      gxmin = fminf(gxmin, pp->xmin);
      gxmax = fmaxf(gxmax, pp->xmax);
      c0n = fminf(c0n, pp->cmin[0]);
      c0x = fmaxf(c0x, pp->cmax[0]);
      c1n = fminf(c1n, pp->cmin[1]);
      c1x = fmaxf(c1x, pp->cmax[1]);
      sum += pp->sum;
      gbad |= pp->bad;
    }
    st.bad = gbad;
    st.clsmin[0] = gxmin;  // provisional (raw range)
    st.clsmax[0] = gxmax;
    part[1].sum = sum;      // stash the total
    part[1].cmin[0] = c0n; part[1].cmax[0] = c0x;
    part[1].cmin[1] = c1n; part[1].cmax[1] = c1x;
    part[1].xmin = gxmin; part[1].xmax = gxmax;
  }
  // the coarse histogram is combined bin-parallel
  __shared__ unsigned hist_all[kMaxFit];
  if (is_tor && P.optimize) {
    for (int k = tid; k < P.nfit; k += blockDim.x) {
      unsigned s = 0;
      for (int q = 0; q < csize; ++q) s += cluster.map_shared_rank(&part[0], q)->hist[k];
      hist_all[k] = s;
    }
  }
  __syncthreads();

  // ---- torsion displacement (largest empty circular run) -----------------
  __shared__ double disp_s;
  __shared__ float xdisp_s;
  // occupancy of the doubled ring as bit words, built by warp 0 with ballots
  __shared__ unsigned ne_s[(2 * kMaxFit + 31) / 32];
  __shared__ unsigned nempty_s;
  if (is_tor && P.optimize && tid < 32) {
    const int nf = P.nfit, n2 = 2 * nf;
    for (int w = 0; w < (n2 + 31) / 32; ++w) {
      const int q = 32 * w + tid;
      const unsigned m = __ballot_sync(0xffffffffu, q < n2 && hist_all[q % nf] != 0);
      if (tid == 0) ne_s[w] = m;
    }
    unsigned e = 0;
    for (int k = tid; k < nf; k += 32) e += (hist_all[k] == 0);
    for (int o = 16; o; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (tid == 0) nempty_s = e;
  }
  __syncthreads();
  if (is_tor && P.optimize && tid == 0) {
    const int nf = P.nfit;
    const unsigned nempty = nempty_s;
    int minidx = 0;
    if (nempty == 0) {
      unsigned rec = hist_all[0];
      for (int j = 1; j < nf; ++j)
        if (hist_all[j] < rec) {
          rec = hist_all[j];
          minidx = j;
        }
    } else {
      // Scan the doubled ring from the first empty bin; a run of empty bins
      // is scored when the next non-empty bin closes it, the first strictly
      // longest run wins (a run still open at the end is not scored).  The
      // occupancy is walked run by run over bit words, not bin by bin.
      const int n2 = 2 * nf;
      const unsigned *ne = ne_s;
      const int nw = (n2 + 31) / 32;
      // first q >= from whose occupancy equals `want` (n2 if none)
      auto next = [&](int from, bool want) {
        for (int w = from >> 5; w < nw; ++w) {
          unsigned m = want ? ne[w] : ~ne[w];
          if (w == (from >> 5)) m &= ~0u << (from & 31);
          if (w == nw - 1 && (n2 & 31)) m &= (1u << (n2 & 31)) - 1u;
          if (m) return 32 * w + __ffs(m) - 1;
        }
        return n2;
      };
      const int j = next(0, false);   // first empty bin (nempty > 0)
      minidx = j;
      int best = 0;
      for (int q = j; q < n2;) {
        const int e = next(q, false);
        if (e >= n2) break;
        const int c = next(e, true);
        if (c >= n2) break;
        if (c - e > best) {
          best = c - e;
          minidx = e;
        }
        q = c;
      }
    }
    if (minidx >= nf) minidx = nf - 1;  // unreachable for valid occupancy
    double center = __dadd_rn(0.0, __dmul_rn(minidx + 0.5, P.fit_bs));
    double disp = __dsub_rn(kTwoPi, center);
    disp_s = disp;
    // smallest float x >= 0 with RN(x + disp) >= 2pi
    float hi = 7.0f;
    xdisp_s = bisect_first(0.0f, hi, [&](float x) {
      return __dadd_rn((double)x, disp) >= kTwoPi;
    });
  }
  __syncthreads();

  // ---- pass 2 (torsions, optimize): displacement-shift sides -------------
  if (is_tor && P.optimize) {
    const float xd = xdisp_s;
    float a0 = FLT_MAX, b0 = -FLT_MAX, a1 = FLT_MAX, b1 = -FLT_MAX;
    for (uint64_t i = tid; i < cnt; i += blockDim.x) {
      float x = src[i];
      if (x >= xd) {
        a1 = fminf(a1, x);
        b1 = fmaxf(b1, x);
      } else {
        a0 = fminf(a0, x);
        b0 = fmaxf(b0, x);
      }
    }
    {
      float mn[2] = {a0, a1}, mx[2] = {b0, b1};
      double dummy = 0.0;
      int nf = 0;
      block_minmax<2>(mn, mx, dummy, nf, &redm[0][0], redd, redb);
      if (tid == 0) {
        part[0].dmin[0] = mn[0];
        part[0].dmax[0] = mx[0];
        part[0].dmin[1] = mn[1];
        part[0].dmax[1] = mx[1];
      }
    }
    cluster.sync();
    if (tid == 0) {
      float d0n = FLT_MAX, d0x = -FLT_MAX, d1n = FLT_MAX, d1x = -FLT_MAX;
      for (int q = 0; q < csize; ++q) {
        const Partial *pp = cluster.map_shared_rank(&part[0], q);
        d0n = fminf(d0n, pp->dmin[0]);
        d0x = fmaxf(d0x, pp->dmax[0]);
        d1n = fminf(d1n, pp->dmin[1]);
        d1x = fmaxf(d1x, pp->dmax[1]);
      }
      part[1].dmin[0] = d0n; part[1].dmax[0] = d0x;
      part[1].dmin[1] = d1n; part[1].dmax[1] = d1x;
    }
  }

  // ---- range selection (src/Real2Int.cpp:49-58, :156-168, :395-452) ------
  if (tid == 0) {
    const double sum = part[1].sum;
    const float gxmin = part[1].xmin, gxmax = part[1].xmax;
    double lo, hi, avg = sum / (double)n, phase = 0.0, c = 0.0;
    int dpind = 0;
    float xfold = FLT_MAX;
    if (P.type != 3) {
      lo = (double)gxmin;
      hi = (double)gxmax;
      lo = __dsub_rn(lo, kDx);
      if (lo < 0.0) lo = 0.0;
      hi = __dadd_rn(hi, kDx);
      if (P.type == 2 && hi > kPi) hi = kPi;
      if (__dsub_rn(hi, lo) < 1.0e-4) hi = __dadd_rn(hi, 0.05);
      st.has[0] = 1;
      st.has[1] = 0;
      st.clsmin[0] = gxmin;
      st.clsmax[0] = gxmax;
    } else {
      // variant 1: raw values (initial values of src/Real2Int.cpp:271-276)
      double lo1 = fmin(6.5, (double)gxmin), hi1 = fmax(0.0, (double)gxmax);
      // variant 2: fmod(x + pi, 2pi), exact from the per-side float extremes
      double lo2 = 6.5, hi2 = 0.0;
      if (part[1].cmin[0] <= part[1].cmax[0]) {  // unfolded side non-empty
        lo2 = fmin(lo2, __dadd_rn((double)part[1].cmin[0], kPi));
        hi2 = fmax(hi2, __dadd_rn((double)part[1].cmax[0], kPi));
      }
      if (part[1].cmin[1] <= part[1].cmax[1]) {
        lo2 = fmin(lo2, __dadd_rn((double)part[1].cmin[1], kPi) - kTwoPi);
        hi2 = fmax(hi2, __dadd_rn((double)part[1].cmax[1], kPi) - kTwoPi);
      }
      if (!P.optimize) {
        double r1 = __dsub_rn(hi1, lo1), r2 = __dsub_rn(hi2, lo2);
        if (fabs(__dsub_rn(r1, r2)) <= 1.0e-1 || r1 < r2) {
          lo = lo1; hi = hi1; dpind = 0;
        } else {
          lo = lo2; hi = hi2; dpind = 1;
          c = kPi;
          xfold = P.xpi;
        }
        phase = dpind * kPi;
      } else {
        const double disp = disp_s;
        double lo3 = 1.0e100, hi3 = 0.0;
        if (part[1].dmin[0] <= part[1].dmax[0]) {
          lo3 = fmin(lo3, __dadd_rn((double)part[1].dmin[0], disp));
          hi3 = fmax(hi3, __dadd_rn((double)part[1].dmax[0], disp));
        }
        if (part[1].dmin[1] <= part[1].dmax[1]) {
          lo3 = fmin(lo3, __dadd_rn((double)part[1].dmin[1], disp) - kTwoPi);
          hi3 = fmax(hi3, __dadd_rn((double)part[1].dmax[1], disp) - kTwoPi);
        }
        lo = lo3; hi = hi3; dpind = 2;
        c = disp;
        xfold = xdisp_s;
        phase = disp;
      }
      lo = __dsub_rn(lo, kDx);
      if (lo < 0.0) lo = 0.0;
      hi = __dadd_rn(hi, kDx);
      if (hi > kTwoPi) hi = kTwoPi;
      if (__dsub_rn(hi, lo) < 1.0e-4) hi = __dadd_rn(hi, 0.05);
      if (dpind == 1) avg = fmod(sum / (double)n + kPi, kTwoPi);
      if (dpind == 2) avg = fmod(sum / (double)n + c, kTwoPi);
      if (dpind == 0) {
        st.has[0] = 1;
        st.has[1] = 0;
        st.clsmin[0] = gxmin;
        st.clsmax[0] = gxmax;
      } else {
        const float *mn = (dpind == 1) ? part[1].cmin : part[1].dmin;
        const float *mx = (dpind == 1) ? part[1].cmax : part[1].dmax;
        for (int s = 0; s < 2; ++s) {
          st.has[s] = mn[s] <= mx[s];
          st.clsmin[s] = mn[s];
          st.clsmax[s] = mx[s];
        }
      }
    }
    st.dpind = dpind;
    st.c = c;
    st.xfold = xfold;
    st.lo = lo;
    st.hi = hi;
    st.avg = avg;
    st.phase = phase;
  }
  __syncthreads();
  // bin range of each side per scheme: one thread per (scheme, side, end)
  __shared__ int kbad;
  if (tid == 0) kbad = 0;
  __syncthreads();
  if (tid < 4 * P.nschemes) {
    const int s = tid >> 2, side = (tid >> 1) & 1, end = tid & 1;
    const int nb = P.schemes[s];
    if (!st.has[side]) {
      if (end == 0) st.kmin[s][side] = 0;
      else st.kmax[s][side] = -1;
    } else {
      const double w = __ddiv_rn(__dsub_rn(st.hi, st.lo), (double)nb);
      const int k = ref_bin(end ? st.clsmax[side] : st.clsmin[side], st.dpind, st.c, st.lo, w);
      if (end == 0) st.kmin[s][side] = k;
      else st.kmax[s][side] = k;
      if ((end == 0 && k < 0) || (end == 1 && k > nb)) atomicOr(&kbad, 1);
    }
  }
  __syncthreads();
  if (tid == 0) {
    if (kbad) st.bad = 1;
    if (rank == 0 && !st.bad) {
      double *e = extremes + 4 * dof;
      e[0] = st.lo;
      e[1] = st.hi;
      e[2] = st.avg;
      e[3] = (P.type == 3) ? st.phase : 0.0;
    }
  }
  __syncthreads();
  if (st.bad) {
    if (rank == 0 && tid == 0) atomicOr(flag, kFlagDomain);
    cluster.sync();
    return;
  }

  // ---- thresholds: thr[s][side][k] = first x of the side with bin >= k ----
  // the cluster's CTAs split the thresholds and exchange them over DSMEM
  const int dpind = st.dpind;
  const double c = st.c, lo = st.lo;
  {
    int total = P.nschemes * 2 * 256;
    for (int i = tid; i < total; i += blockDim.x) {
      int k = i & 255, side = (i >> 8) & 1, s = i >> 9;
      if (k % csize != rank) continue;
      if (!st.has[side] || k <= st.kmin[s][side] || k > st.kmax[s][side]) continue;
      const int nb = P.schemes[s];
      const double w = __ddiv_rn(__dsub_rn(st.hi, lo), (double)nb);
      float a = st.clsmin[side], b = st.clsmax[side];
      // guess: v = lo + k w, x = v - c (+ 2pi on the folded side)
      double vg = lo + k * w;
      double xg = (dpind == 0) ? vg : (side ? vg - c + kTwoPi : vg - c);
      float t = bisect_guess(a, b, (float)xg, [&](float x) {
        return ref_bin(x, dpind, c, lo, w) >= k;
      });
      thr[i] = t;
    }
  }
  cluster.sync();
  if (csize > 1) {
    // pull the thresholds computed by the other CTAs
    int total = P.nschemes * 2 * 256;
    for (int i = tid; i < total; i += blockDim.x) {
      int k = i & 255, side = (i >> 8) & 1, s = i >> 9;
      int owner = k % csize;
      if (owner == rank) continue;
      if (!st.has[side] || k <= st.kmin[s][side] || k > st.kmax[s][side]) continue;
      thr[i] = *cluster.map_shared_rank(&thr[i], owner);
    }
  }
  // no CTA may exit (releasing its shared memory) while others still read it
  cluster.sync();

  // ---- binning pass ------------------------------------------------------
  const float xfold = st.xfold;
  for (int s = 0; s < P.nschemes; ++s) {
    const int nb = P.schemes[s];
    const float lof = (float)lo;
    const float rw = (float)((double)nb / (st.hi - lo));
    const float cf = (float)c;
    const int kmin0 = st.kmin[s][0], kmax0 = st.kmax[s][0];
    const int kmin1 = st.kmin[s][1], kmax1 = st.kmax[s][1];
    const float *t0 = thr + (s * 2 + 0) * 256;
    const float *t1 = thr + (s * 2 + 1) * 256;
    uint8_t *out = bins + (dof * P.nschemes + s) * n + f0;
    auto bin_of = [&](float x) -> uint32_t {
      int side = (dpind != 0 && x >= xfold) ? 1 : 0;
      float v = (dpind == 0) ? x : (side ? x + cf - 6.2831855f : x + cf);
      int k = (int)floorf((v - lof) * rw);
      const float *t = side ? t1 : t0;
      const int kmin = side ? kmin1 : kmin0, kmax = side ? kmax1 : kmax0;
      k = min(max(k, kmin), kmax);
      while (k > kmin && x < t[k]) --k;
      while (k < kmax && x >= t[k + 1]) ++k;
      return (uint32_t)((k == nb) ? nb - 1 : k) & 0xFFu;
    };
    // ---- lookup table over the DOF's raw range --------------------------
    // entry e(x) = floor((x - xlo) * L / (xhi - xlo)) in FP32 is a
    // non-decreasing function of x, so each entry is an interval of floats.
    // Inside an interval that does not hold the fold point, bin_of is
    // non-decreasing; when it rises by at most one there, the entry keeps the
    // two bins and the first float of the upper one, and a frame's bin is one
    // compare.  Other entries (two or more rises, or the fold) fall back to
    // bin_of per frame.  Bins are the same as bin_of's by construction.
    const float xlo = (part[1].xmin == 0.0f) ? 0.0f : part[1].xmin, xhi = part[1].xmax;
    const float lscale = (xhi > xlo) ? (float)kLut / (xhi - xlo) : 0.0f;
    auto entry_of = [&](float x) -> int {
      const int e = (int)__fmul_rn(__fsub_rn(x, xlo), lscale);
      return min(e, kLut - 1);
    };
    __syncthreads();   // the previous scheme's frames are done with the table
    for (int e = tid; e < kLut; e += blockDim.x) {
      // first float of entry e (xhi + 1 ulp when the entry is empty)
      float a;
      if (e == 0) {
        a = xlo;
      } else if (entry_of(xhi) < e) {
        a = __int_as_float(__float_as_int(xhi) + 1);
      } else {
        int l = __float_as_int(xlo), h = __float_as_int(xhi);   // e(l) < e <= e(h)
        while (h - l > 1) {
          const int m = l + ((h - l) >> 1);
          if (entry_of(__int_as_float(m)) >= e) h = m; else l = m;
        }
        a = __int_as_float(h);
      }
      lut_t[e] = a;
    }
    __syncthreads();
    uint32_t my_code[(kLut + 255) / 256];
    float my_t[(kLut + 255) / 256];
    for (int e = tid, q = 0; e < kLut; e += blockDim.x, ++q) {
      const float a = lut_t[e];
      const float b = (e + 1 < kLut) ? __int_as_float(__float_as_int(lut_t[e + 1]) - 1) : xhi;
      uint32_t code = 0;
      float t = INFINITY;
      if (a <= b && a <= xhi) {
        const uint32_t k0 = bin_of(a), k1 = bin_of(b);
        const bool fold = dpind != 0 && a < xfold && xfold <= b;
        if (fold || k1 > k0 + 1) {
          code = 0x10000u;
        } else if (k1 == k0) {
          code = k0 | (k0 << 8);
        } else {
          // one rise inside one side: it happens at that side's threshold
          // for bin k1 (the first float whose bin is >= k1; k1 <= nb - 1
          // here, so the nb -> nb - 1 fold of the top bin is not involved)
          const int side = (dpind != 0 && a >= xfold) ? 1 : 0;
          code = k0 | (k1 << 8);
          t = (side ? t1 : t0)[k1];
        }
      }
      my_code[q] = code;
      my_t[q] = t;
    }
    __syncthreads();
    for (int e = tid, q = 0; e < kLut; e += blockDim.x, ++q) {
      lut_code[e] = my_code[q];
      lut_t[e] = my_t[q];
    }
    __syncthreads();
    auto fast_bin = [&](float x) -> uint32_t {
      const int e = entry_of(x);
      const uint32_t code = lut_code[e];
      if (code & 0x10000u) return bin_of(x);
      return (x >= lut_t[e]) ? (code >> 8) & 0xFFu : code & 0xFFu;
    };
    // four frames at once: table reads first, rare slow entries after
    auto bins4 = [&](float4 v) -> uint32_t {
      const float xs[4] = {v.x, v.y, v.z, v.w};
      uint32_t code[4];
      float tt[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = entry_of(xs[u]);
        code[u] = lut_code[e];
        tt[u] = lut_t[e];
      }
      uint32_t w = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        uint32_t b = (xs[u] >= tt[u]) ? (code[u] >> 8) & 0xFFu : code[u] & 0xFFu;
        if (code[u] & 0x10000u) b = bin_of(xs[u]);
        w |= b << (8 * u);
      }
      return w;
    };
    const bool vout = ((n & 15) == 0) && ((f0 & 15) == 0);
    if (vout) {
      uint64_t n16 = cnt >> 4;
      for (uint64_t g = tid; g < n16; g += blockDim.x) {
        const float *xs = src + g * 16;
        uint32_t w4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float4 v = reinterpret_cast<const float4 *>(xs)[q];
          w4[q] = bins4(v);
        }
        reinterpret_cast<uint4 *>(out)[g] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
      }
      for (uint64_t i = (n16 << 4) + tid; i < cnt; i += blockDim.x)
        out[i] = (uint8_t)fast_bin(src[i]);
    } else {
      for (uint64_t i = tid; i < cnt; i += blockDim.x) out[i] = (uint8_t)fast_bin(src[i]);
    }
  }
}

// Host-side exact thresholds shared by every DOF of a launch.
float host_first_float(double c) {
  // smallest non-negative float x with RN(x + c) >= 2pi
  int lo = 0, hi = 0x40E00000;  // 7.0f
  auto pred = [&](int b) {
    float x;
    memcpy(&x, &b, 4);
    volatile double a = (double)x + c;
    return a >= kTwoPi;
  };
  if (pred(lo)) return 0.0f;
  while (hi - lo > 1) {
    int mid = lo + (hi - lo) / 2;
    if (pred(mid)) hi = mid; else lo = mid;
  }
  float r;
  memcpy(&r, &hi, 4);
  return r;
}

void host_fit_thresholds(int nfit, double bs, float *t) {
  // t[k] = smallest non-negative float with (int)floor(x / bs) >= k
  t[0] = 0.0f;
  for (int k = 1; k <= nfit; ++k) {
    int lo = 0, hi = 0x40E00000;
    auto pred = [&](int b) {
      float x;
      memcpy(&x, &b, 4);
      volatile double q = ((double)x - 0.0) / bs;
      return (int)floor(q) >= k;
    };
    while (hi - lo > 1) {
      int mid = lo + (hi - lo) / 2;
      if (pred(mid)) hi = mid; else lo = mid;
    }
    memcpy(&t[k], &hi, 4);
  }
}

}  // namespace

int launch_discretize(centre_ctx *ctx, int bat_type, const float *d_data, uint32_t ndof,
                      uint64_t nframes, const uint8_t *schemes, uint32_t nschemes,
                      uint8_t bins_ref, int optimize, uint8_t *d_bins, double *d_ext,
                      bool reset_flag) {
  if (bat_type < 1 || bat_type > 3) return set_error(ctx, CENTRE_E_ARG, "bad BAT type");
  if (nschemes < 1 || nschemes > (uint32_t)kMaxSchemes)
    return set_error(ctx, CENTRE_E_ARG, "nschemes must be 1..16");
  for (uint32_t s = 0; s < nschemes; ++s)
    if (schemes[s] == 0) return set_error(ctx, CENTRE_E_ARG, "zero bins in a scheme");
  if (ndof == 0 || nframes == 0) return CENTRE_OK;
  if (bat_type == 3 && optimize && bins_ref == 0)
    return set_error(ctx, CENTRE_E_ARG, "referencenbins must be > 0");

  DiscParams P;
  memset(&P, 0, sizeof(P));
  P.type = bat_type;
  P.optimize = (bat_type == 3) ? (optimize != 0) : 0;
  P.nschemes = (int)nschemes;
  P.nframes = nframes;
  for (uint32_t s = 0; s < nschemes; ++s) P.schemes[s] = schemes[s];
  // cluster size: enough CTAs for the DOF to fit shared memory
  int csize = 1;
  while (csize < kMaxCluster &&
         ((nframes + csize - 1) / csize) * 4 > kStageBytes)
    csize *= 2;
  uint64_t slice = (nframes + csize - 1) / csize;
  slice = (slice + 15) & ~uint64_t(15);
  P.slice = slice;
  P.staged = (slice * 4 <= kStageBytes) ? 1 : 0;
  {
    // largest float whose double value passes the reference's domain
    float lim = FLT_MAX;
    if (P.type == 2) {
      lim = (float)kPi;
      while ((double)lim > kPi) lim = nextafterf(lim, 0.0f);
    } else if (P.type == 3) {
      lim = (float)kTwoPi;
      while ((double)lim >= kTwoPi) lim = nextafterf(lim, 0.0f);
    }
    P.xmax_ok = lim;
  }
  if (P.type == 3) {
    P.nfit = (3 * (int)bins_ref > kMaxFit) ? kMaxFit : 3 * (int)bins_ref;
    P.fit_bs = ((kTwoPi + kDx) - 0.0) / P.nfit;   // src/Real2Int.cpp:281-284
    P.xpi = host_first_float(kPi);
    if (P.optimize) host_fit_thresholds(P.nfit, P.fit_bs, P.tfit);
  }
  size_t smem = (P.staged ? slice * 4 : 0) + (size_t)nschemes * 2 * 256 * 4;
  CENTRE_CUDA(ctx, cudaFuncSetAttribute(discretize_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
  if (reset_flag) CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));

  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(ndof * csize), 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  {
    KernelTimer kt(ctx, CENTRE_TIMER_DISCRETIZE);
    CENTRE_CUDA(ctx, cudaLaunchKernelEx(&cfg, discretize_kernel, d_data, d_bins, d_ext, P,
                                        ctx->d_flag));
  }
  ctx->launches++;
  return CENTRE_OK;
}

}  // namespace centre
