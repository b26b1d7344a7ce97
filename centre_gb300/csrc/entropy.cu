// entropy.cu -- 1-D/2-D counts and plug-in entropies.
//
// Reference: binData1D / binData2D (src/Estimators.cpp:56-205) and
// entropy1D / entropy2D (:217-651), driven by EntropyCalculator::run1d /
// run2d_xx / run2d_xy (src/EntropyCalculator.cpp:6, :281, :674).
//
// Joint entropy factorisation.  For the ML and MM estimators the reference's
// per-cell sum (src/Estimators.cpp:586-642)
//     S = -A * sum_{c>0} J1 J2 p log p,   p = c / (n A J1 J2)
// equals, term by term,
//     S = log n + log A - (1/n) sum c ln c + (1/n)(L_i + L_j)
// with L_i = sum_b R_b ln J_i(b) over the DOF's own 1-D counts R (the row
// marginal of the joint table is the 1-D histogram of the same frames).  So
// per pair and step only two integers are needed: sum over cells of
// round(c ln c * 2^32) (exact, order independent) and the number of
// non-empty cells (for Miller-Madow).  Both count kernels (shared-memory
// atomics here, tensor-core one-hot in pairs_tc.cu) produce exactly these
// integers, so their entropies are bit-identical.  The Chao-Shen and
// James-Stein estimators need every cell; they take the counts path
// (materialised joint counts + per-cell evaluation, as the reference).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {

// ----------------------------------------------------------------------------
// Fixed-point c ln c table at moment scale s (see clnc_fix)
__global__ void fix_table_kernel(unsigned long long *t, int n, int s) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) t[c] = clnc_fix((unsigned)c, s);
}

// ----------------------------------------------------------------------------
// 1-D: counts per step, cumulative; entropies for every estimator; L sums.
// One CTA per (DOF, scheme).
__global__ void __launch_bounds__(256)
entropy1d_kernel(const uint8_t *__restrict__ bins, const uint8_t *__restrict__ types,
                 const double *__restrict__ ext, const __grid_constant__ EntParams P,
                 double *__restrict__ s1, unsigned long long *__restrict__ freq_out,
                 double *__restrict__ lsum, int *__restrict__ flag) {
  const int dof = blockIdx.x / P.nschemes;
  const int s = blockIdx.x % P.nschemes;
  const int nb = P.schemes[s];
  const uint64_t n = P.nframes, ss = P.step_size;
  const uint8_t *row = bins + ((uint64_t)dof * P.nschemes + s) * n;
  __shared__ unsigned hist[256];
  __shared__ unsigned whist[8 * 256];   // per-warp histograms (256 threads)
  __shared__ unsigned long long cum[256];
  __shared__ double mids[256];
  __shared__ int badrange;
  const int tid = threadIdx.x;
  if (tid == 0) badrange = 0;
  for (int b = tid; b < 256; b += blockDim.x) cum[b] = 0;
  const int type = types[dof];
  const double mn = ext[4 * dof], mx = ext[4 * dof + 1];
  double w = __ddiv_rn(__dsub_rn(mx, mn), (double)nb);
  const double hw = w / 2;
  if (P.kde) w = 1.0;
  const bool hj = (type == 1 || type == 2);
  for (int b = tid; b < nb; b += blockDim.x)
    mids[b] = hj ? __dadd_rn(__dadd_rn(mn, __dmul_rn((double)b, w)), hw) : 0.0;
  // the Jacobian factor of each bin and the log the L sum uses do not change
  // with the step: evaluated once (FP64 transcendentals are the bound here)
  __shared__ double jfs[256], ljs[256];
  __syncthreads();
  if (P.jacobian && hj)
    for (int b = tid; b < nb; b += blockDim.x) {
      jfs[b] = (type == 1) ? pow(mids[b], 2) : sin(mids[b]);
      ljs[b] = log(type == 1 ? mids[b] * mids[b] : sin(mids[b]));
    }
  const int nsum = P.nbins_sum;
  const int off = P.scheme_off[s];
  const uint64_t per = (uint64_t)P.nests * P.nschemes * P.nsteps;

  const int warp = tid >> 5, nwarps = blockDim.x >> 5;
  // four frames per 32-bit load; a row that does not start on a 4-byte
  // boundary takes each word from the two aligned words around it
  const uint32_t rsh = 8u * (uint32_t)(reinterpret_cast<uintptr_t>(row) & 3u);
  const uint32_t *rw = reinterpret_cast<const uint32_t *>(row - (rsh >> 3));
  const uint32_t lim = 0x01010101u * (uint32_t)nb;
  for (int t = 0; t < P.nsteps; ++t) {
    for (int b = tid; b < 8 * 256; b += blockDim.x) whist[b] = 0;
    __syncthreads();
    const uint64_t f0 = (uint64_t)t * ss, f1 = f0 + ss;
    unsigned *wh = whist + warp * 256;
    int bad = 0;
    auto one = [&](uint64_t f) {
      const unsigned v = row[f];
      if (v >= (unsigned)nb) bad = 1;
      else atomicAdd(&wh[v], 1u);
    };
    {
      const uint64_t g0 = (f0 + 3) >> 2, g1 = f1 >> 2;
      for (uint64_t f = f0 + tid; f < min(f1, g0 << 2); f += blockDim.x) one(f);
      for (uint64_t f = max(f0, g1 << 2) + tid; f < f1; f += blockDim.x) one(f);
      for (uint64_t g = g0 + tid; g < g1; g += blockDim.x) {
        const uint32_t w = rsh ? __funnelshift_r(__ldg(rw + g), __ldg(rw + g + 1), rsh) : __ldg(rw + g);
        if (__vcmpgeu4(w, lim)) {
          bad = 1;
          continue;
        }
        atomicAdd(&wh[w & 255u], 1u);
        atomicAdd(&wh[(w >> 8) & 255u], 1u);
        atomicAdd(&wh[(w >> 16) & 255u], 1u);
        atomicAdd(&wh[w >> 24], 1u);
      }
    }
    if (bad) badrange = 1;
    __syncthreads();
    for (int b = tid; b < nb; b += blockDim.x) {
      unsigned h = 0;
      for (int w = 0; w < nwarps; ++w) h += whist[w * 256 + b];
      hist[b] = h;
    }
    __syncthreads();
    for (int b = tid; b < nb; b += blockDim.x) cum[b] += hist[b];
    __syncthreads();
    if (freq_out)
      for (int b = tid; b < nb; b += blockDim.x)
        freq_out[((uint64_t)dof * P.nsteps + t) * nsum + off + b] = cum[b];
    // L sum for the 2-D factorisation (deterministic order, one thread)
    if (tid == 0) {
      double L = 0.0;
      if (P.jacobian && hj)
        for (int b = 0; b < nb; ++b)
          if (cum[b]) L += (double)cum[b] * ljs[b];
      lsum[((uint64_t)dof * P.nschemes + s) * P.nsteps + t] = L;
    }
    // entropies: one warp per estimator
    const int e = tid >> 5, lane = tid & 31;
    if (e < P.nests) {
      const int est = P.ests[e];
      const double nd = (t + 1.0) * (double)ss;
      double acc = 0.0;
      if (est == 0 || est == 1) {
        int blank = 0;
        for (int b = lane; b < nb; b += 32) {
          double fq = (double)cum[b] / nd;
          double pd = fq / w;
          if (pd > 0.0) {
            if (P.jacobian && hj) {
              const double jf = jfs[b];
              pd = pd / jf;
              acc += jf * pd * log(pd);
            } else {
              acc += pd * log(pd);
            }
          }
          blank += (cum[b] == 0);
        }
        for (int o = 16; o; o >>= 1) {
          acc += __shfl_xor_sync(0xffffffffu, acc, o);
          blank += __shfl_xor_sync(0xffffffffu, blank, o);
        }
        acc *= -w;
        if (est == 1) acc += ((nb - blank) - 1) / (2.0 * nd);
      } else if (est == 2) {  // Chao-Shen (src/Estimators.cpp:285-345)
        int single = 0;
        for (int b = lane; b < nb; b += 32) single += (cum[b] == 1);
        for (int o = 16; o; o >>= 1) single += __shfl_xor_sync(0xffffffffu, single, o);
        const double g = 1 - ((uint8_t)single / nd);
        for (int b = lane; b < nb; b += 32) {
          double fq = g * ((double)cum[b] / nd);
          double pd = fq / w;
          if (pd > 0.0) {
            double den = 1 - pow((1 - fq), nd);
            if (P.jacobian && hj) {
              const double jf = jfs[b];
              pd = pd / jf;
              acc += jf * pd * log(pd) / den;
            } else {
              acc += pd * log(pd) / den;
            }
          }
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        acc *= -w;
      } else {  // James-Stein (src/Estimators.cpp:298-316)
        const double tk = 1.0 / (double)nb;
        double s2 = 0, t2 = 0;
        for (int b = lane; b < nb; b += 32) {
          double fq = (double)cum[b] / nd;
          s2 += fq * fq;
          t2 += (tk - fq) * (tk - fq);
        }
        for (int o = 16; o; o >>= 1) {
          s2 += __shfl_xor_sync(0xffffffffu, s2, o);
          t2 += __shfl_xor_sync(0xffffffffu, t2, o);
        }
        const double lam = (1 - s2) / ((nd - 1) * t2);
        for (int b = lane; b < nb; b += 32) {
          double fq = (lam * tk) + ((1 - lam) * ((double)cum[b] / nd));
          double pd = fq / w;
          if (pd > 0.0) {
            if (P.jacobian && hj) {
              const double jf = jfs[b];
              pd = pd / jf;
              acc += jf * pd * log(pd);
            } else {
              acc += pd * log(pd);
            }
          }
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        acc *= -w;
      }
      if (lane == 0) s1[(uint64_t)dof * per + ((uint64_t)e * P.nschemes + s) * P.nsteps + t] = acc;
    }
    __syncthreads();
  }
  if (badrange && tid == 0) atomicOr(flag, kFlagBinRange);
}

// ----------------------------------------------------------------------------
// Shared-memory atomic joint histograms.
//
// A CTA owns a tile of R row DOFs x C column DOFs; each of the R*C pairs has
// an nb*nb uint32 histogram in shared memory.  Threads walk the frames of a
// step four at a time: one 32-bit load per DOF gives four bins, each frame's
// R row offsets and C column offsets are formed once, and every increment is
// one add plus one red.shared.add (about three instructions per increment).
// Bin ranges are checked four at a time with one vector compare per word.
// At every step boundary the CTA reduces each histogram to the pair's exact
// moments (sum c ln c as 128-bit fixed point, non-empty cells) or, in counts
// mode, writes the cumulative histograms out.
__device__ __forceinline__ uint64_t tri_index(uint64_t i, uint64_t j, uint64_t n) {
  // row-major index of pair (i, j), i < j, among all pairs of n items
  return i * n - i * (i + 1) / 2 + (j - i - 1);
}

constexpr int kTabF = 2560;     // fixed-point c ln c entries kept in shared memory
constexpr int kRedBatch = 4;    // cells per lane per batch in the moment reduction
#ifndef CENTRE_HIST_MIN_BLOCKS
#define CENTRE_HIST_MIN_BLOCKS 2
#endif
// Resident CTAs per SM the single-trajectory histogram kernel is compiled
// for (its batched moment reduction needs up to 64 registers).  The batch
// kernel keeps the one-cell-at-a-time reduction and fewer registers: its
// autotuned tiles favour more resident CTAs.
constexpr int kHistMinBlocks = CENTRE_HIST_MIN_BLOCKS;
#ifndef CENTRE_HIST_INTERLEAVE
#define CENTRE_HIST_INTERLEAVE 1
#endif
// 4 x 4 tiles of the single-trajectory kernel use interleaved histograms
constexpr bool kHistInterleave = CENTRE_HIST_INTERLEAVE != 0;
#ifndef CENTRE_HIST_PREFETCH
#define CENTRE_HIST_PREFETCH 1
#endif
constexpr bool kHistPrefetch = CENTRE_HIST_PREFETCH != 0;

__device__ __forceinline__ void red_shared_inc(uint32_t addr) {
  asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(addr) : "memory");
}

// F(c) beyond the shared table: the global table, or (counts of 2^16 and
// more) the same expression the table was filled with.
__device__ __forceinline__ unsigned long long fix_far(const unsigned long long *__restrict__ gfix,
                                                      unsigned c, int s) {
  return (c < (unsigned)kTabGlobal) ? __ldg(gfix + c) : clnc_fix(c, s);
}

// One R x C tile of pairs of one trajectory.
struct HistJob {
  const uint8_t *bins;
  uint64_t nframes;
  uint64_t step_size;
  int nsteps;
  int nschemes;
  int scheme;
  int nb;
  int fix_scale;
  unsigned long long *sclnc;
  unsigned *nnz;
  unsigned *counts;
};

// Fill rows/cols/outputs of the all-pairs tile `id` of an upper-triangular
// grid of R x R tiles over ndof DOFs (thread 0).  Tiles (bi, bj), bi <= bj,
// are numbered by column stripe of `stripe` tile columns [c0, c1), then by
// row bi, then by column bj, so that the CTAs running at one time read the
// rows of one stripe and its columns: the stripe's columns (sized to stay in
// L2) are read from DRAM once, instead of every row block streaming all its
// columns through L2.  A stripe of ntile columns is the row-major order.
template <int R>
__device__ void decode_all_pairs_tile(uint64_t id, uint64_t ntile, uint64_t stripe, uint32_t ndof,
                                      uint32_t *rows, uint32_t *cols, uint64_t *outs) {
  uint64_t c0 = 0, w = 0;
  while (true) {
    w = min(ntile, c0 + stripe) - c0;
    const uint64_t cnt = c0 * w + w * (w + 1) / 2;   // full rows above c0, then the triangle
    if (id < cnt) break;
    id -= cnt;
    c0 += w;
  }
  uint64_t bi, bj;
  if (id < c0 * w) {
    bi = id / w;
    bj = c0 + id % w;
  } else {
    id -= c0 * w;
    uint64_t r = 0;   // triangle row r (DOF block c0 + r) holds w - r tiles
    while (id >= w - r) {
      id -= w - r;
      ++r;
    }
    bi = c0 + r;
    bj = bi + id;
  }
  for (int r = 0; r < R; ++r) {
    const uint64_t i = bi * R + r;
    rows[r] = (uint32_t)(i < ndof ? i : bi * R);
  }
  for (int c = 0; c < R; ++c) {
    const uint64_t j = bj * R + c;
    cols[c] = (uint32_t)(j < ndof ? j : bj * R);
  }
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < R; ++c) {
      const uint64_t i = bi * R + r, j = bj * R + c;
      outs[r * R + c] = (i < j && j < ndof) ? tri_index(i, j, ndof) : ~0ull;
    }
}

// Count all frames of one tile and emit its moments (or counts) per step.
// `hist` is zeroed on entry and left zeroed.  Returns non-zero if a bin was
// out of range.  All threads of the CTA call it.
//
// kIlv (interleaved histograms, NP = R*C dividing 32): cell k of pair P is
// word k*NP + P instead of P*nb*nb + k, and lane l counts the pair rotated
// by its slot s = l mod NP (row (r + s/C) mod R, column (c + s%C) mod C at
// unrolled step (r, c)), so the NP lanes of a slot group update NP different
// pairs: for NP = 16 a warp's increments fall on bank P + 16 (k mod 2), at
// most two per bank, where 32 lanes updating one pair at random cells load
// the busiest bank ~3.3 times (shared-memory wavefronts bound this kernel).
// The loaded words are rotated in registers, so the loads stay coalesced.
// The moment reduction then sweeps the whole tile with the CTA: a lane's
// words all belong to pair l mod NP (512 threads: 16 warps combine through
// shared memory).
// With kIlv the next 4-frame group's words are also loaded before the
// current group's increments (kHistPrefetch).
// `tabf` holds F(c) (the fixed-point c ln c of clnc_fix) for c < kTabF in
// shared memory, `gfix` for c < 2^16 in global memory.
template <int R, int C, bool kCounts, bool kBatchedRed, bool kIlv = false, bool kNnz = true,
          bool kAlign = true>
__device__ int hist_tile(const HistJob &J, const uint32_t *rows_s, const uint32_t *cols_s,
                         const uint64_t *out_s, unsigned *hist,
                         const unsigned long long *tabf,
                         const unsigned long long *__restrict__ gfix) {
  constexpr int NP = R * C;
  static_assert(!kIlv || (32 % NP == 0 && NP > 1), "interleaving needs NP | 32");
  static_assert(!kIlv || kBatchedRed, "the interleaved reduction takes cells in batches");
  constexpr bool kPrefetch = kIlv && kHistPrefetch;
  const int tid = threadIdx.x;
  const int nb = J.nb, nb2 = nb * nb;
  const uint64_t n = J.nframes;
  // lane slot of the interleaved layout: row and column rotation
  const int slot = kIlv ? (int)(threadIdx.x & 31) % NP : 0;
  const int rrot = slot / C, crot = slot % C;
  // byte strides of one row bin / one column bin in the histogram words
  const uint32_t rstride = kIlv ? 4u * (uint32_t)nb * NP : 4u * (uint32_t)nb;
  const uint32_t cstride = kIlv ? 4u * NP : 4u;
  const uint8_t *bins = J.bins;
  const uint32_t hist_s = (uint32_t)__cvta_generic_to_shared(hist);
  // DOF rows as 32-bit word offsets from the aligned word at or before the
  // bins pointer.  kAlign (frame count and bins pointer multiples of 4):
  // every row starts on a word.  Otherwise a row that does not start on a
  // 4-byte boundary is read four frames at a time from the two aligned words
  // around them (a funnel shift); the second word holds the group's last
  // byte, so no load leaves the word of a valid byte.
  const uint32_t mis = kAlign ? 0u : (uint32_t)(reinterpret_cast<uintptr_t>(bins) & 3u);
  const uint32_t *bw = reinterpret_cast<const uint32_t *>(bins - mis);
  const uint32_t nb4 = 4u * (uint32_t)nb;
  // Bin range check four bytes at a time.  Up to 128 bins a byte x is out
  // of range (x >= nb) exactly when bit 7 of x | (x + 128 - nb) is set: below
  // 128, x + 128 - nb stays below 256 and reaches 128 exactly when x >= nb;
  // from 128 on, x itself has bit 7.  A carry out of an out-of-range byte can
  // only flag its neighbour, and the word is rejected either way.  Above 128
  // bins the vector compare does it.
  const bool small_nb = nb <= 128;
  const uint32_t range_add = small_nb ? 0x01010101u * (uint32_t)(128 - nb) : 0u;
  const uint32_t lim = 0x01010101u * (uint32_t)nb;
  int bad = 0;

  // row/column word offsets and histogram addresses; with the batched
  // reduction they are recomputed every step so that none of them is live
  // across the reduction, which then has the registers to itself
  uint32_t rw0[R], cw0[C];
  uint32_t rsh[R], csh[C];   // bit shift of each row start within its word
  uint32_t rconst[R], cconst[C];
  auto setup = [&]() {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const uint64_t o = mis + ((uint64_t)rows_s[r] * J.nschemes + J.scheme) * n;
      rw0[r] = (uint32_t)(o >> 2);
      rsh[r] = 8u * (uint32_t)(o & 3u);
      rconst[r] = kIlv ? hist_s + 4u * (uint32_t)(((r + rrot) % R) * C)
                       : hist_s + 4u * (uint32_t)(r * C * nb2);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const uint64_t o = mis + ((uint64_t)cols_s[c] * J.nschemes + J.scheme) * n;
      cw0[c] = (uint32_t)(o >> 2);
      csh[c] = 8u * (uint32_t)(o & 3u);
      cconst[c] = kIlv ? 4u * (uint32_t)((c + crot) % C) : 4u * (uint32_t)(c * nb2);
    }
  };
  // x rotated by k places (y[i] = x[(i + k) mod N]) with selects: no
  // dynamically indexed registers (four entries: by 1, then by 2)
  auto rotate = [](auto &x, int k) {
    constexpr int N = sizeof(x) / sizeof(x[0]);
    if constexpr (N == 4) {
      uint32_t y[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) y[i] = (k & 1) ? x[(i + 1) & 3] : x[i];
#pragma unroll
      for (int i = 0; i < 4; ++i) x[i] = (k & 2) ? y[(i + 2) & 3] : y[i];
    } else {
      uint32_t y[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        uint32_t v = x[i];
#pragma unroll
        for (int j = 1; j < N; ++j) v = (k == j) ? x[(i + j) % N] : v;
        y[i] = v;
      }
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = y[i];
    }
  };
  if (!kBatchedRed) setup();
  for (int t = 0; t < J.nsteps; ++t) {
    const uint64_t f0 = (uint64_t)t * J.step_size, f1 = f0 + J.step_size;
    if (kBatchedRed) setup();
    auto one_frame = [&](uint64_t f) {
      uint32_t a[R], b[C];
      bool ok = true;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        a[r] = bins[((uint64_t)rows_s[r] * J.nschemes + J.scheme) * n + f];
        ok &= a[r] < (uint32_t)nb;
      }
#pragma unroll
      for (int c = 0; c < C; ++c) {
        b[c] = bins[((uint64_t)cols_s[c] * J.nschemes + J.scheme) * n + f];
        ok &= b[c] < (uint32_t)nb;
      }
      if (!ok) {
        bad = 1;
        return;
      }
      if (kIlv) {
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
          for (int c = 0; c < C; ++c)
            red_shared_inc(hist_s + 4u * (uint32_t)(r * C + c) + a[r] * rstride + b[c] * cstride);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
          for (int c = 0; c < C; ++c) red_shared_inc(rconst[r] + a[r] * nb4 + cconst[c] + 4u * b[c]);
      }
    };
    {
      const uint64_t g0 = (f0 + 3) >> 2, g1 = f1 >> 2;   // whole 4-frame groups
      for (uint64_t f = f0 + tid; f < min(f1, g0 << 2); f += blockDim.x) one_frame(f);
      for (uint64_t f = max(f0, g1 << 2) + tid; f < f1; f += blockDim.x) one_frame(f);
      // kPrefetch: the next group's words are loaded before this group's
      // increments (the red.shared asm keeps later loads behind it)
      auto load_group = [&](uint64_t g, uint32_t (&x)[R], uint32_t (&y)[C]) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const uint32_t *w = bw + rw0[r] + (uint32_t)g;
          x[r] = (!kAlign && rsh[r]) ? __funnelshift_r(__ldg(w), __ldg(w + 1), rsh[r]) : __ldg(w);
        }
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const uint32_t *w = bw + cw0[c] + (uint32_t)g;
          y[c] = (!kAlign && csh[c]) ? __funnelshift_r(__ldg(w), __ldg(w + 1), csh[c]) : __ldg(w);
        }
      };
      // one 4-frame group: range check, rotation, 4 x R x C increments
      auto count_group = [&](uint32_t (&rw)[R], uint32_t (&cw)[C]) {
        uint32_t v = 0;
        if (small_nb) {
#pragma unroll
          for (int r = 0; r < R; ++r) v |= rw[r] | (rw[r] + range_add);
#pragma unroll
          for (int c = 0; c < C; ++c) v |= cw[c] | (cw[c] + range_add);
          v &= 0x80808080u;
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) v |= __vcmpgeu4(rw[r], lim);
#pragma unroll
          for (int c = 0; c < C; ++c) v |= __vcmpgeu4(cw[c], lim);
        }
        if (v) {
          bad = 1;
          return;
        }
        if (kIlv) {
          rotate(rw, rrot);
          rotate(cw, crot);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t ro[R], co[C];
#pragma unroll
          for (int r = 0; r < R; ++r) ro[r] = rconst[r] + ((rw[r] >> (8 * q)) & 255u) * rstride;
#pragma unroll
          for (int c = 0; c < C; ++c) co[c] = cconst[c] + ((cw[c] >> (8 * q)) & 255u) * cstride;
#pragma unroll
          for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < C; ++c) red_shared_inc(ro[r] + co[c]);
        }
      };
      if (kPrefetch) {
        // two register sets in turn: the next group's words load while the
        // current group counts, without copies between iterations
        uint32_t ra[R], ca[C], rb[R], cb[C];
        const uint32_t bd = blockDim.x, ge = (uint32_t)g1;
        uint32_t g = (uint32_t)(g0 + tid);
        if (g < ge) load_group(g, ra, ca);
        while (g < ge) {
          if (g + bd < ge) load_group(g + bd, rb, cb);
          count_group(ra, ca);
          g += bd;
          if (g >= ge) break;
          if (g + bd < ge) load_group(g + bd, ra, ca);
          count_group(rb, cb);
          g += bd;
        }
      } else {
        for (uint64_t g = g0 + tid; g < g1; g += blockDim.x) {
          uint32_t rw[R], cw[C];
          load_group(g, rw, cw);
          count_group(rw, cw);
        }
      }
    }
    __syncthreads();
    if (kCounts) {
      for (int q = 0; q < NP; ++q) {
        const uint64_t o = out_s[q];
        if (o == ~0ull) continue;
        unsigned *dst = J.counts + (o * J.nsteps + t) * (uint64_t)nb2;
        for (int i = tid; i < nb2; i += blockDim.x)
          dst[i] = kIlv ? hist[i * NP + q] : hist[q * nb2 + i];
      }
    } else if constexpr (kIlv) {
      // The CTA sweeps all NP * nb2 words, four at a time: quad q holds cell
      // q / 4 of pairs 4 (q mod 4) .. + 3, and a thread's quads all have the
      // same q mod 4 (the stride is a multiple of 4), so it keeps one
      // accumulator per pair of its group.  Sums are exact (integer), so the
      // order does not matter.  kNnz: count the non-empty cells (Miller-Madow).
      static_assert(NP == 16, "the quad sweep assumes 16 interleaved pairs");
      constexpr int kW = 16;   // warps of the 512-thread CTA
      constexpr int kQ = 2;    // quads per lane per iteration
      __shared__ unsigned long long wacc_s[kW][NP];
      __shared__ unsigned wnz_s[kW][NP];
      const int warp = tid >> 5, lane = tid & 31;
      const int nq = NP * nb2 / 4, stride = (int)blockDim.x;
      const uint4 *h4 = reinterpret_cast<const uint4 *>(hist);
      unsigned long long acc[4] = {0ull, 0ull, 0ull, 0ull};
      unsigned cz[4] = {0u, 0u, 0u, 0u};
      // warp-uniform trip count (the warp vote below needs every lane)
      for (int q0 = warp * 32; q0 < nq; q0 += stride * kQ) {
        unsigned c[kQ][4];
        unsigned long long v[kQ][4];
        bool big = false;
#pragma unroll
        for (int u = 0; u < kQ; ++u) {
          const int q = q0 + u * stride + lane;
          const uint4 w = (q < nq) ? h4[q] : make_uint4(0u, 0u, 0u, 0u);
          c[u][0] = w.x;
          c[u][1] = w.y;
          c[u][2] = w.z;
          c[u][3] = w.w;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            big |= c[u][i] >= (unsigned)kTabF;
            v[u][i] = tabf[min(c[u][i], (unsigned)kTabF - 1u)];
          }
        }
        if (__any_sync(0xffffffffu, big)) {
#pragma unroll
          for (int u = 0; u < kQ; ++u)
#pragma unroll
            for (int i = 0; i < 4; ++i)
              if (c[u][i] >= (unsigned)kTabF) v[u][i] = fix_far(gfix, c[u][i], J.fix_scale);
        }
#pragma unroll
        for (int u = 0; u < kQ; ++u)
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            acc[i] += v[u][i];
            if (kNnz) cz[i] += (c[u][i] != 0);
          }
      }
      // lanes l, l + 4, ... hold the same four pairs
#pragma unroll
      for (int off = 4; off < 32; off <<= 1)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
          if (kNnz) cz[i] += __shfl_xor_sync(0xffffffffu, cz[i], off);
        }
      if (lane < 4) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          wacc_s[warp][4 * lane + i] = acc[i];
          wnz_s[warp][4 * lane + i] = cz[i];
        }
      }
      __syncthreads();
      if (tid < NP) {
        const uint64_t o = out_s[tid];
        if (o != ~0ull) {
          unsigned long long sum = 0ull;
          unsigned z = 0;
          for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            sum += wacc_s[w][tid];
            z += wnz_s[w][tid];
          }
          J.sclnc[o * J.nsteps + t] = sum;
          if (kNnz) J.nnz[o * J.nsteps + t] = z;
        }
      }
    } else {
      // one warp per pair: the moment and the non-empty cells
      const int warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
      for (int q = warp; q < NP; q += nwarps) {
        const uint64_t o = out_s[q];
        if (o == ~0ull) continue;
        unsigned long long acc = 0ull;
        unsigned cz = 0;
        const unsigned *h = hist + q * nb2;
        if (kBatchedRed) {
          for (int i0 = 0; i0 < nb2; i0 += 32 * kRedBatch) {
            // kRedBatch cells per lane, table loads issued together; counts
            // beyond the shared table (common at few bins) from the global one
            unsigned c[kRedBatch];
            unsigned long long v[kRedBatch];
            bool big = false;
#pragma unroll
            for (int u = 0; u < kRedBatch; ++u) {
              const int i = i0 + 32 * u + lane;
              c[u] = (i < nb2) ? h[i] : 0u;
              big |= c[u] >= (unsigned)kTabF;
              v[u] = tabf[min(c[u], (unsigned)kTabF - 1u)];
            }
            if (__any_sync(0xffffffffu, big)) {
#pragma unroll
              for (int u = 0; u < kRedBatch; ++u)
                if (c[u] >= (unsigned)kTabF) v[u] = fix_far(gfix, c[u], J.fix_scale);
            }
#pragma unroll
            for (int u = 0; u < kRedBatch; ++u) {
              acc += v[u];
              cz += (c[u] != 0);
            }
          }
        } else {
          // one cell at a time (fewer registers: more resident CTAs)
          for (int i = lane; i < nb2; i += 32) {
            const unsigned c = h[i];
            acc += (c < (unsigned)kTabF) ? tabf[c] : fix_far(gfix, c, J.fix_scale);
            cz += (c != 0);
          }
        }
        for (int off = 16; off; off >>= 1) {
          acc += __shfl_xor_sync(0xffffffffu, acc, off);
          cz += __shfl_xor_sync(0xffffffffu, cz, off);
        }
        if (lane == 0) {
          J.sclnc[o * J.nsteps + t] = acc;
          J.nnz[o * J.nsteps + t] = cz;
        }
      }
    }
    __syncthreads();
  }
  // leave the histograms zeroed for the next tile of a persistent CTA
  for (int i = tid; i < NP * nb2; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  return bad;
}

template <int R, int C, bool kCounts, int kMinBlocks = kHistMinBlocks, bool kNnz = true>
__global__ void __launch_bounds__(512, kMinBlocks)
pairs_hist_kernel(const uint8_t *__restrict__ bins, const PairTask *__restrict__ tasks,
                  const __grid_constant__ PairParams P,
                  const unsigned long long *__restrict__ gfix,
                  unsigned long long *__restrict__ sclnc, unsigned *__restrict__ nnz,
                  unsigned *__restrict__ counts, int *__restrict__ flag) {
  constexpr int NP = R * C;
  extern __shared__ __align__(16) unsigned char dyn[];
  const int nb2 = P.nb * P.nb;
  unsigned *hist = reinterpret_cast<unsigned *>(dyn);
  unsigned long long *tabf =
      reinterpret_cast<unsigned long long *>(dyn + (((size_t)NP * nb2 * 4 + 15) & ~size_t(15)));
  __shared__ uint32_t rows_s[R], cols_s[C];
  __shared__ uint64_t out_s[NP];
  const int tid = threadIdx.x;
  if (tid == 0) {
    if (P.all_pairs) {
      decode_all_pairs_tile<R>(blockIdx.x, P.ntile, P.stripe, P.ndof, rows_s, cols_s, out_s);
    } else {
      const PairTask &tk = tasks[blockIdx.x];
      for (int r = 0; r < R; ++r) rows_s[r] = tk.rows[r < tk.nr ? r : 0];
      for (int c = 0; c < C; ++c) cols_s[c] = tk.cols[c < tk.nc ? c : 0];
      for (int r = 0; r < R; ++r)
        for (int c = 0; c < C; ++c)
          out_s[r * C + c] = (r < tk.nr && c < tk.nc) ? tk.out[r * tk.nc + c] : ~0ull;
    }
  }
  if (!kCounts)   // the counts mode writes counts and reads no table
    for (int i = tid; i < kTabF; i += blockDim.x) tabf[i] = __ldg(gfix + i);
  for (int i = tid; i < NP * nb2; i += blockDim.x) hist[i] = 0;
  __syncthreads();
  HistJob J;
  J.bins = bins;
  J.nframes = P.nframes;
  J.step_size = P.step_size;
  J.nsteps = P.nsteps;
  J.nschemes = P.nschemes;
  J.scheme = P.scheme;
  J.nb = P.nb;
  J.fix_scale = P.fix_scale;
  J.sclnc = sclnc;
  J.nnz = nnz;
  J.counts = counts;
  constexpr bool kIlv = kHistInterleave && R == 4 && C == 4;
  // rows on word boundaries take the plain 32-bit loads
  const bool aligned = ((P.nframes & 3) == 0) && ((reinterpret_cast<uintptr_t>(bins) & 3) == 0);
  const int bad =
      aligned ? hist_tile<R, C, kCounts, true, kIlv, kNnz, true>(J, rows_s, cols_s, out_s, hist, tabf, gfix)
              : hist_tile<R, C, kCounts, true, kIlv, kNnz, false>(J, rows_s, cols_s, out_s, hist, tabf, gfix);
  if (bad) atomicOr(flag, kFlagBinRange);   // any thread may have seen it
}

// Persistent all-pairs histogram counts over several trajectories: the work
// list is every (trajectory, tile) pair; CTAs stride through it.
template <int R>
__global__ void __launch_bounds__(512)
pairs_hist_batch_kernel(const BatchSys *__restrict__ sys, int nsys, uint64_t nitems,
                        const __grid_constant__ BatchCommon B,
                        const unsigned long long *__restrict__ gfix, int *__restrict__ flag) {
  constexpr int NP = R * R;
  extern __shared__ __align__(16) unsigned char dyn[];
  const int nb2 = B.nb * B.nb;
  unsigned *hist = reinterpret_cast<unsigned *>(dyn);
  unsigned long long *tabf =
      reinterpret_cast<unsigned long long *>(dyn + (((size_t)NP * nb2 * 4 + 15) & ~size_t(15)));
  __shared__ uint32_t rows_s[R], cols_s[R];
  __shared__ uint64_t out_s[NP];
  __shared__ int sys_s;
  const int tid = threadIdx.x;
  for (int i = tid; i < kTabF; i += blockDim.x) tabf[i] = __ldg(gfix + i);
  for (int i = tid; i < NP * nb2; i += blockDim.x) hist[i] = 0;
  int bad = 0;
  for (uint64_t item = blockIdx.x + B.item0; item < nitems; item += gridDim.x) {
    __syncthreads();
    if (tid == 0) {
      int lo = 0, hi = nsys - 1;   // last trajectory whose first item <= item
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sys[mid].item_begin <= item) lo = mid; else hi = mid - 1;
      }
      const int s = lo;
      sys_s = s;
      decode_all_pairs_tile<R>(item - sys[s].item_begin, sys[s].ntile, sys[s].stripe, sys[s].ndof,
                               rows_s,
                               cols_s, out_s);
    }
    __syncthreads();
    const BatchSys &S = sys[sys_s];
    HistJob J;
    J.bins = S.bins;
    J.nframes = S.nframes;
    J.step_size = S.step_size;
    J.nsteps = B.nsteps;
    J.nschemes = B.nschemes;
    J.scheme = B.scheme;
    J.nb = B.nb;
    J.fix_scale = B.fix_scale;
    J.sclnc = S.sclnc;
    J.nnz = S.nnz;
    J.counts = nullptr;
    // 4 x 4 tiles: interleaved histograms and the batched quad-sweep
    // reduction, as in the single-trajectory kernel
    constexpr bool kIlvB = kHistInterleave && R == 4;
    const bool aligned = ((J.nframes & 3) == 0) && ((reinterpret_cast<uintptr_t>(J.bins) & 3) == 0);
    bad |= aligned ? hist_tile<R, R, false, kIlvB, kIlvB, true, true>(J, rows_s, cols_s, out_s, hist, tabf, gfix)
                   : hist_tile<R, R, false, kIlvB, kIlvB, true, false>(J, rows_s, cols_s, out_s, hist, tabf, gfix);
  }
  if (bad) atomicOr(flag, kFlagBinRange);
}

// ----------------------------------------------------------------------------
// Joint counts for bin counts whose histograms do not fit shared memory
// (more than 217 bins): each CTA owns one nb x nb histogram in global
// memory (L2-resident) and counts a pair's frames into it with global
// atomics, one pair at a time.  At every step it emits the pair's moments
// (or copies the cumulative counts), then clears the histogram.  Reads of
// the histogram bypass L1 (the atomics update L2).
__global__ void __launch_bounds__(512)
pairs_global_kernel(const uint8_t *__restrict__ bins, const __grid_constant__ PairParams P,
                    const uint32_t *__restrict__ pairs, uint64_t p0, uint64_t np,
                    const unsigned long long *__restrict__ gfix,
                    unsigned long long *__restrict__ sclnc, unsigned *__restrict__ nnz,
                    unsigned *__restrict__ counts, unsigned *__restrict__ hist_all,
                    int *__restrict__ flag) {
  const int nb = P.nb, nb2 = nb * nb;
  unsigned *h = hist_all + (uint64_t)blockIdx.x * nb2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  __shared__ unsigned long long wacc[32];
  __shared__ unsigned wnz[32];
  int bad = 0;
  for (uint64_t q = blockIdx.x; q < np; q += gridDim.x) {
    const uint64_t gp = p0 + q;
    uint32_t i, j;
    if (pairs) {
      i = pairs[2 * gp];
      j = pairs[2 * gp + 1];
    } else {
      tri_pair(gp, P.ndof, i, j);
    }
    const uint8_t *bi = bins + ((uint64_t)i * P.nschemes + P.scheme) * P.nframes;
    const uint8_t *bj = bins + ((uint64_t)j * P.nschemes + P.scheme) * P.nframes;
    for (int t = 0; t < P.nsteps; ++t) {
      const uint64_t f0 = (uint64_t)t * P.step_size, f1 = f0 + P.step_size;
      for (uint64_t f = f0 + tid; f < f1; f += blockDim.x) {
        const unsigned a = bi[f], b = bj[f];
        if (a >= (unsigned)nb || b >= (unsigned)nb) {
          bad = 1;
          continue;
        }
        atomicAdd(&h[a * nb + b], 1u);
      }
      __syncthreads();
      if (counts) {
        unsigned *dst = counts + (q * P.nsteps + t) * (uint64_t)nb2;
        for (int c = tid; c < nb2; c += blockDim.x) dst[c] = __ldcg(h + c);
      } else {
        unsigned long long acc = 0ull;
        unsigned cz = 0;
        for (int c = tid; c < nb2; c += blockDim.x) {
          const unsigned v = __ldcg(h + c);
          acc += fix_far(gfix, v, P.fix_scale);
          cz += (v != 0);
        }
        for (int off = 16; off; off >>= 1) {
          acc += __shfl_xor_sync(0xffffffffu, acc, off);
          cz += __shfl_xor_sync(0xffffffffu, cz, off);
        }
        if (lane == 0) {
          wacc[warp] = acc;
          wnz[warp] = cz;
        }
        __syncthreads();
        if (tid == 0) {
          unsigned long long tot = wacc[0];
          unsigned z = wnz[0];
          for (int w = 1; w < nwarps; ++w) {
            tot += wacc[w];
            z += wnz[w];
          }
          sclnc[gp * P.nsteps + t] = tot;
          nnz[gp * P.nsteps + t] = z;
        }
      }
      __syncthreads();
    }
    for (int c = tid; c < nb2; c += blockDim.x) h[c] = 0u;
    __threadfence_block();
    __syncthreads();
  }
  if (bad) atomicOr(flag, kFlagBinRange);
}

int launch_pairs_global(centre_ctx *ctx, const PairParams &P, const uint32_t *d_pairs,
                        uint64_t p0, uint64_t np, const unsigned long long *d_fix,
                        unsigned long long *d_sclnc, unsigned *d_nnz, unsigned *d_counts) {
  if (np == 0) return CENTRE_OK;
  const uint64_t grid = std::min<uint64_t>(np, (uint64_t)ctx->sm_count * 4);
  int st = CENTRE_OK;
  unsigned *d_hist = (unsigned *)scratch(ctx, kSlotAux3,
                                         sizeof(unsigned) * grid * (uint64_t)P.nb * P.nb, &st);
  if (!d_hist) return st;
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_hist, 0, sizeof(unsigned) * grid * (uint64_t)P.nb * P.nb,
                                   ctx->stream));
  KernelTimer kt(ctx, CENTRE_TIMER_PAIRS);
  pairs_global_kernel<<<(unsigned)grid, 512, 0, ctx->stream>>>(P.bins, P, d_pairs, p0, np, d_fix,
                                                             d_sclnc, d_nnz, d_counts, d_hist,
                                                             ctx->d_flag);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

// ----------------------------------------------------------------------------
// S2 from the integer moments (ML, MM), every step of one scheme.
__global__ void finalize2d_kernel(const uint32_t *__restrict__ pairs, int all_pairs,
                                  uint32_t ndof, const double *__restrict__ logw,
                                  const double *__restrict__ lsum,
                                  const unsigned long long *__restrict__ sclnc,
                                  const unsigned *__restrict__ nnz,
                                  const __grid_constant__ EntParams P, int scheme,
                                  uint64_t npairs, double *__restrict__ s2) {
  // One thread per pair over all its steps: the pair is decoded once, and
  // the per-step 1/n (the only divisions, FP64 being scarce here) and log n
  // are formed once per block.
  __shared__ double inv_n[256], log_n[256];
  for (int t = threadIdx.x; t < P.nsteps; t += blockDim.x) {
    inv_n[t] = 1.0 / ((t + 1.0) * (double)P.step_size);
    log_n[t] = logw[(uint64_t)ndof * P.nschemes + t];
  }
  __syncthreads();
  const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  uint32_t i, j;
  if (all_pairs) {
    tri_pair(p, ndof, i, j);
  } else {
    i = pairs[2 * p];
    j = pairs[2 * p + 1];
  }
  // log(n A) = log n + log w_i + log w_j (per-step and per-DOF logs hoisted)
  const double lw = logw[(uint64_t)i * P.nschemes + scheme] + logw[(uint64_t)j * P.nschemes + scheme];
  const double *li = lsum + ((uint64_t)i * P.nschemes + scheme) * P.nsteps;
  const double *lj = lsum + ((uint64_t)j * P.nschemes + scheme) * P.nsteps;
  const uint64_t per = (uint64_t)P.nests * P.nschemes * P.nsteps;
  for (int t = 0; t < P.nsteps; ++t) {
    const uint64_t idx = p * P.nsteps + t;
    const double X = (double)sclnc[idx] * P.fix_inv;
    const double S = log_n[t] + lw + (li[t] + lj[t] - X) * inv_n[t];
    for (int e = 0; e < P.nests; ++e) {
      double v = S;
      if (P.ests[e] == 1) v += ((double)nnz[idx] - 1.0) * (0.5 * inv_n[t]);
      s2[p * per + ((uint64_t)e * P.nschemes + scheme) * P.nsteps + t] = v;
    }
  }
}

// log of each DOF's bin width per scheme (width 1 in KDE mode) followed by
// log of the frame count of each step: the per-pair log(n A) is their sum.
__global__ void logw_kernel(const double *__restrict__ ext, uint32_t ndof,
                            const __grid_constant__ EntParams P, double *__restrict__ logw) {
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t nw = (uint64_t)ndof * P.nschemes;
  if (idx < nw) {
    const uint64_t d = idx / P.nschemes;
    const int s = (int)(idx % P.nschemes);
    const double w = __ddiv_rn(__dsub_rn(ext[4 * d + 1], ext[4 * d]), (double)P.schemes[s]);
    logw[idx] = P.kde ? 0.0 : log(w);
  } else if (idx < nw + (uint64_t)P.nsteps) {
    const int t = (int)(idx - nw);
    logw[idx] = log((t + 1.0) * (double)P.step_size);
  }
}

// ----------------------------------------------------------------------------
// Per-cell entropy2D on materialised counts (every estimator), one CTA per
// pair.  Mirrors src/Estimators.cpp:455-645 including the Chao-Shen branch's
// use of the row bin centre for the second DOF's Jacobian (:555-566).
__global__ void __launch_bounds__(256)
entropy2d_counts_kernel(const uint32_t *__restrict__ pairs, const uint8_t *__restrict__ types,
                        const double *__restrict__ ext, const unsigned *__restrict__ counts,
                        const __grid_constant__ EntParams P, int scheme, uint64_t p0,
                        uint64_t npairs, double *__restrict__ s2) {
  const uint64_t p = p0 + blockIdx.x;
  if (p >= npairs) return;
  const uint32_t i = pairs[2 * p], j = pairs[2 * p + 1];
  const int nb = P.schemes[scheme];
  const unsigned nb2 = (unsigned)nb * nb;
  const int t1 = types[i], t2 = types[j];
  const bool hj1 = (t1 == 1 || t1 == 2), hj2 = (t2 == 1 || t2 == 2);
  double w1 = __ddiv_rn(__dsub_rn(ext[4 * i + 1], ext[4 * i]), (double)nb);
  double w2 = __ddiv_rn(__dsub_rn(ext[4 * j + 1], ext[4 * j]), (double)nb);
  const double hw1 = w1 / 2, hw2 = w2 / 2;
  if (P.kde) w1 = w2 = 1.0;
  __shared__ double mid1[256], mid2[256], red[32];
  __shared__ unsigned long long redu[32];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    mid1[b] = hj1 ? __dadd_rn(__dadd_rn(ext[4 * i], __dmul_rn((double)b, w1)), hw1) : 0.0;
    mid2[b] = hj2 ? __dadd_rn(__dadd_rn(ext[4 * j], __dmul_rn((double)b, w2)), hw2) : 0.0;
  }
  __syncthreads();
  const double area = w1 * w2;
  const uint64_t per = (uint64_t)P.nests * P.nschemes * P.nsteps;
  auto jac = [](int type, double m) { return type == 1 ? pow(m, 2) : sin(m); };
  auto bsum_d = [&](double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    return s;
  };
  auto bsum_u = [&](unsigned long long v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) redu[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long s = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += redu[q];
    return s;
  };
  for (int t = 0; t < P.nsteps; ++t) {
    const unsigned *c = counts + ((p - p0) * P.nsteps + t) * (uint64_t)nb2;
    const double nd = (t + 1.0) * (double)P.step_size;
    for (int e = 0; e < P.nests; ++e) {
      const int est = P.ests[e];
      double g = 1.0, lam = 0.0;
      const double tk = 1.0 / (double)nb;
      unsigned long long blank = 0;
      if (est == 1) {
        unsigned long long z = 0;
        for (unsigned q = threadIdx.x; q < nb2; q += blockDim.x) z += (c[q] == 0);
        blank = bsum_u(z);
      } else if (est == 2) {
        unsigned long long z = 0;
        for (unsigned q = threadIdx.x; q < nb2; q += blockDim.x) z += (c[q] == 1);
        unsigned single = (unsigned)bsum_u(z);
        g = 1 - (single / nd);
      } else if (est == 3) {
        double a = 0, b = 0;
        for (unsigned q = threadIdx.x; q < nb2; q += blockDim.x) {
          double f = c[q] / nd;
          a += f * f;
          b += (tk - f) * (tk - f);
        }
        a = bsum_d(a);
        b = bsum_d(b);
        lam = (1 - a) / ((nd - 1) * b);
      }
      double acc = 0.0;
      for (unsigned q = threadIdx.x; q < nb2; q += blockDim.x) {
        const int jj = q / nb, kk = q % nb;
        double f = c[q] / nd;
        if (est == 2) f = g * (c[q] / nd);
        if (est == 3) f = (lam * tk) + ((1 - lam) * f);
        double pd = f / area;
        if (pd > 0.0) {
          const double jf1 = hj1 ? jac(t1, mid1[jj]) : 1.0;
          double jf2 = 1.0;
          if (hj2) jf2 = jac(t2, est == 2 ? mid2[jj] : mid2[kk]);
          double den = (est == 2) ? 1 - pow((1 - f), nd) : 1.0;
          if (P.jacobian) {
            const double jf = jf1 * jf2;
            pd = pd / jf;
            acc += jf * pd * log(pd) / den;
          } else {
            acc += pd * log(pd) / den;
          }
        }
      }
      acc = bsum_d(acc) * -area;
      if (est == 1) acc += ((nb2 - (unsigned)blank) - 1) / (2.0 * nd);
      if (threadIdx.x == 0) s2[p * per + ((uint64_t)e * P.nschemes + scheme) * P.nsteps + t] = acc;
    }
  }
}

// ----------------------------------------------------------------------------
uint64_t all_pairs_stripe(int tile, uint64_t nframes, uint64_t ntile) {
  // the columns of a stripe (tile DOFs per tile column, nframes bytes each)
  // take at most kStripeBytes of L2
  constexpr uint64_t kStripeBytes = 48ull << 20;
  const uint64_t per = (uint64_t)std::max(tile, 1) * std::max<uint64_t>(nframes, 1);
  return std::max<uint64_t>(1, std::min<uint64_t>(ntile, kStripeBytes / per));
}

int moment_scale(uint64_t n) {
  if (n < 3) return 52;
  const double L = (double)n * std::log((double)n);   // largest possible moment
  const int s = 63 - (int)std::ceil(std::log2(L));
  return std::max(0, std::min(52, s));
}

int fill_fix_table(centre_ctx *ctx, unsigned long long *tab, int s) {
  fix_table_kernel<<<(kTabGlobal + 255) / 256, 256, 0, ctx->stream>>>(tab, kTabGlobal, s);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

const unsigned long long *fix_table(centre_ctx *ctx, int s, int *status) {
  if (s < 0 || s > 52) {
    *status = set_error(ctx, CENTRE_E_ARG, "moment scale out of range");
    return nullptr;
  }
  if (!ctx->d_fix[s]) {
    void *p = nullptr;
    const cudaError_t e = cudaMalloc(&p, sizeof(unsigned long long) * kTabGlobal);
    if (e != cudaSuccess) {
      *status = check_cuda(ctx, e, "cudaMalloc(c ln c table)");
      return nullptr;
    }
    const int rc = fill_fix_table(ctx, static_cast<unsigned long long *>(p), s);
    if (rc != CENTRE_OK) {
      cudaFree(p);
      *status = rc;
      return nullptr;
    }
    ctx->d_fix[s] = p;
  }
  return static_cast<const unsigned long long *>(ctx->d_fix[s]);
}

int launch_entropy1d(centre_ctx *ctx, const EntParams &P, uint32_t ndof, const uint8_t *d_types,
                     const uint8_t *d_bins, const double *d_ext, double *d_s1,
                     unsigned long long *d_freq, double *d_lsum) {
  if (ndof == 0) return CENTRE_OK;
  KernelTimer kt(ctx, CENTRE_TIMER_COUNTS1D);
  entropy1d_kernel<<<ndof * P.nschemes, 256, 0, ctx->stream>>>(d_bins, d_types, d_ext, P, d_s1,
                                                               d_freq, d_lsum, ctx->d_flag);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

// Shared-memory budget of the histograms (the fixed-point c ln c table and the
// kernel's static data take the rest of the 227 KB).
#ifndef CENTRE_HIST_BUDGET_KB
#define CENTRE_HIST_BUDGET_KB 184
#endif
static constexpr size_t kHistBudget = CENTRE_HIST_BUDGET_KB * 1024;

int pair_tile_for(int nb) {
  // pairs whose nb*nb uint32 histograms fit the shared-memory budget
  const size_t per = (size_t)nb * nb * 4;
  return (int)std::min<size_t>(16, kHistBudget / per);
}

template <int R, int C, int kMinB>
static int launch_hist_mb(centre_ctx *ctx, const PairParams &P, const PairTask *d_tasks,
                          uint64_t ntasks, const unsigned long long *d_fix,
                          unsigned long long *d_sclnc, unsigned *d_nnz,
                          unsigned *d_counts, size_t smem) {
  if (d_counts) {
    CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_hist_kernel<R, C, true, kMinB>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pairs_hist_kernel<R, C, true, kMinB><<<(unsigned)ntasks, 512, smem, ctx->stream>>>(
        P.bins, d_tasks, P, d_fix, d_sclnc, d_nnz, d_counts, ctx->d_flag);
  } else if (P.want_nnz) {
    CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_hist_kernel<R, C, false, kMinB>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pairs_hist_kernel<R, C, false, kMinB><<<(unsigned)ntasks, 512, smem, ctx->stream>>>(
        P.bins, d_tasks, P, d_fix, d_sclnc, d_nnz, d_counts, ctx->d_flag);
  } else {
    // no estimator needs the non-empty cell counts: they are not kept
    CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_hist_kernel<R, C, false, kMinB, false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pairs_hist_kernel<R, C, false, kMinB, false><<<(unsigned)ntasks, 512, smem, ctx->stream>>>(
        P.bins, d_tasks, P, d_fix, d_sclnc, d_nnz, d_counts, ctx->d_flag);
  }
  return CENTRE_OK;
}

template <int R, int C>
static int launch_hist(centre_ctx *ctx, const PairParams &P, const PairTask *d_tasks,
                       uint64_t ntasks, const unsigned long long *d_fix,
                          unsigned long long *d_sclnc, unsigned *d_nnz,
                       unsigned *d_counts) {
  const size_t smem =
      (((size_t)R * C * P.nb * P.nb * 4 + 15) & ~size_t(15)) + 8 * kTabF;
  if (R == 4 && C == 4 && kHistPrefetch) {
    // the prefetching 4 x 4 kernel is built twice: capped at 64 registers
    // for two resident CTAs, and uncapped (~120 registers) for histograms
    // so large that one CTA fills an SM's shared memory anyway (50 bins:
    // 218 vs 233 ms for the 2994-DOF chain)
    int per_sm = 0;
    CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_hist_kernel<R, C, false, 2>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CENTRE_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                         &per_sm, pairs_hist_kernel<R, C, false, 2>, 512, smem));
    if (per_sm < 2)
      return launch_hist_mb<R, C, 1>(ctx, P, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts,
                                     smem);
    return launch_hist_mb<R, C, 2>(ctx, P, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts,
                                   smem);
  }
  if (d_counts) {
    CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_hist_kernel<R, C, true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pairs_hist_kernel<R, C, true><<<(unsigned)ntasks, 512, smem, ctx->stream>>>(
        P.bins, d_tasks, P, d_fix, d_sclnc, d_nnz, d_counts, ctx->d_flag);
  } else {
    CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_hist_kernel<R, C, false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    pairs_hist_kernel<R, C, false><<<(unsigned)ntasks, 512, smem, ctx->stream>>>(
        P.bins, d_tasks, P, d_fix, d_sclnc, d_nnz, d_counts, ctx->d_flag);
  }
  return CENTRE_OK;
}

// Sets the dynamic shared-memory limit of the batch kernel for tiles of
// tile x tile pairs with up to nb bins (outside any stream capture).
int prepare_pairs_hist_batch(centre_ctx *ctx, int tile, int nb) {
  const size_t smem = (((size_t)tile * tile * nb * nb * 4 + 15) & ~size_t(15)) + 8 * kTabF;
  auto set = [&](auto kern) {
    return check_cuda(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem), "batch smem attribute");
  };
  switch (tile) {
    case 4: return set(pairs_hist_batch_kernel<4>);
    case 3: return set(pairs_hist_batch_kernel<3>);
    case 2: return set(pairs_hist_batch_kernel<2>);
    default: return set(pairs_hist_batch_kernel<1>);
  }
}

size_t pairs_hist_batch_smem(int tile, int nb) {
  return (((size_t)tile * tile * nb * nb * 4 + 15) & ~size_t(15)) + 8 * kTabF;
}

// Resident CTAs per SM of the batch kernel for a tile shape and block size.
int pairs_hist_batch_occupancy(centre_ctx *ctx, int tile, int threads, int nb, int *per_sm) {
  const size_t smem = pairs_hist_batch_smem(tile, nb);
  cudaError_t e;
  switch (tile) {
    case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, pairs_hist_batch_kernel<4>, threads, smem); break;
    case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, pairs_hist_batch_kernel<3>, threads, smem); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, pairs_hist_batch_kernel<2>, threads, smem); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, pairs_hist_batch_kernel<1>, threads, smem); break;
  }
  return check_cuda(ctx, e, "batch occupancy");
}

int launch_pairs_hist_batch(centre_ctx *ctx, const BatchSys *d_sys, int nsys, uint64_t nitems,
                            const BatchCommon &B, int tile, int threads, int grid,
                            const unsigned long long *d_fix) {
  if (nitems <= B.item0 || grid <= 0) return CENTRE_OK;
  KernelTimer kt(ctx, CENTRE_TIMER_PAIRS);
  const size_t smem = pairs_hist_batch_smem(tile, B.nb);
  switch (tile) {
    case 4: pairs_hist_batch_kernel<4><<<grid, threads, smem, ctx->stream>>>(d_sys, nsys, nitems, B, d_fix, ctx->d_flag); break;
    case 3: pairs_hist_batch_kernel<3><<<grid, threads, smem, ctx->stream>>>(d_sys, nsys, nitems, B, d_fix, ctx->d_flag); break;
    case 2: pairs_hist_batch_kernel<2><<<grid, threads, smem, ctx->stream>>>(d_sys, nsys, nitems, B, d_fix, ctx->d_flag); break;
    default: pairs_hist_batch_kernel<1><<<grid, threads, smem, ctx->stream>>>(d_sys, nsys, nitems, B, d_fix, ctx->d_flag); break;
  }
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

int launch_pairs_atomic(centre_ctx *ctx, const PairParams &P, const PairTask *d_tasks,
                        uint64_t ntasks, const unsigned long long *d_fix,
                          unsigned long long *d_sclnc, unsigned *d_nnz,
                        unsigned *d_counts) {
  if (ntasks == 0) return CENTRE_OK;
  if ((uint64_t)P.ndof * P.nschemes * P.nframes >= kMaxHistBinBytes)
    return set_error(ctx, CENTRE_E_ARG, "bin matrix of 16 GiB or more (histogram counts)");
  PairParams Q = P;
  if (Q.all_pairs) Q.stripe = all_pairs_stripe(Q.tile, Q.nframes, Q.ntile);
  KernelTimer kt(ctx, CENTRE_TIMER_PAIRS);
  int rc;
  if (Q.all_pairs) {
    switch (Q.tile) {
      case 4: rc = launch_hist<4, 4>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts); break;
      case 3: rc = launch_hist<3, 3>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts); break;
      case 2: rc = launch_hist<2, 2>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts); break;
      default: rc = launch_hist<1, 1>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts); break;
    }
  } else {
    const int w = pair_tile_for(Q.nb);
    if (w >= 16) rc = launch_hist<1, 16>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts);
    else if (w >= 8) rc = launch_hist<1, 8>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts);
    else if (w >= 4) rc = launch_hist<1, 4>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts);
    else if (w >= 2) rc = launch_hist<1, 2>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts);
    else rc = launch_hist<1, 1>(ctx, Q, d_tasks, ntasks, d_fix, d_sclnc, d_nnz, d_counts);
  }
  ctx->launches++;
  if (rc != CENTRE_OK) return rc;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

int launch_finalize2d(centre_ctx *ctx, const EntParams &P, int scheme, const uint32_t *d_pairs,
                      int all_pairs, uint32_t ndof, const double *d_ext, const double *d_lsum,
                      const unsigned long long *d_sclnc, const unsigned *d_nnz, uint64_t npairs,
                      double *d_s2) {
  const uint64_t total = npairs * P.nsteps;
  if (total == 0) return CENTRE_OK;
  int st = CENTRE_OK;
  const uint64_t nl = (uint64_t)ndof * P.nschemes + P.nsteps;
  double *d_logw = (double *)scratch(ctx, kSlotAux2, sizeof(double) * nl, &st);
  if (!d_logw) return st;
  // the table is rebuilt for each scheme (the same buffer serves all)
  logw_kernel<<<(unsigned)((nl + 255) / 256), 256, 0, ctx->stream>>>(d_ext, ndof, P, d_logw);
  finalize2d_kernel<<<(unsigned)((npairs + 255) / 256), 256, 0, ctx->stream>>>(
      d_pairs, all_pairs, ndof, d_logw, d_lsum, d_sclnc, d_nnz, P, scheme, npairs, d_s2);
  ctx->launches += 2;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

// As launch_finalize2d, with the log table supplied by the caller instead of
// context scratch (used by the entry point that allocates nothing).
int launch_finalize2d_into(centre_ctx *ctx, const EntParams &P, int scheme, uint32_t ndof,
                           const double *d_ext, const double *d_lsum, const unsigned long long *d_sclnc,
                           const unsigned *d_nnz, uint64_t npairs, double *d_logw,
                           double *d_s2) {
  const uint64_t total = npairs * P.nsteps;
  if (total == 0) return CENTRE_OK;
  const uint64_t nl = (uint64_t)ndof * P.nschemes + P.nsteps;
  logw_kernel<<<(unsigned)((nl + 255) / 256), 256, 0, ctx->stream>>>(d_ext, ndof, P, d_logw);
  finalize2d_kernel<<<(unsigned)((npairs + 255) / 256), 256, 0, ctx->stream>>>(
      nullptr, 1, ndof, d_logw, d_lsum, d_sclnc, d_nnz, P, scheme, npairs, d_s2);
  ctx->launches += 2;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

int launch_entropy2d_counts(centre_ctx *ctx, const EntParams &P, int scheme,
                            const uint32_t *d_pairs, const uint8_t *d_types, const double *d_ext,
                            const unsigned *d_counts, uint64_t p0, uint64_t np, uint64_t npairs,
                            double *d_s2) {
  if (np == 0) return CENTRE_OK;
  entropy2d_counts_kernel<<<(unsigned)np, 256, 0, ctx->stream>>>(d_pairs, d_types, d_ext,
                                                                  d_counts, P, scheme, p0, npairs,
                                                                  d_s2);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

}  // namespace centre
