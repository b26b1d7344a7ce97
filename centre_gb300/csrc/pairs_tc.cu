// pairs_tc.cu -- exact joint counts as an FP8 one-hot contraction on tcgen05.
//
// Reference: binData2D (src/Estimators.cpp:130-205) for every pair i<j, with
// the per-pair entropy2D cell sum (:586-631) reduced to the exact integer
// moments sum_c round-free(c ln c) and the non-empty cell count (see
// entropy.cu for the factorisation).
//
// Formulation.  Rows of the one-hot matrix O are (DOF, bin) packed without
// padding: row = dof * nb + bin.  O[frame][row] = 1 when DOF's bin at frame is
// bin.  The joint counts of every pair are blocks of O^T O.  A CTA computes a
// 128 x 256 tile of O^T O (rows [rb, rb+128), columns [cb, cb+256)) over all
// frames with tcgen05.mma kind::f8f6f4 (E4M3 operands, FP32 accumulator in
// TMEM): 1.0 and 0.0 are exact in E4M3 and FP32 sums of integers below 2^24
// are exact, so the counts are exact.
//
// Operand tiles stay zero in shared memory; producer warps write one E4M3 1.0
// byte per (frame, DOF) into the K-major, 128-byte-swizzled tiles and clear
// exactly those bytes again once the MMA has consumed the stage, so building
// a one-hot tile costs two byte stores per (frame, DOF) instead of writing
// the whole tile.  Lane l of a producer warp owns frames 4l..4l+3 of the
// chunk for every DOF of the tile: its bins arrive in one coalesced 32-bit
// load per DOF, and the stores of one instruction spread over all 32 banks.
//
// Convergence steps are prefixes of the frame axis: K-chunks never straddle a
// step boundary, and at each boundary the epilogue warps read the running
// accumulator from TMEM (tcgen05.ld), reduce each (row DOF, column DOF) block
// to sum c ln c (exact 128-bit fixed point) and the non-empty cell count, and
// add them into the pair's moments with integer atomics (tiles split pair
// blocks; integer addition keeps the result independent of the split).
//
// Warp roles (288 threads): warp 0 allocates TMEM and one lane issues the
// MMAs; warps 1-4 produce operand stages, warp 1+p owning stage p, so four
// stages are built concurrently without cross-warp barriers, each warp
// prefetching the bins of its next chunk into registers while it marks the
// current one; warps 5-8 run the epilogue (TMEM lane group = warp % 4).  Every
// mbarrier wait is bounded: on expiry the kernel sets an error flag, lets the
// MMAs it issued drain (again bounded), frees its TMEM and returns.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {
namespace {

constexpr int kTileM = 128;                 // A rows (row DOF bins)
constexpr int kTileN = 256;                 // B rows (column DOF bins)
constexpr int kChunk = 128;                 // frames per stage (one 128 B row)
constexpr int kStages = 4;
constexpr int kABytes = kTileM * kChunk;    // 16 KB
constexpr int kBBytes = kTileN * kChunk;    // 32 KB
constexpr int kStageBytes = kABytes + kBBytes;
constexpr int kMinBins = 16;                // DOF slots per tile bounded below
constexpr int kMaxSlotsA = kTileM / kMinBins + 1;  // 9
constexpr int kMaxSlotsB = kTileN / kMinBins + 1;  // 17
constexpr int kMaxSlots = kMaxSlotsA + kMaxSlotsB;
constexpr int kTabTc = 2048;                // c ln c doubles in shared memory
constexpr int kProducerWarps = kStages;     // producer warp p owns stage p
constexpr int kEpilogue = 128;
constexpr int kThreads = 32 * (1 + kProducerWarps + 4);   // 288
constexpr int kFramesPerLane = kChunk / 32;              // 4
constexpr unsigned kTmemCols = 256;
constexpr long long kWaitCycles = 20000000000ll;  // ~10 s at 2 GHz
constexpr uint8_t kOne = 0x38;              // 1.0 in E4M3

struct TcParams {
  const uint8_t *bins;
  const uint2 *tiles;     // (row tile, column tile)
  uint64_t ntiles;
  uint64_t nframes;
  uint64_t step_size;
  uint32_t ndof;
  uint32_t nrows;         // ndof * nb
  int nschemes;
  int scheme;
  int nb;
  int nsteps;
};

struct StageMeta {
  int rb, cb;       // tile rows / columns base
  int d0a, nda;     // first DOF and DOF count of the A tile
  int d0b, ndb;
  int nvalid;       // frames in this chunk
  int used;
};

struct Smem {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t accfull;
  uint64_t accempty;
  uint64_t drain;
  uint32_t tmem_base;
  int abort_flag;
  int ego[2];       // epilogue's per-snapshot go/abort decision
  double tab[kTabTc];
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the kernel is aborting (timeout here or elsewhere).
__device__ bool wait_bar(Smem &S, uint64_t *bar, uint32_t parity, int *flag) {
  const long long t0 = clock64();
  uint32_t it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (*(volatile int *)&S.abort_flag) return false;
    if ((++it & 255u) == 0 && clock64() - t0 > kWaitCycles) {
      atomicOr(flag, kFlagTimeout);
      *(volatile int *)&S.abort_flag = 1;
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void named_bar(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), version 1, base offset 0.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;                 // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;       // SBO
  d |= (uint64_t)1u << 46;                 // descriptor version
  d |= (uint64_t)2u << 61;                 // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D = F32, A = B = E4M3, both K-major, N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kTileN >> 3) << 17) |
                            ((uint32_t)(kTileM >> 4) << 24);

__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// Byte offset of element (row, k) in a K-major 128B-swizzled tile.
__device__ __forceinline__ uint32_t swz(uint32_t row, uint32_t k) {
  return (row >> 3) * 1024u + (row & 7u) * 128u + ((((k >> 4) ^ row) & 7u) << 4) + (k & 15u);
}

struct ChunkIter {
  // walks (step, chunk) of the frame axis; chunks end at step boundaries
  uint64_t ss;
  int nsteps;
  int t;
  uint64_t f;   // next frame
  __device__ void start(uint64_t step_size, int ns) {
    ss = step_size;
    nsteps = ns;
    t = 0;
    f = 0;
  }
  // returns false when done; sets [f0, f1) and whether it closes a step
  __device__ bool next(uint64_t &f0, uint64_t &f1, bool &last_of_step) {
    if (t >= nsteps) return false;
    const uint64_t end = (uint64_t)(t + 1) * ss;
    f0 = f;
    f1 = min(end, f0 + (uint64_t)kChunk);
    last_of_step = (f1 == end);
    f = f1;
    if (last_of_step) ++t;
    return true;
  }
};

__device__ __forceinline__ void tile_geometry(const TcParams &P, uint2 tl, StageMeta &m) {
  m.rb = (int)tl.x * kTileM;
  m.cb = (int)tl.y * kTileN;
  m.d0a = m.rb / P.nb;
  const int lasta = min((int)P.nrows, m.rb + kTileM) - 1;
  m.nda = lasta / P.nb - m.d0a + 1;
  m.d0b = m.cb / P.nb;
  const int lastb = min((int)P.nrows, m.cb + kTileN) - 1;
  m.ndb = lastb / P.nb - m.d0b + 1;
}

// Chunk c of a CTA's work: tile and frame range.  Walks the per-tile chunk
// sequence (steps x 128-frame chunks, a chunk never straddles a step).
struct ChunkPos {
  uint64_t ti;      // tile index (global)
  uint64_t f0, f1;
  bool last;        // closes a convergence step
  bool valid;
};

struct ChunkWalker {
  uint64_t ti;
  ChunkIter it;
  uint64_t stride;
  uint64_t ntiles;
  __device__ void start(uint64_t first, uint64_t stride_, uint64_t ntiles_, uint64_t ss, int ns) {
    ti = first;
    stride = stride_;
    ntiles = ntiles_;
    it.start(ss, ns);
  }
  __device__ ChunkPos next() {
    ChunkPos p;
    p.valid = false;
    while (ti < ntiles) {
      if (it.next(p.f0, p.f1, p.last)) {
        p.ti = ti;
        p.valid = true;
        return p;
      }
      ti += stride;
      it.start(it.ss, it.nsteps);
    }
    return p;
  }
};

// Slot geometry of a stage: DOF slot -> (A or B tile, first row of the DOF's
// bins relative to the tile).
__device__ __forceinline__ void slot_info(const TcParams &P, const StageMeta &m, int slot,
                                          bool &isA, int &dof, int &base) {
  isA = slot < m.nda;
  dof = isA ? m.d0a + slot : m.d0b + (slot - m.nda);
  base = dof * P.nb - (isA ? m.rb : m.cb);
}

// Load lane's 4 frames (4*lane .. +3 of the chunk) of every DOF slot into
// registers.  The values are first used one chunk later (prefetch); the
// range check happens when they are marked.
__device__ __forceinline__ void load_lane_bins(const TcParams &P, const StageMeta &m, uint64_t f0,
                                               int lane, uint32_t (&pb)[kMaxSlots], int *flag) {
  const int nslots = m.nda + m.ndb;
  const uint64_t n = P.nframes;
  const int k0 = kFramesPerLane * lane;
  const int avail = max(0, min(kFramesPerLane, m.nvalid - k0));
#pragma unroll
  for (int slot = 0; slot < kMaxSlots; ++slot) {
    uint32_t w = 0;
    if (slot < nslots && avail > 0) {
      bool isA;
      int dof, base;
      slot_info(P, m, slot, isA, dof, base);
      if (dof < (int)P.ndof) {
        const uint8_t *src = P.bins + ((uint64_t)dof * P.nschemes + P.scheme) * n + f0 + k0;
        if (avail == kFramesPerLane && ((reinterpret_cast<uintptr_t>(src) & 3u) == 0)) {
          w = __ldg(reinterpret_cast<const uint32_t *>(src));
        } else {
#pragma unroll
          for (int q = 0; q < kFramesPerLane; ++q)
            if (q < avail) w |= (uint32_t)__ldg(src + q) << (8 * q);
        }
      }
    }
    pb[slot] = w;
  }
}

// c ln c for counts beyond the shared-memory table (rare): the global table,
// then the expression itself.  Kept out of line so the unrolled epilogue
// loop stays small.
__device__ __noinline__ double clnc_far(const double *__restrict__ gtab, unsigned c) {
  return (c < (unsigned)kTabGlobal) ? __ldg(gtab + c) : clnc_value(c);
}

__device__ __forceinline__ void sts_u8(uint32_t addr, uint32_t v) {
  asm volatile("st.shared.u8 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// Write val at the one-hot positions of the lane's frames.  In a K-major
// 128B-swizzled tile, element (row, k) sits at
//   (row << 7) + ((((k >> 4) ^ row) & 7) << 4) + (k & 15).
__device__ __forceinline__ void mark_lane(const TcParams &P, const StageMeta &m, uint32_t stage_s,
                                          int lane, uint32_t (&pb)[kMaxSlots], uint32_t val,
                                          bool check, int *flag) {
  const int nslots = m.nda + m.ndb;
  const int k0 = kFramesPerLane * lane;
  const uint32_t g = (uint32_t)(k0 >> 4);
  const uint32_t q0 = (uint32_t)(k0 & 15);
  const int kv = m.nvalid - k0;
#pragma unroll
  for (int slot = 0; slot < kMaxSlots; ++slot) {
    if (slot >= nslots) break;
    bool isA;
    int dof, base;
    slot_info(P, m, slot, isA, dof, base);
    const uint32_t rows = isA ? kTileM : kTileN;
    const uint32_t T = stage_s + (isA ? 0u : (uint32_t)kABytes);
    if (check && __vcmpgeu4(pb[slot], 0x01010101u * (uint32_t)P.nb)) {
      // a bin >= nb: report it and keep every store inside the tile
      atomicOr(flag, kFlagBinRange);
      pb[slot] = 0;
    }
#pragma unroll
    for (int q = 0; q < kFramesPerLane; ++q) {
      if (q >= kv) break;
      const uint32_t row = (uint32_t)(base + (int)((pb[slot] >> (8 * q)) & 255u));
      if (row < rows) sts_u8(T + (row << 7) + (((g ^ row) & 7u) << 4) + q0 + q, val);
    }
  }
}

// Add one row segment's (sum c ln c, non-empty cells) to pair (rd, cd): the
// lanes of a warp hold consecutive rows, so rows of the same DOF are
// contiguous lanes; a segmented shuffle reduction leaves each DOF's total in
// its first lane, which adds it to the pair's moments.
__device__ __noinline__ void flush_segment(const TcParams &P, U128 a, unsigned z, int rd,
                                              bool rowvalid, int cd, int t, int lane,
                                              U128 *__restrict__ sclnc,
                                              unsigned *__restrict__ nnz) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    U128 od;
    od.lo = __shfl_down_sync(0xffffffffu, a.lo, off);
    od.hi = __shfl_down_sync(0xffffffffu, a.hi, off);
    const unsigned oz = __shfl_down_sync(0xffffffffu, z, off);
    const int ord = __shfl_down_sync(0xffffffffu, rd, off);
    if (lane + off < 32 && ord == rd) {
      a = u128_add(a, od);
      z += oz;
    }
  }
  const int prd = __shfl_up_sync(0xffffffffu, rd, 1);
  const bool head = (lane == 0) || (prd != rd);
  if (head && rowvalid && rd < cd && cd < (int)P.ndof) {
    const uint64_t pidx =
        (uint64_t)rd * P.ndof - (uint64_t)rd * (rd + 1) / 2 + (uint64_t)(cd - rd - 1);
    U128 *dst = sclnc + pidx * P.nsteps + t;
    const unsigned long long old = atomicAdd(&dst->lo, a.lo);
    const unsigned long long carry = (old + a.lo < old) ? 1ull : 0ull;
    atomicAdd(&dst->hi, a.hi + carry);
    atomicAdd(&nnz[pidx * P.nsteps + t], z);
  }
}

__global__ void __launch_bounds__(kThreads, 1)
pairs_tc_kernel(const __grid_constant__ TcParams P, const double *__restrict__ gtab,
                U128 *__restrict__ sclnc, unsigned *__restrict__ nnz, int *__restrict__ flag) {
  extern __shared__ __align__(1024) unsigned char dyn[];
  // stages first (1024-aligned), then the bookkeeping block
  const uint32_t pad = (1024u - (smem_u32(dyn) & 1023u)) & 1023u;
  uint8_t *stages = dyn + pad;
  const uint32_t stages_s = smem_u32(stages);
  Smem &S = *reinterpret_cast<Smem *>(stages + kStages * kStageBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // ---- set-up ------------------------------------------------------------
  {
    uint4 z = make_uint4(0, 0, 0, 0);
    uint4 *p = reinterpret_cast<uint4 *>(stages);
    for (int i = tid; i < kStages * kStageBytes / 16; i += kThreads) p[i] = z;
    for (int i = tid; i < kTabTc; i += kThreads) S.tab[i] = gtab[i];
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&S.full[s], 32);
      mbar_init(&S.empty[s], 1);
    }
    mbar_init(&S.accfull, 1);
    mbar_init(&S.accempty, kEpilogue);
    mbar_init(&S.drain, 1);
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_proxy_async();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&S.tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;

  if (warp == 0) {
    // ---- MMA issuer --------------------------------------------------------
    if (lane == 0) {
      int s = 0;
      uint32_t ph[kStages] = {0, 0, 0, 0};
      uint32_t nsnap = 0;
      bool issued = false;
      bool ok = true;
      for (uint64_t ti = blockIdx.x; ti < P.ntiles && ok; ti += gridDim.x) {
        ChunkIter it;
        it.start(P.step_size, P.nsteps);
        uint64_t f0, f1;
        bool last;
        bool first = true;
        while (ok && it.next(f0, f1, last)) {
          if (!wait_bar(S, &S.full[s], ph[s], flag)) { ok = false; break; }
          ph[s] ^= 1u;
          tc_fence_after();
          const uint32_t a0 = smem_u32(stages + s * kStageBytes);
          const uint32_t b0 = a0 + kABytes;
          const int nk = (int)((f1 - f0 + 31) / 32);
          for (int k = 0; k < nk; ++k) {
            mma_f8(tmem, sw128_desc(a0 + 32u * k), sw128_desc(b0 + 32u * k),
                   (first && k == 0) ? 0u : 1u);
          }
          issued = true;
          first = false;
          mma_commit(&S.empty[s]);
          s = (s + 1) % kStages;
          if (last) {
            mma_commit(&S.accfull);
            ++nsnap;
            // wait until the epilogue has read this snapshot
            if (!wait_bar(S, &S.accempty, (nsnap - 1) & 1u, flag)) { ok = false; break; }
            tc_fence_after();
          }
        }
      }
      if (issued) {
        // drain: every MMA issued by this thread has completed
        mma_commit(&S.drain);
        const long long t0 = clock64();
        while (!mbar_try_wait(&S.drain, 0)) {
          if (clock64() - t0 > kWaitCycles) {
            atomicOr(flag, kFlagTimeout);
            break;
          }
        }
      }
    }
    __syncwarp();
  } else if (warp <= kProducerWarps) {
    // ---- producers: warp 1+p builds every chunk c with c % 4 == p ------------
    const int p = warp - 1;
    const uint32_t stage_s = stages_s + (uint32_t)(p * kStageBytes);
    uint32_t ph = 0;
    bool used = false;
    StageMeta old;            // previous occupant of this stage
    uint32_t oldb[kMaxSlots];
    uint32_t pb[kMaxSlots];
    ChunkWalker walk;
    walk.start(blockIdx.x, gridDim.x, P.ntiles, P.step_size, P.nsteps);
    ChunkPos cur;
    for (int i = 0; i <= p; ++i) cur = walk.next();   // this warp's first chunk
    StageMeta m;
    if (cur.valid) {
      tile_geometry(P, P.tiles[cur.ti], m);
      m.nvalid = (int)(cur.f1 - cur.f0);
      load_lane_bins(P, m, cur.f0, lane, pb, flag);
    }
    while (cur.valid) {
      // wait until the MMA has consumed this stage's previous chunk
      int go = 1;
      if (lane == 0 && used) go = wait_bar(S, &S.empty[p], ph, flag) ? 1 : 0;
      go = __shfl_sync(0xffffffffu, go, 0);
      if (!go) break;
      if (used) {
        ph ^= 1u;
        mark_lane(P, old, stage_s, lane, oldb, 0u, false, flag);
      }
      __syncwarp();
      mark_lane(P, m, stage_s, lane, pb, kOne, true, flag);
      fence_proxy_async();
      mbar_arrive(&S.full[p]);
      // remember what was set, then fetch this warp's next chunk
      old = m;
#pragma unroll
      for (int i = 0; i < kMaxSlots; ++i) oldb[i] = pb[i];
      used = true;
      for (int i = 0; i < kProducerWarps; ++i) cur = walk.next();
      if (cur.valid) {
        tile_geometry(P, P.tiles[cur.ti], m);
        m.nvalid = (int)(cur.f1 - cur.f0);
        load_lane_bins(P, m, cur.f0, lane, pb, flag);
      }
    }
  } else {
    // ---- epilogue ------------------------------------------------------------
    const int ew = warp & 3;             // TMEM lane group of this warp
    const int etid = 32 * ew + lane;     // accumulator row
    uint32_t nsnap = 0;
    bool ok = true;
    const int nb = P.nb;
    for (uint64_t ti = blockIdx.x; ti < P.ntiles && ok; ti += gridDim.x) {
      StageMeta m;
      tile_geometry(P, P.tiles[ti], m);
      const int grow = m.rb + etid;
      const int rd = grow / nb;
      const bool rowvalid = grow < (int)P.nrows;
      for (int t = 0; t < P.nsteps; ++t) {
        if (etid == 0) {
          bool go = wait_bar(S, &S.accfull, nsnap & 1u, flag);
          if (*(volatile int *)&S.abort_flag) go = false;
          S.ego[nsnap & 1u] = go ? 1 : 0;
        }
        named_bar(2, kEpilogue);
        if (!*(volatile int *)&S.ego[nsnap & 1u]) { ok = false; break; }
        tc_fence_after();
        U128 acc;
        acc.lo = acc.hi = 0ull;
        unsigned cnz = 0;
        int cur = m.cb / nb;                       // column DOF of column 0
        int nextb = (cur + 1) * nb - m.cb;         // first column of the next DOF
        for (int chunk = 0; chunk < kTileN / 32; ++chunk) {
          uint32_t v[32];
          const uint32_t taddr = tmem + ((uint32_t)(32 * ew) << 16) + (uint32_t)(chunk * 32);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
              "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
              "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]),
                "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
                "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                "=r"(v[30]), "=r"(v[31])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const int c = chunk * 32 + q;
            if (c == nextb) {
              flush_segment(P, acc, cnz, rd, rowvalid, cur, t, lane, sclnc, nnz);
              acc.lo = acc.hi = 0ull;
              cnz = 0;
              ++cur;
              nextb += nb;
            }
            // exact integer count from the FP32 accumulator
            const unsigned cnt = __float_as_uint(__uint_as_float(v[q]) + 8388608.0f) - 0x4B000000u;
            if (cnt) {
              const double dv = (cnt < (unsigned)kTabTc) ? S.tab[cnt] : clnc_far(gtab, cnt);
              acc = u128_add(acc, u128_from_double(dv));
              ++cnz;
            }
          }
        }
        flush_segment(P, acc, cnz, rd, rowvalid, cur, t, lane, sclnc, nnz);
        tc_fence_before();
        mbar_arrive(&S.accempty);
        ++nsnap;
      }
    }
  }

  // ---- tear-down -----------------------------------------------------------
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

size_t tc_smem_bytes() { return 1024 + (size_t)kStages * kStageBytes + sizeof(Smem); }

}  // namespace

bool tc_supported(centre_ctx *ctx, int nb, uint64_t nframes) {
  if (ctx->cc_major != 10 || ctx->cc_minor != 3) return false;  // sm_103a build
  if (nb < kMinBins || nb > 255) return false;
  if (nframes >= (1ull << 24)) return false;  // FP32 accumulation stays exact
  return true;
}

int launch_pairs_tc(centre_ctx *ctx, const PairParams &PP, const double *d_tab, U128 *d_sclnc,
                    unsigned *d_nnz) {
  const int nb = PP.nb;
  const uint32_t ndof = PP.ndof;
  const uint64_t nrows = (uint64_t)ndof * nb;
  if (nrows >= (1ull << 31)) return set_error(ctx, CENTRE_E_UNSUPPORTED, "too many DOF bins");
  // tiles (row tile, column tile) holding at least one pair i < j
  const int ntr = (int)((nrows + kTileM - 1) / kTileM);
  const int ntc = (int)((nrows + kTileN - 1) / kTileN);
  std::vector<uint2> tiles;
  for (int a = 0; a < ntr; ++a) {
    const int mind = (a * kTileM) / nb;
    for (int b = 0; b < ntc; ++b) {
      const uint64_t lastrow = std::min<uint64_t>(nrows, (uint64_t)(b + 1) * kTileN) - 1;
      const int maxd = (int)(lastrow / nb);
      if (maxd > mind) tiles.push_back(make_uint2((unsigned)a, (unsigned)b));
    }
  }
  if (tiles.empty()) return CENTRE_OK;
  int st = CENTRE_OK;
  uint2 *d_tiles = (uint2 *)scratch(ctx, kSlotPairs, sizeof(uint2) * tiles.size(), &st);
  if (!d_tiles) return st;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_tiles, tiles.data(), sizeof(uint2) * tiles.size(),
                                   cudaMemcpyHostToDevice, ctx->stream));
  const uint64_t npairs = (uint64_t)ndof * (ndof - 1) / 2;
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_sclnc, 0, sizeof(U128) * npairs * PP.nsteps, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_nnz, 0, sizeof(unsigned) * npairs * PP.nsteps, ctx->stream));
  TcParams P;
  P.bins = PP.bins;
  P.tiles = d_tiles;
  P.ntiles = tiles.size();
  P.nframes = PP.nframes;
  P.step_size = PP.step_size;
  P.ndof = ndof;
  P.nrows = (uint32_t)nrows;
  P.nschemes = PP.nschemes;
  P.scheme = PP.scheme;
  P.nb = nb;
  P.nsteps = PP.nsteps;
  const size_t smem = tc_smem_bytes();
  CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
  const unsigned grid = (unsigned)std::min<uint64_t>(tiles.size(), (uint64_t)ctx->sm_count);
  {
    KernelTimer kt(ctx, CENTRE_TIMER_PAIRS);
    pairs_tc_kernel<<<grid, kThreads, smem, ctx->stream>>>(P, d_tab, d_sclnc, d_nnz, ctx->d_flag);
  }
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

}  // namespace centre
