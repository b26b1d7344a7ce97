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
// exactly those bytes again (at addresses kept in registers) once the MMA has
// consumed the stage, so building a one-hot tile costs two byte stores per
// (frame, DOF) instead of writing the whole tile.  Lane l of a producer warp
// owns frames 4l..4l+3 of the chunk: its bins arrive in one coalesced 32-bit
// load per DOF, and the stores of one instruction spread over the banks.
//
// Convergence steps are prefixes of the frame axis: K-chunks never straddle a
// step boundary.  The MMAs of a step accumulate into TMEM columns [256, 512)
// starting from zero; at the step's end the epilogue warps add them to the
// cumulative counts in columns [0, 256) and release the accumulator at once,
// so the next step's MMAs overlap the rest of the epilogue: reading the
// cumulative counts (tcgen05.ld), reducing each (row DOF, column DOF) block to
// sum F(c) (the 64-bit fixed-point c ln c of entropy.cuh) and the non-empty
// cell count, and
// adding them into the pair's moments with integer atomics (tiles split pair
// blocks; integer addition keeps the result independent of the split).
//
// Warp roles (672 threads): warp 0 allocates TMEM and one lane issues the
// MMAs; warps 1-12 produce operand stages, three per stage (warp 1+p+4h marks
// the DOF slots h, h+3, ... of stage p, from a per-tile slot table in shared
// memory), so the four stages are built concurrently without cross-warp
// barriers, each warp prefetching the bins of its next chunk into registers
// while it marks the current one (the marking is bound by instruction issue
// and latency; more warps hide it); warps 13-20 run the epilogue as two
// quartets over the two column halves (TMEM lane group = warp % 4).  Every
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
constexpr int kTabTc = 2048;                // fixed-point c ln c entries in shared memory
#ifndef CENTRE_TC_PRODUCERS_PER_STAGE
#define CENTRE_TC_PRODUCERS_PER_STAGE 3
#endif
// Producer warps p, p + kStages, ... fill stage p, each the DOF slots
// congruent to its rank modulo kPerStage (the marking is issue-bound: more
// warps hide its latency).
constexpr int kPerStage = CENTRE_TC_PRODUCERS_PER_STAGE;
constexpr int kProducerWarps = kStages * kPerStage;
constexpr int kSlotsPerWarp = (kMaxSlots + kPerStage - 1) / kPerStage;
// Epilogue: kEpiGroups warp quartets, quartet g reading accumulator columns
// [g * kEpiCols, (g + 1) * kEpiCols) of all 128 rows (a warp reads the TMEM
// lanes of its warp index modulo 4).
#ifndef CENTRE_TC_EPI_GROUPS
#define CENTRE_TC_EPI_GROUPS 2
#endif
constexpr int kEpiGroups = CENTRE_TC_EPI_GROUPS;
constexpr int kEpiCols = kTileN / kEpiGroups;
constexpr int kEpilogue = 128 * kEpiGroups;
constexpr int kThreads = 32 * (1 + kProducerWarps + 4 * kEpiGroups);
constexpr int kFramesPerLane = kChunk / 32;              // 4
// TMEM columns: [0, 256) the cumulative counts of the current step, read by
// the epilogue; [256, 512) the MMA accumulator of the step's own frames
constexpr unsigned kTmemCols = 512;
constexpr uint32_t kIncCol = 256;
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
  int fix_scale;          // moment scale s (counts beyond the table)
};

// Geometry of one 128 x 256 tile of O^T O.
struct StageMeta {
  int rb, cb;       // tile rows / columns base
  int d0a, nda;     // first DOF and DOF count of the A tile
  int d0b, ndb;
};

// A producer warp's DOF slot of the current tile: the DOF's bins row
// (element offset), the stage address of the slot's row 0 (tile row
// `base` = row of the DOF's bin 0 relative to the tile, may be negative), and
// the tile's row count.
struct SlotInfo {
  uint64_t src;
  uint32_t tb;
  int base;
  int rows;
  int pad;
};

struct Smem {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  // per stage: the producer warps of the stage have cleared their previous
  // chunk's bytes (needed when the stage moves to another tile, where the
  // warps' DOF slots cover other rows)
  uint64_t cleared[kStages];
  uint64_t accfull;
  uint64_t accempty;
  uint64_t drain;
  uint32_t tmem_base;
  int abort_flag;
  int ego[2];       // epilogue's per-snapshot go/abort decision
  uint32_t sink;    // target of one-hot stores that fall outside a tile
  // per producer warp, its DOF slots of the current tile (see SlotInfo)
  SlotInfo slots[kProducerWarps][kSlotsPerWarp];
  __align__(16) unsigned long long tab[kTabTc];   // F(c), fixed-point c ln c
  // per (row DOF slot, column DOF slot) block of the tile: the sum of F over
  // its cells and the non-empty cell count, filled with shared-memory
  // reductions
  unsigned long long blk_x[kMaxSlotsA * kMaxSlotsB];
  unsigned blk_nz[kMaxSlotsA * kMaxSlotsB];
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
  // the waiting thread may be suspended up to the hint (ns) instead of
  // spinning, which leaves the issue slots to the warps doing work
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void red_shared_u64(uint32_t addr, unsigned long long v) {
  asm volatile("red.shared.add.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}
__device__ __forceinline__ void red_shared_u32(uint32_t addr, unsigned v) {
  asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
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
// 16 consecutive TMEM columns of the warp's 32 lanes (one row per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
      "%13,%14,%15,%16};" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
      "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
      "r"(v[15])
      : "memory");
}
// Wait for the thread's TMEM loads; the registers are operands so that no
// use of them is scheduled before the wait.
__device__ __forceinline__ void tmem_wait_ld16(uint32_t (&v)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]),
                 "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]),
                 "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
               :
               : "memory");
}
// The epilogue's column chunk: kEpiW columns of the warp's 32 lanes.
constexpr int kEpiW = 4;
__device__ __forceinline__ void tmem_ld_w(uint32_t taddr, uint32_t (&v)[kEpiW]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld_w(uint32_t (&v)[kEpiW]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3])
               :
               : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

struct ChunkIter {
  // walks (step, chunk) of the frame axis; chunks end at step boundaries
  uint64_t ss;
  int nsteps;
  int t;
  uint64_t f;     // next frame
  uint64_t end;   // end of step t
  __device__ void start(uint64_t step_size, int ns) {
    ss = step_size;
    nsteps = ns;
    t = 0;
    f = 0;
    end = step_size;
  }
  // returns false when done; sets [f0, f1) and whether it closes a step
  __device__ bool next(uint64_t &f0, uint64_t &f1, bool &last_of_step) {
    if (t >= nsteps) return false;
    f0 = f;
    f1 = min(end, f0 + (uint64_t)kChunk);
    last_of_step = (f1 == end);
    f = f1;
    if (last_of_step) {
      ++t;
      end += ss;
    }
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

// F(c) for counts beyond the global table (rare).  Kept out of line so the
// unrolled epilogue loop stays small.
__device__ __noinline__ unsigned long long clnc_far(unsigned c, int s) { return clnc_fix(c, s); }

// Load the lane's 4 frames (4*lane .. +3 of the chunk) of the warp's DOF
// slots into registers.  The values are first used one chunk later
// (prefetch); the range check happens when they are marked.
__device__ __forceinline__ void load_lane_bins(const TcParams &P, const SlotInfo *sl, int nmine,
                                               int nvalid, uint64_t f0, int lane,
                                               uint32_t (&pb)[kSlotsPerWarp]) {
  const int k0 = kFramesPerLane * lane;
  const int avail = max(0, min(kFramesPerLane, nvalid - k0));
#pragma unroll
  for (int i = 0; i < kSlotsPerWarp; ++i) {
    uint32_t w = 0;
    if (i < nmine && avail > 0) {
      const uint8_t *src = P.bins + sl[i].src + f0 + k0;
      if (avail == kFramesPerLane && ((reinterpret_cast<uintptr_t>(src) & 3u) == 0)) {
        w = __ldg(reinterpret_cast<const uint32_t *>(src));
      } else {
#pragma unroll
        for (int q = 0; q < kFramesPerLane; ++q)
          if (q < avail) w |= (uint32_t)__ldg(src + q) << (8 * q);
      }
    }
    pb[i] = w;
  }
}

__device__ __forceinline__ void sts_u8(uint32_t addr, uint32_t v) {
  asm volatile("st.shared.u8 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// Set the one-hot bytes (E4M3 1.0) of the lane's frames and remember their
// addresses for clearing.  In a K-major 128B-swizzled tile, element (row, k)
// sits at (row << 7) + ((((k >> 4) ^ row) & 7) << 4) + (k & 15).  Positions
// outside the tile (first/last DOF of a tile cut by its edge, frames past
// the chunk's end) go to a scratch byte instead, so that clearing is one
// unconditional store per position.  Slots whose DOF lies inside the tile
// take the path without those checks when the chunk is full.
constexpr int kLaneMarks = kSlotsPerWarp * kFramesPerLane;

__device__ __forceinline__ void mark_set(const TcParams &P, const SlotInfo *sl, int nmine,
                                         uint32_t edgemask, int nvalid, uint32_t sink, int lane,
                                         uint32_t (&pb)[kSlotsPerWarp],
                                         uint32_t (&addr)[kLaneMarks], int *flag) {
  const int k0 = kFramesPerLane * lane;
  const uint32_t g = (uint32_t)(k0 >> 4);
  const uint32_t q0 = (uint32_t)(k0 & 15);
  const int kv = nvalid - k0;
  const bool full = nvalid == kChunk;
#pragma unroll
  for (int i = 0; i < kSlotsPerWarp; ++i) {
    if (i < nmine) {
      const int base = sl[i].base;
      const uint32_t tbq = sl[i].tb + q0;
      if (__vcmpgeu4(pb[i], 0x01010101u * (uint32_t)P.nb)) {
        // a bin >= nb: report it and keep every store inside the tile
        atomicOr(flag, kFlagBinRange);
        pb[i] = 0;
      }
      if (full && !((edgemask >> i) & 1u)) {
#pragma unroll
        for (int q = 0; q < kFramesPerLane; ++q) {
          const uint32_t b = (pb[i] >> (8 * q)) & 255u;
          const uint32_t row = (uint32_t)base + b;
          addr[i * kFramesPerLane + q] = tbq + (b << 7) + (((g ^ row) & 7u) << 4) + q;
        }
      } else {
        const uint32_t rows = (uint32_t)sl[i].rows;
#pragma unroll
        for (int q = 0; q < kFramesPerLane; ++q) {
          const uint32_t b = (pb[i] >> (8 * q)) & 255u;
          const uint32_t row = (uint32_t)base + b;
          const uint32_t a = tbq + (b << 7) + (((g ^ row) & 7u) << 4) + q;
          addr[i * kFramesPerLane + q] = (row < rows && q < kv) ? a : sink;
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < kFramesPerLane; ++q) addr[i * kFramesPerLane + q] = sink;
    }
  }
#pragma unroll
  for (int j = 0; j < kLaneMarks; ++j) sts_u8(addr[j], kOne);
}

__device__ __forceinline__ void mark_clear(const uint32_t (&addr)[kLaneMarks]) {
#pragma unroll
  for (int j = 0; j < kLaneMarks; ++j) sts_u8(addr[j], 0u);
}

__global__ void __launch_bounds__(kThreads, 1)
pairs_tc_kernel(const __grid_constant__ TcParams P, const unsigned long long *__restrict__ gfix,
                unsigned long long *__restrict__ sclnc, unsigned *__restrict__ nnz,
                int *__restrict__ flag) {
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
    for (int i = tid; i < kTabTc; i += kThreads) S.tab[i] = gfix[i];
    for (int i = tid; i < kMaxSlotsA * kMaxSlotsB; i += kThreads) {
      S.blk_x[i] = 0ull;
      S.blk_nz[i] = 0u;
    }
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&S.full[s], 32 * kPerStage);
      mbar_init(&S.empty[s], 1);
      mbar_init(&S.cleared[s], kPerStage);
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
      uint32_t ph[kStages] = {};
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
            mma_f8(tmem + kIncCol, sw128_desc(a0 + 32u * k), sw128_desc(b0 + 32u * k),
                   (first && k == 0) ? 0u : 1u);
          }
          issued = true;
          first = false;
          mma_commit(&S.empty[s]);
          s = (s + 1) % kStages;
          if (last) {
            mma_commit(&S.accfull);
            ++nsnap;
            // wait until the epilogue has added this step's counts to the
            // cumulative ones; the next step starts from zero
            if (!wait_bar(S, &S.accempty, (nsnap - 1) & 1u, flag)) { ok = false; break; }
            tc_fence_after();
            first = true;
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
    // ---- producers: warps 1+p, 1+p+kStages, ... build every chunk c with
    // c % kStages == p, warp rank h marking the DOF slots h, h+kPerStage, ...
    const int p = (warp - 1) % kStages;
    const int h = (warp - 1) / kStages;
    const uint32_t stage_s = stages_s + (uint32_t)(p * kStageBytes);
    uint32_t ph = 0;
    bool used = false;
    const uint32_t sink = smem_u32(&S.sink);
    const int pw = warp - 1;
    SlotInfo *sl = S.slots[pw];
    uint32_t addr[kLaneMarks];   // one-hot positions set for the stage's occupant
    uint32_t pb[kSlotsPerWarp];
    ChunkWalker walk;
    walk.start(blockIdx.x, gridDim.x, P.ntiles, P.step_size, P.nsteps);
    ChunkPos cur;
    for (int i = 0; i <= p; ++i) cur = walk.next();   // this warp's first chunk
    uint64_t tile = ~0ull;       // tile whose slots are in sl[]
    int nmine = 0;               // this warp's DOF slots in that tile
    uint32_t edgemask = 0;       // slots whose DOF is cut by the tile's edge
    // slot table of tile ti: lane i describes this warp's slot i
    auto set_tile = [&](uint64_t ti) {
      // every lane has finished reading the previous tile's slot table
      // (mark_set, load_lane_bins) before any lane overwrites its entry: a
      // lane still marking the last chunk of the old tile would otherwise
      // combine the old edge mask with the new slot geometry
      __syncwarp();
      StageMeta m;
      tile_geometry(P, P.tiles[ti], m);
      const int slot = h + lane * kPerStage;
      const bool valid = lane < kSlotsPerWarp && slot < m.nda + m.ndb;
      bool edge = false;
      if (valid) {
        bool isA;
        int dof, base;
        slot_info(P, m, slot, isA, dof, base);
        const int rows = isA ? kTileM : kTileN;
        SlotInfo si;
        si.src = ((uint64_t)dof * P.nschemes + P.scheme) * P.nframes;
        si.tb = stage_s + (isA ? 0u : (uint32_t)kABytes) + ((uint32_t)base << 7);
        si.base = base;
        si.rows = rows;
        si.pad = 0;
        sl[lane] = si;
        edge = base < 0 || base + P.nb > rows;
      }
      nmine = __popc(__ballot_sync(0xffffffffu, valid));
      edgemask = __ballot_sync(0xffffffffu, edge);
      tile = ti;
      __syncwarp();
    };
    int nvalid = 0;
    if (cur.valid) {
      set_tile(cur.ti);
      nvalid = (int)(cur.f1 - cur.f0);
      load_lane_bins(P, sl, nmine, nvalid, cur.f0, lane, pb);
    }
    // Fetch this warp's next chunk (kStages on); true when it lies in the
    // same tile as the chunk just marked.
    auto fetch = [&]() -> bool {
      for (int i = 0; i < kStages; ++i) cur = walk.next();
      if (!cur.valid) return false;
      const bool same = cur.ti == tile;
      if (!same) set_tile(cur.ti);
      nvalid = (int)(cur.f1 - cur.f0);
      load_lane_bins(P, sl, nmine, nvalid, cur.f0, lane, pb);
      return same;
    };
    uint32_t cph = 0;            // phase of S.cleared[p]
    bool aborted = false;
    // Outer loop: one pass per tile.  Its first chunk is marked here; when
    // the stage comes from another tile, the other warps of this stage own
    // rows this warp may have marked (and the reverse), so every warp of the
    // stage clears its previous chunk before any sets the new one.  All
    // warps of a stage walk the same chunks, so they all meet here.  The
    // tile's other chunks are marked by the inner loop, which holds no
    // barrier code (with it, the marking loop compiles to slower code).
    while (cur.valid && !aborted) {
      int go = 1;
      if (lane == 0 && used) go = wait_bar(S, &S.empty[p], ph, flag) ? 1 : 0;
      go = __shfl_sync(0xffffffffu, go, 0);
      if (!go) break;
      if (used) {
        ph ^= 1u;
        mark_clear(addr);
        __syncwarp();
        int ok = 1;
        if (lane == 0) {
          mbar_arrive(&S.cleared[p]);
          ok = wait_bar(S, &S.cleared[p], cph, flag) ? 1 : 0;
        }
        cph ^= 1u;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
      }
      __syncwarp();
      mark_set(P, sl, nmine, edgemask, nvalid, sink, lane, pb, addr, flag);
      fence_proxy_async();
      mbar_arrive(&S.full[p]);
      used = true;
      bool more = fetch();
      while (more) {
        // wait until the MMA has consumed this stage's previous chunk
        go = 1;
        if (lane == 0) go = wait_bar(S, &S.empty[p], ph, flag) ? 1 : 0;
        go = __shfl_sync(0xffffffffu, go, 0);
        if (!go) {
          aborted = true;
          break;
        }
        ph ^= 1u;
        mark_clear(addr);
        __syncwarp();
        mark_set(P, sl, nmine, edgemask, nvalid, sink, lane, pb, addr, flag);
        fence_proxy_async();
        mbar_arrive(&S.full[p]);
        more = fetch();
      }
    }
  } else {
    // ---- epilogue ------------------------------------------------------------
    const int ew = warp & 3;             // TMEM lane group of this warp
    const int etid = 32 * ew + lane;     // accumulator row
    const int eth = 32 * (warp - 1 - kProducerWarps) + lane;   // 0 .. kEpilogue-1
    const int col0 = (eth / 128) * kEpiCols;                  // this quartet's columns
    uint32_t nsnap = 0;
    bool ok = true;
    const int nb = P.nb;
    for (uint64_t ti = blockIdx.x; ti < P.ntiles && ok; ti += gridDim.x) {
      StageMeta m;
      tile_geometry(P, P.tiles[ti], m);
      const int grow = m.rb + etid;
      const int rd = grow / nb;
      const bool rowvalid = grow < (int)P.nrows;
      // this lane's row DOF segment within the warp: lanes [first, seg_end)
      const int wrow0 = m.rb + 32 * ew;
      const int seg_end = rowvalid ? min(32, (rd + 1) * nb - wrow0) : 32;
      const bool seg_head = rowvalid && lane == max(0, rd * nb - wrow0);
      const int seg_max = min(32, nb);       // longest segment (warp-uniform)
      for (int t = 0; t < P.nsteps; ++t) {
        if (eth == 0) {
          bool go = wait_bar(S, &S.accfull, nsnap & 1u, flag);
          if (*(volatile int *)&S.abort_flag) go = false;
          S.ego[nsnap & 1u] = go ? 1 : 0;
        }
        named_bar(2, kEpilogue);
        if (!*(volatile int *)&S.ego[nsnap & 1u]) { ok = false; break; }
        tc_fence_after();
        const uint32_t trow = tmem + ((uint32_t)(32 * ew) << 16);
        // Add the step's counts to the cumulative ones (the first step of a
        // tile replaces them) and release the MMA accumulator at once.
#pragma unroll 1
        for (int c = col0; c < col0 + kEpiCols; c += 16) {
          uint32_t inc[16], cum[16];
          tmem_ld16(trow + kIncCol + (uint32_t)c, inc);
          if (t > 0) {
            tmem_ld16(trow + (uint32_t)c, cum);
            tmem_wait_ld16(cum);
          }
          tmem_wait_ld16(inc);
#pragma unroll
          for (int j = 0; j < 16; ++j)
            cum[j] = (t > 0) ? __float_as_uint(__uint_as_float(inc[j]) + __uint_as_float(cum[j]))
                             : inc[j];
          tmem_st16(trow + (uint32_t)c, cum);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        tc_fence_before();
        mbar_arrive(&S.accempty);
        // Each thread reads its row of the cumulative counts in chunks of 8
        // columns and sums the exact c ln c of its cells per column DOF in
        // registers.  At each column DOF boundary the rows of one row DOF
        // (consecutive lanes) are summed with a segmented warp reduction and
        // the segment's first lane adds the sum to the tile's (row DOF,
        // column DOF) block in shared memory (one atomic per warp segment:
        // 64-bit shared-memory atomics on one address from many lanes
        // serialise).  The blocks are then added to their pairs' moments,
        // one thread per block.
        const int rs = rowvalid ? rd - m.d0a : -1;     // row DOF slot
        unsigned long long acc = 0ull;
        unsigned cnz = 0;
        const int dcol = (m.cb + col0) / nb;           // DOF of the first column
        int cs = dcol - m.d0b;                         // column DOF slot
        int nextb = (dcol + 1) * nb - m.cb;            // first column of the next DOF
        auto flush = [&]() {
          unsigned long long x = acc;
          unsigned z = cnz;
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            if (off >= seg_max) break;
            const unsigned long long x2 = __shfl_down_sync(0xffffffffu, x, off);
            const unsigned z2 = __shfl_down_sync(0xffffffffu, z, off);
            if (lane + off < seg_end) {
              x += x2;
              z += z2;
            }
          }
          if (seg_head && z) {
            const uint32_t bi = (uint32_t)(rs * kMaxSlotsB + cs);
            red_shared_u64(smem_u32(&S.blk_x[bi]), x);
            red_shared_u32(smem_u32(&S.blk_nz[bi]), z);
          }
          acc = 0ull;
          cnz = 0;
        };
#pragma unroll 1
        for (int chunk = col0 / kEpiW; chunk < (col0 + kEpiCols) / kEpiW; ++chunk) {
          uint32_t v[kEpiW];
          tmem_ld_w(trow + (uint32_t)(chunk * kEpiW), v);
          tmem_wait_ld_w(v);
          // exact integer counts from the FP32 accumulator; F(c) from the
          // shared table, larger counts from the global table
          unsigned cnt[kEpiW];
          unsigned long long cv[kEpiW];
          bool big = false;
#pragma unroll
          for (int q = 0; q < kEpiW; ++q) {
            cnt[q] = __float_as_uint(__uint_as_float(v[q]) + 8388608.0f) - 0x4B000000u;
            big |= cnt[q] >= (unsigned)kTabTc;
            cv[q] = S.tab[min(cnt[q], (unsigned)kTabTc - 1u)];
          }
          if (__any_sync(0xffffffffu, big)) {
            // counts beyond the shared table
#pragma unroll
            for (int q = 0; q < kEpiW; ++q)
              if (cnt[q] >= (unsigned)kTabTc)
                cv[q] = (cnt[q] < (unsigned)kTabGlobal) ? __ldg(gfix + cnt[q])
                                                        : clnc_far(cnt[q], P.fix_scale);
          }
          // at most one column DOF boundary per kEpiW columns (nb >= 16):
          // cells before it close the current segment, the rest open the next
          const int qb = nextb - chunk * kEpiW;
          if (qb >= kEpiW) {
#pragma unroll
            for (int q = 0; q < kEpiW; ++q) {
              acc += cv[q];
              cnz += (cnt[q] != 0u);
            }
            continue;
          }
          unsigned long long a1 = 0ull;
          unsigned z1 = 0;
#pragma unroll
          for (int q = 0; q < kEpiW; ++q) {
            if (q < qb) {
              acc += cv[q];
              cnz += (cnt[q] != 0u);
            } else {
              a1 += cv[q];
              z1 += (cnt[q] != 0u);
            }
          }
          flush();
          ++cs;
          nextb += nb;
          acc = a1;
          cnz = z1;
        }
        flush();
        named_bar(2, kEpilogue);
        for (int i = eth; i < kMaxSlotsA * kMaxSlotsB; i += kEpilogue) {
          const unsigned z = S.blk_nz[i];
          if (z) {
            const int rdb = m.d0a + i / kMaxSlotsB, cdb = m.d0b + i % kMaxSlotsB;
            if (rdb < cdb && cdb < (int)P.ndof) {
              const uint64_t pidx = (uint64_t)rdb * P.ndof - (uint64_t)rdb * (rdb + 1) / 2 +
                                    (uint64_t)(cdb - rdb - 1);
              atomicAdd(&sclnc[pidx * P.nsteps + t], S.blk_x[i]);
              atomicAdd(&nnz[pidx * P.nsteps + t], z);
            }
          }
          S.blk_x[i] = 0ull;
          S.blk_nz[i] = 0u;
        }
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

int launch_pairs_tc(centre_ctx *ctx, const PairParams &PP, const unsigned long long *d_fix,
                    unsigned long long *d_sclnc, unsigned *d_nnz) {
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
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_sclnc, 0, sizeof(unsigned long long) * npairs * PP.nsteps,
                                   ctx->stream));
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
  P.fix_scale = PP.fix_scale;
  const size_t smem = tc_smem_bytes();
  CENTRE_CUDA(ctx, cudaFuncSetAttribute(pairs_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
  const unsigned grid = (unsigned)std::min<uint64_t>(tiles.size(), (uint64_t)ctx->sm_count);
  {
    KernelTimer kt(ctx, CENTRE_TIMER_PAIRS);
    pairs_tc_kernel<<<grid, kThreads, smem, ctx->stream>>>(P, d_fix, d_sclnc, d_nnz, ctx->d_flag);
  }
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

}  // namespace centre
