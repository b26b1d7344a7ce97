// pairs_tc.cu -- exact joint counts as an FP8 one-hot contraction on tcgen05.
//
// Reference: binData2D (src/Estimators.cpp:130-205) for every pair i<j, with
// the per-pair entropy2D cell sum (:586-631) reduced to the exact integer
// moments sum_c round-free(c ln c) and the non-empty cell count (see
// entropy.cu for the factorisation).
//
// Formulation.  Rows of the one-hot matrix O are (DOF, bin) packed without
// padding: row = dof * nb + bin.  O[frame][row] = 2 when DOF's bin at frame is
// bin, else 0.  The joint counts of every pair are blocks of O^T O / 4.  A
// pair of CTAs (a cluster of two on one TPC) computes a 256 x 256 tile of
// O^T O over all frames with tcgen05.mma.cta_group::2 kind::f8f6f4 (E4M3
// operands, FP32 accumulator in TMEM; M = 256, N = 256, K = 32): CTA r holds
// A rows [rb + 128r, +128), B rows (tile columns) [cb + 128r, +128) and the
// accumulator rows of its A half, all 256 columns.  2.0 and 0.0 are exact in
// E4M3 and FP32 sums of multiples of 4 up to 2^24 are exact, so the counts are
// exact for up to 2^22 frames.  Against one CTA per 128 x 256 tile, each SM
// builds 256 instead of 384 operand rows per 128 frames and its tensor core
// reads 2/3 of the operand bytes for the same accumulator area.
//
// Operands.  The frame axis is cut into 128-frame blocks (one 128-byte
// K-major row of an operand tile); a block that holds the end of a
// convergence step is used twice, once per side of the step boundary (a
// "piece" is a block and a frame range inside it).  In each CTA a loader warp
// stages the bins of its halves' DOFs for each piece with two TMA loads
// (cp.async.bulk.tensor.2d: 9 DOF rows for the A half, 9 for the B half, 128
// frames each) into a 16-slot ring.  Producer warps then rewrite the CTA's
// whole operand stage (128 + 128 rows x 128 bytes, 128-byte swizzled) from
// those bins: lane (g, s) owns segment g (16 frames) of 8 rows of a 32-row
// group, in every piece the warp's stage takes, so no producer ever writes
// where another does and no stage needs clearing.  For each row it compares
// the 16 bins of its DOF with the row's bin four at a time with integer
// arithmetic (no per-byte work) and writes the 16 one-hot bytes with one
// 128-bit shared store; the stores of one instruction hit the eight 16-byte
// bank groups of a swizzled row group once each.  Frames of a piece's block
// outside the piece are zeroed in the A operand only.
//
// Pair protocol.  The even CTA's full barrier of a stage counts the producer
// lanes of both CTAs (the odd CTA arrives through its shared::cluster
// address); its MMA thread issues the pair's MMAs and commits the stage's and
// the accumulator's release to both CTAs at once (multicast).  Both CTAs
// allocate TMEM together (cta_group::2: the same columns in both SMs), meet
// on a cluster barrier after initialising their barriers and again before
// freeing TMEM.
//
// Accumulation.  Convergence steps are prefixes of the frame axis.  The MMAs
// of a step accumulate into TMEM columns [256, 512) starting from zero; at the
// step's end the epilogue warps of each CTA add them to the cumulative counts
// in columns [0, 256) and release the accumulator (to the even CTA's
// barrier) at once, so the next step's MMAs overlap the rest of the epilogue:
// reading the cumulative counts (tcgen05.ld), reducing each (row DOF, column
// DOF) block to sum F(c) (the 64-bit fixed-point c ln c of entropy.cuh) and
// the non-empty cell count, and adding them into the pair's moments with
// integer atomics (tiles split pair blocks; integer addition keeps the result
// independent of the split).
//
// Warp roles (640 threads per CTA): warp 0 allocates TMEM and, in the even
// CTA, one lane issues the MMAs; one lane of warp 1 issues the TMA loads of
// the bins; warps 2-11 produce operand stages (two per stage, four 32-row
// groups each); warps 12-19 run the epilogue as two quartets over the two
// column halves (TMEM lane group = warp % 4).  Every mbarrier wait is
// bounded: on expiry the kernel sets an error flag, lets the MMAs and loads it
// issued drain (again bounded), frees its TMEM and returns.
//
// Bins outside [0, nb) never steer an address here (the operand stores go to
// fixed places); a check pass ahead of the contraction reports them.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {
namespace {

constexpr int kPairM = 256;                 // tile rows (A rows of both CTAs)
constexpr int kHalfM = 128;                 // A rows of one CTA (its TMEM lanes)
constexpr int kTileN = 256;                 // tile columns (B rows of both CTAs)
constexpr int kHalfN = 128;                 // B rows of one CTA
constexpr int kChunk = 128;                 // frames per block (one 128 B row)
constexpr int kStages = 5;
constexpr int kABytes = kHalfM * kChunk;    // 16 KB
constexpr int kBBytes = kHalfN * kChunk;    // 16 KB
constexpr int kStageBytes = kABytes + kBBytes;
constexpr int kMinBins = 16;                // DOF slots per tile bounded below
constexpr int kSlotsHalf = kHalfM / kMinBins + 1;  // 9 DOFs in 128 rows
constexpr int kMaxSlotsA = kSlotsHalf;             // row DOFs of a CTA's A half
constexpr int kMaxSlotsB = kTileN / kMinBins + 1;  // 17 column DOFs of a tile
constexpr int kBinRows = 2 * kSlotsHalf;           // DOF rows staged per piece
constexpr int kBinBytes = kBinRows * kChunk;       // 2,304
constexpr int kBinStages = 16;
constexpr int kTabTc = 512;                 // fixed-point c ln c entries in shared memory
constexpr int kGroupsA = kHalfM / 32;       // 32-row groups of the A half
constexpr int kRowGroups = (kHalfM + kHalfN) / 32;   // 32-row groups of a stage
// Producer warps: a team of kPerTeam warps per operand stage, each warp
// rewriting kGroupsPerWarp row groups of every piece its stage takes.
constexpr int kPerTeam = 2;
constexpr int kGroupsPerWarp = kRowGroups / kPerTeam;
constexpr int kProducers = kStages * kPerTeam;
// Epilogue: kEpiGroups warp quartets, quartet g reading accumulator columns
// [g * kEpiCols, (g + 1) * kEpiCols) of all 128 rows (a warp reads the TMEM
// lanes of its warp index modulo 4).
constexpr int kEpiGroups = 2;
constexpr int kEpiCols = kTileN / kEpiGroups;
constexpr int kEpilogue = 128 * kEpiGroups;
constexpr int kWarpMma = 0;
constexpr int kWarpLoad = 1;
constexpr int kWarpProd = 2;
constexpr int kWarpEpi = kWarpProd + kProducers;
constexpr int kThreads = 32 * (kWarpEpi + 4 * kEpiGroups);
// TMEM columns: [0, 256) the cumulative counts of the current step, read by
// the epilogue; [256, 512) the MMA accumulator of the step's own frames
constexpr unsigned kTmemCols = 512;
constexpr uint32_t kIncCol = 256;
constexpr long long kWaitCycles = 20000000000ll;  // ~10 s at 2 GHz

struct TcParams {
  const uint2 *tiles;     // (row tile of 256, column tile of 256)
  uint64_t ntiles;
  uint64_t step_size;
  uint32_t ndof;
  uint32_t nrows;         // ndof * nb
  int nb;
  int nsteps;
  int fix_scale;          // moment scale s (counts beyond the table)
};

// Geometry of a CTA's half of one 256 x 256 tile of O^T O: its 128 A rows
// (the accumulator rows in its TMEM) and 128 B rows, and the tile's 256
// columns (the accumulator columns of both CTAs).
struct StageMeta {
  int rb;           // first row of this CTA's A half
  int cb;           // first column of the tile
  int cbh;          // first row of this CTA's B half (= a column)
  int d0a;          // first DOF of the A half
  int d0b;          // first DOF of the tile's columns
  int d0bh;         // first DOF of the B half
};

struct Smem {
  uint64_t full[kStages];      // operand stage built (producer lanes of both CTAs;
                               // the even CTA's is the one used)
  uint64_t empty[kStages];     // operand stage consumed (MMA commit)
  uint64_t bfull[kBinStages];  // bins of a piece landed (TMA bytes)
  uint64_t bempty[kBinStages]; // bins of a piece read (all producer lanes)
  uint64_t accfull;
  uint64_t accempty;           // both CTAs' epilogue threads (the even CTA's)
  uint64_t drain;
  uint32_t tmem_base;
  int abort_flag;
  int ego[2];       // epilogue's per-snapshot go/abort decision
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
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n\t"
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
// kSleepNs > 0 backs off between polls: for waits off the critical path
// (the loader, the epilogue's step wait), whose polling would otherwise take
// issue slots from the producers on the same scheduler.
template <int kSleepNs = 0>
__device__ bool wait_bar(Smem &S, uint64_t *bar, uint32_t parity, int *flag) {
  const long long t0 = clock64();
  uint32_t it = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (kSleepNs > 0) __nanosleep(kSleepNs);
    if (*(volatile int *)&S.abort_flag) return false;
    if ((++it & 255u) == 0 && clock64() - t0 > kWaitCycles) {
      atomicOr(flag, kFlagTimeout);
      *(volatile int *)&S.abort_flag = 1;
      return false;
    }
  }
  return true;
}
// Generic-proxy writes of this thread to shared memory become visible to the
// tensor cores of both CTAs of the pair (the MMA reads each CTA's operand
// halves).
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cluster;" ::: "memory");
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

// Instruction descriptor: D = F32, A = B = E4M3, both K-major, N = 256,
// M = 256 (the CTA pair: each CTA holds 128 rows of A, 128 rows of B and 128
// rows of D).
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kTileN >> 3) << 17) |
                            ((uint32_t)(kPairM >> 4) << 24);

__device__ __forceinline__ void mma_f8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
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
// Arrive on `bar` in both CTAs of the pair once every MMA issued so far has
// completed.
__device__ __forceinline__ void mma_commit_both(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
      "[%0], %1;" ::"r"(smem_u32(bar)),
      "h"((unsigned short)3)
      : "memory");
}
// The same, on this CTA's `bar` only.
__device__ __forceinline__ void mma_commit_local(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Address of this CTA's shared variable `p` in the even CTA of the pair.
__device__ __forceinline__ uint32_t leader_addr(const void *p) {
  uint32_t a;
  asm volatile("mapa.shared::cluster.u32 %0, %1, 0;" : "=r"(a) : "r"(smem_u32(p)));
  return a;
}
// Arrive on an mbarrier of the pair (a shared::cluster address).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t caddr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr)
               : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// Bounded wait that ignores the abort flag: for copies the kernel issued,
// which land whatever the other warps do.
__device__ void wait_landed(uint64_t *bar, uint32_t parity, int *flag) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) {
      atomicOr(flag, kFlagTimeout);
      return;
    }
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ uint4 lds128(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}

// The pieces of a CTA's work, in order: its tiles (first, first + stride,
// ...), each over the convergence steps, each step over the 128-frame blocks
// it touches.  Step t adds frames [t * step_size, (t + 1) * step_size); a
// block that holds a step boundary is visited once per side of it.
struct Piece {
  uint32_t ti;      // tile index
  uint32_t blk;     // block: frames [blk * 128, blk * 128 + 128)
  int lo, hi;       // the piece's frames within the block
  bool last;        // closes a convergence step
  bool valid;
};

// (32-bit state: at most 2^22 frames, fewer than 2^32 tiles)
struct PieceWalker {
  uint32_t ti, stride, ntiles, ss, f, end;
  int t, nsteps;
  __device__ void start(uint32_t first, uint32_t stride_, uint32_t ntiles_, uint32_t ss_,
                        int nsteps_) {
    ti = first;
    stride = stride_;
    ntiles = ntiles_;
    ss = ss_;
    nsteps = nsteps_;
    t = 0;
    f = 0;
    end = ss_;
  }
  __device__ Piece next() {
    Piece p;
    p.valid = false;
    while (ti < ntiles) {
      if (t < nsteps) {
        const uint32_t blk = f / kChunk;
        const uint32_t hi = min(end, (blk + 1) * kChunk);
        p.ti = ti;
        p.blk = blk;
        p.lo = (int)(f - blk * kChunk);
        p.hi = (int)(hi - blk * kChunk);
        p.last = hi == end;
        p.valid = true;
        f = hi;
        if (p.last) {
          ++t;
          end += ss;
        }
        return p;
      }
      ti += stride;
      t = 0;
      f = 0;
      end = ss;
    }
    return p;
  }
};

__device__ __forceinline__ void tile_geometry(const TcParams &P, uint2 tl, uint32_t rank,
                                              StageMeta &m) {
  m.rb = (int)tl.x * kPairM + (int)rank * kHalfM;
  m.cb = (int)tl.y * kTileN;
  m.cbh = m.cb + (int)rank * kHalfN;
  m.d0a = m.rb / P.nb;
  m.d0b = m.cb / P.nb;
  m.d0bh = m.cbh / P.nb;
}

// F(c) for counts beyond the global table (rare).  Kept out of line so the
// unrolled epilogue loop stays small.
__device__ __noinline__ unsigned long long clnc_far(unsigned c, int s) { return clnc_fix(c, s); }

// One-hot of four frames: byte q of the result is 0x40 (E4M3 2.0) where byte
// q of w (a bin) equals the row's bin (every byte of bb), else 0.  With x =
// w ^ bb the byte is zero exactly on a match:
//   bins < 64:  0xC0 - x lies in [0x81, 0xC0] and has bit 6 set only for x = 0;
//   bins < 128: 0x80 - x lies in [0x01, 0x80] and has bit 7 set only for x = 0;
//   otherwise:  (x & 0x7F) + 0x7F has bit 7 set iff the low 7 bits are not all
//               zero, and x's own bit 7 covers the rest.
// No byte borrows from or carries into its neighbour in any of the three.
template <int kMode>
__device__ __forceinline__ uint32_t onehot4(uint32_t w, uint32_t bb) {
  const uint32_t x = w ^ bb;
  if (kMode == 0) return (0xC0C0C0C0u - x) & 0x40404040u;
  if (kMode == 1) return ((0x80808080u - x) >> 1) & 0x40404040u;
  const uint32_t t = (x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
  return (~(t | x) & 0x80808080u) >> 1;
}

// Byte mask of frames [a, b) among the four frames 0..3 of a word.
__device__ __forceinline__ uint32_t frame_mask(int a, int b) {
  a = min(max(a, 0), 4);
  b = min(max(b, 0), 4);
  return (uint32_t)(0xFFFFFFFFull << (8 * a)) & (uint32_t)~(0xFFFFFFFFull << (8 * b));
}

// The lane's 8 rows of one piece: row i (tile row rowbase + i) is the bin
// bin0 + i of the DOF whose bins are wc, or, from row `split` on when the rows
// cross into the next DOF, bin i - split of the DOF whose bins are wn.  The
// rows' segment g lands at byte 128 i + 16 (g ^ i) of the 1024-byte row
// group (the 128-byte swizzle, with rowbase a multiple of 8).
template <int kMode, bool kSplit, bool kMask>
__device__ __forceinline__ void build_rows(uint8_t *group, uint32_t g16, const uint4 &wc,
                                           const uint4 &wn, int bin0, int split, int nb,
                                           const uint32_t (&fm)[4]) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    uint4 w = wc;
    int b = bin0 + i;
    if (kSplit && i >= split) {
      w = wn;
      b -= nb;
    }
    const uint32_t bb = (uint32_t)b * 0x01010101u;
    uint4 o;
    o.x = onehot4<kMode>(w.x, bb);
    o.y = onehot4<kMode>(w.y, bb);
    o.z = onehot4<kMode>(w.z, bb);
    o.w = onehot4<kMode>(w.w, bb);
    if (kMask) {
      o.x &= fm[0];
      o.y &= fm[1];
      o.z &= fm[2];
      o.w &= fm[3];
    }
    *reinterpret_cast<uint4 *>(group + (((uint32_t)i << 7) | (g16 ^ ((uint32_t)i << 4)))) = o;
  }
}

template <int kMode, bool kSplit>
__global__ void __maxnreg__(80)
pairs_tc_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                const __grid_constant__ TcParams P, const unsigned long long *__restrict__ gfix,
                unsigned long long *__restrict__ sclnc, unsigned *__restrict__ nnz,
                int *__restrict__ flag) {
  extern __shared__ __align__(1024) unsigned char dyn[];
  // operand stages first (1024-aligned), then the bins ring, then the
  // bookkeeping block
  const uint32_t pad = (1024u - (smem_u32(dyn) & 1023u)) & 1023u;
  uint8_t *stages = dyn + pad;
  const uint32_t stages_s = smem_u32(stages);
  const uint32_t bins_s = stages_s + (uint32_t)(kStages * kStageBytes);
  Smem &S = *reinterpret_cast<Smem *>(stages + kStages * kStageBytes + kBinStages * kBinBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // the CTA pair (a cluster of two) walks the pair's tiles; the even CTA
  // issues the MMAs
  const uint32_t rank = cluster_rank();
  const uint32_t pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;

  // ---- set-up ------------------------------------------------------------
  for (int i = tid; i < kTabTc; i += kThreads) S.tab[i] = gfix[i];
  for (int i = tid; i < kMaxSlotsA * kMaxSlotsB; i += kThreads) {
    S.blk_x[i] = 0ull;
    S.blk_nz[i] = 0u;
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&S.full[s], 2 * 32 * kPerTeam);
      mbar_init(&S.empty[s], 1);
    }
    for (int s = 0; s < kBinStages; ++s) {
      mbar_init(&S.bfull[s], 1);
      mbar_init(&S.bempty[s], 32 * kPerTeam);
    }
    mbar_init(&S.accfull, 1);
    mbar_init(&S.accempty, 2 * kEpilogue);
    mbar_init(&S.drain, 1);
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_proxy_async();
  if (warp == kWarpMma) {
    // one warp in each CTA of the pair allocates, together: the same
    // columns in both SMs
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&S.tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  // both CTAs' barriers are initialised before either arrives on the other's
  cluster_sync();
  tc_fence_after();
  const uint32_t tmem = S.tmem_base;

  if (warp == kWarpMma) {
    // ---- MMA issuer (the even CTA) ------------------------------------------
    if (lane == 0 && rank == 0) {
      PieceWalker walk;
      walk.start(pair, npairs, (uint32_t)P.ntiles, (uint32_t)P.step_size, P.nsteps);
      int s = 0;
      uint32_t ph = 0;
      uint32_t nsnap = 0;
      bool issued = false;
      bool first = true;
      // descriptors of stage 0's halves; a stage adds kStageBytes and a K
      // step 32 bytes to the start-address field (16-byte units, no carry
      // out of its 14 bits below 256 KB)
      const uint64_t desc0 = sw128_desc(stages_s);
      for (;;) {
        const Piece pc = walk.next();
        if (!pc.valid) break;
        if (!wait_bar(S, &S.full[s], ph, flag)) break;
        tc_fence_after();
        const uint64_t da = desc0 + (uint64_t)(s * (kStageBytes >> 4));
        const uint64_t db = da + (uint64_t)(kABytes >> 4);
        // the K steps (32 frames each) the piece touches
        const int k0 = pc.lo >> 5, k1 = (pc.hi + 31) >> 5;
        for (int k = k0; k < k1; ++k)
          mma_f8(tmem + kIncCol, da + (uint64_t)(2 * k), db + (uint64_t)(2 * k),
                 (first && k == k0) ? 0u : 1u);
        issued = true;
        first = false;
        mma_commit_both(&S.empty[s]);
        if (++s == kStages) {
          s = 0;
          ph ^= 1u;
        }
        if (pc.last) {
          mma_commit_both(&S.accfull);
          ++nsnap;
          // wait until the epilogue has added this step's counts to the
          // cumulative ones; the next step starts from zero
          if (!wait_bar(S, &S.accempty, (nsnap - 1) & 1u, flag)) break;
          tc_fence_after();
          first = true;
        }
      }
      if (issued) {
        // drain: every MMA issued by this thread has completed
        mma_commit_local(&S.drain);
        wait_landed(&S.drain, 0, flag);
      }
    }
    __syncwarp();
  } else if (warp == kWarpLoad) {
    // ---- bins loader -------------------------------------------------------
    if (lane == 0) {
      PieceWalker walk;
      walk.start(pair, npairs, (uint32_t)P.ntiles, (uint32_t)P.step_size, P.nsteps);
      int bs = 0;
      uint32_t round = 0;        // uses of the ring so far, per slot
      uint32_t tile = ~0u;
      int d0a = 0, d0b = 0;
      uint64_t n = 0;
      for (;;) {
        const Piece pc = walk.next();
        if (!pc.valid) break;
        // the producers have read this slot's previous piece
        if (round > 0 && !wait_bar<128>(S, &S.bempty[bs], (round - 1) & 1u, flag)) break;
        if (pc.ti != tile) {
          StageMeta m;
          tile_geometry(P, P.tiles[pc.ti], rank, m);
          d0a = m.d0a;
          d0b = m.d0bh;
          tile = pc.ti;
        }
        const uint32_t dst = bins_s + (uint32_t)(bs * kBinBytes);
        mbar_expect_tx(&S.bfull[bs], kBinBytes);
        tma_load_2d(dst, &map_a, (int)(pc.blk * kChunk), d0a, &S.bfull[bs]);
        tma_load_2d(dst + kSlotsHalf * kChunk, &map_b, (int)(pc.blk * kChunk), d0b, &S.bfull[bs]);
        ++n;
        if (++bs == kBinStages) {
          bs = 0;
          ++round;
        }
      }
      // every load issued has landed before the CTA may exit
      for (int b = 0; b < kBinStages; ++b) {
        const uint64_t uses = n > (uint64_t)b ? (n - b + kBinStages - 1) / kBinStages : 0;
        if (uses) wait_landed(&S.bfull[b], (uint32_t)((uses - 1) & 1u), flag);
      }
    }
    __syncwarp();
  } else if (warp < kWarpEpi) {
    // ---- producers: the team of warps 2 + p, 2 + p + kStages, ... builds
    // the pieces n with n % kStages == p into operand stage p of this CTA;
    // its warp h rewrites row groups h, h + kPerTeam, ... (groups 0-3 the A
    // half, 4-7 the B half), lane (g, s) segment g of rows 32 * group + 8s
    // .. + 7
    const int pw = warp - kWarpProd;
    const int team = pw % kStages;
    const int h = pw / kStages;
    const int g = lane & 7;
    const uint32_t g16 = (uint32_t)g << 4;
    const int sub8 = 8 * (lane >> 3);
    const int nb = P.nb;
    const uint32_t nomask[4] = {~0u, ~0u, ~0u, ~0u};
    // per row group k of this warp, the lane's rows in the current tile:
    // the first is bin bin0 of the DOF whose bins row lies at lds0 in a ring
    // slot; from row `split` on, the next DOF's (at lds1)
    int bin0[kGroupsPerWarp], split[kGroupsPerWarp];
    uint32_t lds0[kGroupsPerWarp], lds1[kGroupsPerWarp];
    auto geometry = [&](uint32_t ti) {
      StageMeta m;
      tile_geometry(P, P.tiles[ti], rank, m);
#pragma unroll
      for (int k = 0; k < kGroupsPerWarp; ++k) {
        const int rg = h + kPerTeam * k;
        const bool isA = rg < kGroupsA;
        const int r0 = (isA ? m.rb + 32 * rg : m.cbh + 32 * (rg - kGroupsA)) + sub8;
        const int dof0 = r0 / nb;
        bin0[k] = r0 - dof0 * nb;
        split[k] = nb - bin0[k];
        // staged DOF rows: the A half's from row 0, the B half's from row
        // kSlotsHalf; rows past the matrix read the zero fill
        const int first = isA ? 0 : kSlotsHalf;
        const int lastrow = isA ? kSlotsHalf - 1 : kBinRows - 1;
        const int slot = min(first + dof0 - (isA ? m.d0a : m.d0bh), lastrow);
        lds0[k] = (uint32_t)slot * kChunk + g16;
        lds1[k] = (uint32_t)min(slot + 1, lastrow) * kChunk + g16;
      }
    };
    // bounded wait by lane 0, then every lane acquires the completed phase
    auto warp_wait = [&](uint64_t *bar, uint32_t parity) -> bool {
      int go = 1;
      if (lane == 0) go = wait_bar(S, bar, parity, flag) ? 1 : 0;
      go = __shfl_sync(0xffffffffu, go, 0);
      if (go) mbar_try_wait(bar, parity);
      return go != 0;
    };
    PieceWalker walk;
    walk.start(pair, npairs, (uint32_t)P.ntiles, (uint32_t)P.step_size, P.nsteps);
    Piece pc;
    for (int i = 0; i <= team; ++i) pc = walk.next();
    // this stage's full barrier in the even CTA
    const uint32_t full_pair = leader_addr(&S.full[team]);
    uint32_t n = (uint32_t)team;   // index of the piece among the CTA's pieces
    uint32_t tile = ~0u;
    uint32_t use = 0;              // earlier pieces built into this stage
    uint8_t *const stage = stages + team * kStageBytes;
    while (pc.valid) {
      if (pc.ti != tile) {
        geometry(pc.ti);
        tile = pc.ti;
      }
      const int bs = (int)(n & (kBinStages - 1));
      if (!warp_wait(&S.bfull[bs], (n / kBinStages) & 1u)) break;
      // the MMA has consumed this stage's previous piece
      if (use > 0 && !warp_wait(&S.empty[team], (use - 1) & 1u)) break;
      const uint32_t src = bins_s + (uint32_t)(bs * kBinBytes);
      uint4 wc[kGroupsPerWarp], wn[kGroupsPerWarp];
#pragma unroll
      for (int k = 0; k < kGroupsPerWarp; ++k) {
        wc[k] = lds128(src + lds0[k]);
        wn[k] = kSplit ? lds128(src + lds1[k]) : wc[k];
      }
      const bool partial = pc.lo > 0 || pc.hi < kChunk;
      uint32_t fm[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) fm[j] = frame_mask(pc.lo - 16 * g - 4 * j, pc.hi - 16 * g - 4 * j);
#pragma unroll
      for (int k = 0; k < kGroupsPerWarp; ++k) {
        const int rg = h + kPerTeam * k;
        const bool isA = rg < kGroupsA;
        uint8_t *group = stage + (isA ? 32 * rg * kChunk : kABytes + 32 * (rg - kGroupsA) * kChunk) +
                         sub8 * kChunk;
        if (isA && partial)   // frames of the block outside the piece read zero in A
          build_rows<kMode, kSplit, true>(group, g16, wc[k], wn[k], bin0[k], split[k], nb, fm);
        else
          build_rows<kMode, kSplit, false>(group, g16, wc[k], wn[k], bin0[k], split[k], nb, nomask);
      }
      // the ring slot is released once its values have been used: an
      // arrive right after the loads did not keep them ahead of the
      // loader's next copy into the slot
      mbar_arrive(&S.bempty[bs]);
      fence_proxy_async();
      mbar_arrive_cluster(full_pair);
      ++use;
      for (int i = 0; i < kStages; ++i) pc = walk.next();
      n += kStages;
    }
  } else {
    // ---- epilogue ------------------------------------------------------------
    const int ew = warp & 3;             // TMEM lane group of this warp
    const int etid = 32 * ew + lane;     // accumulator row
    const int eth = 32 * (warp - kWarpEpi) + lane;   // 0 .. kEpilogue-1
    const int col0 = (eth / 128) * kEpiCols;                  // this quartet's columns
    uint32_t nsnap = 0;
    bool ok = true;
    const int nb = P.nb;
    // the accumulator's release goes to the even CTA's barrier
    const uint32_t accempty_pair = leader_addr(&S.accempty);
    for (uint64_t ti = pair; ti < P.ntiles && ok; ti += npairs) {
      StageMeta m;
      tile_geometry(P, P.tiles[ti], rank, m);
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
          bool go = wait_bar<256>(S, &S.accfull, nsnap & 1u, flag);
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
        mbar_arrive_cluster(accempty_pair);
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
          // exact integer counts from the FP32 accumulator (4 per frame);
          // F(c) from the shared table, larger counts from the global table
          unsigned cnt[kEpiW];
          unsigned long long cv[kEpiW];
          bool big = false;
#pragma unroll
          for (int q = 0; q < kEpiW; ++q) {
            cnt[q] = __float_as_uint(fmaf(__uint_as_float(v[q]), 0.25f, 8388608.0f)) -
                     0x4B000000u;
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
  // the pair leaves together: the even CTA's MMAs read this CTA's operands
  // and write its TMEM until they drain, and the odd CTA arrives on the even
  // CTA's barriers until its last piece
  cluster_sync();
  if (warp == kWarpMma) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// Checks every bin of the scheme against nb (a bin outside [0, nb) sets
// kFlagBinRange) and, when dst is set, copies the scheme's rows to dst with
// a row pitch of `pitch` bytes (a multiple of 16, as TMA needs).  Thread x of
// block row y handles 16 frames of DOF y, y + gridDim.y, ...
__global__ void tc_bins_kernel(const uint8_t *__restrict__ bins, uint64_t nframes, int nschemes,
                               int scheme, uint32_t ndof, int nb, uint8_t *__restrict__ dst,
                               uint64_t pitch, int *__restrict__ flag) {
  const uint64_t f0 = 16ull * (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x);
  if (f0 >= nframes) return;
  const int nv = (int)(nframes - f0 < 16 ? nframes - f0 : 16);
  const uint32_t lim = 0x01010101u * (uint32_t)nb;
  bool bad = false;
  for (uint32_t d = blockIdx.y; d < ndof; d += gridDim.y) {
    const uint8_t *src = bins + ((uint64_t)d * nschemes + scheme) * nframes + f0;
    uint32_t w[4];
    if (nv == 16 && (reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
      const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src));
      w[0] = v.x;
      w[1] = v.y;
      w[2] = v.z;
      w[3] = v.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        uint32_t x = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (4 * j + q < nv) x |= (uint32_t)__ldg(src + 4 * j + q) << (8 * q);
        w[j] = x;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) bad |= __vcmpgeu4(w[j], lim) != 0u;
    if (dst)
      *reinterpret_cast<uint4 *>(dst + (uint64_t)d * pitch + f0) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  if (bad) atomicOr(flag, kFlagBinRange);
}

size_t tc_smem_bytes() {
  return 1024 + (size_t)kStages * kStageBytes + (size_t)kBinStages * kBinBytes + sizeof(Smem);
}
static_assert(1024 + kStages * kStageBytes + kBinStages * kBinBytes + sizeof(Smem) <= 232448,
              "shared memory of the tensor-core count kernel above 227 KB");
static_assert(kThreads == 640 && kRowGroups == kPerTeam * kGroupsPerWarp, "warp roles");
static_assert((kBinStages & (kBinStages - 1)) == 0, "bins ring slots: a power of two");

template <int kMode, bool kSplit>
int launch_tc(centre_ctx *ctx, const CUtensorMap &ma, const CUtensorMap &mb, const TcParams &P,
              unsigned grid, const unsigned long long *d_fix, unsigned long long *d_sclnc,
              unsigned *d_nnz) {
  auto kern = pairs_tc_kernel<kMode, kSplit>;
  const size_t smem = tc_smem_bytes();
  CENTRE_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
  // clusters of two CTAs (the pair of one MMA)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, 1, 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  {
    KernelTimer kt(ctx, CENTRE_TIMER_PAIRS);
    CENTRE_CUDA(ctx, cudaLaunchKernelEx(&cfg, kern, ma, mb, P, d_fix, d_sclnc, d_nnz,
                                        ctx->d_flag));
  }
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

}  // namespace

bool tc_supported(centre_ctx *ctx, int nb, uint64_t nframes) {
  if (ctx->cc_major != 10 || ctx->cc_minor != 3) return false;  // sm_103a build
  if (nb < kMinBins || nb > 255) return false;
  if (nframes > (1ull << 22)) return false;  // FP32 sums of 4 per frame stay exact
  return true;
}

int launch_pairs_tc(centre_ctx *ctx, const PairParams &PP, const unsigned long long *d_fix,
                    unsigned long long *d_sclnc, unsigned *d_nnz) {
  const int nb = PP.nb;
  const uint32_t ndof = PP.ndof;
  const uint64_t nframes = PP.nframes;
  const uint64_t nrows = (uint64_t)ndof * nb;
  if (nrows >= (1ull << 31)) return set_error(ctx, CENTRE_E_UNSUPPORTED, "too many DOF bins");
  // tiles (row tile, column tile) holding at least one pair i < j
  const int ntr = (int)((nrows + kPairM - 1) / kPairM);
  const int ntc = (int)((nrows + kTileN - 1) / kTileN);
  std::vector<uint2> tiles;
  for (int a = 0; a < ntr; ++a) {
    const int mind = (a * kPairM) / nb;
    for (int b = 0; b < ntc; ++b) {
      const uint64_t lastrow = std::min<uint64_t>(nrows, (uint64_t)(b + 1) * kTileN) - 1;
      const int maxd = (int)(lastrow / nb);
      if (maxd > mind) tiles.push_back(make_uint2((unsigned)a, (unsigned)b));
    }
  }
  if (tiles.empty()) return CENTRE_OK;
  if (tiles.size() >= (1ull << 32)) return set_error(ctx, CENTRE_E_UNSUPPORTED, "too many tiles");
  auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encoder());
  if (!encode) return set_error(ctx, CENTRE_E_CUDA, "cuTensorMapEncodeTiled unavailable");
  int st = CENTRE_OK;
  uint2 *d_tiles = (uint2 *)scratch(ctx, kSlotPairs, sizeof(uint2) * tiles.size(), &st);
  if (!d_tiles) return st;
  // The scheme's bins as a 2-D tensor of nframes bytes per DOF row.  TMA
  // wants a 16-byte aligned base and row pitch: the bins array itself when
  // nframes is a multiple of 16, else a copy with the pitch rounded up.
  const uint8_t *base = PP.bins + (uint64_t)PP.scheme * nframes;
  uint64_t pitch = (uint64_t)PP.nschemes * nframes;
  uint8_t *copy = nullptr;
  if (nframes % 16 != 0 || (reinterpret_cast<uintptr_t>(PP.bins) & 15u) != 0) {
    pitch = (nframes + 15) / 16 * 16;
    copy = (uint8_t *)scratch(ctx, kSlotTcBins, pitch * ndof, &st);
    if (!copy) return st;
    base = copy;
  }
  {
    const uint64_t nthr = (nframes + 15) / 16;
    const dim3 grid((unsigned)((nthr + 255) / 256), std::min<uint32_t>(ndof, 2048u));
    tc_bins_kernel<<<grid, 256, 0, ctx->stream>>>(PP.bins, nframes, PP.nschemes, PP.scheme, ndof,
                                                  nb, copy, pitch, ctx->d_flag);
    ctx->launches++;
    CENTRE_CUDA(ctx, cudaGetLastError());
  }
  CUtensorMap ma, mb;
  {
    const cuuint64_t gdim[2] = {nframes, ndof};
    const cuuint64_t gstride[1] = {pitch};
    const cuuint32_t box_a[2] = {(cuuint32_t)kChunk, (cuuint32_t)kSlotsHalf};
    const cuuint32_t box_b[2] = {(cuuint32_t)kChunk, (cuuint32_t)kSlotsHalf};
    const cuuint32_t estride[2] = {1, 1};
    CUresult cr = encode(&ma, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t *>(base), gdim,
                         gstride, box_a, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr == CUDA_SUCCESS)
      cr = encode(&mb, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t *>(base), gdim,
                  gstride, box_b, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(ctx, CENTRE_E_CUDA, "cuTensorMapEncodeTiled failed");
  }
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_tiles, tiles.data(), sizeof(uint2) * tiles.size(),
                                   cudaMemcpyHostToDevice, ctx->stream));
  const uint64_t npairs = (uint64_t)ndof * (ndof - 1) / 2;
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_sclnc, 0, sizeof(unsigned long long) * npairs * PP.nsteps,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_nnz, 0, sizeof(unsigned) * npairs * PP.nsteps, ctx->stream));
  TcParams P;
  P.tiles = d_tiles;
  P.ntiles = tiles.size();
  P.step_size = PP.step_size;
  P.ndof = ndof;
  P.nrows = (uint32_t)nrows;
  P.nb = nb;
  P.nsteps = PP.nsteps;
  P.fix_scale = PP.fix_scale;
  // one CTA pair per two SMs
  const unsigned grid =
      2u * (unsigned)std::min<uint64_t>(tiles.size(), (uint64_t)(ctx->sm_count / 2));
  const bool split = nb % 8 != 0;   // a lane's 8 rows may span two DOFs
  if (nb <= 64)
    return split ? launch_tc<0, true>(ctx, ma, mb, P, grid, d_fix, d_sclnc, d_nnz)
                 : launch_tc<0, false>(ctx, ma, mb, P, grid, d_fix, d_sclnc, d_nnz);
  if (nb <= 128)
    return split ? launch_tc<1, true>(ctx, ma, mb, P, grid, d_fix, d_sclnc, d_nnz)
                 : launch_tc<1, false>(ctx, ma, mb, P, grid, d_fix, d_sclnc, d_nnz);
  return split ? launch_tc<2, true>(ctx, ma, mb, P, grid, d_fix, d_sclnc, d_nnz)
               : launch_tc<2, false>(ctx, ma, mb, P, grid, d_fix, d_sclnc, d_nnz);
}

}  // namespace centre
