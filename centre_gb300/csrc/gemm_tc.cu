// gemm_tc.cu -- the pair screen's correlation matrix R = X X^T on tcgen05.
//
// X is n x K bf16, row-major with a leading dimension ldx (each row one
// column of standardised DOF values over the screen's frames, K-major); R is
// n x n fp32, row-major with leading dimension ldr.  No counterpart in the
// reference (it reads neighbour lists from files, src/Centre.cpp:459-593).
//
// A persistent CTA per SM walks 128 x 256 tiles of R.  Warp 0 (one lane)
// loads the two operand panels of each 64-element K chunk with TMA
// (cp.async.bulk.tensor.2d, 128-byte swizzle: a 128 x 64 box of the tile's
// rows and two of its 256 columns, 48 KB per stage) into a four-stage
// ring; warp 1 (one lane) issues tcgen05.mma kind::f16 (bf16 operands, fp32
// accumulator in TMEM, M = 128, N = 256, K = 16 per instruction) and
// releases each stage with tcgen05.commit; warps 2-5 read the finished
// accumulator (tcgen05.ld) and store it.  The accumulator is double
// buffered in TMEM (2 x 256 columns), so a tile's epilogue overlaps the next
// tile's MMAs.  Tiles are walked in groups of eight row tiles, column tile
// by column tile, so the CTAs running at one time share their rows (and the
// current K window of them) in L2.  Every wait is bounded: on expiry the
// kernel sets an error flag, drains its MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {
namespace {

constexpr int kBM = 128;                  // tile rows (A panel rows)
constexpr int kBN = 256;                  // tile columns (B panel rows)
constexpr int kBK = 64;                   // bf16 elements per K chunk (128 bytes)
constexpr int kStages = 4;
constexpr int kABytes = kBM * kBK * 2;    // 16 KB
constexpr int kBBytes = kBN * kBK * 2;    // 32 KB
constexpr int kStageBytes = kABytes + kBBytes;
constexpr int kGroupRows = 8;             // row tiles per group of the tile order
constexpr int kThreads = 192;             // producer, MMA, 4 epilogue warps
constexpr int kEpi = 128;
constexpr unsigned kTmemCols = 512;       // two 256-column accumulators
constexpr long long kWaitCycles = 20000000000ll;   // ~10 s at 2 GHz

// D = F32, A = B = BF16, both K-major, N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

struct GemmSmem {
  uint64_t full[kStages];
  uint64_t empty[kStages];
  uint64_t tfull[2];
  uint64_t tempty[2];
  uint64_t drain;
  uint32_t tmem_base;
  int abort_flag;
};

struct GemmParams {
  float *R;
  uint32_t n;
  uint32_t nk;            // K chunks
  uint32_t ldr;
  uint32_t ntm, ntn;      // row and column tiles
  uint64_t ntiles;
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
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
      : "memory");
  return ok != 0;
}
// Bounded wait: false when the kernel is aborting (timeout here or elsewhere).
__device__ bool wait_bar(GemmSmem &S, uint64_t *bar, uint32_t parity, int *flag) {
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
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// K-major operand in 128-byte swizzled rows, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1u << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)2u << 61;
  return d;
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld16(uint32_t (&v)[16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]),
                 "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]),
                 "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
               :
               : "memory");
}

// Tile id -> (row tile, column tile): groups of kGroupRows row tiles, each
// walked column tile by column tile.
__device__ __forceinline__ void tile_of(const GemmParams &P, uint64_t id, uint32_t &tr,
                                        uint32_t &tc) {
  const uint64_t per_group = (uint64_t)kGroupRows * P.ntn;
  const uint32_t g = (uint32_t)(id / per_group);
  const uint64_t in = id - (uint64_t)g * per_group;
  const uint32_t gr = min((uint32_t)kGroupRows, P.ntm - g * kGroupRows);
  tc = (uint32_t)(in / gr);
  tr = g * kGroupRows + (uint32_t)(in % gr);
}

__global__ void __launch_bounds__(kThreads, 1)
corr_gemm_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ GemmParams P,
                 int *__restrict__ flag) {
  extern __shared__ __align__(1024) unsigned char dyn[];
  const uint32_t pad = (1024u - (smem_u32(dyn) & 1023u)) & 1023u;
  unsigned char *stages = dyn + pad;
  GemmSmem &S = *reinterpret_cast<GemmSmem *>(stages + kStages * kStageBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&S.tfull[b], 1);
      mbar_init(&S.tempty[b], kEpi);
    }
    mbar_init(&S.drain, 1);
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
  }
  if (warp == 1) {
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
  const uint32_t stages_s = smem_u32(stages);

  if (warp == 0) {
    // ---- TMA producer ------------------------------------------------------
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (uint64_t id = blockIdx.x; id < P.ntiles && ok; id += gridDim.x) {
        uint32_t tr, tc;
        tile_of(P, id, tr, tc);
        for (uint32_t kc = 0; kc < P.nk; ++kc, ++it) {
          const uint32_t s = it % kStages, u = it / kStages;
          if (u >= 1 && !wait_bar(S, &S.empty[s], (u - 1) & 1u, flag)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&S.full[s], (uint32_t)kStageBytes);
          const uint32_t a = stages_s + s * kStageBytes;
          // the column panel's 256 rows as two 128-row boxes, one after the
          // other: the same swizzled layout as one 256-row panel
          tma_load_2d(a, &tmap, (int)(kc * kBK), (int)(tr * kBM), &S.full[s]);
          tma_load_2d(a + kABytes, &tmap, (int)(kc * kBK), (int)(tc * kBN), &S.full[s]);
          tma_load_2d(a + kABytes + kABytes, &tmap, (int)(kc * kBK), (int)(tc * kBN + kBM),
                      &S.full[s]);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer --------------------------------------------------------
    if (lane == 0) {
      uint32_t it = 0, tcount = 0;
      bool ok = true, issued = false;
      for (uint64_t id = blockIdx.x; id < P.ntiles && ok; id += gridDim.x, ++tcount) {
        const uint32_t b = tcount & 1u, ub = tcount >> 1;
        if (ub >= 1 && !wait_bar(S, &S.tempty[b], (ub - 1) & 1u, flag)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + b * (uint32_t)kBN;
        for (uint32_t kc = 0; kc < P.nk; ++kc, ++it) {
          const uint32_t s = it % kStages, u = it / kStages;
          if (!wait_bar(S, &S.full[s], u & 1u, flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a = stages_s + s * kStageBytes;
#pragma unroll
          for (int k = 0; k < kBK / 16; ++k)
            mma_bf16(d, sw128_desc(a + 32u * k), sw128_desc(a + kABytes + 32u * k),
                     (kc == 0 && k == 0) ? 0u : 1u);
          issued = true;
          mma_commit(&S.empty[s]);
        }
        if (!ok) break;
        mma_commit(&S.tfull[b]);
      }
      if (issued) {
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
  } else {
    // ---- epilogue: TMEM -> registers -> R --------------------------------------
    const int ew = warp & 3;   // TMEM lane group
    uint32_t tcount = 0;
    for (uint64_t id = blockIdx.x; id < P.ntiles; id += gridDim.x, ++tcount) {
      const uint32_t b = tcount & 1u, ub = tcount >> 1;
      if (!wait_bar(S, &S.tfull[b], ub & 1u, flag)) break;
      tc_fence_after();
      uint32_t tr, tc;
      tile_of(P, id, tr, tc);
      const uint32_t row = tr * kBM + 32 * ew + lane;
      const uint32_t taddr = tmem + ((uint32_t)(32 * ew) << 16) + b * (uint32_t)kBN;
      float *dst = P.R + (uint64_t)row * P.ldr;
#pragma unroll 1
      for (int c = 0; c < kBN; c += 16) {
        uint32_t v[16];
        tmem_ld16(taddr + (uint32_t)c, v);
        tmem_wait_ld16(v);
        const uint32_t col = tc * kBN + (uint32_t)c;
        if (row < P.n) {
#pragma unroll
          for (int q = 0; q < 16; q += 4) {
            const uint32_t cq = col + q;
            if (cq + 4 <= P.n) {
              *reinterpret_cast<float4 *>(dst + cq) =
                  make_float4(__uint_as_float(v[q]), __uint_as_float(v[q + 1]),
                              __uint_as_float(v[q + 2]), __uint_as_float(v[q + 3]));
            } else {
#pragma unroll
              for (int e = 0; e < 4; ++e)
                if (cq + e < P.n) dst[cq + e] = __uint_as_float(v[q + e]);
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&S.tempty[b]);
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
}

size_t gemm_smem_bytes() { return 1024 + (size_t)kStages * kStageBytes + sizeof(GemmSmem); }

std::once_flag g_encode_once;
void *g_encode_fn = nullptr;

}  // namespace

void *tensor_map_encoder() {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode_fn = fn;
  });
  return g_encode_fn;
}

int launch_corr_gemm(centre_ctx *ctx, const void *X, uint32_t n, uint32_t K, uint32_t ldx,
                     float *R, uint32_t ldr) {
  if (n == 0 || K == 0) return CENTRE_OK;
  if (ldx % 8 != 0 || ldx < K || ldr % 4 != 0 || ldr < n ||
      (reinterpret_cast<uintptr_t>(X) & 15u) != 0 || (reinterpret_cast<uintptr_t>(R) & 15u) != 0)
    return set_error(ctx, CENTRE_E_ARG, "correlation GEMM: bad layout");
  auto g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encoder());
  if (!g_encode) return set_error(ctx, CENTRE_E_CUDA, "cuTensorMapEncodeTiled unavailable");
  // X as a 2-D tensor: K elements per row (the inner dimension; loads past
  // it, and rows past n, read zeros), n rows, ldx elements apart; boxes of
  // 64 elements x 128 rows (a tile's rows, and each half of its columns).
  CUtensorMap map;
  const cuuint64_t gdim[2] = {K, n};
  const cuuint64_t gstride[1] = {(cuuint64_t)ldx * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)kBM};
  const cuuint32_t estride[2] = {1, 1};
  const CUresult cr = g_encode(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(X),
                               gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(ctx, CENTRE_E_CUDA, "cuTensorMapEncodeTiled failed");
  GemmParams P;
  P.R = R;
  P.n = n;
  P.nk = (K + kBK - 1) / kBK;
  P.ldr = ldr;
  P.ntm = (n + kBM - 1) / kBM;
  P.ntn = (n + kBN - 1) / kBN;
  P.ntiles = (uint64_t)P.ntm * P.ntn;
  const size_t smem = gemm_smem_bytes();
  CENTRE_CUDA(ctx, cudaFuncSetAttribute(corr_gemm_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)std::min<uint64_t>(P.ntiles, (uint64_t)ctx->sm_count);
  corr_gemm_kernel<<<grid, kThreads, smem, ctx->stream>>>(map, P, ctx->d_flag);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

}  // namespace centre

using namespace centre;

extern "C" int centre_gpu_corr_gemm_dev(centre_ctx *ctx, const void *X, uint32_t n, uint32_t K,
                                        uint32_t ldx, float *R, uint32_t ldr) {
  if (!ctx || !X || !R) return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  CENTRE_TRY(launch_corr_gemm(ctx, X, n, K, ldx, R, ldr));
  int f = 0;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(&f, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag_status(f) != CENTRE_OK) return set_error(ctx, flag_status(f), "correlation GEMM flag");
  return CENTRE_OK;
}
