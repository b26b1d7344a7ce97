// common.cuh -- shared definitions of the CENTRE GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "centre_gpu.h"

namespace centre {

// Largest bin count the reference can express (hbin_t is uint8_t,
// src/configcentre.h:24).
constexpr int kMaxBins = 255;
constexpr int kMaxSchemes = 16;
constexpr int kMaxSteps = 255;

// Largest frame count (counts and the 64-bit moment sums stay exact below
// it; see clnc_fix in entropy.cuh).
constexpr uint64_t kMaxFrames = 1ull << 27;

// Grow-only device scratch owned by a context.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace centre

struct centre_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uint64_t launches = 0;
  std::string last_error;
  centre::DevBuf scratch[9];   // one per ScratchSlot (below)
  int *d_flag = nullptr;   // device error flag (bin range, timeouts)
  // copy-in and copy-out streams and their events for the host-pointer
  // entry points that overlap transfers with kernels (created on first use)
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t copy_ev[16] = {};
  int *h_flag = nullptr;   // pinned mirror
  int cc_major = 0, cc_minor = 0;
  // fixed-point c ln c tables (2^16 entries), one per moment scale s in use
  void *d_fix[64] = {};
  // event timing of the hot kernels (centre_gpu_enable_timing)
  bool timing = false;
  struct TimerRec {
    int which;
    cudaEvent_t a, b;
  };
  std::vector<TimerRec> timers;
  std::vector<cudaEvent_t> event_pool;
  double timer_ms[4] = {0, 0, 0, 0};
  uint64_t timer_n[4] = {0, 0, 0, 0};
  void *batch_state = nullptr;  // tuned tiles and the cached batch graph
};

namespace centre {

// Scratch slots of a context.
enum ScratchSlot {
  kSlotIn = 0,     // staged host inputs
  kSlotBins = 1,
  kSlotOut = 2,
  kSlotMoments = 3,  // per pair/step sum(c ln c), nnz
  kSlotAux = 4,
  kSlotPairs = 5,
  kSlotAux2 = 6,
  kSlotAux3 = 7,
  kSlotTcBins = 8,  // bins re-pitched for TMA (tensor-core counts)
};

int set_error(centre_ctx *ctx, int status, const std::string &msg);
int check_cuda(centre_ctx *ctx, cudaError_t e, const char *what);
void *scratch(centre_ctx *ctx, int slot, size_t bytes, int *status);
void batch_state_free(centre_ctx *ctx);
void screen_state_free(centre_ctx *ctx);

// Scoped event timer around a launch on the context's stream (no-op unless
// timing is enabled).
struct KernelTimer {
  centre_ctx *ctx;
  int which;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelTimer(centre_ctx *c, int w);
  ~KernelTimer();
};

#define CENTRE_TRY(expr)        \
  do {                          \
    int _rc = (expr);           \
    if (_rc != CENTRE_OK) return _rc; \
  } while (0)

#define CENTRE_CUDA(ctx, expr) CENTRE_TRY(::centre::check_cuda((ctx), (expr), #expr))

// Device error-flag bits.
enum : int {
  kFlagBinRange = 1,
  kFlagTimeout = 2,
  kFlagDomain = 4,
};

// The status a device error flag maps to (every entry point uses this
// mapping, so the same input gives the same status everywhere).
inline int flag_status(int f) {
  if (f & kFlagDomain) return CENTRE_E_ARG;
  if (f & kFlagBinRange) return CENTRE_E_BINRANGE;
  if (f & kFlagTimeout) return CENTRE_E_TIMEOUT;
  return f ? CENTRE_E_CUDA : CENTRE_OK;
}

// The shared-memory histogram kernels address bin rows with 32-bit word
// offsets from the aligned word at or before the bins pointer (up to 3 bytes
// before it, and a row's last word may be followed by one more for an
// unaligned row): a bin matrix (DOFs x schemes x frames bytes) must stay
// 16 bytes below 16 GiB for them.
constexpr uint64_t kMaxHistBinBytes = (1ull << 34) - 16;

// Order-preserving map of a double onto uint64 (larger double -> larger key).
__host__ __device__ inline uint64_t order_key(double v) {
  union {
    double d;
    uint64_t u;
  } c;
  c.d = v;
  return (c.u & 0x8000000000000000ull) ? ~c.u : (c.u | 0x8000000000000000ull);
}

}  // namespace centre
