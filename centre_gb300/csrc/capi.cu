// capi.cu -- the C ABI of the library (declared in include/centre_gpu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {

int set_error(centre_ctx *ctx, int status, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return status;
}

int check_cuda(centre_ctx *ctx, cudaError_t e, const char *what) {
  if (e == cudaSuccess) return CENTRE_OK;
  int st = (e == cudaErrorMemoryAllocation) ? CENTRE_E_NOMEM : CENTRE_E_CUDA;
  char buf[512];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return set_error(ctx, st, buf);
}

void *scratch(centre_ctx *ctx, int slot, size_t bytes, int *status) {
  DevBuf &b = ctx->scratch[slot];
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return b.ptr;
  if (b.ptr) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.ptr, bytes);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    *status = check_cuda(ctx, e, "cudaMalloc(scratch)");
    return nullptr;
  }
  b.bytes = bytes;
  return b.ptr;
}

static cudaEvent_t pool_event(centre_ctx *ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

KernelTimer::KernelTimer(centre_ctx *c, int w) : ctx(c), which(w) {
  if (!ctx->timing) return;
  a = pool_event(ctx);
  b = pool_event(ctx);
  cudaEventRecord(a, ctx->stream);
}

KernelTimer::~KernelTimer() {
  if (!a) return;
  cudaEventRecord(b, ctx->stream);
  ctx->timers.push_back({which, a, b});
}

static int drain_timers(centre_ctx *ctx) {
  if (ctx->timers.empty()) return CENTRE_OK;
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto &t : ctx->timers) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t.a, t.b);
    ctx->timer_ms[t.which] += ms;
    ctx->timer_n[t.which] += 1;
    ctx->event_pool.push_back(t.a);
    ctx->event_pool.push_back(t.b);
  }
  ctx->timers.clear();
  return CENTRE_OK;
}

namespace {

int validate_params(centre_ctx *ctx, const centre_entropy_params *p, EntParams *E) {
  if (!p) return set_error(ctx, CENTRE_E_ARG, "null entropy params");
  if (p->nsteps == 0) return set_error(ctx, CENTRE_E_ARG, "nsteps must be > 0");
  if (p->nschemes == 0 || p->nschemes > kMaxSchemes)
    return set_error(ctx, CENTRE_E_ARG, "nschemes must be 1..16");
  if (p->nestimators == 0 || p->nestimators > 4)
    return set_error(ctx, CENTRE_E_ARG, "nestimators must be 1..4");
  if (p->nframes < p->nsteps) return set_error(ctx, CENTRE_E_ARG, "fewer frames than steps");
  if (p->nframes > kMaxFrames) return set_error(ctx, CENTRE_E_ARG, "more than 2^27 frames");
  memset(E, 0, sizeof(*E));
  E->nframes = p->nframes;
  E->step_size = p->nframes / p->nsteps;
  E->nsteps = p->nsteps;
  E->nschemes = p->nschemes;
  E->nests = p->nestimators;
  E->jacobian = p->jacobian ? 1 : 0;
  E->kde = p->kde ? 1 : 0;
  int off = 0;
  for (int s = 0; s < p->nschemes; ++s) {
    if (p->bin_schemes[s] == 0) return set_error(ctx, CENTRE_E_ARG, "zero bins in a scheme");
    E->schemes[s] = p->bin_schemes[s];
    E->scheme_off[s] = off;
    off += p->bin_schemes[s];
  }
  E->nbins_sum = off;
  for (int e = 0; e < p->nestimators; ++e) {
    if (p->estimators[e] > 3) return set_error(ctx, CENTRE_E_ARG, "unknown estimator");
    E->ests[e] = p->estimators[e];
  }
  E->fix_scale = moment_scale(E->step_size * E->nsteps);
  E->fix_inv = std::ldexp(1.0, -E->fix_scale);
  return CENTRE_OK;
}

int read_flag(centre_ctx *ctx) {
  CENTRE_CUDA(ctx, cudaMemcpyAsync(ctx->h_flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int f = *ctx->h_flag;
  switch (flag_status(f)) {
    case CENTRE_OK: return CENTRE_OK;
    case CENTRE_E_ARG:
      return set_error(ctx, CENTRE_E_ARG,
                       "input outside the reference's domain (bonds >= 0, angles in [0, pi], "
                       "torsions in [0, 2pi), finite)");
    case CENTRE_E_BINRANGE: return set_error(ctx, CENTRE_E_BINRANGE, "bin index >= bin count");
    case CENTRE_E_TIMEOUT: return set_error(ctx, CENTRE_E_TIMEOUT, "device wait limit reached");
    default: return set_error(ctx, CENTRE_E_CUDA, "unknown device error flag");
  }
}

// Tasks for an explicit pair list: pairs grouped by first DOF, up to `width`
// partner DOFs per task.  out[] holds the pair's position (minus `base`).
void plan_tasks(const uint32_t *pairs, uint64_t p0, uint64_t p1, int width,
                std::vector<PairTask> &tasks) {
  std::vector<uint64_t> idx(p1 - p0);
  std::iota(idx.begin(), idx.end(), p0);
  std::stable_sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
    if (pairs[2 * a] != pairs[2 * b]) return pairs[2 * a] < pairs[2 * b];
    return pairs[2 * a + 1] < pairs[2 * b + 1];
  });
  size_t q = 0;
  while (q < idx.size()) {
    PairTask t;
    memset(&t, 0, sizeof(t));
    t.nr = 1;
    t.rows[0] = pairs[2 * idx[q]];
    while (q < idx.size() && t.nc < width && pairs[2 * idx[q]] == t.rows[0]) {
      t.cols[t.nc] = pairs[2 * idx[q] + 1];
      t.out[t.nc] = idx[q] - p0;
      t.nc++;
      q++;
    }
    tasks.push_back(t);
  }
}

int atomic_pair_width(int nb) {
  // task widths are the kernel's instantiated column counts: 16, 8, 4, 2, 1
  const int w = pair_tile_for(nb);
  return w >= 16 ? 16 : w >= 8 ? 8 : w >= 4 ? 4 : w >= 2 ? 2 : 1;
}

bool atomic_fits(int nb) { return pair_tile_for(nb) >= 1; }

// Counts of a chunk of an explicit pair list: [np][nsteps][nb^2] uint32.
int counts_chunk(centre_ctx *ctx, const EntParams &E, int scheme, uint32_t ndof,
                 const uint8_t *d_bins, const uint32_t *h_pairs, uint64_t p0, uint64_t p1,
                 unsigned *d_counts) {
  const int nb = E.schemes[scheme];
  const int width = atomic_pair_width(nb);
  if (!atomic_fits(nb)) {
    // histograms too large for shared memory: the global-histogram kernel
    // over the chunk's pairs (uploaded as a device list)
    int st2 = CENTRE_OK;
    uint32_t *d_pl = (uint32_t *)scratch(ctx, kSlotPairs, sizeof(uint32_t) * 2 * (p1 - p0), &st2);
    if (!d_pl) return st2;
    CENTRE_CUDA(ctx, cudaMemcpyAsync(d_pl, h_pairs + 2 * p0, sizeof(uint32_t) * 2 * (p1 - p0),
                                     cudaMemcpyHostToDevice, ctx->stream));
    PairParams P;
    memset(&P, 0, sizeof(P));
    P.bins = d_bins;
    P.nframes = E.nframes;
    P.step_size = E.step_size;
    P.ndof = ndof;
    P.nschemes = E.nschemes;
    P.scheme = scheme;
    P.nb = nb;
    P.nsteps = E.nsteps;
    CENTRE_TRY(launch_pairs_global(ctx, P, d_pl, 0, p1 - p0, nullptr, nullptr, nullptr,
                                   d_counts));
    CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CENTRE_OK;
  }
  std::vector<PairTask> tasks;
  plan_tasks(h_pairs, p0, p1, width, tasks);
  int st = CENTRE_OK;
  PairTask *d_tasks = (PairTask *)scratch(ctx, kSlotPairs, sizeof(PairTask) * tasks.size(), &st);
  if (!d_tasks) return st;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_tasks, tasks.data(), sizeof(PairTask) * tasks.size(),
                                   cudaMemcpyHostToDevice, ctx->stream));
  PairParams P;
  memset(&P, 0, sizeof(P));
  P.bins = d_bins;
  P.nframes = E.nframes;
  P.step_size = E.step_size;
  P.ndof = ndof;
  P.nschemes = E.nschemes;
  P.scheme = scheme;
  P.nb = nb;
  P.nsteps = E.nsteps;
  P.all_pairs = 0;
  CENTRE_TRY(launch_pairs_atomic(ctx, P, d_tasks, tasks.size(), nullptr, nullptr, nullptr,
                                 d_counts));
  // the task buffer is reused by the next chunk: finish this one first
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

std::vector<uint32_t> all_pairs_list(uint32_t ndof) {
  std::vector<uint32_t> v;
  v.reserve((size_t)ndof * (ndof ? ndof - 1 : 0));
  for (uint32_t i = 0; i < ndof; ++i)
    for (uint32_t j = i + 1; j < ndof; ++j) {
      v.push_back(i);
      v.push_back(j);
    }
  return v;
}

}  // namespace

// ---------------------------------------------------------------------------
int entropy2d_dev(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                  const uint8_t *d_types, const uint8_t *d_bins, const double *d_ext,
                  uint64_t npairs, const uint32_t *d_pairs, double *d_s2) {
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  const bool all = (d_pairs == nullptr);
  if (all) npairs = (uint64_t)ndof * (ndof ? ndof - 1 : 0) / 2;
  if (npairs == 0 || ndof < 2) return CENTRE_OK;
  CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  int st = CENTRE_OK;
  bool moments = true;
  for (int e = 0; e < E.nests; ++e)
    if (E.ests[e] >= 2) moments = false;

  if (moments) {
    // L sums from the 1-D counts (and throw-away S1)
    const uint64_t per = (uint64_t)E.nests * E.nschemes * E.nsteps;
    double *d_tmp = (double *)scratch(ctx, kSlotAux,
                                      sizeof(double) * ((uint64_t)ndof * per +
                                                        (uint64_t)ndof * E.nschemes * E.nsteps),
                                      &st);
    if (!d_tmp) return st;
    double *d_lsum = d_tmp + (uint64_t)ndof * per;
    CENTRE_TRY(launch_entropy1d(ctx, E, ndof, d_types, d_bins, d_ext, d_tmp, nullptr, d_lsum));
    const unsigned long long *d_fix = fix_table(ctx, E.fix_scale, &st);
    if (!d_fix) return st;
    unsigned long long *d_sclnc = (unsigned long long *)scratch(
        ctx, kSlotMoments, (sizeof(unsigned long long) + sizeof(unsigned)) * npairs * E.nsteps,
        &st);
    if (!d_sclnc) return st;
    unsigned *d_nnz = reinterpret_cast<unsigned *>(d_sclnc + npairs * E.nsteps);
    std::vector<uint32_t> h_pairs;
    for (int s = 0; s < E.nschemes; ++s) {
      const int nb = E.schemes[s];
      PairParams P;
      memset(&P, 0, sizeof(P));
      P.bins = d_bins;
      P.nframes = E.nframes;
      P.step_size = E.step_size;
      P.ndof = ndof;
      P.nschemes = E.nschemes;
      P.scheme = s;
      P.nb = nb;
      P.nsteps = E.nsteps;
      P.fix_scale = E.fix_scale;
      for (int e = 0; e < E.nests; ++e)
        if (E.ests[e] == CENTRE_MM) P.want_nnz = 1;
      const int form = p->counts_form;
      // AUTO takes the tensor-core contraction only where the histograms
      // do not fit shared memory (more than 217 bins; kTcAutoMaxBins is 0).
      // Everywhere else the shared-memory histogram is about as fast or faster: it
      // does one increment per frame and pair where the contraction does
      // B^2 multiply-adds (all pairs of 2994 DOFs x 100,000 frames: 120.2
      // against 118.7 ms at 16 bins, 172.6 against 1,423 ms at 50).
      const bool use_tc =
          all && tc_supported(ctx, nb, E.nframes) &&
          (form == CENTRE_COUNTS_TC ||
           (form == CENTRE_COUNTS_AUTO && (!atomic_fits(nb) || nb <= kTcAutoMaxBins)));
      if (form == CENTRE_COUNTS_TC && !use_tc)
        return set_error(ctx, CENTRE_E_UNSUPPORTED,
                         "tensor-core counts need the all-pairs form and a supported bin count");
      if (use_tc) {
        P.all_pairs = 1;
        CENTRE_TRY(launch_pairs_tc(ctx, P, d_fix, d_sclnc, d_nnz));
      } else if (!atomic_fits(nb)) {
        // histograms too large for shared memory: one global histogram per CTA
        P.all_pairs = all ? 1 : 0;
        CENTRE_TRY(launch_pairs_global(ctx, P, d_pairs, 0, npairs, d_fix, d_sclnc, d_nnz,
                                       nullptr));
      } else {
        if (all) {
          int ppair = atomic_pair_width(nb);
          int tile = 1;
          while ((tile + 1) * (tile + 1) <= ppair && tile < 4) ++tile;
          P.all_pairs = 1;
          P.tile = tile;
          P.ntile = (ndof + tile - 1) / tile;
          const uint64_t ntasks = P.ntile * (P.ntile + 1) / 2;
          CENTRE_TRY(launch_pairs_atomic(ctx, P, nullptr, ntasks, d_fix, d_sclnc, d_nnz,
                                         nullptr));
        } else {
          if (h_pairs.empty()) {
            h_pairs.resize(2 * npairs);
            CENTRE_CUDA(ctx, cudaMemcpyAsync(h_pairs.data(), d_pairs, 8 * npairs,
                                             cudaMemcpyDeviceToHost, ctx->stream));
            CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (uint64_t q = 0; q < 2 * npairs; ++q)
              if (h_pairs[q] >= ndof) return set_error(ctx, CENTRE_E_ARG, "pair index >= ndof");
          }
          std::vector<PairTask> tasks;
          plan_tasks(h_pairs.data(), 0, npairs, atomic_pair_width(nb), tasks);
          PairTask *d_tasks =
              (PairTask *)scratch(ctx, kSlotPairs, sizeof(PairTask) * tasks.size(), &st);
          if (!d_tasks) return st;
          CENTRE_CUDA(ctx, cudaMemcpyAsync(d_tasks, tasks.data(), sizeof(PairTask) * tasks.size(),
                                           cudaMemcpyHostToDevice, ctx->stream));
          CENTRE_TRY(launch_pairs_atomic(ctx, P, d_tasks, tasks.size(), d_fix, d_sclnc,
                                         d_nnz, nullptr));
          CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        }
      }
      CENTRE_TRY(launch_finalize2d(ctx, E, s, d_pairs, all ? 1 : 0, ndof, d_ext, d_lsum, d_sclnc,
                                   d_nnz, npairs, d_s2));
    }
    return CENTRE_OK;
  }

  // counts path (Chao-Shen / James-Stein present): materialise per-pair
  // counts in chunks and evaluate every cell as the reference does
  std::vector<uint32_t> h_pairs;
  const uint32_t *dp = d_pairs;
  if (all) {
    h_pairs = all_pairs_list(ndof);
    uint32_t *d_all = (uint32_t *)scratch(ctx, kSlotAux2, sizeof(uint32_t) * h_pairs.size(), &st);
    if (!d_all) return st;
    CENTRE_CUDA(ctx, cudaMemcpyAsync(d_all, h_pairs.data(), sizeof(uint32_t) * h_pairs.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
    dp = d_all;
  } else {
    h_pairs.resize(2 * npairs);
    CENTRE_CUDA(ctx, cudaMemcpyAsync(h_pairs.data(), d_pairs, 8 * npairs, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (uint64_t q = 0; q < 2 * npairs; ++q)
      if (h_pairs[q] >= ndof) return set_error(ctx, CENTRE_E_ARG, "pair index >= ndof");
  }
  for (int s = 0; s < E.nschemes; ++s) {
    const int nb = E.schemes[s];
    const size_t per_pair = (size_t)E.nsteps * nb * nb * 4;
    const uint64_t chunk = std::max<uint64_t>(1, std::min<uint64_t>(npairs, (1ull << 30) / per_pair));
    unsigned *d_counts = (unsigned *)scratch(ctx, kSlotAux, per_pair * chunk, &st);
    if (!d_counts) return st;
    for (uint64_t p0 = 0; p0 < npairs; p0 += chunk) {
      const uint64_t p1 = std::min(npairs, p0 + chunk);
      CENTRE_TRY(counts_chunk(ctx, E, s, ndof, d_bins, h_pairs.data(), p0, p1, d_counts));
      CENTRE_TRY(launch_entropy2d_counts(ctx, E, s, dp, d_types, d_ext, d_counts, p0, p1 - p0,
                                         npairs, d_s2));
    }
  }
  return CENTRE_OK;
}

}  // namespace centre

using namespace centre;

// ===========================================================================
extern "C" {

const char *centre_gpu_strerror(int status) {
  switch (status) {
    case CENTRE_OK: return "ok";
    case CENTRE_E_ARG: return "invalid argument";
    case CENTRE_E_CUDA: return "CUDA runtime error";
    case CENTRE_E_NOMEM: return "device out of memory";
    case CENTRE_E_BINRANGE: return "bin index out of range";
    case CENTRE_E_TIMEOUT: return "device wait limit reached";
    case CENTRE_E_UNSUPPORTED: return "unsupported on this path";
    case CENTRE_E_NODEVICE: return "no usable sm_103 device";
    default: return "unknown status";
  }
}

const char *centre_gpu_last_error(const centre_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int centre_gpu_create(centre_ctx **out, int device) {
  if (!out) return CENTRE_E_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return CENTRE_E_NODEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return CENTRE_E_NODEVICE;
  if (prop.major < 10) return CENTRE_E_NODEVICE;
  if (cudaSetDevice(device) != cudaSuccess) return CENTRE_E_NODEVICE;
  centre_ctx *ctx = new centre_ctx();
  ctx->device = device;
  ctx->sm_count = prop.multiProcessorCount;
  ctx->cc_major = prop.major;
  ctx->cc_minor = prop.minor;
  int rc = CENTRE_OK;
  if ((rc = check_cuda(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking),
                       "stream")) != CENTRE_OK ||
      (rc = check_cuda(ctx, cudaMalloc(&ctx->d_flag, sizeof(int)), "flag")) != CENTRE_OK ||
      (rc = check_cuda(ctx, cudaMallocHost(&ctx->h_flag, sizeof(int)), "flag")) != CENTRE_OK) {
    centre_gpu_destroy(ctx);
    return rc;
  }
  ctx->own_stream = true;
  *out = ctx;
  return CENTRE_OK;
}

void centre_gpu_destroy(centre_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto &b : ctx->scratch)
    if (b.ptr) cudaFree(b.ptr);
  if (ctx->d_flag) cudaFree(ctx->d_flag);
  if (ctx->h_flag) cudaFreeHost(ctx->h_flag);
  for (void *t : ctx->d_fix)
    if (t) cudaFree(t);
  for (auto &t : ctx->timers) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->copy_in) cudaStreamSynchronize(ctx->copy_in), cudaStreamDestroy(ctx->copy_in);
  if (ctx->copy_out) cudaStreamSynchronize(ctx->copy_out), cudaStreamDestroy(ctx->copy_out);
  for (auto e : ctx->copy_ev)
    if (e) cudaEventDestroy(e);
  centre::batch_state_free(ctx);
  centre::screen_state_free(ctx);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int centre_gpu_set_stream(centre_ctx *ctx, void *stream) {
  if (!ctx) return CENTRE_E_ARG;
  if (ctx->own_stream && ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  return CENTRE_OK;
}

int centre_gpu_synchronize(centre_ctx *ctx) {
  if (!ctx) return CENTRE_E_ARG;
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

uint64_t centre_gpu_launch_count(const centre_ctx *ctx) { return ctx ? ctx->launches : 0; }

int centre_gpu_enable_timing(centre_ctx *ctx, int enable) {
  if (!ctx) return CENTRE_E_ARG;
  CENTRE_TRY(drain_timers(ctx));
  ctx->timing = enable != 0;
  for (int i = 0; i < CENTRE_TIMER_CLASSES; ++i) {
    ctx->timer_ms[i] = 0;
    ctx->timer_n[i] = 0;
  }
  return CENTRE_OK;
}

int centre_gpu_timer(centre_ctx *ctx, int which, double *ms, uint64_t *launches) {
  if (!ctx || which < 0 || which >= CENTRE_TIMER_CLASSES) return CENTRE_E_ARG;
  CENTRE_TRY(drain_timers(ctx));
  if (ms) *ms = ctx->timer_ms[which];
  if (launches) *launches = ctx->timer_n[which];
  return CENTRE_OK;
}

// ---- discretisation --------------------------------------------------------
int centre_gpu_discretize_dev(centre_ctx *ctx, int bat_type, const float *data, uint32_t ndof,
                              uint64_t nframes, const uint8_t *bin_schemes, uint32_t nschemes,
                              uint8_t bins_ref, int optimize_dih, uint8_t *bins,
                              double *extremes) {
  if (!ctx || !bin_schemes) return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  return launch_discretize(ctx, bat_type, data, ndof, nframes, bin_schemes, nschemes, bins_ref,
                           optimize_dih, bins, extremes);
}

// DOFs per chunk below which the discretiser's transfers are not split
static constexpr uint32_t kDiscChunkMinDofs = 64;

// The context's copy-in / copy-out streams and events, created on first use
// (not under stream capture: host-pointer entry points are never captured).
static int copy_streams(centre_ctx *ctx) {
  if (!ctx->copy_in)
    CENTRE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
  if (!ctx->copy_out)
    CENTRE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
  for (auto &e : ctx->copy_ev)
    if (!e) CENTRE_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return CENTRE_OK;
}

int centre_gpu_discretize(centre_ctx *ctx, int bat_type, const float *data, uint32_t ndof,
                          uint64_t nframes, const uint8_t *bin_schemes, uint32_t nschemes,
                          uint8_t bins_ref, int optimize_dih, uint8_t *bins, double *extremes) {
  if (!ctx || !data || !bins || !extremes || !bin_schemes)
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  if (ndof == 0 || nframes == 0) return CENTRE_OK;
  cudaSetDevice(ctx->device);
  int st = CENTRE_OK;
  const size_t nin = (size_t)ndof * nframes * 4;
  const size_t nbins = (size_t)ndof * nschemes * nframes;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, nin, &st);
  if (!d_in) return st;
  unsigned char *d_out = (unsigned char *)scratch(ctx, kSlotBins, nbins + 32 * (size_t)ndof + 256, &st);
  if (!d_out) return st;
  double *d_ext = reinterpret_cast<double *>(d_out + ((nbins + 255) & ~size_t(255)));
  // DOFs are binned independently: chunks of them stream in, are binned and
  // stream out on three streams, so the transfers overlap the kernels (and
  // each other) instead of running before and after them
  CENTRE_TRY(copy_streams(ctx));
  // Every path below ends by waiting for all three streams: copies that read
  // the caller's BAT or write its bins must not outlive the call, also when
  // a step fails part way.
  int rc = CENTRE_OK;
  auto step = [&](cudaError_t e, const char *what) {
    if (rc == CENTRE_OK && e != cudaSuccess) rc = check_cuda(ctx, e, what);
    return rc == CENTRE_OK;
  };
  // one flag for all chunks: the chunk launches do not reset it
  step(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream), "flag reset");
  // the first upload waits for work already queued on the context's stream
  // (it may still read the scratch the upload fills)
  step(cudaEventRecord(ctx->copy_ev[15], ctx->stream), "event");
  step(cudaStreamWaitEvent(ctx->copy_in, ctx->copy_ev[15], 0), "stream wait");
  const uint32_t nchunk = ndof >= 4 * kDiscChunkMinDofs ? 4u : 1u;
  const size_t fin = (size_t)nframes * 4, fout = (size_t)nschemes * nframes;
  for (uint32_t c = 0; c < nchunk && rc == CENTRE_OK; ++c) {
    const uint32_t d0 = (uint32_t)((uint64_t)ndof * c / nchunk);
    const uint32_t d1 = (uint32_t)((uint64_t)ndof * (c + 1) / nchunk);
    cudaEvent_t in_ev = ctx->copy_ev[2 * c], done_ev = ctx->copy_ev[2 * c + 1];
    if (!step(cudaMemcpyAsync(d_in + d0 * fin, data + (size_t)d0 * nframes, (d1 - d0) * fin,
                              cudaMemcpyHostToDevice, ctx->copy_in), "BAT upload") ||
        !step(cudaEventRecord(in_ev, ctx->copy_in), "event") ||
        !step(cudaStreamWaitEvent(ctx->stream, in_ev, 0), "stream wait"))
      break;
    rc = launch_discretize(ctx, bat_type, (const float *)(d_in + d0 * fin), d1 - d0, nframes,
                           bin_schemes, nschemes, bins_ref, optimize_dih, d_out + d0 * fout,
                           d_ext + 4 * (size_t)d0, false);
    if (rc != CENTRE_OK) break;
    if (!step(cudaEventRecord(done_ev, ctx->stream), "event") ||
        !step(cudaStreamWaitEvent(ctx->copy_out, done_ev, 0), "stream wait") ||
        !step(cudaMemcpyAsync(bins + d0 * fout, d_out + d0 * fout, (d1 - d0) * fout,
                              cudaMemcpyDeviceToHost, ctx->copy_out), "bins download") ||
        !step(cudaMemcpyAsync(extremes + 4 * (size_t)d0, d_ext + 4 * (size_t)d0,
                              32 * (size_t)(d1 - d0), cudaMemcpyDeviceToHost, ctx->copy_out),
              "extremes download"))
      break;
  }
  step(cudaStreamSynchronize(ctx->copy_in), "copy-in sync");
  step(cudaStreamSynchronize(ctx->stream), "stream sync");
  step(cudaStreamSynchronize(ctx->copy_out), "copy-out sync");
  if (rc != CENTRE_OK) return rc;
  return read_flag(ctx);
}

// ---- 1-D -------------------------------------------------------------------
int centre_gpu_entropy1d_dev(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                             const uint8_t *types, const uint8_t *bins, const double *extremes,
                             double *s1, uint64_t *freq) {
  if (!ctx) return CENTRE_E_ARG;
  cudaSetDevice(ctx->device);
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  int st = CENTRE_OK;
  double *d_l = (double *)scratch(ctx, kSlotAux3, sizeof(double) * ndof * E.nschemes * E.nsteps + 8,
                                  &st);
  if (!d_l) return st;
  CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  return launch_entropy1d(ctx, E, ndof, types, bins, extremes, s1,
                          reinterpret_cast<unsigned long long *>(freq), d_l);
}

int centre_gpu_entropy1d(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                         const uint8_t *types, const uint8_t *bins, const double *extremes,
                         double *s1, uint64_t *freq) {
  if (!ctx || !p || !types || !bins || !extremes || !s1)
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  if (ndof == 0) return CENTRE_OK;
  cudaSetDevice(ctx->device);
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  int st = CENTRE_OK;
  const size_t nb = (size_t)ndof * E.nschemes * E.nframes;
  const size_t per = (size_t)E.nests * E.nschemes * E.nsteps;
  const size_t nfreq = freq ? (size_t)ndof * E.nsteps * E.nbins_sum : 0;
  const size_t bytes = nb + 256 + 32 * (size_t)ndof + 256 + ndof + 256;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, bytes, &st);
  if (!d_in) return st;
  double *d_ext = reinterpret_cast<double *>(d_in + ((nb + 255) & ~size_t(255)));
  uint8_t *d_types = reinterpret_cast<uint8_t *>(d_ext + 4 * (size_t)ndof);
  double *d_s1 = (double *)scratch(ctx, kSlotOut, sizeof(double) * ndof * per + 8 * nfreq + 8, &st);
  if (!d_s1) return st;
  uint64_t *d_freq = freq ? reinterpret_cast<uint64_t *>(d_s1 + ndof * per) : nullptr;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_in, bins, nb, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_ext, extremes, 32 * (size_t)ndof, cudaMemcpyHostToDevice,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_types, types, ndof, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_TRY(centre_gpu_entropy1d_dev(ctx, p, ndof, d_types, d_in, d_ext, d_s1, d_freq));
  CENTRE_TRY(read_flag(ctx));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(s1, d_s1, sizeof(double) * ndof * per, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  if (freq)
    CENTRE_CUDA(ctx, cudaMemcpyAsync(freq, d_freq, 8 * nfreq, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

// ---- 2-D -------------------------------------------------------------------
int centre_gpu_entropy2d_dev(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                             const uint8_t *types, const uint8_t *bins, const double *extremes,
                             uint64_t npairs, const uint32_t *pairs, double *s2) {
  if (!ctx) return CENTRE_E_ARG;
  cudaSetDevice(ctx->device);
  return entropy2d_dev(ctx, p, ndof, types, bins, extremes, npairs, pairs, s2);
}

int centre_gpu_entropy2d(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                         const uint8_t *types, const uint8_t *bins, const double *extremes,
                         uint64_t npairs, const uint32_t *pairs, double *s2) {
  if (!ctx || !p || !types || !bins || !extremes || !s2)
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  const uint64_t np = pairs ? npairs : (uint64_t)ndof * (ndof ? ndof - 1 : 0) / 2;
  if (np == 0) return CENTRE_OK;
  int st = CENTRE_OK;
  const size_t nb = (size_t)ndof * E.nschemes * E.nframes;
  const size_t per = (size_t)E.nests * E.nschemes * E.nsteps;
  const size_t off_ext = (nb + 255) & ~size_t(255);
  const size_t off_ty = off_ext + ((32 * (size_t)ndof + 255) & ~size_t(255));
  const size_t off_pr = off_ty + (((size_t)ndof + 255) & ~size_t(255));
  const size_t bytes = off_pr + (pairs ? 8 * np : 0) + 16;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, bytes, &st);
  if (!d_in) return st;
  double *d_ext = reinterpret_cast<double *>(d_in + off_ext);
  uint8_t *d_types = d_in + off_ty;
  uint32_t *d_pairs = pairs ? reinterpret_cast<uint32_t *>(d_in + off_pr) : nullptr;
  double *d_s2 = (double *)scratch(ctx, kSlotOut, sizeof(double) * np * per, &st);
  if (!d_s2) return st;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_in, bins, nb, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_ext, extremes, 32 * (size_t)ndof, cudaMemcpyHostToDevice,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_types, types, ndof, cudaMemcpyHostToDevice, ctx->stream));
  if (pairs)
    CENTRE_CUDA(ctx, cudaMemcpyAsync(d_pairs, pairs, 8 * np, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_TRY(entropy2d_dev(ctx, p, ndof, d_types, d_in, d_ext, np, d_pairs, d_s2));
  CENTRE_TRY(read_flag(ctx));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(s2, d_s2, sizeof(double) * np * per, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

int centre_gpu_counts2d(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                        const uint8_t *bins, uint64_t npairs, const uint32_t *pairs,
                        uint64_t *freq) {
  if (!ctx || !p || !bins || !pairs || !freq) return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  if (npairs == 0) return CENTRE_OK;
  for (uint64_t q = 0; q < 2 * npairs; ++q)
    if (pairs[q] >= ndof) return set_error(ctx, CENTRE_E_ARG, "pair index >= ndof");
  int st = CENTRE_OK;
  const size_t nb = (size_t)ndof * E.nschemes * E.nframes;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, nb, &st);
  if (!d_in) return st;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_in, bins, nb, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  int nsq = 0;
  for (int s = 0; s < E.nschemes; ++s) nsq += E.schemes[s] * E.schemes[s];
  std::vector<unsigned> h;
  int off = 0;
  for (int s = 0; s < E.nschemes; ++s) {
    const int b = E.schemes[s];
    const size_t per_pair = (size_t)E.nsteps * b * b;
    unsigned *d_counts = (unsigned *)scratch(ctx, kSlotAux, 4 * per_pair * npairs, &st);
    if (!d_counts) return st;
    CENTRE_TRY(counts_chunk(ctx, E, s, ndof, d_in, pairs, 0, npairs, d_counts));
    CENTRE_TRY(read_flag(ctx));
    h.resize(per_pair * npairs);
    CENTRE_CUDA(ctx, cudaMemcpy(h.data(), d_counts, 4 * h.size(), cudaMemcpyDeviceToHost));
    for (uint64_t q = 0; q < npairs; ++q)
      for (int t = 0; t < E.nsteps; ++t)
        for (int c = 0; c < b * b; ++c)
          freq[(q * E.nsteps + t) * nsq + off + c] = h[(q * E.nsteps + t) * (size_t)b * b + c];
    off += b * b;
  }
  return CENTRE_OK;
}

int centre_gpu_pair_moments(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                            const uint8_t *bins, int scheme, uint64_t *clnc, uint32_t *nnz,
                            int *scale) {
  if (!ctx || !p || !bins || !clnc || !nnz || !scale)
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  if (scheme < 0 || scheme >= E.nschemes) return set_error(ctx, CENTRE_E_ARG, "bad scheme");
  *scale = E.fix_scale;
  if (ndof < 2) return CENTRE_OK;
  const uint64_t npairs = (uint64_t)ndof * (ndof - 1) / 2;
  int st = CENTRE_OK;
  const unsigned long long *d_fix = fix_table(ctx, E.fix_scale, &st);
  if (!d_fix) return st;
  const size_t nbb = (size_t)ndof * E.nschemes * E.nframes;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, nbb, &st);
  if (!d_in) return st;
  unsigned long long *d_m = (unsigned long long *)scratch(
      ctx, kSlotMoments, (sizeof(unsigned long long) + 4) * npairs * E.nsteps, &st);
  if (!d_m) return st;
  unsigned *d_z = reinterpret_cast<unsigned *>(d_m + npairs * E.nsteps);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_in, bins, nbb, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
  PairParams P;
  memset(&P, 0, sizeof(P));
  P.bins = d_in;
  P.nframes = E.nframes;
  P.step_size = E.step_size;
  P.ndof = ndof;
  P.nschemes = E.nschemes;
  P.scheme = scheme;
  P.nb = E.schemes[scheme];
  P.nsteps = E.nsteps;
  P.all_pairs = 1;
  P.fix_scale = E.fix_scale;
  P.want_nnz = 1;
  if (p->counts_form == CENTRE_COUNTS_TC) {
    if (!tc_supported(ctx, P.nb, E.nframes))
      return set_error(ctx, CENTRE_E_UNSUPPORTED, "tensor-core counts not supported here");
    CENTRE_TRY(launch_pairs_tc(ctx, P, d_fix, d_m, d_z));
  } else {
    if (!atomic_fits(P.nb))
      return set_error(ctx, CENTRE_E_UNSUPPORTED, "bin count too large for shared-memory counts");
    int ppair = atomic_pair_width(P.nb);
    int tile = 1;
    while ((tile + 1) * (tile + 1) <= ppair && tile < 4) ++tile;
    P.tile = tile;
    P.ntile = (ndof + tile - 1) / tile;
    CENTRE_TRY(launch_pairs_atomic(ctx, P, nullptr, P.ntile * (P.ntile + 1) / 2, d_fix, d_m, d_z,
                                   nullptr));
  }
  CENTRE_TRY(read_flag(ctx));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(clnc, d_m, sizeof(unsigned long long) * npairs * E.nsteps,
                                   cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(nnz, d_z, 4 * npairs * E.nsteps, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

// ---- scoring ---------------------------------------------------------------
static int score_impl(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                      const uint8_t *d_types, const uint8_t *h_types, const double *d_s1,
                      uint64_t npairs, const uint32_t *d_pairs, const double *d_s2, int build_tree,
                      double *d_mi, double *mie, double *mist, uint32_t *tree, uint32_t *ntree) {
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  ScoreParams S;
  memset(&S, 0, sizeof(S));
  S.ndof = ndof;
  S.all_pairs = d_pairs ? 0 : 1;
  S.npairs = d_pairs ? npairs : (uint64_t)ndof * (ndof ? ndof - 1 : 0) / 2;
  S.G = E.nests * E.nschemes * E.nsteps;
  S.sorted_types = 1;
  for (uint32_t d = 0; d < ndof; ++d) {
    const int t = h_types[d];
    if (t < 1 || t > 3) return set_error(ctx, CENTRE_E_ARG, "DOF type must be 1, 2 or 3");
    if (d > 0 && t < h_types[d - 1]) S.sorted_types = 0;
    if (S.type_count[t] == 0) S.type_start[t] = d;
    S.type_count[t]++;
  }
  if (build_tree && (!mist || !tree || !ntree))
    return set_error(ctx, CENTRE_E_ARG, "tree outputs required when build_tree is set");
  if (!mie) return set_error(ctx, CENTRE_E_ARG, "mie_sums is required");
  return launch_score(ctx, S, d_types, d_pairs, d_s1, d_s2, d_mi, mie, build_tree, mist, tree,
                      ntree);
}

int centre_gpu_score_dev(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                         const uint8_t *types, const double *s1, uint64_t npairs,
                         const uint32_t *pairs, const double *s2, int build_tree, double *mi,
                         double *mie_sums, double *mist_sums, uint32_t *tree, uint32_t *ntree) {
  if (!ctx) return CENTRE_E_ARG;
  cudaSetDevice(ctx->device);
  std::vector<uint8_t> ht(ndof);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(ht.data(), types, ndof, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return score_impl(ctx, p, ndof, types, ht.data(), s1, npairs, pairs, s2, build_tree, mi,
                    mie_sums, mist_sums, tree, ntree);
}

int centre_gpu_score(centre_ctx *ctx, const centre_entropy_params *p, uint32_t ndof,
                     const uint8_t *types, const double *s1, uint64_t npairs,
                     const uint32_t *pairs, const double *s2, int build_tree, double *mi,
                     double *mie_sums, double *mist_sums, uint32_t *tree, uint32_t *ntree) {
  if (!ctx || !p || !types || !s1 || !s2) return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  EntParams E;
  CENTRE_TRY(validate_params(ctx, p, &E));
  const uint64_t np = pairs ? npairs : (uint64_t)ndof * (ndof ? ndof - 1 : 0) / 2;
  const size_t G = (size_t)E.nests * E.nschemes * E.nsteps;
  int st = CENTRE_OK;
  const size_t off_s1 = 0;
  const size_t off_s2 = ((8 * ndof * G) + 255) & ~size_t(255);
  const size_t off_ty = off_s2 + (((8 * np * G) + 255) & ~size_t(255));
  const size_t off_pr = off_ty + ((ndof + 255) & ~size_t(255));
  const size_t bytes = off_pr + (pairs ? 8 * np : 0) + 16;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, bytes, &st);
  if (!d_in) return st;
  double *d_s1 = reinterpret_cast<double *>(d_in + off_s1);
  double *d_s2 = reinterpret_cast<double *>(d_in + off_s2);
  uint8_t *d_types = d_in + off_ty;
  uint32_t *d_pairs = pairs ? reinterpret_cast<uint32_t *>(d_in + off_pr) : nullptr;
  double *d_mi = nullptr;
  if (mi) {
    d_mi = (double *)scratch(ctx, kSlotOut, 8 * np * G, &st);
    if (!d_mi) return st;
  }
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_s1, s1, 8 * ndof * G, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_s2, s2, 8 * np * G, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_types, types, ndof, cudaMemcpyHostToDevice, ctx->stream));
  if (pairs)
    CENTRE_CUDA(ctx, cudaMemcpyAsync(d_pairs, pairs, 8 * np, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_TRY(score_impl(ctx, p, ndof, d_types, types, d_s1, np, d_pairs, d_s2, build_tree, d_mi,
                        mie_sums, mist_sums, tree, ntree));
  if (mi) {
    CENTRE_CUDA(ctx, cudaMemcpyAsync(mi, d_mi, 8 * np * G, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

int centre_gpu_discretize_vmkde(centre_ctx *ctx, const float *data, uint32_t ndof,
                                uint64_t nframes, uint8_t nmaxconf, double kappa,
                                uint32_t sdo_nstep, double sdo_conv, uint32_t sdo_niter,
                                uint8_t *bins, double *minima, uint8_t *nfound) {
  if (!ctx || !data || !bins || !minima || !nfound)
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  if (ndof == 0 || nframes == 0) return CENTRE_OK;
  cudaSetDevice(ctx->device);
  int st = CENTRE_OK;
  const size_t nin = (size_t)ndof * nframes * 4;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, nin, &st);
  if (!d_in) return st;
  uint8_t *d_bins = (uint8_t *)scratch(ctx, kSlotBins, (size_t)ndof * nframes, &st);
  if (!d_bins) return st;
  const size_t nw = vmkde_work_doubles(ndof);
  double *d_work = (double *)scratch(ctx, kSlotAux,
                                     sizeof(double) * (nw + (size_t)ndof * nmaxconf) + ndof + 16,
                                     &st);
  if (!d_work) return st;
  double *d_min = d_work + nw;
  uint8_t *d_nf = reinterpret_cast<uint8_t *>(d_min + (size_t)ndof * nmaxconf);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_in, data, nin, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_TRY(launch_vmkde(ctx, (const float *)d_in, ndof, nframes, nmaxconf, kappa, sdo_nstep,
                          sdo_conv, sdo_niter, d_bins, d_min, d_nf, d_work));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(bins, d_bins, (size_t)ndof * nframes, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(minima, d_min, sizeof(double) * ndof * nmaxconf,
                                   cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(nfound, d_nf, ndof, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

int centre_gpu_df_exp_eval(centre_ctx *ctx, const double *y, uint64_t n, double *out) {
  if (!ctx || ((!y || !out) && n)) return set_error(ctx, CENTRE_E_ARG, "null argument");
  if (n == 0) return CENTRE_OK;
  cudaSetDevice(ctx->device);
  int st = CENTRE_OK;
  double *d = (double *)scratch(ctx, kSlotAux, sizeof(double) * 2 * n, &st);
  if (!d) return st;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d, y, sizeof(double) * n, cudaMemcpyHostToDevice,
                                   ctx->stream));
  CENTRE_TRY(launch_df_exp_eval(ctx, d, n, d + n));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

int centre_gpu_discretize_gridkde_dev(centre_ctx *ctx, int bat_type, const float *data,
                                      uint32_t ndof, uint64_t nframes, uint32_t ngrid,
                                      double kappa, uint8_t *bins, double *minima,
                                      uint8_t *nmin, uint8_t *nbins) {
  if (!ctx || ((!data || !bins || !minima || !nmin || !nbins) && ndof && nframes))
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  cudaSetDevice(ctx->device);
  int st = CENTRE_OK;
  void *d_work = scratch(ctx, kSlotAux, gridkde_work_bytes(ndof) + 16, &st);
  if (!d_work) return st;
  CENTRE_TRY(launch_gridkde(ctx, bat_type, data, ndof, nframes, (int)ngrid, kappa, bins, minima,
                            nmin, nbins, d_work));
  return read_flag(ctx);
}

int centre_gpu_discretize_gridkde(centre_ctx *ctx, int bat_type, const float *data,
                                  uint32_t ndof, uint64_t nframes, uint32_t ngrid, double kappa,
                                  uint8_t *bins, double *minima, uint8_t *nmin, uint8_t *nbins) {
  if (!ctx || !data || !bins || !minima || !nmin || !nbins)
    return set_error(ctx, CENTRE_E_ARG, "null argument");
  if (ndof == 0 || nframes == 0) return CENTRE_OK;
  cudaSetDevice(ctx->device);
  int st = CENTRE_OK;
  const size_t nin = (size_t)ndof * nframes * 4;
  unsigned char *d_in = (unsigned char *)scratch(ctx, kSlotIn, nin, &st);
  if (!d_in) return st;
  uint8_t *d_bins = (uint8_t *)scratch(ctx, kSlotBins, (size_t)ndof * nframes, &st);
  if (!d_bins) return st;
  const size_t nmn = sizeof(double) * (size_t)ndof * ngrid;
  unsigned char *d_out = (unsigned char *)scratch(ctx, kSlotOut, nmn + 2 * (size_t)ndof + 16, &st);
  if (!d_out) return st;
  double *d_min = reinterpret_cast<double *>(d_out);
  uint8_t *d_nmin = d_out + nmn;
  uint8_t *d_nb = d_nmin + ndof;
  void *d_work = scratch(ctx, kSlotAux, gridkde_work_bytes(ndof) + 16, &st);
  if (!d_work) return st;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(d_in, data, nin, cudaMemcpyHostToDevice, ctx->stream));
  CENTRE_TRY(launch_gridkde(ctx, bat_type, (const float *)d_in, ndof, nframes, (int)ngrid, kappa,
                            d_bins, d_min, d_nmin, d_nb, d_work));
  CENTRE_TRY(read_flag(ctx));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(bins, d_bins, (size_t)ndof * nframes, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(minima, d_min, nmn, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(nmin, d_nmin, ndof, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(nbins, d_nb, ndof, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CENTRE_OK;
}

}  // extern "C"
