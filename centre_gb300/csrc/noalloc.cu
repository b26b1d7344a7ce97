// noalloc.cu -- 2-D joint entropies of all pairs without allocating memory.
//
// Some callers cannot call cudaMalloc: plug-ins living inside an application
// whose memory manager owns every device byte and forbids foreign
// allocations, and latency-critical loops where an allocation could stall on
// a device-wide synchronisation.  For them centre_gpu_entropy2d_static()
// computes what centre_gpu_entropy2d_dev()
// computes for the all-pairs case, with every piece of scratch memory taken
// from one file-scope device array of fixed size (kStaticScratchBytes, 16
// MiB) instead of the context's allocator.  The caller passes its inputs and
// outputs as device pointers and a stream; no context is needed.
//
// The array exists once per device for the life of the process and every
// call shares it: the first call on a device records the array's address
// (cudaGetSymbolAddress, with that device current); a call fills the
// fixed-point c*ln(c) table kept at the array's start when its moment scale
// (which follows from the frame count) differs from the previous call's, and
// reuses it otherwise.  Calls that overlap on the GPU (different streams, or
// different host threads on one device) race on the array and must be
// serialised by the caller.
#include <cmath>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {
namespace {

constexpr size_t kStaticScratchBytes = 16u << 20;   // 16 MiB per device
constexpr int kMaxDevices = 64;

// Scratch layout: [error flag | c ln c table | 1-D entropies | L sums |
// log table | pair moments (sum c ln c) | pair non-empty counts].
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr size_t kFlagBytes = 256;
constexpr size_t kTableBytes = sizeof(unsigned long long) * kTabGlobal;   // 512 KiB

std::mutex g_setup_mutex;
unsigned char *g_base[kMaxDevices] = {};   // device address of the array
int g_scale[kMaxDevices];                  // moment scale of the table in it (-1: none)

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// With the device current: the array's device address (recorded on the
// first call on the device) and the c ln c table at its start for moment
// scale s (filled, on the call's stream, when the previous call on the device
// used another scale).  Returns 0 or a CENTRE_E_* status.
int setup_device(int dev, cudaStream_t stream, int s, unsigned char **base) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_base[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || p == nullptr)
      return CENTRE_E_CUDA;
    g_base[dev] = static_cast<unsigned char *>(p);
    g_scale[dev] = -1;
  }
  unsigned char *b = g_base[dev];
  if (g_scale[dev] != s) {
    centre_ctx c;
    c.device = dev;
    c.stream = stream;
    if (fill_fix_table(&c, reinterpret_cast<unsigned long long *>(b + kFlagBytes), s) !=
        CENTRE_OK)
      return CENTRE_E_CUDA;
    g_scale[dev] = s;
  }
  *base = b;
  return CENTRE_OK;
}

}  // namespace
}  // namespace centre

using namespace centre;

extern "C" int centre_gpu_entropy2d_static(const centre_entropy_params *p, uint32_t ndof,
                                           const uint8_t *types, const uint8_t *bins,
                                           const double *extremes, double *s2, void *stream) {
  if (!p || !types || !bins || !extremes || !s2) return CENTRE_E_ARG;
  if (p->nsteps == 0 || p->nschemes == 0 || p->nschemes > kMaxSchemes || p->nestimators == 0 ||
      p->nestimators > 4 || p->nframes < p->nsteps || p->nframes > kMaxFrames)
    return CENTRE_E_ARG;
  if (p->counts_form == CENTRE_COUNTS_TC) return CENTRE_E_UNSUPPORTED;
  EntParams E;
  memset(&E, 0, sizeof(E));
  E.nframes = p->nframes;
  E.step_size = p->nframes / p->nsteps;
  E.nsteps = p->nsteps;
  E.nschemes = p->nschemes;
  E.nests = p->nestimators;
  E.jacobian = p->jacobian ? 1 : 0;
  E.kde = p->kde ? 1 : 0;
  int off = 0;
  for (int s = 0; s < p->nschemes; ++s) {
    if (p->bin_schemes[s] == 0) return CENTRE_E_ARG;
    if (pair_tile_for(p->bin_schemes[s]) < 1) return CENTRE_E_UNSUPPORTED;
    E.schemes[s] = p->bin_schemes[s];
    E.scheme_off[s] = off;
    off += p->bin_schemes[s];
  }
  E.nbins_sum = off;
  for (int e = 0; e < p->nestimators; ++e) {
    // the factorised (integer-moment) estimators only: ML and Miller-Madow
    if (p->estimators[e] > CENTRE_MM) return CENTRE_E_UNSUPPORTED;
    E.ests[e] = p->estimators[e];
  }
  E.fix_scale = moment_scale(E.step_size * E.nsteps);
  E.fix_inv = ldexp(1.0, -E.fix_scale);
  if (ndof < 2) return CENTRE_OK;

  // sizes against the fixed array: reject what does not fit
  const uint64_t npairs = (uint64_t)ndof * (ndof - 1) / 2;
  const uint64_t per1 = (uint64_t)E.nests * E.nschemes * E.nsteps;
  const size_t b_s1 = align256(sizeof(double) * ndof * per1);
  const size_t b_l = align256(sizeof(double) * ndof * E.nschemes * E.nsteps);
  const size_t b_logw = align256(sizeof(double) * ((uint64_t)ndof * E.nschemes + E.nsteps));
  const size_t b_mom = align256(sizeof(unsigned long long) * npairs * E.nsteps);
  const size_t b_nnz = align256(sizeof(unsigned) * npairs * E.nsteps);
  const size_t need = kFlagBytes + kTableBytes + b_s1 + b_l + b_logw + b_mom + b_nnz;
  if (need > kStaticScratchBytes) return CENTRE_E_ARG;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CENTRE_E_NODEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char *base = nullptr;
  int rc = setup_device(dev, st, E.fix_scale, &base);
  if (rc != CENTRE_OK) return rc;

  int *d_flag = reinterpret_cast<int *>(base);
  const unsigned long long *d_fix = reinterpret_cast<const unsigned long long *>(base + kFlagBytes);
  size_t o = kFlagBytes + kTableBytes;
  double *d_s1 = reinterpret_cast<double *>(base + o);
  o += b_s1;
  double *d_lsum = reinterpret_cast<double *>(base + o);
  o += b_l;
  double *d_logw = reinterpret_cast<double *>(base + o);
  o += b_logw;
  unsigned long long *d_mom = reinterpret_cast<unsigned long long *>(base + o);
  o += b_mom;
  unsigned *d_nnz = reinterpret_cast<unsigned *>(base + o);

  // a context on the stack: it carries the stream and the flag only and is
  // never given to anything that allocates
  centre_ctx c;
  c.device = dev;
  c.stream = st;
  c.d_flag = d_flag;
  // the array keeps the previous call's contents: the error flag must start
  // at zero (moments, sums and tables below are overwritten before use)
  if (cudaMemsetAsync(d_flag, 0, sizeof(int), st) != cudaSuccess) return CENTRE_E_CUDA;
  if ((rc = launch_entropy1d(&c, E, ndof, types, bins, extremes, d_s1, nullptr, d_lsum)) != CENTRE_OK)
    return rc;
  for (int s = 0; s < E.nschemes; ++s) {
    const int nb = E.schemes[s];
    const int width = pair_tile_for(nb);
    int tile = 1;
    while ((tile + 1) * (tile + 1) <= width && tile < 4) ++tile;
    PairParams P;
    memset(&P, 0, sizeof(P));
    P.bins = bins;
    P.nframes = E.nframes;
    P.step_size = E.step_size;
    P.ndof = ndof;
    P.nschemes = E.nschemes;
    P.scheme = s;
    P.nb = nb;
    P.nsteps = E.nsteps;
    P.all_pairs = 1;
    P.tile = tile;
    P.ntile = (ndof + tile - 1) / tile;
    P.fix_scale = E.fix_scale;
    for (int e = 0; e < E.nests; ++e)
      if (E.ests[e] == CENTRE_MM) P.want_nnz = 1;
    if ((rc = launch_pairs_atomic(&c, P, nullptr, P.ntile * (P.ntile + 1) / 2, d_fix, d_mom, d_nnz,
                                  nullptr)) != CENTRE_OK)
      return rc;
    if ((rc = launch_finalize2d_into(&c, E, s, ndof, extremes, d_lsum, d_mom, d_nnz, npairs, d_logw,
                                     s2)) != CENTRE_OK)
      return rc;
  }
  int h_flag = 0;
  if (cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return CENTRE_E_CUDA;
  return flag_status(h_flag);
}
