// score.cu -- mutual information, MIE sums and the MIST spanning tree.
//
// Reference: EntropyScorer::run (src/EntropyScorer.cpp:287-866),
// getMaxMI2D (src/Convergance.cpp:183-194), boruvkaMST (src/Centre.cpp:5-115).
//
// Sums are reduced in a fixed order (per-thread strided partials, then a
// fixed tree over threads and CTAs), so they are identical from run to run.
//
// The spanning tree is Boruvka's algorithm on the GPU over all (estimator,
// scheme, step) graphs at once.  The reference lets every component keep the
// first edge, in its edge-list order, of strictly largest MI; that is the
// strict total order (MI descending, edge rank ascending), under which the
// maximum spanning tree is unique, so any Boruvka schedule that picks per
// component the maximum under the same order returns the reference's tree.
// Each round takes the maximum MI key per component with 64-bit atomicMax,
// then the smallest edge rank among edges carrying that key with atomicMin,
// hooks components along the picked edges (a mutual pick is added once) and
// compresses the component labels by pointer jumping.
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {
namespace {

constexpr int kCols = CENTRE_SUMS_COLS;

// block index of a DOF-type pair, in the reference's CSV column order:
// 0 B/B, 1 A/A, 2 D/D, 3 B/A, 4 B/D, 5 A/D; -1 when a type is unknown
__device__ __forceinline__ int block_of(int a, int b) {
  if (a > b) {
    int t = a;
    a = b;
    b = t;
  }
  if (a == 1 && b == 1) return 0;
  if (a == 2 && b == 2) return 1;
  if (a == 3 && b == 3) return 2;
  if (a == 1 && b == 2) return 3;
  if (a == 1 && b == 3) return 4;
  if (a == 2 && b == 3) return 5;
  return -1;
}

__device__ __forceinline__ void pair_of(const ScoreParams &S, const uint32_t *pairs, uint64_t p,
                                        uint32_t &i, uint32_t &j) {
  if (!S.all_pairs) {
    i = pairs[2 * p];
    j = pairs[2 * p + 1];
    return;
  }
  tri_pair(p, S.ndof, i, j);
}

// Rank of a pair in the reference's edge list: blocks B/B, B/A, B/D, A/A,
// A/D, D/D (src/EntropyScorer.cpp:675-741), row-major inside a block.  Used
// in all-pairs mode with types sorted bonds, angles, torsions; an explicit
// pair list is already in edge order, its rank is its position.
__device__ __forceinline__ uint64_t edge_rank(const ScoreParams &S, uint64_t p, uint32_t i,
                                              uint32_t j, const uint8_t *types) {
  if (!S.all_pairs || !S.sorted_types) return p;
  const int ti = types[i], tj = types[j];
  const uint64_t nb = S.type_count[1], na = S.type_count[2], nd = S.type_count[3];
  const uint64_t sz_bb = nb * (nb ? nb - 1 : 0) / 2, sz_ba = nb * na, sz_bd = nb * nd;
  const uint64_t sz_aa = na * (na ? na - 1 : 0) / 2, sz_ad = na * nd;
  const uint64_t li = i - S.type_start[ti], lj = j - S.type_start[tj];
  auto tri = [](uint64_t a, uint64_t b, uint64_t m) { return a * m - a * (a + 1) / 2 + (b - a - 1); };
  if (ti == 1 && tj == 1) return tri(li, lj, nb);
  if (ti == 1 && tj == 2) return sz_bb + li * na + lj;
  if (ti == 1 && tj == 3) return sz_bb + sz_ba + li * nd + lj;
  if (ti == 2 && tj == 2) return sz_bb + sz_ba + sz_bd + tri(li, lj, na);
  if (ti == 2 && tj == 3) return sz_bb + sz_ba + sz_bd + sz_aa + li * nd + lj;
  return sz_bb + sz_ba + sz_bd + sz_aa + sz_ad + tri(li, lj, nd);
}

// MI per (pair, g) and per-CTA partial block sums.  blockDim = G * k, each
// thread owns one g and strides over the CTA's pair chunk.
__global__ void mi_sums_kernel(const __grid_constant__ ScoreParams S, const uint8_t *__restrict__ types,
                               const uint32_t *__restrict__ pairs, const double *__restrict__ s1,
                               const double *__restrict__ s2, double *__restrict__ mi,
                               double *__restrict__ partial, uint64_t chunk) {
  const int G = S.G;
  const int k = blockDim.x / G;
  const int g = threadIdx.x % G, lane = threadIdx.x / G;
  double acc[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) acc[q] = 0.0;
  const uint64_t p0 = (uint64_t)blockIdx.x * chunk;
  const uint64_t p1 = min(S.npairs, p0 + chunk);
  if (lane < k) {
    for (uint64_t p = p0 + lane; p < p1; p += k) {
      uint32_t i, j;
      pair_of(S, pairs, p, i, j);
      const double v2 = s2[p * G + g];
      const double m = s1[(uint64_t)i * G + g] + s1[(uint64_t)j * G + g] - v2;
      if (mi) mi[p * G + g] = m;
      const int b = block_of(types[i], types[j]);
      if (b >= 0) {
        acc[2 * b] += v2;
        acc[2 * b + 1] += m;
      }
    }
  }
  extern __shared__ double red[];  // [blockDim][12]
  for (int q = 0; q < 12; ++q) red[threadIdx.x * 12 + q] = acc[q];
  __syncthreads();
  // thread (g, q) sums over lanes in order
  for (int idx = threadIdx.x; idx < G * 12; idx += blockDim.x) {
    const int gg = idx / 12, q = idx % 12;
    double s = 0.0;
    for (int l = 0; l < k; ++l) s += red[(l * G + gg) * 12 + q];
    partial[((uint64_t)blockIdx.x * G + gg) * 12 + q] = s;
  }
}

// Final sums: per g the 1-D sums by type and the CTA partials in order.
__global__ void sums_final_kernel(const __grid_constant__ ScoreParams S,
                                  const uint8_t *__restrict__ types, const double *__restrict__ s1,
                                  const double *__restrict__ partial, int nchunks,
                                  double *__restrict__ out) {
  const int g = blockIdx.x;
  __shared__ double r1[3][256];
  double a[3] = {0, 0, 0};
  for (uint32_t d = threadIdx.x; d < S.ndof; d += blockDim.x) {
    int t = types[d];
    if (t >= 1 && t <= 3) a[t - 1] += s1[(uint64_t)d * S.G + g];
  }
  for (int q = 0; q < 3; ++q) r1[q][threadIdx.x] = a[q];
  __syncthreads();
  if (threadIdx.x < 12) {
    const int q = threadIdx.x;
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += partial[((uint64_t)c * S.G + g) * 12 + q];
    // columns: 3 + 2*block + {0: S2, 1: I2}
    out[(uint64_t)g * kCols + 3 + q] = s;
  }
  if (threadIdx.x == 0) {
    double t3[3];
    for (int q = 0; q < 3; ++q) {
      double s = 0.0;
      for (int l = 0; l < (int)blockDim.x; ++l) s += r1[q][l];
      t3[q] = s;
      out[(uint64_t)g * kCols + q] = s;
    }
    out[(uint64_t)g * kCols + 15] = t3[0] + t3[1] + t3[2];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // doublet = singlet - sum of I2 (src/EntropyScorer.cpp:567)
    double d = out[(uint64_t)g * kCols + 15];
    const int i2[6] = {4, 6, 8, 10, 12, 14};
    for (int q = 0; q < 6; ++q) d -= out[(uint64_t)g * kCols + i2[q]];
    out[(uint64_t)g * kCols + 16] = d;
  }
}

// ---- Boruvka -------------------------------------------------------------
__global__ void mst_reset_kernel(unsigned long long *bestkey, unsigned long long *bestedge,
                                 uint64_t n) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    bestkey[i] = 0ull;
    bestedge[i] = ~0ull;
  }
}

__global__ void mst_init_kernel(uint32_t *comp, uint32_t V, uint64_t n) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) comp[i] = (uint32_t)(i % V);
}

// One thread per pair, looping over the G graphs: the pair's DOFs and edge
// rank are found once (no 64-bit division or conversion per graph) and its
// G MI values are contiguous.
template <int kPass>
__global__ void mst_pick_kernel(const __grid_constant__ ScoreParams S, const uint8_t *__restrict__ types,
                                const uint32_t *__restrict__ pairs, const double *__restrict__ mi,
                                const uint32_t *__restrict__ comp, unsigned long long *bestkey,
                                unsigned long long *bestedge) {
  const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (p >= S.npairs) return;
  uint32_t i, j;
  pair_of(S, pairs, p, i, j);
  const unsigned long long r = (kPass == 1) ? edge_rank(S, p, i, j, types) : 0ull;
  const double *m = mi + p * S.G;
  for (int g = 0; g < S.G; ++g) {
    const uint32_t *cg_ = comp + (uint64_t)g * S.ndof;
    const uint32_t ci = cg_[i], cj = cg_[j];
    if (ci == cj) continue;
    const unsigned long long key = order_key(m[g]);
    unsigned long long *bk = bestkey + (uint64_t)g * S.ndof;
    if (kPass == 0) {
      if (key > bk[ci]) atomicMax(&bk[ci], key);
      if (key > bk[cj]) atomicMax(&bk[cj], key);
    } else {
      unsigned long long *be = bestedge + (uint64_t)g * S.ndof;
      if (key == bk[ci]) atomicMin(&be[ci], r);
      if (key == bk[cj]) atomicMin(&be[cj], r);
    }
  }
}

// Map winning edge ranks back to pair indices and hook components.
__global__ void mst_hook_kernel(const __grid_constant__ ScoreParams S, const uint8_t *__restrict__ types,
                                const uint32_t *__restrict__ pairs, const double *__restrict__ mi,
                                uint32_t *comp, uint32_t *parent,
                                const unsigned long long *__restrict__ bestkey,
                                const unsigned long long *__restrict__ bestedge,
                                unsigned long long *winpair, uint32_t *tree, uint32_t *ntree,
                                uint32_t cap, unsigned *added) {
  // pass A (one thread per pair, every graph): record the pair index of
  // each winning rank
  const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (p >= S.npairs) return;
  uint32_t i, j;
  pair_of(S, pairs, p, i, j);
  const unsigned long long r = edge_rank(S, p, i, j, types);
  for (int g = 0; g < S.G; ++g) {
    const uint32_t *cg_ = comp + (uint64_t)g * S.ndof;
    const uint32_t ci = cg_[i], cj = cg_[j];
    if (ci == cj) continue;
    const unsigned long long *be = bestedge + (uint64_t)g * S.ndof;
    unsigned long long *wp = winpair + (uint64_t)g * S.ndof;
    if (be[ci] == r) wp[ci] = p;
    if (be[cj] == r) wp[cj] = p;
  }
}

__global__ void mst_link_kernel(const __grid_constant__ ScoreParams S, const uint32_t *__restrict__ pairs,
                                const uint32_t *__restrict__ comp, uint32_t *parent,
                                const unsigned long long *__restrict__ bestedge,
                                const unsigned long long *__restrict__ winpair, uint32_t *tree,
                                uint32_t *ntree, uint32_t cap, unsigned *added) {
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)S.G * S.ndof) return;
  const int g = (int)(idx / S.ndof);
  const uint32_t v = (uint32_t)(idx % S.ndof);
  const uint32_t *cg_ = comp + (uint64_t)g * S.ndof;
  if (cg_[v] != v) return;  // not a component root
  const unsigned long long *be = bestedge + (uint64_t)g * S.ndof;
  if (be[v] == ~0ull) return;
  const uint64_t p = winpair[(uint64_t)g * S.ndof + v];
  uint32_t i, j;
  pair_of(S, pairs, p, i, j);
  const uint32_t o = (cg_[i] == v) ? cg_[j] : cg_[i];
  // mutual pick: the smaller root stays, the larger one hooks and records
  if (be[o] == be[v] && v < o) return;
  parent[(uint64_t)g * S.ndof + v] = o;
  const uint32_t slot = atomicAdd(&ntree[g], 1u);
  if (slot < cap) tree[(uint64_t)g * (cap + 1) + slot] = (uint32_t)p;
  atomicAdd(added, 1u);
}

__global__ void mst_jump_kernel(const __grid_constant__ ScoreParams S, uint32_t *comp,
                                const uint32_t *parent) {
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)S.G * S.ndof) return;
  const int g = (int)(idx / S.ndof);
  const uint32_t *pg = parent + (uint64_t)g * S.ndof;
  uint32_t v = comp[idx];
  // follow the hooks to the new root (chains are acyclic, depth < ndof)
  for (uint32_t it = 0; it < S.ndof && pg[v] != v; ++it) v = pg[v];
  comp[idx] = v;
}

__global__ void mst_parent_sync_kernel(const __grid_constant__ ScoreParams S, const uint32_t *comp,
                                       uint32_t *parent) {
  // after a round every vertex's parent is its root
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)S.G * S.ndof) return;
  parent[idx] = comp[idx];
}

__global__ void mst_gather_kernel(const __grid_constant__ ScoreParams S,
                                  const uint32_t *__restrict__ pairs, const double *__restrict__ mi,
                                  const uint32_t *__restrict__ tree, const uint32_t *__restrict__ ntree,
                                  uint32_t cap, double *__restrict__ w, uint32_t *__restrict__ ij) {
  const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)S.G * (cap + 1)) return;
  const int g = (int)(idx / (cap + 1));
  const uint32_t e = (uint32_t)(idx % (cap + 1));
  if (e >= min(ntree[g], cap)) return;
  const uint64_t p = tree[idx];
  uint32_t i, j;
  pair_of(S, pairs, p, i, j);
  w[idx] = mi[p * S.G + g];
  ij[2 * idx] = i;
  ij[2 * idx + 1] = j;
}

// MIST rows on the device: tree MI summed per type block, S2 = S1 - sum
// (src/EntropyScorer.cpp:769-799).  One CTA per graph.
__global__ void mist_sums_kernel(const __grid_constant__ ScoreParams S,
                                 const uint8_t *__restrict__ types,
                                 const uint32_t *__restrict__ pairs,
                                 const double *__restrict__ mi, const uint32_t *__restrict__ tree,
                                 const uint32_t *__restrict__ ntree, uint32_t cap,
                                 const double *__restrict__ mie, double *__restrict__ mist) {
  const int g = blockIdx.x;
  __shared__ double blk[6][256];
  double a[6] = {0, 0, 0, 0, 0, 0};
  const uint32_t nt = min(ntree[g], cap);
  for (uint32_t e = threadIdx.x; e < nt; e += blockDim.x) {
    const uint64_t p = tree[(uint64_t)g * (cap + 1) + e];
    uint32_t i, j;
    pair_of(S, pairs, p, i, j);
    const int b = block_of(types[i], types[j]);
    if (b >= 0) a[b] += mi[p * S.G + g];
  }
  for (int q = 0; q < 6; ++q) blk[q][threadIdx.x] = a[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    const double *row = mie + (uint64_t)g * kCols;
    double *out = mist + (uint64_t)g * kCols;
    for (int c = 0; c < kCols; ++c) out[c] = row[c];
    double d = row[15];
    for (int q = 0; q < 6; ++q) {
      double sum = 0.0;
      for (int l = 0; l < (int)blockDim.x; ++l) sum += blk[q][l];
      out[4 + 2 * q] = sum;
      d -= sum;
    }
    out[16] = d;
  }
}

}  // namespace

size_t score_scratch_bytes(const ScoreParams &S, bool tree) {
  const int G = S.G;
  const uint64_t chunk = 4096;
  const uint64_t nchunks = std::max<uint64_t>(1, (S.npairs + chunk - 1) / chunk);
  size_t b = sizeof(double) * nchunks * G * 12 + 256;
  if (tree) {
    const uint64_t GV = (uint64_t)G * S.ndof;
    const uint64_t cap = S.ndof > 0 ? S.ndof - 1 : 0;
    b += sizeof(uint32_t) * GV * 2 + sizeof(unsigned long long) * GV * 3 +
         sizeof(uint32_t) * ((uint64_t)G * (cap + 1) + G + 1) + 256;
  }
  return b;
}

// Everything on the stream, no host synchronisation (capturable): MI, the
// MIE rows into d_mie, and with d_mist the spanning tree after a fixed
// number of Boruvka rounds (each round at least halves the component count,
// so ceil(log2 V) + 1 rounds always finish; extra rounds change nothing) and
// the MIST rows into d_mist.
int launch_score_async(centre_ctx *ctx, const ScoreParams &S, const uint8_t *d_types,
                       const uint32_t *d_pairs, const double *d_s1, const double *d_s2,
                       double *d_mi, double *d_mie, double *d_mist, void *d_scratch) {
  const int G = S.G;
  if (G <= 0 || G > 256)
    return set_error(ctx, CENTRE_E_UNSUPPORTED, "estimators*schemes*steps must be <= 256");
  const int k = std::max(1, 256 / G);
  const int threads = G * k;
  const uint64_t chunk = 4096;
  const int nchunks = (int)std::max<uint64_t>(1, (S.npairs + chunk - 1) / chunk);
  double *d_part = reinterpret_cast<double *>(d_scratch);
  KernelTimer kt(ctx, CENTRE_TIMER_SCORE);
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_part, 0, sizeof(double) * (size_t)nchunks * G * 12, ctx->stream));
  if (S.npairs) {
    mi_sums_kernel<<<nchunks, threads, sizeof(double) * threads * 12, ctx->stream>>>(
        S, d_types, d_pairs, d_s1, d_s2, d_mi, d_part, chunk);
    ctx->launches++;
  }
  sums_final_kernel<<<G, 256, 0, ctx->stream>>>(S, d_types, d_s1, d_part, nchunks, d_mie);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  if (!d_mist) return CENTRE_OK;
  unsigned char *base = reinterpret_cast<unsigned char *>(d_scratch) +
                        ((sizeof(double) * (size_t)nchunks * G * 12 + 255) & ~size_t(255));
  const uint64_t GV = (uint64_t)G * S.ndof;
  const uint32_t cap = S.ndof > 0 ? S.ndof - 1 : 0;
  uint32_t *comp = reinterpret_cast<uint32_t *>(base);
  uint32_t *parent = comp + GV;
  unsigned long long *bestkey = reinterpret_cast<unsigned long long *>(parent + GV);
  unsigned long long *bestedge = bestkey + GV;
  unsigned long long *winpair = bestedge + GV;
  uint32_t *tree = reinterpret_cast<uint32_t *>(winpair + GV);
  uint32_t *ntree = tree + (uint64_t)G * (cap + 1);
  unsigned *added = ntree + G;
  const unsigned TB = 256;
  auto blocks = [&](uint64_t n) { return (unsigned)((n + TB - 1) / TB); };
  mst_init_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(comp, S.ndof, GV);
  mst_init_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(parent, S.ndof, GV);
  ctx->launches += 2;
  CENTRE_CUDA(ctx, cudaMemsetAsync(ntree, 0, sizeof(uint32_t) * (G + 1), ctx->stream));
  const uint64_t PG = S.npairs * (uint64_t)G;
  int rounds = 1;
  while ((1u << (rounds - 1)) < S.ndof) ++rounds;
  for (int r = 0; r < rounds && PG > 0; ++r) {
    mst_reset_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(bestkey, bestedge, GV);
    mst_pick_kernel<0><<<blocks(S.npairs), TB, 0, ctx->stream>>>(S, d_types, d_pairs, d_mi,
                                                                 comp, bestkey, bestedge);
    mst_pick_kernel<1><<<blocks(S.npairs), TB, 0, ctx->stream>>>(S, d_types, d_pairs, d_mi,
                                                                 comp, bestkey, bestedge);
    mst_hook_kernel<<<blocks(S.npairs), TB, 0, ctx->stream>>>(S, d_types, d_pairs, d_mi, comp, parent,
                                                        bestkey, bestedge, winpair, tree, ntree,
                                                        cap, added);
    mst_link_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(S, d_pairs, comp, parent, bestedge,
                                                        winpair, tree, ntree, cap, added);
    mst_jump_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(S, comp, parent);
    mst_parent_sync_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(S, comp, parent);
    ctx->launches += 7;
  }
  mist_sums_kernel<<<G, 256, 0, ctx->stream>>>(S, d_types, d_pairs, d_mi, tree, ntree, cap, d_mie,
                                               d_mist);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  return CENTRE_OK;
}

int launch_score(centre_ctx *ctx, const ScoreParams &S, const uint8_t *d_types,
                 const uint32_t *d_pairs, const double *d_s1, const double *d_s2, double *d_mi,
                 double *h_mie, int build_tree, double *h_mist, uint32_t *h_tree,
                 uint32_t *h_ntree) {
  const int G = S.G;
  if (G <= 0 || G > 256)
    return set_error(ctx, CENTRE_E_UNSUPPORTED, "estimators*schemes*steps must be <= 256");
  int st = CENTRE_OK;
  const int k = std::max(1, 256 / G);
  const int threads = G * k;
  const uint64_t chunk = 4096;
  const int nchunks = (int)std::max<uint64_t>(1, (S.npairs + chunk - 1) / chunk);
  double *d_part = (double *)scratch(ctx, kSlotAux, sizeof(double) * (size_t)nchunks * G * 12, &st);
  if (!d_part) return st;
  double *d_sums = (double *)scratch(ctx, kSlotAux2, sizeof(double) * (size_t)G * kCols * 2, &st);
  if (!d_sums) return st;
  const bool need_mi = build_tree || d_mi;
  double *mi = d_mi;
  if (need_mi && !mi) {
    mi = (double *)scratch(ctx, kSlotOut, sizeof(double) * S.npairs * G, &st);
    if (!mi) return st;
  }
  CENTRE_CUDA(ctx, cudaMemsetAsync(d_part, 0, sizeof(double) * (size_t)nchunks * G * 12, ctx->stream));
  KernelTimer kt(ctx, CENTRE_TIMER_SCORE);
  if (S.npairs) {
    mi_sums_kernel<<<nchunks, threads, sizeof(double) * threads * 12, ctx->stream>>>(
        S, d_types, d_pairs, d_s1, d_s2, mi, d_part, chunk);
    ctx->launches++;
    CENTRE_CUDA(ctx, cudaGetLastError());
  }
  sums_final_kernel<<<G, 256, 0, ctx->stream>>>(S, d_types, d_s1, d_part, nchunks, d_sums);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  CENTRE_CUDA(ctx, cudaMemcpyAsync(h_mie, d_sums, sizeof(double) * G * kCols,
                                   cudaMemcpyDeviceToHost, ctx->stream));
  if (!build_tree) return check_cuda(ctx, cudaStreamSynchronize(ctx->stream), "score sync");

  // ---- Boruvka over all G graphs ----------------------------------------
  const uint64_t GV = (uint64_t)G * S.ndof;
  const uint32_t cap = S.ndof > 0 ? S.ndof - 1 : 0;
  uint32_t *comp = (uint32_t *)scratch(ctx, kSlotAux, sizeof(uint32_t) * GV * 2 +
                                                         sizeof(unsigned long long) * GV * 3 +
                                                         sizeof(uint32_t) * ((uint64_t)G * (cap + 1) + G + 1),
                                       &st);
  if (!comp) return st;
  uint32_t *parent = comp + GV;
  unsigned long long *bestkey = reinterpret_cast<unsigned long long *>(parent + GV);
  unsigned long long *bestedge = bestkey + GV;
  unsigned long long *winpair = bestedge + GV;
  uint32_t *tree = reinterpret_cast<uint32_t *>(winpair + GV);
  uint32_t *ntree = tree + (uint64_t)G * (cap + 1);
  unsigned *added = ntree + G;
  const unsigned TB = 256;
  auto blocks = [&](uint64_t n) { return (unsigned)((n + TB - 1) / TB); };
  mst_init_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(comp, S.ndof, GV);
  mst_init_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(parent, S.ndof, GV);
  ctx->launches += 2;
  CENTRE_CUDA(ctx, cudaMemsetAsync(ntree, 0, sizeof(uint32_t) * (G + 1), ctx->stream));
  const uint64_t PG = S.npairs * (uint64_t)G;
  unsigned h_added = 0;
  for (uint32_t round = 0; round < 64 && PG > 0; ++round) {
    CENTRE_CUDA(ctx, cudaMemsetAsync(added, 0, sizeof(unsigned), ctx->stream));
    mst_reset_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(bestkey, bestedge, GV);
    mst_pick_kernel<0><<<blocks(S.npairs), TB, 0, ctx->stream>>>(S, d_types, d_pairs, mi, comp,
                                                                 bestkey, bestedge);
    mst_pick_kernel<1><<<blocks(S.npairs), TB, 0, ctx->stream>>>(S, d_types, d_pairs, mi, comp,
                                                                 bestkey, bestedge);
    mst_hook_kernel<<<blocks(S.npairs), TB, 0, ctx->stream>>>(S, d_types, d_pairs, mi, comp, parent,
                                                        bestkey, bestedge, winpair, tree, ntree,
                                                        cap, added);
    mst_link_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(S, d_pairs, comp, parent, bestedge,
                                                        winpair, tree, ntree, cap, added);
    mst_jump_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(S, comp, parent);
    mst_parent_sync_kernel<<<blocks(GV), TB, 0, ctx->stream>>>(S, comp, parent);
    ctx->launches += 7;
    CENTRE_CUDA(ctx, cudaGetLastError());
    CENTRE_CUDA(ctx, cudaMemcpyAsync(&h_added, added, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     ctx->stream));
    CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_added == 0) break;
  }
  std::vector<uint32_t> tr((size_t)G * (cap + 1));
  std::vector<uint32_t> nt(G);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(tr.data(), tree, sizeof(uint32_t) * tr.size(),
                                   cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(nt.data(), ntree, sizeof(uint32_t) * G, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int g = 0; g < G; ++g) nt[g] = std::min(nt[g], cap);
  // gather MI and endpoints of the tree edges (G * (ndof - 1) values)
  const uint64_t nslots = (uint64_t)G * (cap + 1);
  double *d_w = (double *)scratch(ctx, kSlotAux2, nslots * (sizeof(double) + 8) + 16, &st);
  if (!d_w) return st;
  uint32_t *d_ij = reinterpret_cast<uint32_t *>(d_w + nslots);
  mst_gather_kernel<<<blocks(nslots), TB, 0, ctx->stream>>>(S, d_pairs, mi, tree, ntree, cap,
                                                             d_w, d_ij);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  std::vector<double> wt(nslots);
  std::vector<uint32_t> ij(2 * nslots);
  std::vector<uint8_t> ty(S.ndof);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(wt.data(), d_w, sizeof(double) * nslots, cudaMemcpyDeviceToHost,
                                   ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(ij.data(), d_ij, sizeof(uint32_t) * 2 * nslots,
                                   cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(ty.data(), d_types, S.ndof, cudaMemcpyDeviceToHost, ctx->stream));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (int g = 0; g < G; ++g)
    if (nt[g] > cap) return set_error(ctx, CENTRE_E_CUDA, "spanning tree overflow");
  for (int g = 0; g < G; ++g) {
    const size_t base = (size_t)g * (cap + 1);
    std::vector<uint32_t> ord(nt[g]);
    for (uint32_t e = 0; e < nt[g]; ++e) ord[e] = e;
    // sort by MI descending, then pair index (src/EntropyScorer.cpp:753)
    std::sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) {
      const double wa = wt[base + a], wb = wt[base + b];
      if (wa != wb) return wa > wb;
      return tr[base + a] < tr[base + b];
    });
    h_ntree[g] = nt[g];
    double blk[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t e = 0; e < nt[g]; ++e) {
      const uint32_t q = ord[e];
      h_tree[(size_t)g * cap + e] = tr[base + q];
      int a = ty[ij[2 * (base + q)]], b = ty[ij[2 * (base + q) + 1]];
      if (a > b) std::swap(a, b);
      int bi = (a == 1 && b == 1) ? 0 : (a == 2 && b == 2) ? 1 : (a == 3 && b == 3) ? 2
             : (a == 1 && b == 2) ? 3 : (a == 1 && b == 3) ? 4 : (a == 2 && b == 3) ? 5 : -1;
      if (bi >= 0) blk[bi] += wt[base + q];
    }
    // MIST sums (src/EntropyScorer.cpp:769-799): I2 columns hold tree MI
    double *row = h_mist + (size_t)g * kCols;
    const double *mrow = h_mie + (size_t)g * kCols;
    for (int c = 0; c < kCols; ++c) row[c] = mrow[c];
    double d = row[15];
    for (int b = 0; b < 6; ++b) {
      row[4 + 2 * b] = blk[b];
      d -= blk[b];
    }
    row[16] = d;
  }
  return CENTRE_OK;
}

}  // namespace centre
