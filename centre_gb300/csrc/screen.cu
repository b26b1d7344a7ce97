// screen.cu -- learned pair screen for A-MIE / A-MIST neighbour selection.
//
// The reference scores only the DOF pairs of a neighbour file for its
// approximate methods (scoringmethod MIST/MIE with useneighbor=true,
// src/Inputs.cpp:660-690, Neighbors(fname), src/Centre.cpp:459-593); the
// file comes from outside the program (geometric neighbours).  This file
// builds that list on the GPU instead, from the data:
//
//   1. per-DOF columns over the first nframes/feat_div frames: a torsion
//      gives (cos, sin) of its bin-centre angle, a bond or angle its bin
//      index; each column standardised, stored bf16 DOF-major;
//   2. their correlation matrix R = X X^T (X standardised and scaled by
//      1/sqrt(F): one bf16 GEMM on the tensor cores, gemm_tc.cu);
//   3. per DOF, the nprefilter partners with the largest squared Frobenius
//      norm of their 2x2 correlation block (radix select in shared memory);
//   4. a BF16 MLP 12 -> 64 -> 64 -> 1 (ReLU) scores those partners from 12
//      cheap features (prefix marginal entropies, types, index distance,
//      the correlation block and a Gaussian MI proxy); the nneigh best per
//      DOF are kept and the union of (i, j) is the pair list, row-major.
//
// The network is trained here, on exact MI of random pairs over the same
// frame prefix (the method's own 2-D entropies at the first convergence
// step), by hand-written forward, backward and Adam kernels.  Exact MI of
// the selected pairs (centre_gpu_entropy2d_dev) remains the judge; the
// caller compares against all pairs when it wants the error.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "entropy.cuh"

namespace centre {
namespace {

constexpr int kFeat = 12;
constexpr int kHid = 64;
// parameter layout: W1 [64][12], b1 [64], W2 [64][64], b2 [64], W3 [64], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kFeat;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid;
constexpr int kNParams = kOffB3 + 1;
static_assert(kNParams == CENTRE_SCREEN_NPARAMS, "parameter count");

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Device memory owned for the duration of one call.
struct Buf {
  void *p = nullptr;
  ~Buf() {
    if (p) cudaFree(p);
  }
};

int dalloc(centre_ctx *ctx, Buf &b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  const cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return set_error(ctx, CENTRE_E_NOMEM, "screen: device allocation failed");
  }
  return CENTRE_OK;
}

// ------------------------------------------------------------ columns ----
// Per-DOF column statistics over the first F frames of scheme 0.
__global__ void column_stats_kernel(const uint8_t *__restrict__ bins, const uint8_t *__restrict__ types,
                                    uint64_t nframes, int nschemes, uint32_t F, int nb,
                                    float *__restrict__ stats /*[ndof][4]*/) {
  const uint32_t d = blockIdx.x;
  const uint8_t *row = bins + (uint64_t)d * nschemes * nframes;
  const bool tor = types[d] == 3;
  double su = 0, sv = 0, suu = 0, svv = 0;
  for (uint32_t f = threadIdx.x; f < F; f += blockDim.x) {
    const float b = (float)row[f];
    float u, v;
    if (tor) {
      sincospif((2.f * b + 1.f) / (float)nb, &v, &u);
    } else {
      u = b;
      v = 0.f;
    }
    su += u;
    sv += v;
    suu += (double)u * u;
    svv += (double)v * v;
  }
  __shared__ double red[4][32];
  double vals[4] = {su, sv, suu, svv};
  for (int q = 0; q < 4; ++q) {
    double x = vals[q];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double x = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += red[threadIdx.x][w];
    red[threadIdx.x][0] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double mu = red[0][0] / F, mv = red[1][0] / F;
    const double vu = red[2][0] / F - mu * mu, vv = red[3][0] / F - mv * mv;
    stats[d * 4 + 0] = (float)mu;
    stats[d * 4 + 1] = vu > 1e-12 ? (float)(1.0 / sqrt(vu)) : 0.f;
    stats[d * 4 + 2] = (float)mv;
    stats[d * 4 + 3] = vv > 1e-12 ? (float)(1.0 / sqrt(vv)) : 0.f;
  }
}

// X [2*ndof][ldx] bf16, DOF-major: row 2d = u, 2d+1 = v over the F frames,
// standardised and scaled by 1/sqrt(F) so that X X^T is the correlation
// matrix (ldx >= F; the GEMM reads nothing past F).
__global__ void columns_kernel(const uint8_t *__restrict__ bins, const uint8_t *__restrict__ types,
                               uint64_t nframes, int nschemes, uint32_t F, int nb,
                               const float *__restrict__ stats, uint32_t ldx,
                               __nv_bfloat16 *__restrict__ X) {
  const uint32_t d = blockIdx.y;
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  const float b = (float)bins[(uint64_t)d * nschemes * nframes + f];
  float u, v;
  if (types[d] == 3) {
    sincospif((2.f * b + 1.f) / (float)nb, &v, &u);
  } else {
    u = b;
    v = 0.f;
  }
  const float s = rsqrtf((float)F);
  X[(uint64_t)(2 * d) * ldx + f] = __float2bfloat16_rn((u - stats[d * 4]) * stats[d * 4 + 1] * s);
  X[(uint64_t)(2 * d + 1) * ldx + f] =
      __float2bfloat16_rn((v - stats[d * 4 + 2]) * stats[d * 4 + 3] * s);
}

// ------------------------------------------------------------ features ---
struct FeatCtx {
  const float *R;        // [2D][ld], symmetric
  const float *s1p;      // prefix entropy per DOF
  const uint8_t *types;
  const uint32_t *tid;   // index within its type
  uint32_t ndof;
  uint32_t ld;           // R's leading dimension (>= 2D)
};

__device__ __forceinline__ float block_frob2(const FeatCtx &F, uint32_t i, uint32_t j) {
  const uint64_t ld = F.ld;
  const float a = F.R[(2ull * j) + (2ull * i) * ld], b = F.R[(2ull * j + 1) + (2ull * i) * ld];
  const float c = F.R[(2ull * j) + (2ull * i + 1) * ld], e = F.R[(2ull * j + 1) + (2ull * i + 1) * ld];
  return a * a + b * b + c * c + e * e;
}

__device__ void pair_features(const FeatCtx &F, uint32_t i, uint32_t j, float *f) {
  const uint64_t ld = F.ld;
  const float ruu = F.R[(2ull * j) + (2ull * i) * ld];
  const float rvu = F.R[(2ull * j + 1) + (2ull * i) * ld];
  const float ruv = F.R[(2ull * j) + (2ull * i + 1) * ld];
  const float rvv = F.R[(2ull * j + 1) + (2ull * i + 1) * ld];
  const float fr = ruu * ruu + ruv * ruv + rvu * rvu + rvv * rvv;
  const float si = F.s1p[i], sj = F.s1p[j];
  const uint32_t ti = F.tid[i], tj = F.tid[j];
  f[0] = si;
  f[1] = sj;
  f[2] = (float)F.types[i] * (1.f / 3.f);
  f[3] = (float)F.types[j] * (1.f / 3.f);
  f[4] = log1pf((float)(ti > tj ? ti - tj : tj - ti));
  f[5] = fabsf(ruu);
  f[6] = fabsf(ruv);
  f[7] = fabsf(rvu);
  f[8] = fabsf(rvv);
  f[9] = fr;
  f[10] = -0.5f * logf(1.f - fminf(fr, 0.999f));
  f[11] = fminf(si, sj);
}

__global__ void features_kernel(FeatCtx F, const uint32_t *__restrict__ pairs, uint64_t n,
                                float *__restrict__ X) {
  const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  float f[kFeat];
  pair_features(F, pairs[2 * k], pairs[2 * k + 1], f);
  for (int q = 0; q < kFeat; ++q) X[k * kFeat + q] = f[q];
}

// ------------------------------------------------------------------ MLP --
// Weights as the kernels use them: bf16 values held as float in shared
// memory.  Activations are rounded to bf16 between layers; sums in FP32.
__device__ __forceinline__ float mlp_forward(const float *__restrict__ W, const float *x,
                                             float *h1, float *z1, float *h2, float *z2) {
  for (int m = 0; m < kHid; ++m) {
    float z = W[kOffB1 + m];
    for (int q = 0; q < kFeat; ++q) z = fmaf(W[kOffW1 + m * kFeat + q], x[q], z);
    z1[m] = z;
    h1[m] = bf16r(fmaxf(z, 0.f));
  }
  float out = W[kOffB3];
  for (int k = 0; k < kHid; ++k) {
    float z = W[kOffB2 + k];
    for (int m = 0; m < kHid; ++m) z = fmaf(W[kOffW2 + k * kHid + m], h1[m], z);
    if (z2) z2[k] = z;
    const float h = bf16r(fmaxf(z, 0.f));
    if (h2) h2[k] = h;
    out = fmaf(W[kOffW3 + k], h, out);
  }
  return out;
}

__device__ void load_weights(const float *__restrict__ wbf, float *W) {
  for (int q = threadIdx.x; q < kNParams; q += blockDim.x) W[q] = wbf[q];
  __syncthreads();
}

// Forward and the backward pass down to the activations, one thread per
// sample of a minibatch: stores x, h1, h2 (bf16 values), dh1, dh2 (FP32)
// and dout, and adds the squared error to *loss.
__global__ void __launch_bounds__(128)
mlp_fwd_bwd_kernel(const float *__restrict__ wbf, const float *__restrict__ X,
                   const float *__restrict__ y, const uint32_t *__restrict__ order, uint64_t first,
                   uint32_t B, float *__restrict__ xs, float *__restrict__ h1s,
                   float *__restrict__ h2s, float *__restrict__ dh1s, float *__restrict__ dh2s,
                   float *__restrict__ douts, float *__restrict__ preds, double *__restrict__ loss) {
  __shared__ float W[kNParams];
  load_weights(wbf, W);
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  float err2 = 0.f;
  if (s < B) {
    const uint64_t row = order ? order[first + s] : first + s;
    float x[kFeat], h1[kHid], z1[kHid], z2[kHid], h2[kHid];
    for (int q = 0; q < kFeat; ++q) x[q] = bf16r(X[row * kFeat + q]);
    const float out = mlp_forward(W, x, h1, z1, h2, z2);
    const float e = out - y[row];
    err2 = e * e;
    const float dout = 2.f * e / (float)B;
    if (preds) preds[s] = out;
    douts[s] = dout;
    for (int q = 0; q < kFeat; ++q) xs[(uint64_t)s * kFeat + q] = x[q];
    float dh2[kHid];
    for (int k = 0; k < kHid; ++k) {
      dh2[k] = z2[k] > 0.f ? dout * W[kOffW3 + k] : 0.f;
      dh2s[(uint64_t)s * kHid + k] = dh2[k];
      h2s[(uint64_t)s * kHid + k] = h2[k];
      h1s[(uint64_t)s * kHid + k] = h1[k];
    }
    for (int m = 0; m < kHid; ++m) {
      float g = 0.f;
      for (int k = 0; k < kHid; ++k) g = fmaf(W[kOffW2 + k * kHid + m], dh2[k], g);
      dh1s[(uint64_t)s * kHid + m] = z1[m] > 0.f ? g : 0.f;
    }
  }
  for (int o = 16; o; o >>= 1) err2 += __shfl_xor_sync(0xffffffffu, err2, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)err2);
}

// Weight gradients: sums over the minibatch of outer products, 256 threads
// per block splitting the samples, partial sums reduced in shared memory.
//   block k < 64      : row k of W2 (lane m = t & 63) and b2[k]
//   block 64 + m      : row m of W1 (lane q = t & 15, q < 12) and b1[m]
//   block 128         : W3 (lane k = t & 63) and b3
// Blocks along y take disjoint sample ranges and write their own partial
// gradient rows (grad + y * kNParams); reduce_grad_kernel or the Adam kernel
// sums the rows in a fixed order.
constexpr int kGradSplit = 8;

__global__ void __launch_bounds__(256)
mlp_grad_kernel(const float *__restrict__ xs, const float *__restrict__ h1s,
                const float *__restrict__ h2s, const float *__restrict__ dh1s,
                const float *__restrict__ dh2s, const float *__restrict__ douts, uint32_t B,
                float *__restrict__ gradpart) {
  __shared__ float pw[256], pb[256];
  const int b = blockIdx.x, t = threadIdx.x;
  const uint32_t per = (B + gridDim.y - 1) / gridDim.y;
  const uint32_t sb = blockIdx.y * per, se = min(B, sb + per);
  float *grad = gradpart + (uint64_t)blockIdx.y * kNParams;
  float aw = 0.f, ab = 0.f;
  if (b < kHid) {
    const int m = t & 63, part = t >> 6;
    for (uint32_t s = sb + part; s < se; s += 4) {
      const float d = dh2s[(uint64_t)s * kHid + b];
      aw = fmaf(d, h1s[(uint64_t)s * kHid + m], aw);
      ab += d;
    }
  } else if (b < 2 * kHid) {
    const int m = b - kHid, q = t & 15, part = t >> 4;
    for (uint32_t s = sb + part; s < se; s += 16) {
      const float d = dh1s[(uint64_t)s * kHid + m];
      if (q < kFeat) aw = fmaf(d, xs[(uint64_t)s * kFeat + q], aw);
      ab += d;
    }
  } else {
    const int k = t & 63, part = t >> 6;
    for (uint32_t s = sb + part; s < se; s += 4) {
      const float d = douts[s];
      aw = fmaf(d, h2s[(uint64_t)s * kHid + k], aw);
      ab += d;
    }
  }
  pw[t] = aw;
  pb[t] = ab;
  __syncthreads();
  if (b < kHid || b == 2 * kHid) {
    if (t < 64) {
      const float w = pw[t] + pw[t + 64] + pw[t + 128] + pw[t + 192];
      if (b < kHid) grad[kOffW2 + b * kHid + t] = w;
      else grad[kOffW3 + t] = w;
    } else if (t == 64) {
      // every lane of a part saw the same bias terms: take lane 0 of each part
      const float bb = pb[0] + pb[64] + pb[128] + pb[192];
      if (b < kHid) grad[kOffB2 + b] = bb;
      else grad[kOffB3] = bb;
    }
  } else {
    const int m = b - kHid;
    if (t < kFeat) {
      float w = 0.f;
      for (int part = 0; part < 16; ++part) w += pw[part * 16 + t];
      grad[kOffW1 + m * kFeat + t] = w;
    } else if (t == 16) {
      float bb = 0.f;
      for (int part = 0; part < 16; ++part) bb += pb[part * 16];
      grad[kOffB1 + m] = bb;
    }
  }
}

// Adam on the FP32 master weights; the bf16-rounded copy feeds the kernels.
__global__ void reduce_grad_kernel(const float *__restrict__ gradpart, float *__restrict__ g) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kNParams) return;
  float v = 0.f;
  for (int k = 0; k < kGradSplit; ++k) v += gradpart[(uint64_t)k * kNParams + q];
  g[q] = v;
}

__global__ void adam_kernel(float *__restrict__ w, float *__restrict__ wbf,
                            const float *__restrict__ gradpart, float *__restrict__ m1,
                            float *__restrict__ m2, float lr, float c1, float c2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kNParams) return;
  float gq = 0.f;
  for (int k = 0; k < kGradSplit; ++k) gq += gradpart[(uint64_t)k * kNParams + q];
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  m1[q] = b1 * m1[q] + (1.f - b1) * gq;
  m2[q] = b2 * m2[q] + (1.f - b2) * gq * gq;
  w[q] -= lr * (m1[q] / c1) / (sqrtf(m2[q] / c2) + eps);
  wbf[q] = bf16r(w[q]);
}

__global__ void round_weights_kernel(const float *__restrict__ w, float *__restrict__ wbf) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < kNParams) wbf[q] = bf16r(w[q]);
}

// ------------------------------------------------------------ selection --
// Per DOF i: the P partners with the largest squared correlation-block norm
// (ties: lower index first), in index order; rows with fewer than P
// partners pad with 0xffffffff.
__global__ void __launch_bounds__(512)
prefilter_kernel(FeatCtx F, uint32_t P, uint32_t *__restrict__ cand) {
  extern __shared__ uint32_t keys[];   // [ndof]
  __shared__ uint32_t hist[256];
  __shared__ uint32_t sh_prefix, sh_need;
  __shared__ uint32_t scan[512];
  const uint32_t i = blockIdx.x, D = F.ndof, T = blockDim.x, tid = threadIdx.x;
  for (uint32_t j = tid; j < D; j += T)
    keys[j] = (j == i) ? 0u : (__float_as_uint(fmaxf(block_frob2(F, i, j), 0.f)) | 0u) + 1u;
  // key 0 marks i itself; every real partner has key >= 1
  uint32_t *out = cand + (uint64_t)i * P;
  if (D - 1 <= P) {
    __syncthreads();
    if (tid == 0) {
      uint32_t c = 0;
      for (uint32_t j = 0; j < D; ++j)
        if (j != i) out[c++] = j;
      for (; c < P; ++c) out[c] = 0xffffffffu;
    }
    return;
  }
  if (tid == 0) {
    sh_prefix = 0;
    sh_need = P;
  }
  uint32_t mask = 0;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (uint32_t b = tid; b < 256; b += T) hist[b] = 0;
    __syncthreads();
    const uint32_t prefix = sh_prefix;
    for (uint32_t j = tid; j < D; j += T)
      if ((keys[j] & mask) == prefix && keys[j] != 0u) atomicAdd(&hist[(keys[j] >> shift) & 255u], 1u);
    __syncthreads();
    if (tid == 0) {
      uint32_t need = sh_need, b = 255;
      for (;; --b) {
        if (hist[b] >= need || b == 0) break;
        need -= hist[b];
      }
      sh_prefix = prefix | (b << shift);
      sh_need = need;
    }
    mask |= 255u << shift;
    __syncthreads();
  }
  const uint32_t thr = sh_prefix, ties = sh_need;   // take `ties` keys equal to thr
  // contiguous chunks per thread keep index order
  const uint32_t chunk = (D + T - 1) / T, j0 = tid * chunk, j1 = min(D, j0 + chunk);
  uint32_t gt = 0, eq = 0;
  for (uint32_t j = j0; j < j1; ++j) {
    gt += keys[j] > thr;
    eq += keys[j] == thr;
  }
  scan[tid] = eq;
  __syncthreads();
  for (uint32_t o = 1; o < T; o <<= 1) {
    const uint32_t v = tid >= o ? scan[tid - o] : 0;
    __syncthreads();
    scan[tid] += v;
    __syncthreads();
  }
  const uint32_t eq_before = scan[tid] - eq;
  const uint32_t take = eq_before >= ties ? 0 : min(eq, ties - eq_before);
  __syncthreads();
  scan[tid] = gt + take;
  __syncthreads();
  for (uint32_t o = 1; o < T; o <<= 1) {
    const uint32_t v = tid >= o ? scan[tid - o] : 0;
    __syncthreads();
    scan[tid] += v;
    __syncthreads();
  }
  uint32_t pos = scan[tid] - (gt + take), taken = 0;
  for (uint32_t j = j0; j < j1; ++j) {
    if (keys[j] > thr || (keys[j] == thr && taken < take)) {
      if (keys[j] == thr) ++taken;
      if (pos < P) out[pos] = j;
      ++pos;
    }
  }
}

// Per DOF i: the network's score of each prefilter candidate, the nneigh
// best kept (ties: lower index first); pads with 0xffffffff.
__global__ void __launch_bounds__(256)
rank_kernel(FeatCtx F, const float *__restrict__ wbf, const uint32_t *__restrict__ cand,
            uint32_t P, uint32_t K, uint32_t *__restrict__ neigh) {
  __shared__ float W[kNParams];
  __shared__ float score[1024];
  __shared__ uint32_t who[1024];
  load_weights(wbf, W);
  const uint32_t i = blockIdx.x;
  for (uint32_t t = threadIdx.x; t < P; t += blockDim.x) {
    const uint32_t j = cand[(uint64_t)i * P + t];
    float s = -INFINITY;
    if (j != 0xffffffffu) {
      float x[kFeat], h1[kHid], z1[kHid];
      const uint32_t a = min(i, j), b = max(i, j);
      pair_features(F, a, b, x);
      for (int q = 0; q < kFeat; ++q) x[q] = bf16r(x[q]);
      s = mlp_forward(W, x, h1, z1, nullptr, nullptr);
    }
    score[t] = s;
    who[t] = j;
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < P; t += blockDim.x) {
    const float s = score[t];
    const uint32_t j = who[t];
    uint32_t rank = 0;
    for (uint32_t u = 0; u < P; ++u)
      rank += (score[u] > s) || (score[u] == s && (who[u] < j || (who[u] == j && u < t)));
    if (rank < K) neigh[(uint64_t)i * K + rank] = (j != 0xffffffffu && s > -INFINITY) ? j : 0xffffffffu;
  }
}

// Union of the neighbour lists as an upper-triangular bitmap.
__global__ void mark_pairs_kernel(const uint32_t *__restrict__ neigh, uint32_t D, uint32_t K,
                                  uint32_t *__restrict__ bitmap) {
  const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= (uint64_t)D * K) return;
  const uint32_t i = (uint32_t)(k / K), j = neigh[k];
  if (j == 0xffffffffu || j == i || j >= D) return;
  const uint64_t a = min(i, j), b = max(i, j);
  const uint64_t bit = a * D + b;
  atomicOr(&bitmap[bit >> 5], 1u << (bit & 31));
}

__global__ void row_count_kernel(const uint32_t *__restrict__ bitmap, uint32_t D,
                                 uint32_t *__restrict__ counts) {
  const uint32_t a = blockIdx.x;
  uint32_t c = 0;
  for (uint32_t b = a + 1 + threadIdx.x; b < D; b += blockDim.x) {
    const uint64_t bit = (uint64_t)a * D + b;
    c += (bitmap[bit >> 5] >> (bit & 31)) & 1u;
  }
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  __shared__ uint32_t red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (uint32_t w = 0; w < blockDim.x / 32; ++w) t += red[w];
    counts[a] = t;
  }
}

__global__ void write_pairs_kernel(const uint32_t *__restrict__ bitmap, uint32_t D,
                                   const uint64_t *__restrict__ offsets,
                                   uint32_t *__restrict__ pairs) {
  const uint32_t a = blockIdx.x;
  if (threadIdx.x != 0) return;
  uint64_t o = offsets[a];
  for (uint32_t b = a + 1; b < D; ++b) {
    const uint64_t bit = (uint64_t)a * D + b;
    if ((bitmap[bit >> 5] >> (bit & 31)) & 1u) {
      pairs[2 * o] = a;
      pairs[2 * o + 1] = b;
      ++o;
    }
  }
}

__global__ void mi_labels_kernel(const uint32_t *__restrict__ pairs, uint64_t n,
                                 const double *__restrict__ s1, const double *__restrict__ s2,
                                 int G, float *__restrict__ y) {
  const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  // scheme 0, estimator 0, step 0 is element 0 of each record
  y[k] = (float)(s1[(uint64_t)pairs[2 * k] * G] + s1[(uint64_t)pairs[2 * k + 1] * G] - s2[k * G]);
}

__global__ void gather_s1_kernel(const double *__restrict__ s1, uint32_t D, int G,
                                 float *__restrict__ s1p) {
  const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d < D) s1p[d] = (float)s1[(uint64_t)d * G];
}

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double uniform01(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

void screen_state_free(centre_ctx *) {}

// He-uniform initial weights, zero biases (host, seeded).
void screen_init_weights(uint64_t seed, float *w) {
  uint64_t s = seed ^ 0x5eed5eedull;
  memset(w, 0, sizeof(float) * kNParams);
  auto fill = [&](int off, int n, int fan_in) {
    const double a = sqrt(6.0 / fan_in);
    for (int q = 0; q < n; ++q) w[off + q] = (float)((2.0 * uniform01(s) - 1.0) * a);
  };
  fill(kOffW1, kHid * kFeat, kFeat);
  fill(kOffW2, kHid * kHid, kHid);
  fill(kOffW3, kHid, kHid);
}

}  // namespace centre

using namespace centre;

extern "C" int centre_gpu_screen_mlp_grad(centre_ctx *ctx, const float *weights, uint64_t n,
                                          const float *feats, const float *targets, float *pred,
                                          float *grad, double *loss) {
  if (!ctx || !weights || !feats || !targets || !grad || n == 0 || n > (1u << 20))
    return set_error(ctx, CENTRE_E_ARG, "screen_mlp_grad: bad arguments");
  cudaSetDevice(ctx->device);
  const uint32_t B = (uint32_t)n;
  Buf w, wbf, X, y, xs, h1, h2, dh1, dh2, dout, pr, g, ls;
  CENTRE_TRY(dalloc(ctx, w, sizeof(float) * kNParams));
  CENTRE_TRY(dalloc(ctx, wbf, sizeof(float) * kNParams));
  CENTRE_TRY(dalloc(ctx, X, sizeof(float) * n * kFeat));
  CENTRE_TRY(dalloc(ctx, y, sizeof(float) * n));
  CENTRE_TRY(dalloc(ctx, xs, sizeof(float) * n * kFeat));
  CENTRE_TRY(dalloc(ctx, h1, sizeof(float) * n * kHid));
  CENTRE_TRY(dalloc(ctx, h2, sizeof(float) * n * kHid));
  CENTRE_TRY(dalloc(ctx, dh1, sizeof(float) * n * kHid));
  CENTRE_TRY(dalloc(ctx, dh2, sizeof(float) * n * kHid));
  CENTRE_TRY(dalloc(ctx, dout, sizeof(float) * n));
  CENTRE_TRY(dalloc(ctx, pr, sizeof(float) * n));
  CENTRE_TRY(dalloc(ctx, g, sizeof(float) * kNParams));
  CENTRE_TRY(dalloc(ctx, ls, sizeof(double)));
  cudaStream_t st = ctx->stream;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(w.p, weights, sizeof(float) * kNParams, cudaMemcpyHostToDevice, st));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(X.p, feats, sizeof(float) * n * kFeat, cudaMemcpyHostToDevice, st));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(y.p, targets, sizeof(float) * n, cudaMemcpyHostToDevice, st));
  CENTRE_CUDA(ctx, cudaMemsetAsync(ls.p, 0, sizeof(double), st));
  round_weights_kernel<<<(kNParams + 255) / 256, 256, 0, st>>>((float *)w.p, (float *)wbf.p);
  mlp_fwd_bwd_kernel<<<(B + 127) / 128, 128, 0, st>>>(
      (float *)wbf.p, (float *)X.p, (float *)y.p, nullptr, 0, B, (float *)xs.p, (float *)h1.p,
      (float *)h2.p, (float *)dh1.p, (float *)dh2.p, (float *)dout.p, (float *)pr.p, (double *)ls.p);
  Buf gp;
  CENTRE_TRY(dalloc(ctx, gp, sizeof(float) * kNParams * kGradSplit));
  mlp_grad_kernel<<<dim3(2 * kHid + 1, kGradSplit), 256, 0, st>>>(
      (float *)xs.p, (float *)h1.p, (float *)h2.p, (float *)dh1.p, (float *)dh2.p,
      (float *)dout.p, B, (float *)gp.p);
  reduce_grad_kernel<<<(kNParams + 255) / 256, 256, 0, st>>>((float *)gp.p, (float *)g.p);
  ctx->launches += 4;
  CENTRE_CUDA(ctx, cudaGetLastError());
  double l = 0;
  CENTRE_CUDA(ctx, cudaMemcpyAsync(grad, g.p, sizeof(float) * kNParams, cudaMemcpyDeviceToHost, st));
  if (pred) CENTRE_CUDA(ctx, cudaMemcpyAsync(pred, pr.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(&l, ls.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(st));
  if (loss) *loss = l / (double)n;
  return CENTRE_OK;
}

extern "C" int centre_gpu_screen_dev(centre_ctx *ctx, const centre_entropy_params *p,
                                     const centre_screen_params *sp, uint32_t ndof,
                                     const uint8_t *types, const uint8_t *bins,
                                     const double *extremes, float *weights, float *losses,
                                     uint64_t capacity, uint32_t *pairs, uint64_t *npairs) {
  if (!ctx || !p || !sp || !types || !bins || !extremes || !weights || !pairs || !npairs)
    return set_error(ctx, CENTRE_E_ARG, "screen: null argument");
  cudaSetDevice(ctx->device);
  if (ndof < 3 || sp->feat_div == 0 || p->nframes / sp->feat_div < 16 || sp->nprefilter == 0 ||
      sp->nprefilter > 1024 || sp->nneigh == 0 || sp->nneigh > sp->nprefilter ||
      (sp->train && (sp->batch == 0 || sp->batch > 65536 || sp->ntrain < sp->batch)))
    return set_error(ctx, CENTRE_E_ARG, "screen: bad parameters");
  if ((uint64_t)ndof * 4 > 200 * 1024)
    return set_error(ctx, CENTRE_E_UNSUPPORTED, "screen: more than 51200 DOFs");
  if (p->nschemes == 0 || p->bin_schemes[0] == 0)
    return set_error(ctx, CENTRE_E_ARG, "screen: no bin scheme");
  cudaStream_t st = ctx->stream;
  const uint32_t D = ndof;
  const uint32_t F = (uint32_t)(p->nframes / sp->feat_div);
  const int nb = p->bin_schemes[0];
  // DOF index within its type (types are bonds, angles, torsions in order)
  std::vector<uint8_t> ht(D);
  CENTRE_CUDA(ctx, cudaMemcpy(ht.data(), types, D, cudaMemcpyDeviceToHost));
  std::vector<uint32_t> tid(D);
  uint32_t start[4] = {0, 0, 0, 0};
  for (uint32_t d = 0; d < D; ++d) {
    if (ht[d] < 1 || ht[d] > 3) return set_error(ctx, CENTRE_E_ARG, "screen: DOF type must be 1..3");
    if (d == 0 || ht[d] != ht[d - 1]) start[ht[d]] = d;
    tid[d] = d - start[ht[d]];
  }
  // prefix entropies: the first of feat_div convergence steps, ML, scheme 0
  centre_entropy_params pl = *p;
  pl.nsteps = (uint8_t)sp->feat_div;
  pl.nestimators = 1;
  pl.estimators[0] = CENTRE_ML;
  pl.counts_form = CENTRE_COUNTS_AUTO;
  const int Gl = pl.nschemes * pl.nsteps;
  Buf s1l, s1p, dtid, stats, X, R, cand, neigh, bitmap, counts, offs;
  CENTRE_TRY(dalloc(ctx, s1l, sizeof(double) * D * Gl));
  CENTRE_TRY(dalloc(ctx, s1p, sizeof(float) * D));
  CENTRE_TRY(dalloc(ctx, dtid, sizeof(uint32_t) * D));
  CENTRE_TRY(dalloc(ctx, stats, sizeof(float) * D * 4));
  // row strides the tensor-core GEMM takes: X rows 16-byte aligned, R rows
  // of whole float4s
  const uint32_t ldx = (F + 7u) & ~7u, ldr = (2 * D + 3u) & ~3u;
  CENTRE_TRY(dalloc(ctx, X, sizeof(__nv_bfloat16) * 2ull * D * ldx));
  CENTRE_TRY(dalloc(ctx, R, sizeof(float) * 2ull * D * ldr));
  CENTRE_CUDA(ctx, cudaMemcpyAsync(dtid.p, tid.data(), sizeof(uint32_t) * D, cudaMemcpyHostToDevice, st));
  int rc = centre_gpu_entropy1d_dev(ctx, &pl, D, types, bins, extremes, (double *)s1l.p, nullptr);
  if (rc != CENTRE_OK) return rc;
  gather_s1_kernel<<<(D + 255) / 256, 256, 0, st>>>((double *)s1l.p, D, Gl, (float *)s1p.p);
  column_stats_kernel<<<D, 256, 0, st>>>(bins, types, p->nframes, p->nschemes, F, nb, (float *)stats.p);
  columns_kernel<<<dim3((F + 255) / 256, D), 256, 0, st>>>(bins, types, p->nframes, p->nschemes, F,
                                                           nb, (float *)stats.p, ldx,
                                                           (__nv_bfloat16 *)X.p);
  ctx->launches += 3;
  CENTRE_CUDA(ctx, cudaGetLastError());
  // R = X X^T on the tensor cores (hand-written tcgen05 GEMM, gemm_tc.cu)
  CENTRE_TRY(launch_corr_gemm(ctx, X.p, 2 * D, F, ldx, (float *)R.p, ldr));
  FeatCtx FC{(const float *)R.p, (const float *)s1p.p, types, (const uint32_t *)dtid.p, D, ldr};
  // ---- training on exact MI of random pairs over the prefix -------------
  Buf w, wbf, m1, m2, g, ls;
  CENTRE_TRY(dalloc(ctx, w, sizeof(float) * kNParams));
  CENTRE_TRY(dalloc(ctx, wbf, sizeof(float) * kNParams));
  std::vector<float> hw(kNParams);
  if (sp->train && sp->init_weights) screen_init_weights(sp->seed, hw.data());
  else memcpy(hw.data(), weights, sizeof(float) * kNParams);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(w.p, hw.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice, st));
  round_weights_kernel<<<(kNParams + 255) / 256, 256, 0, st>>>((float *)w.p, (float *)wbf.p);
  ctx->launches++;
  if (sp->train) {
    const uint64_t n = sp->ntrain;
    const uint32_t B = sp->batch;
    Buf tp, ts2, tX, ty, ord, xs, h1, h2, dh1, dh2, dout;
    CENTRE_TRY(dalloc(ctx, tp, sizeof(uint32_t) * 2 * n));
    CENTRE_TRY(dalloc(ctx, ts2, sizeof(double) * n * Gl));
    CENTRE_TRY(dalloc(ctx, tX, sizeof(float) * n * kFeat));
    CENTRE_TRY(dalloc(ctx, ty, sizeof(float) * n));
    CENTRE_TRY(dalloc(ctx, ord, sizeof(uint32_t) * n));
    CENTRE_TRY(dalloc(ctx, xs, sizeof(float) * (size_t)B * kFeat));
    CENTRE_TRY(dalloc(ctx, h1, sizeof(float) * (size_t)B * kHid));
    CENTRE_TRY(dalloc(ctx, h2, sizeof(float) * (size_t)B * kHid));
    CENTRE_TRY(dalloc(ctx, dh1, sizeof(float) * (size_t)B * kHid));
    CENTRE_TRY(dalloc(ctx, dh2, sizeof(float) * (size_t)B * kHid));
    CENTRE_TRY(dalloc(ctx, dout, sizeof(float) * (size_t)B));
    CENTRE_TRY(dalloc(ctx, m1, sizeof(float) * kNParams));
    CENTRE_TRY(dalloc(ctx, m2, sizeof(float) * kNParams));
    CENTRE_TRY(dalloc(ctx, g, sizeof(float) * kNParams * kGradSplit));
    CENTRE_TRY(dalloc(ctx, ls, sizeof(double) * std::max<uint32_t>(sp->epochs, 1)));
    uint64_t s = sp->seed;
    std::vector<uint32_t> hp(2 * n);
    for (uint64_t k = 0; k < n; ++k) {
      uint32_t a, b;
      do {
        a = (uint32_t)(splitmix(s) % D);
        b = (uint32_t)(splitmix(s) % D);
      } while (a == b);
      hp[2 * k] = std::min(a, b);
      hp[2 * k + 1] = std::max(a, b);
    }
    CENTRE_CUDA(ctx, cudaMemcpyAsync(tp.p, hp.data(), sizeof(uint32_t) * 2 * n, cudaMemcpyHostToDevice, st));
    rc = centre_gpu_entropy2d_dev(ctx, &pl, D, types, bins, extremes, n, (const uint32_t *)tp.p,
                                  (double *)ts2.p);
    if (rc != CENTRE_OK) return rc;
    mi_labels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((uint32_t *)tp.p, n,
                                                                  (double *)s1l.p, (double *)ts2.p,
                                                                  Gl, (float *)ty.p);
    features_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(FC, (uint32_t *)tp.p, n, (float *)tX.p);
    CENTRE_CUDA(ctx, cudaMemsetAsync(m1.p, 0, sizeof(float) * kNParams, st));
    CENTRE_CUDA(ctx, cudaMemsetAsync(m2.p, 0, sizeof(float) * kNParams, st));
    CENTRE_CUDA(ctx, cudaMemsetAsync(ls.p, 0, sizeof(double) * std::max<uint32_t>(sp->epochs, 1), st));
    ctx->launches += 2;
    std::vector<uint32_t> perm(n);
    const uint64_t steps = n / B;
    uint64_t t = 0;
    for (uint32_t ep = 0; ep < sp->epochs; ++ep) {
      for (uint64_t k = 0; k < n; ++k) perm[k] = (uint32_t)k;
      for (uint64_t k = n - 1; k > 0; --k) std::swap(perm[k], perm[splitmix(s) % (k + 1)]);
      CENTRE_CUDA(ctx, cudaMemcpyAsync(ord.p, perm.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st));
      for (uint64_t q = 0; q < steps; ++q) {
        ++t;
        mlp_fwd_bwd_kernel<<<(B + 127) / 128, 128, 0, st>>>(
            (float *)wbf.p, (float *)tX.p, (float *)ty.p, (uint32_t *)ord.p, q * B, B,
            (float *)xs.p, (float *)h1.p, (float *)h2.p, (float *)dh1.p, (float *)dh2.p,
            (float *)dout.p, nullptr, (double *)ls.p + ep);
        mlp_grad_kernel<<<dim3(2 * kHid + 1, kGradSplit), 256, 0, st>>>(
            (float *)xs.p, (float *)h1.p, (float *)h2.p, (float *)dh1.p, (float *)dh2.p,
            (float *)dout.p, B, (float *)g.p);
        const float c1 = 1.f - powf(0.9f, (float)t), c2 = 1.f - powf(0.999f, (float)t);
        adam_kernel<<<(kNParams + 255) / 256, 256, 0, st>>>((float *)w.p, (float *)wbf.p,
                                                            (float *)g.p, (float *)m1.p,
                                                            (float *)m2.p, sp->lr, c1, c2);
        ctx->launches += 3;
      }
      // the host copy of perm is reused next epoch: wait for the upload
      CENTRE_CUDA(ctx, cudaStreamSynchronize(st));
    }
    CENTRE_CUDA(ctx, cudaGetLastError());
    if (losses && sp->epochs) {
      std::vector<double> l(sp->epochs);
      CENTRE_CUDA(ctx, cudaMemcpyAsync(l.data(), ls.p, sizeof(double) * sp->epochs, cudaMemcpyDeviceToHost, st));
      CENTRE_CUDA(ctx, cudaStreamSynchronize(st));
      for (uint32_t e = 0; e < sp->epochs; ++e) losses[e] = (float)(l[e] / (double)(steps * B));
    }
    CENTRE_CUDA(ctx, cudaMemcpyAsync(weights, w.p, sizeof(float) * kNParams, cudaMemcpyDeviceToHost, st));
  }
  // ---- selection --------------------------------------------------------
  const uint32_t P = sp->nprefilter, K = sp->nneigh;
  CENTRE_TRY(dalloc(ctx, cand, sizeof(uint32_t) * (uint64_t)D * P));
  CENTRE_TRY(dalloc(ctx, neigh, sizeof(uint32_t) * (uint64_t)D * K));
  const uint64_t nbits = (uint64_t)D * D;
  CENTRE_TRY(dalloc(ctx, bitmap, sizeof(uint32_t) * ((nbits + 31) / 32)));
  CENTRE_TRY(dalloc(ctx, counts, sizeof(uint32_t) * D));
  CENTRE_TRY(dalloc(ctx, offs, sizeof(uint64_t) * D));
  const size_t pre_smem = sizeof(uint32_t) * D;
  CENTRE_CUDA(ctx, cudaFuncSetAttribute(prefilter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)pre_smem));
  CENTRE_CUDA(ctx, cudaMemsetAsync(neigh.p, 0xff, sizeof(uint32_t) * (uint64_t)D * K, st));
  prefilter_kernel<<<D, 512, pre_smem, st>>>(FC, P, (uint32_t *)cand.p);
  rank_kernel<<<D, 256, 0, st>>>(FC, (float *)wbf.p, (uint32_t *)cand.p, P, K, (uint32_t *)neigh.p);
  CENTRE_CUDA(ctx, cudaMemsetAsync(bitmap.p, 0, sizeof(uint32_t) * ((nbits + 31) / 32), st));
  mark_pairs_kernel<<<(unsigned)(((uint64_t)D * K + 255) / 256), 256, 0, st>>>(
      (uint32_t *)neigh.p, D, K, (uint32_t *)bitmap.p);
  row_count_kernel<<<D, 256, 0, st>>>((uint32_t *)bitmap.p, D, (uint32_t *)counts.p);
  ctx->launches += 4;
  CENTRE_CUDA(ctx, cudaGetLastError());
  std::vector<uint32_t> hc(D);
  std::vector<uint64_t> ho(D);
  CENTRE_CUDA(ctx, cudaMemcpyAsync(hc.data(), counts.p, sizeof(uint32_t) * D, cudaMemcpyDeviceToHost, st));
  CENTRE_CUDA(ctx, cudaStreamSynchronize(st));
  uint64_t total = 0;
  for (uint32_t d = 0; d < D; ++d) {
    ho[d] = total;
    total += hc[d];
  }
  *npairs = total;
  if (total > capacity)
    return set_error(ctx, CENTRE_E_ARG, "screen: pair capacity too small");
  CENTRE_CUDA(ctx, cudaMemcpyAsync(offs.p, ho.data(), sizeof(uint64_t) * D, cudaMemcpyHostToDevice, st));
  write_pairs_kernel<<<D, 32, 0, st>>>((uint32_t *)bitmap.p, D, (uint64_t *)offs.p, pairs);
  ctx->launches++;
  CENTRE_CUDA(ctx, cudaGetLastError());
  CENTRE_CUDA(ctx, cudaStreamSynchronize(st));
  return CENTRE_OK;
}

extern "C" int centre_gpu_screen(centre_ctx *ctx, const centre_entropy_params *p,
                                 const centre_screen_params *sp, uint32_t ndof,
                                 const uint8_t *types, const uint8_t *bins,
                                 const double *extremes, float *weights, float *losses,
                                 uint64_t capacity, uint32_t *pairs, uint64_t *npairs) {
  if (!ctx || !p || !sp || !types || !bins || !extremes || !pairs || !npairs)
    return set_error(ctx, CENTRE_E_ARG, "screen: null argument");
  cudaSetDevice(ctx->device);
  const uint64_t nbytes = (uint64_t)ndof * p->nschemes * p->nframes;
  Buf dt, db, de, dp;
  CENTRE_TRY(dalloc(ctx, dt, ndof));
  CENTRE_TRY(dalloc(ctx, db, nbytes));
  CENTRE_TRY(dalloc(ctx, de, sizeof(double) * 4 * ndof));
  CENTRE_TRY(dalloc(ctx, dp, sizeof(uint32_t) * 2 * std::max<uint64_t>(capacity, 1)));
  CENTRE_CUDA(ctx, cudaMemcpy(dt.p, types, ndof, cudaMemcpyHostToDevice));
  CENTRE_CUDA(ctx, cudaMemcpy(db.p, bins, nbytes, cudaMemcpyHostToDevice));
  CENTRE_CUDA(ctx, cudaMemcpy(de.p, extremes, sizeof(double) * 4 * ndof, cudaMemcpyHostToDevice));
  CENTRE_TRY(centre_gpu_screen_dev(ctx, p, sp, ndof, (const uint8_t *)dt.p, (const uint8_t *)db.p,
                                   (const double *)de.p, weights, losses, capacity,
                                   (uint32_t *)dp.p, npairs));
  CENTRE_CUDA(ctx, cudaMemcpy(pairs, dp.p, sizeof(uint32_t) * 2 * *npairs, cudaMemcpyDeviceToHost));
  return CENTRE_OK;
}
