// gi_mlp.cu -- the learned reconstructor: a 32 -> 64 -> 64 -> 64 -> 3 ReLU MLP
// that maps a few-ray interleaved gather plus G-buffer features to the many-ray
// indirect light.  BF16 weights and activations, FP32 accumulation on the tensor
// cores, FP32 master weights and Adam state.
//
// Kernels
//   features_kernel   32 bf16 features per pixel (layout below), for a full frame
//                     or for a list of march tiles (tile-major pixel order).
//   adam_kernel       Adam update of the FP32 masters, bf16 copies refreshed.
//   mlp_grad_partials_kernel  the allocation-free entry point's gradients on
//                     16x16x16 bf16 MMA fragments, one scratch slot per CTA.
//   (inference and training run on the 5th-generation tensor cores, in
//   gi_mlp_tc.cu: mlp_reconstruct_kernel -- features fused, or given rows for
//   gi_mlp_forward -- and mlp_train_tc_kernel -- forward with saved activations,
//   loss gradient, backward through all layers, per-CTA gradient sums added to
//   the FP32 gradient sums)
//
// Feature layout (channel: meaning), I = the few-ray indirect light:
//   0        linear depth d (depth moments .x)
//   1-3      world normal
//   4-6      albedo (linear)
//   7-9      I at the pixel (rgb)
//   10-12    F: I after the 5x5 bilateral filter, at the pixel (rgb)
//   13-18    luminance of I at (x-1,y), (x+1,y), (x,y-1), (x,y+1), (x-1,y-1), (x+1,y+1), clamp-to-edge
//   19-21    I at mip level 2 (rgb, bilinear at the pixel centre): the 4x4 box that spans all
//            16 interleave patterns
//   22-24    I at mip level 4 (rgb, bilinear)
//   25       depth deviation sqrt(max(0, E[d^2] - E[d]^2)) of the blurred moments at level 2
//   26-28    direct light at the pixel (rgb)
//   29-30    Hammersley offsets (angular, linear) of the pixel's interleave pattern
//   31       screen-space distance to the nearest viewport edge, min(u, 1-u, v, 1-v)
//
// Output head: the 3 outputs are softmax logits; the result is the weighted blend
// of three candidate estimates in the pixel's own feature row -- the bilaterally
// filtered few-ray light (10-12) and the few-ray light at mip 2 (19-21; its 4x4
// box spans all 16 interleave patterns once) and mip 4 (22-24).  The network thus
// chooses, per pixel, how far to average (edges keep the 5x5 bilateral, flat
// regions take the pattern-complete mip averages) and cannot add noise of its own.
//
// Exposure normalisation: light transport is linear in the light, so every
// light-dependent channel (7-24, 26-28) is divided by a per-pixel scale
// s = |lum(I at mip 2)| + |lum(I at mip 4)| + 1e-3 (the march's indirect light can be
// slightly negative), written beside the features, and the divided values are
// clamped to [-32, 32]; the
// blend is in units of s and is multiplied by s.  The network is then independent
// of the light's intensity; training weighs each pixel's squared error (in units
// of s) by a caller-given weight (s over its batch mean, so that pixels count by
// their light, as in a frame's relative L1 error).
#include <cuda_bf16.h>
#include <mma.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <type_traits>
#include <vector>

#include "gi_device.cuh"
#include "gi_internal.h"
#include "gi_kernels.h"
#include "gi_mlp.h"
#include "gi_features.cuh"
#include "gi_mlp_layout.h"

namespace gi {
namespace {

using namespace nvcuda;
using bf16 = __nv_bfloat16;
using namespace dev;

constexpr int kTileP = 64;   // pixels per CTA
constexpr int kThreads = 128;

// Shared memory layout of the MLP kernels (bytes, each region 1 KB aligned).
constexpr int sW = 0;                                   // bf16 weights, kWbf elements
constexpr int sX = sW + ((kWbf * 2 + 1023) / 1024) * 1024;  // bf16 [64 x 32]
constexpr int sH1 = sX + kTileP * kIn * 2;              // bf16 [64 x 64]
constexpr int sH2 = sH1 + kTileP * kHid * 2;
constexpr int sH3 = sH2 + kTileP * kHid * 2;
constexpr int sZ = sH3 + kTileP * kHid * 2;             // fp32 [64 x 64]
constexpr int sD = sZ + kTileP * kHid * 4;              // bf16 [64 x 64] (dZ of the current layer)
constexpr int sDY = sD + kTileP * kHid * 2;             // bf16 [64 x 16]
constexpr int sT = sDY + kTileP * kOutPad * 2;          // fp32 [64 x 4] targets
constexpr int sG = sT + kTileP * 4 * 4;                 // fp32 [64 x 64] gradient staging
constexpr int kSmemTrain = sG + kHid * kHid * 4;

template <int K, int N, typename BL>
__device__ __forceinline__ void gemm_rows(const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc) {
  // C[64 x N] = A[64 x K] * B[K x N]; warp w owns rows 16w..16w+15.
  const int warp = threadIdx.x >> 5;
  wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc[N / 16];
#pragma unroll
  for (int n = 0; n < N / 16; n++) wmma::fill_fragment(acc[n], 0.0f);
#pragma unroll
  for (int k = 0; k < K; k += 16) {
    wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::row_major> a;
    wmma::load_matrix_sync(a, A + warp * 16 * lda + k, lda);
#pragma unroll
    for (int n = 0; n < N / 16; n++) {
      wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, BL> b;
      if (std::is_same<BL, wmma::row_major>::value) wmma::load_matrix_sync(b, B + k * ldb + n * 16, ldb);
      else wmma::load_matrix_sync(b, B + n * 16 * ldb + k, ldb);
      wmma::mma_sync(acc[n], a, b, acc[n]);
    }
  }
#pragma unroll
  for (int n = 0; n < N / 16; n++)
    wmma::store_matrix_sync(C + warp * 16 * ldc + n * 16, acc[n], ldc, wmma::mem_row_major);
}

// G[M x N] = A^T * B over the tile's 64 pixels: A is [64 x M] row-major (read
// as an M x 64 column-major matrix), B is [64 x N] row-major.  Fragments are
// spread over the 4 warps; each is added into `grad` (row-major, N columns).
template <int M, int N>
__device__ __forceinline__ void grad_AtB(const bf16* A, int lda, const bf16* B, int ldb, float* stage,
                                         float* grad) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int FM = M / 16, FN = N / 16;
  for (int f = warp; f < FM * FN; f += 4) {
    const int fm = f / FN, fn = f % FN;
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
#pragma unroll
    for (int k = 0; k < kTileP; k += 16) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::col_major> a;
      wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> b;
      wmma::load_matrix_sync(a, A + k * lda + fm * 16, lda);
      wmma::load_matrix_sync(b, B + k * ldb + fn * 16, ldb);
      wmma::mma_sync(acc, a, b, acc);
    }
    float* st = stage + warp * 256;
    wmma::store_matrix_sync(st, acc, 16, wmma::mem_row_major);
    __syncwarp();
    for (int e = lane; e < 256; e += 32) {
      const int r = fm * 16 + e / 16, c = fn * 16 + e % 16;
      if (c < (N == kOutPad ? kOut : N)) atomicAdd(grad + r * (N == kOutPad ? kOut : N) + c, st[e]);
    }
    __syncwarp();
  }
}

// The three candidate estimates of a feature row (bf16 as the network sees them).
__device__ __forceinline__ void load_candidates(const bf16* x, float (&c)[3][3]) {
#pragma unroll
  for (int ch = 0; ch < 3; ch++) {
    c[0][ch] = __bfloat162float(x[kCand0 + ch]);
    c[1][ch] = __bfloat162float(x[kCand1 + ch]);
    c[2][ch] = __bfloat162float(x[kCand2 + ch]);
  }
}

// Loss term of one pixel and the gradient d of the summed weighted squared loss
// with respect to its 3 logits: y = the head's blend, e = y - T (T already divided
// by the exposure scale), g = 2 w clip(e, -1, 1) (a Huber-style gradient: a
// target the few-ray signal cannot explain does not swamp the batch), d = the
// head's backward of g.  z: the pixel's layer-4 accumulator row (before bias).
__device__ __forceinline__ float head_loss_grad(const float* z, const float* __restrict__ params, const bf16* x,
                                                const float* T, float (&d)[3]) {
  const float lo[3] = {z[0] + __ldg(params + ob4 + 0), z[1] + __ldg(params + ob4 + 1), z[2] + __ldg(params + ob4 + 2)};
  float c[3][3];
  load_candidates(x, c);
  return head_loss_grad_logits(lo, c, T, d);
}

__device__ __forceinline__ void stage_weights(const bf16* __restrict__ wb, char* smem) {
  const int4* src = reinterpret_cast<const int4*>(wb);
  int4* dst = reinterpret_cast<int4*>(smem + sW);
  for (int i = threadIdx.x; i < kWbf * 2 / 16; i += kThreads) dst[i] = src[i];
}

// bias + ReLU epilogue: Z (fp32, smem) -> H (bf16, smem).
__device__ __forceinline__ void relu_epilogue(const float* Z, const float* __restrict__ bias, bf16* H) {
  for (int i = threadIdx.x; i < kTileP * kHid; i += kThreads) {
    const float z = Z[i] + __ldg(bias + (i % kHid));
    H[i] = __float2bfloat16_rn(z > 0.0f ? z : 0.0f);
  }
}

// Forward through the 4 layers; leaves H1..H3 in shared memory and the output
// (before bias 4) in Z[:, 0:16].
__device__ void forward_tile(char* smem, const float* __restrict__ params) {
  bf16* W = reinterpret_cast<bf16*>(smem + sW);
  bf16* X = reinterpret_cast<bf16*>(smem + sX);
  bf16* H1 = reinterpret_cast<bf16*>(smem + sH1);
  bf16* H2 = reinterpret_cast<bf16*>(smem + sH2);
  bf16* H3 = reinterpret_cast<bf16*>(smem + sH3);
  float* Z = reinterpret_cast<float*>(smem + sZ);
  gemm_rows<kIn, kHid, wmma::row_major>(X, kIn, W + qW1, kHid, Z, kHid);
  __syncthreads();
  relu_epilogue(Z, params + ob1, H1);
  __syncthreads();
  gemm_rows<kHid, kHid, wmma::row_major>(H1, kHid, W + qW2, kHid, Z, kHid);
  __syncthreads();
  relu_epilogue(Z, params + ob2, H2);
  __syncthreads();
  gemm_rows<kHid, kHid, wmma::row_major>(H2, kHid, W + qW3, kHid, Z, kHid);
  __syncthreads();
  relu_epilogue(Z, params + ob3, H3);
  __syncthreads();
  gemm_rows<kHid, kOutPad, wmma::row_major>(H3, kHid, W + qW4, kOutPad, Z, kOutPad);
  __syncthreads();
}

__device__ __forceinline__ void load_x(char* smem, const bf16* __restrict__ feats, int base, int n) {
  int4* X = reinterpret_cast<int4*>(smem + sX);
  const int4* src = reinterpret_cast<const int4*>(feats);
  for (int i = threadIdx.x; i < kTileP * kIn * 2 / 16; i += kThreads) {
    const int row = i / (kIn * 2 / 16);
    X[i] = (base + row < n) ? src[(size_t)base * (kIn * 2 / 16) + i] : make_int4(0, 0, 0, 0);
  }
}

// Backward of one hidden layer: dH (fp32 in Z) -> dZ (bf16 in D) masked by the
// ReLU of H; bias gradient = column sums.
__device__ __forceinline__ void relu_backward(const float* dH, const bf16* H, bf16* D, float* __restrict__ gbias) {
  for (int i = threadIdx.x; i < kTileP * kHid; i += kThreads) {
    const float g = __bfloat162float(H[i]) > 0.0f ? dH[i] : 0.0f;
    D[i] = __float2bfloat16_rn(g);
  }
  __syncthreads();
  if (threadIdx.x < kHid) {
    float s = 0.0f;
    for (int r = 0; r < kTileP; r++) s += __bfloat162float(D[r * kHid + threadIdx.x]);
    atomicAdd(gbias + threadIdx.x, s);
  }
}

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ wb, float inv_batch, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  float gi_ = g[i] * inv_batch;
  g[i] = 0.0f;
  if (!isfinite(gi_)) gi_ = 0.0f;  // a non-finite gradient element counts as zero
  const float mi = b1 * m[i] + (1.0f - b1) * gi_;
  const float vi = b2 * v[i] + (1.0f - b2) * gi_ * gi_;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / c1, vh = vi / c2;
  const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
  p[i] = pi;
  // Refresh the bf16 copy of a weight.
  int q = -1;
  if (i >= oW1 && i < ob1) q = qW1 + (i - oW1);
  else if (i >= oW2 && i < ob2) q = qW2 + (i - oW2);
  else if (i >= oW3 && i < ob3) q = qW3 + (i - oW3);
  else if (i >= oW4 && i < ob4) q = qW4 + ((i - oW4) / kOut) * kOutPad + (i - oW4) % kOut;
  if (q >= 0) wb[q] = __float2bfloat16_rn(pi);
}

__global__ void sync_bf16_kernel(const float* __restrict__ p, bf16* __restrict__ wb) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kWbf) return;
  float v = 0.0f;
  if (q < qW2) v = p[oW1 + q];
  else if (q < qW3) v = p[oW2 + (q - qW2)];
  else if (q < qW4) v = p[oW3 + (q - qW3)];
  else {
    const int r = (q - qW4) / kOutPad, c = (q - qW4) % kOutPad;
    v = c < kOut ? p[oW4 + r * kOut + c] : 0.0f;
  }
  wb[q] = __float2bfloat16_rn(v);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) features_kernel(const __grid_constant__ FeatureArgs a) {
  const int P = a.pattern;
  const int tw = kMarchTileSubX * P, th = kMarchTileSubY * P;
  int x, y;
  size_t out_idx;
  if (a.tiles) {
    const int t = blockIdx.y;
    const int tile = __ldg(a.tiles + t);
    const int txn = (a.width + tw - 1) / tw;
    const int tyn = (a.height + th - 1) / th;
    if (tile < 0 || tile >= txn * tyn) return;
    const int local = blockIdx.x * blockDim.x + threadIdx.x;
    if (local >= tw * th) return;
    x = (tile % txn) * tw + local % tw;
    y = (tile / txn) * th + local / tw;
    out_idx = (size_t)t * tw * th + local;
    if (x >= a.width || y >= a.height) {
      int4* o = reinterpret_cast<int4*>(a.out + out_idx * kIn);
      for (int k = 0; k < 4; k++) o[k] = make_int4(0, 0, 0, 0);
      a.scale[out_idx] = 1.0f;
      return;
    }
  } else {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.width * a.height) return;
    x = p % a.width;
    y = p / a.width;
    out_idx = p;
  }
  float f[kIn];
  float scale;
  pixel_features(a, x, y, f, scale);
  a.scale[out_idx] = scale;
  __align__(16) bf16 q[kIn];
#pragma unroll
  for (int i = 0; i < kIn; i++) q[i] = __float2bfloat16_rn(f[i]);
  int4* o = reinterpret_cast<int4*>(a.out + out_idx * kIn);
  const int4* qi = reinterpret_cast<const int4*>(q);
#pragma unroll
  for (int i = 0; i < 4; i++) o[i] = qi[i];
}

// Gathers 4-channel pixels of the listed march tiles into tile-major order.
__global__ void gather_tiles_kernel(const float* __restrict__ img, int W, int H, int P, const int* __restrict__ tiles,
                                    float* __restrict__ out) {
  const int tw = kMarchTileSubX * P, th = kMarchTileSubY * P;
  const int t = blockIdx.y, local = blockIdx.x * blockDim.x + threadIdx.x;
  if (local >= tw * th) return;
  const int txn = (W + tw - 1) / tw, tyn = (H + th - 1) / th;
  const int tile = __ldg(tiles + t);
  const size_t o = (size_t)t * tw * th + local;
  float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (tile >= 0 && tile < txn * tyn) {
    const int x = (tile % txn) * tw + local % tw, y = (tile / txn) * th + local / tw;
    if (x < W && y < H) v = ld4(img, y * W + x);
  }
  reinterpret_cast<float4*>(out)[o] = v;
}

// Writes tile-major 4-channel values back into the image at the tiles' pixels.
__global__ void scatter_tiles_kernel(const float* __restrict__ vals, int W, int H, int P,
                                     const int* __restrict__ tiles, float* __restrict__ img) {
  const int tw = kMarchTileSubX * P, th = kMarchTileSubY * P;
  const int t = blockIdx.y, local = blockIdx.x * blockDim.x + threadIdx.x;
  if (local >= tw * th) return;
  const int txn = (W + tw - 1) / tw, tyn = (H + th - 1) / th;
  const int tile = __ldg(tiles + t);
  if (tile < 0 || tile >= txn * tyn) return;
  const int x = (tile % txn) * tw + local % tw, y = (tile / txn) * th + local / tw;
  if (x >= W || y >= H) return;
  reinterpret_cast<float4*>(img)[y * W + x] = ld4(vals, (int)((size_t)t * tw * th + local));
}

// Tile judge: one CTA per judged tile compares the learned indirect light with
// the plain gather over the tile (relative L1 over rgb); above `threshold` the
// tile falls back to the plain result.  counters[0] += judged, [1] += fell back.
__global__ void __launch_bounds__(256) judge_tiles_kernel(float* __restrict__ learned,
                                                          const float* __restrict__ plain, int W, int H, int P,
                                                          const int* __restrict__ tiles, float threshold,
                                                          int* __restrict__ counters) {
  __shared__ float s_num[8], s_den[8];
  __shared__ int s_fall;
  const int tw = kMarchTileSubX * P, th = kMarchTileSubY * P;
  const int txn = (W + tw - 1) / tw, tyn = (H + th - 1) / th;
  const int tile = __ldg(tiles + blockIdx.x);
  if (tile < 0 || tile >= txn * tyn) return;
  const int x0 = (tile % txn) * tw, y0 = (tile / txn) * th;
  float num = 0.0f, den = 0.0f;
  for (int i = threadIdx.x; i < tw * th; i += blockDim.x) {
    const int x = x0 + i % tw, y = y0 + i / tw;
    if (x >= W || y >= H) continue;
    const float4 l = ld4(learned, y * W + x), p = ld4(plain, y * W + x);
    num += fabsf(l.x - p.x) + fabsf(l.y - p.y) + fabsf(l.z - p.z);
    den += fabsf(p.x) + fabsf(p.y) + fabsf(p.z);
  }
  for (int o = 16; o > 0; o >>= 1) {
    num += __shfl_xor_sync(0xffffffffu, num, o);
    den += __shfl_xor_sync(0xffffffffu, den, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_num[threadIdx.x >> 5] = num;
    s_den[threadIdx.x >> 5] = den;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float n = 0.0f, d = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      n += s_num[k];
      d += s_den[k];
    }
    s_fall = n > threshold * fmaxf(d, 1e-20f);
    atomicAdd(counters + 0, 1);
    if (s_fall) atomicAdd(counters + 1, 1);
  }
  __syncthreads();
  if (!s_fall) return;
  for (int i = threadIdx.x; i < tw * th; i += blockDim.x) {
    const int x = x0 + i % tw, y = y0 + i / tw;
    if (x >= W || y >= H) continue;
    reinterpret_cast<float4*>(learned)[y * W + x] = ld4(plain, y * W + x);
  }
}

// ---------------------------------------------------------------------------
// Allocation-free gradients (gi_mlp_gradients_noalloc).  Its scratch is one
// file-scope device array: a bf16 copy of the caller's weights and one slot of
// gradient sums per 64-pixel CTA, summed by a second kernel in CTA order (so the
// result is also the same bits from call to call).  Every slot a call reads is
// written earlier in the same call, so nothing in it needs clearing.
constexpr int kNoAllocMaxPixels = 8192;
constexpr int kNoAllocMaxCtas = kNoAllocMaxPixels / kTileP;

struct NoAllocScratch {
  bf16 wb[kWbf];                          // 22,528 bytes
  float loss[kNoAllocMaxCtas];            // per-CTA summed squared error
  float grads[kNoAllocMaxCtas][kParams];  // per-CTA gradient sums, 5.4 MB
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// grad_AtB with the fragment written (not added) into `grad`.
template <int M, int N>
__device__ __forceinline__ void grad_AtB_store(const bf16* A, int lda, const bf16* B, int ldb, float* stage,
                                               float* grad) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int FM = M / 16, FN = N / 16;
  for (int f = warp; f < FM * FN; f += 4) {
    const int fm = f / FN, fn = f % FN;
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc;
    wmma::fill_fragment(acc, 0.0f);
#pragma unroll
    for (int k = 0; k < kTileP; k += 16) {
      wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::col_major> a;
      wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> b;
      wmma::load_matrix_sync(a, A + k * lda + fm * 16, lda);
      wmma::load_matrix_sync(b, B + k * ldb + fn * 16, ldb);
      wmma::mma_sync(acc, a, b, acc);
    }
    float* st = stage + warp * 256;
    wmma::store_matrix_sync(st, acc, 16, wmma::mem_row_major);
    __syncwarp();
    for (int e = lane; e < 256; e += 32) {
      const int r = fm * 16 + e / 16, c = fn * 16 + e % 16;
      if (c < (N == kOutPad ? kOut : N)) grad[r * (N == kOutPad ? kOut : N) + c] = st[e];
    }
    __syncwarp();
  }
}

__device__ __forceinline__ void relu_backward_store(const float* dH, const bf16* H, bf16* D, float* gbias) {
  for (int i = threadIdx.x; i < kTileP * kHid; i += kThreads) {
    const float g = __bfloat162float(H[i]) > 0.0f ? dH[i] : 0.0f;
    D[i] = __float2bfloat16_rn(g);
  }
  __syncthreads();
  if (threadIdx.x < kHid) {
    float s = 0.0f;
    for (int r = 0; r < kTileP; r++) s += __bfloat162float(D[r * kHid + threadIdx.x]);
    gbias[threadIdx.x] = s;
  }
}

// One 64-pixel tile's forward, loss gradient and backward on 16x16x16 bf16 MMA
// fragments (the roundings of the training kernel: bf16 operands, FP32 sums,
// FP32 bias and head), with each CTA's sums stored in its own scratch slot
// instead of added to shared sums.
__global__ void __launch_bounds__(kThreads) mlp_grad_partials_kernel(const bf16* __restrict__ feats,
                                                                     const float* __restrict__ targets,
                                                                     const float* __restrict__ scale, int n,
                                                                     const float* __restrict__ params,
                                                                     NoAllocScratch* __restrict__ scratch) {
  extern __shared__ __align__(1024) char smem[];
  __shared__ float s_loss[kThreads / 32];
  const int base = blockIdx.x * kTileP;
  float* gout = scratch->grads[blockIdx.x];
  stage_weights(scratch->wb, smem);
  load_x(smem, feats, base, n);
  float* T = reinterpret_cast<float*>(smem + sT);
  for (int i = threadIdx.x; i < kTileP * 4; i += kThreads) {
    const int r = base + i / 4;
    // rgb divided by the exposure scale; channel 3 is the pixel's loss weight, as given
    const float raw = (r < n) ? __ldg(targets + (size_t)base * 4 + i) : 0.0f;
    T[i] = ((i & 3) == 3 || !scale || r >= n) ? raw : raw / __ldg(scale + r);
  }
  __syncthreads();
  forward_tile(smem, params);
  bf16* W = reinterpret_cast<bf16*>(smem + sW);
  bf16* X = reinterpret_cast<bf16*>(smem + sX);
  bf16* H1 = reinterpret_cast<bf16*>(smem + sH1);
  bf16* H2 = reinterpret_cast<bf16*>(smem + sH2);
  bf16* H3 = reinterpret_cast<bf16*>(smem + sH3);
  float* Z = reinterpret_cast<float*>(smem + sZ);
  bf16* D = reinterpret_cast<bf16*>(smem + sD);
  bf16* DY = reinterpret_cast<bf16*>(smem + sDY);
  float* G = reinterpret_cast<float*>(smem + sG);
  float lsum = 0.0f;
  for (int r = threadIdx.x; r < kTileP; r += kThreads) {
    float d[3] = {0.0f, 0.0f, 0.0f};
    if (base + r < n) lsum += head_loss_grad(Z + r * kOutPad, params, X + r * kIn, T + r * 4, d);
#pragma unroll
    for (int c = 0; c < kOutPad; c++) DY[r * kOutPad + c] = __float2bfloat16_rn(c < kOut ? d[c] : 0.0f);
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int k = 0; k < kThreads / 32; k++) t += s_loss[k];
    scratch->loss[blockIdx.x] = t;
  }
  if (threadIdx.x < kOut) {
    float s = 0.0f;
    for (int r = 0; r < kTileP; r++) s += __bfloat162float(DY[r * kOutPad + threadIdx.x]);
    gout[ob4 + threadIdx.x] = s;
  }
  grad_AtB_store<kHid, kOutPad>(H3, kHid, DY, kOutPad, G, gout + oW4);
  gemm_rows<kOutPad, kHid, wmma::col_major>(DY, kOutPad, W + qW4, kOutPad, Z, kHid);
  __syncthreads();
  relu_backward_store(Z, H3, D, gout + ob3);
  __syncthreads();
  grad_AtB_store<kHid, kHid>(H2, kHid, D, kHid, G, gout + oW3);
  gemm_rows<kHid, kHid, wmma::col_major>(D, kHid, W + qW3, kHid, Z, kHid);
  __syncthreads();
  relu_backward_store(Z, H2, D, gout + ob2);
  __syncthreads();
  grad_AtB_store<kHid, kHid>(H1, kHid, D, kHid, G, gout + oW2);
  gemm_rows<kHid, kHid, wmma::col_major>(D, kHid, W + qW2, kHid, Z, kHid);
  __syncthreads();
  relu_backward_store(Z, H1, D, gout + ob1);
  __syncthreads();
  grad_AtB_store<kIn, kHid>(X, kIn, D, kHid, G, gout + oW1);
}

// Sums the per-CTA slots in CTA order and divides by the batch (mean-loss gradient).
__global__ void noalloc_reduce_kernel(const NoAllocScratch* __restrict__ scratch, int ctas, int n,
                                      float* __restrict__ grads, float* __restrict__ loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kParams) {
    float s = 0.0f;
    for (int c = 0; c < ctas; c++) s += scratch->grads[c][p];
    grads[p] = s / (float)n;
  } else if (p == kParams) {
    float s = 0.0f;
    for (int c = 0; c < ctas; c++) s += scratch->loss[c];
    *loss = s / (float)(n * kOut);
  }
}

uint32_t crc32(const void* data, size_t n, uint32_t crc = 0) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  crc = ~crc;
  const uint8_t* p = static_cast<const uint8_t*>(data);
  for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

}  // namespace

int launch_features(const FeatureArgs& a, int num_tiles, cudaStream_t stream) {
  if (a.tiles) {
    const int tp = kMarchTileSubX * kMarchTileSubY * a.pattern * a.pattern;
    if (num_tiles == 0) return GI_OK;
    features_kernel<<<dim3((tp + 255) / 256, num_tiles), 256, 0, stream>>>(a);
  } else {
    const int n = a.width * a.height;
    features_kernel<<<(n + 255) / 256, 256, 0, stream>>>(a);
  }
  GI_CHECK_LAUNCH("features_kernel");
  count_launches(1);
  return GI_OK;
}

int launch_tiles_copy(const float* src, float* dst, int W, int H, int P, const int* tiles, int num_tiles,
                      bool scatter, cudaStream_t stream) {
  if (num_tiles == 0) return GI_OK;
  const int tp = kMarchTileSubX * kMarchTileSubY * P * P;
  dim3 grid((tp + 255) / 256, num_tiles);
  if (scatter) scatter_tiles_kernel<<<grid, 256, 0, stream>>>(src, W, H, P, tiles, dst);
  else gather_tiles_kernel<<<grid, 256, 0, stream>>>(src, W, H, P, tiles, dst);
  GI_CHECK_LAUNCH("tiles_copy_kernel");
  count_launches(1);
  return GI_OK;
}

int launch_judge(float* learned, const float* plain, int W, int H, int P, const int* tiles, int num_tiles,
                 float threshold, int* counters, cudaStream_t stream) {
  if (num_tiles == 0) return GI_OK;
  judge_tiles_kernel<<<num_tiles, 256, 0, stream>>>(learned, plain, W, H, P, tiles, threshold, counters);
  GI_CHECK_LAUNCH("judge_tiles_kernel");
  count_launches(1);
  return GI_OK;
}

struct Mlp {
  float* params = nullptr;
  float* grads = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* loss = nullptr;
  bf16* wb = nullptr;
  int step = 0;
  int loss_kind = GI_MLP_LOSS_SQUARED;  // training loss (gi_mlp_set_loss)
  ~Mlp() {
    dfree(params);
    dfree(grads);
    dfree(m);
    dfree(v);
    dfree(loss);
    dfree(wb);
  }
};

// gi_mlp_forward: the fused reconstruction kernel on given feature rows (tcgen05).
int mlp_forward(const Mlp* m, const void* feats, const float* scale, int n, float* out, cudaStream_t s) {
  return launch_forward_tc(static_cast<const bf16*>(feats), scale, n, m->wb, m->params, out, s);
}

}  // namespace gi

struct gi_mlp {
  gi::Mlp impl;
};

using namespace gi;

extern "C" int gi_mlp_param_count(void) { return kParams; }

extern "C" int gi_mlp_create(gi_mlp** out) {
  GI_CHECK_ARG(out, "gi_mlp_create: null");
  *out = nullptr;
  std::unique_ptr<gi_mlp> m(new gi_mlp);
  Mlp& M = m->impl;
  int e = GI_OK;
  e = e ? e : check_cuda(dmalloc(&M.params, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(dmalloc(&M.grads, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(dmalloc(&M.m, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(dmalloc(&M.v, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(dmalloc(&M.loss, 4), "gi_mlp_create");
  e = e ? e : check_cuda(dmalloc(&M.wb, kWbf * 2), "gi_mlp_create");
  if (e) return e;
  e = check_cuda(cudaMemset(M.grads, 0, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(cudaMemset(M.m, 0, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(cudaMemset(M.v, 0, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(cudaMemset(M.loss, 0, 4), "gi_mlp_create");
  e = e ? e : check_cuda(cudaMemset(M.params, 0, kParams * 4), "gi_mlp_create");
  e = e ? e : check_cuda(cudaMemset(M.wb, 0, kWbf * 2), "gi_mlp_create");
  if (e) return e;
  *out = m.release();
  return GI_OK;
}

extern "C" int gi_mlp_destroy(gi_mlp* m) {
  delete m;
  return GI_OK;
}

extern "C" int gi_mlp_set_params(gi_mlp* m, const float* host, int count) {
  GI_CHECK_ARG(m && host && count == kParams, "gi_mlp_set_params: bad arguments");
  int e = check_cuda(cudaMemcpy(m->impl.params, host, kParams * 4, cudaMemcpyHostToDevice), "gi_mlp_set_params");
  if (e) return e;
  sync_bf16_kernel<<<(kWbf + 255) / 256, 256>>>(m->impl.params, m->impl.wb);
  GI_CHECK_LAUNCH("sync_bf16_kernel");
  count_launches(1);
  return check_cuda(cudaDeviceSynchronize(), "gi_mlp_set_params");
}

extern "C" int gi_mlp_get_params(const gi_mlp* m, float* host, int count) {
  GI_CHECK_ARG(m && host && count == kParams, "gi_mlp_get_params: bad arguments");
  return check_cuda(cudaMemcpy(host, m->impl.params, kParams * 4, cudaMemcpyDeviceToHost), "gi_mlp_get_params");
}

extern "C" int gi_mlp_init(gi_mlp* m, uint64_t seed) {
  GI_CHECK_ARG(m, "gi_mlp_init: null");
  std::vector<float> p(kParams, 0.0f);
  std::mt19937_64 g(seed);
  auto fill = [&](int off, int fan_in, int count) {
    const double lim = std::sqrt(6.0 / fan_in);  // He-uniform for ReLU layers
    for (int i = 0; i < count; i++) p[off + i] = (float)((((g() >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0) * lim);
  };
  fill(oW1, kIn, kIn * kHid);
  fill(oW2, kHid, kHid * kHid);
  fill(oW3, kHid, kHid * kHid);
  fill(oW4, kHid, kHid * kOut);
  m->impl.step = 0;
  int e = check_cuda(cudaMemset(m->impl.m, 0, kParams * 4), "gi_mlp_init");
  e = e ? e : check_cuda(cudaMemset(m->impl.v, 0, kParams * 4), "gi_mlp_init");
  e = e ? e : check_cuda(cudaMemset(m->impl.grads, 0, kParams * 4), "gi_mlp_init");
  if (e) return e;
  return gi_mlp_set_params(m, p.data(), kParams);
}

extern "C" int gi_mlp_forward(const gi_mlp* m, const void* features, const float* scale, int n, float* out,
                              void* stream) {
  GI_CHECK_ARG(m && features && out && n >= 0, "gi_mlp_forward: bad arguments");
  GI_CHECK_ARG(aligned16(features) && aligned16(out), "gi_mlp_forward: unaligned buffer");
  return mlp_forward(&m->impl, features, scale, n, out, (cudaStream_t)stream);
}

extern "C" int gi_mlp_train_step(gi_mlp* m, const void* features, const float* targets, const float* scale, int n,
                                 float lr, float* loss_out, void* stream) {
  GI_CHECK_ARG(m && features && targets && n > 0, "gi_mlp_train_step: bad arguments");
  GI_CHECK_ARG(aligned16(features) && aligned16(targets), "gi_mlp_train_step: unaligned buffer");
  cudaStream_t s = (cudaStream_t)stream;
  Mlp& M = m->impl;
  int e = check_cuda(cudaMemsetAsync(M.loss, 0, 4, s), "gi_mlp_train_step");
  e = e ? e : launch_train_tc(static_cast<const bf16*>(features), targets, scale, n, M.wb, M.params, M.grads, M.loss,
                              M.loss_kind, s);
  if (e) return e;
  M.step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - (float)std::pow((double)b1, M.step), c2 = 1.0f - (float)std::pow((double)b2, M.step);
  adam_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(M.params, M.grads, M.m, M.v, M.wb, 1.0f / (float)n, lr, b1, b2,
                                                    1e-8f, c1, c2);
  GI_CHECK_LAUNCH("adam_kernel");
  count_launches(1);
  if (loss_out) {
    float l = 0.0f;
    e = check_cuda(cudaMemcpyAsync(&l, M.loss, 4, cudaMemcpyDeviceToHost, s), "gi_mlp_train_step: loss");
    if (e) return e;
    e = check_cuda(cudaStreamSynchronize(s), "gi_mlp_train_step: sync");
    if (e) return e;
    *loss_out = l / (float)(n * kOut);
  }
  return GI_OK;
}

extern "C" int gi_mlp_set_loss(gi_mlp* m, int loss) {
  GI_CHECK_ARG(m, "gi_mlp_set_loss: null network");
  GI_CHECK_ARG(loss == GI_MLP_LOSS_SQUARED || loss == GI_MLP_LOSS_ABSOLUTE, "gi_mlp_set_loss: unknown loss");
  m->impl.loss_kind = loss;
  return GI_OK;
}

extern "C" int gi_mlp_gradients(gi_mlp* m, const void* features, const float* targets, const float* scale, int n,
                                float* grads_host, float* loss_host, void* stream) {
  GI_CHECK_ARG(m && features && targets && n > 0 && grads_host, "gi_mlp_gradients: bad arguments");
  GI_CHECK_ARG(aligned16(features) && aligned16(targets), "gi_mlp_gradients: unaligned buffer");
  cudaStream_t s = (cudaStream_t)stream;
  Mlp& M = m->impl;
  int e = check_cuda(cudaMemsetAsync(M.loss, 0, 4, s), "gi_mlp_gradients");
  e = e ? e : check_cuda(cudaMemsetAsync(M.grads, 0, kParams * 4, s), "gi_mlp_gradients");
  e = e ? e : launch_train_tc(static_cast<const bf16*>(features), targets, scale, n, M.wb, M.params, M.grads, M.loss,
                              M.loss_kind, s);
  if (e) return e;
  std::vector<float> g(kParams);
  float l = 0.0f;
  e = check_cuda(cudaMemcpyAsync(g.data(), M.grads, kParams * 4, cudaMemcpyDeviceToHost, s), "gi_mlp_gradients");
  e = e ? e : check_cuda(cudaMemcpyAsync(&l, M.loss, 4, cudaMemcpyDeviceToHost, s), "gi_mlp_gradients");
  e = e ? e : check_cuda(cudaMemsetAsync(M.grads, 0, kParams * 4, s), "gi_mlp_gradients");
  e = e ? e : check_cuda(cudaStreamSynchronize(s), "gi_mlp_gradients");
  if (e) return e;
  for (int i = 0; i < kParams; i++) grads_host[i] = g[i] / (float)n;
  if (loss_host) *loss_host = l / (float)(n * kOut);
  return GI_OK;
}

// Checkpoint: "GIMLP001", u32 param count, u32 Adam step, params, m, v (fp32),
// u32 CRC-32 of everything before it.
extern "C" int gi_mlp_save(const gi_mlp* m, const char* path) {
  GI_CHECK_ARG(m && path, "gi_mlp_save: bad arguments");
  std::vector<float> buf(3 * kParams);
  int e = check_cuda(cudaMemcpy(buf.data(), m->impl.params, kParams * 4, cudaMemcpyDeviceToHost), "gi_mlp_save");
  e = e ? e : check_cuda(cudaMemcpy(buf.data() + kParams, m->impl.m, kParams * 4, cudaMemcpyDeviceToHost), "gi_mlp_save");
  e = e ? e : check_cuda(cudaMemcpy(buf.data() + 2 * kParams, m->impl.v, kParams * 4, cudaMemcpyDeviceToHost), "gi_mlp_save");
  if (e) return e;
  std::vector<char> out(8 + 8 + buf.size() * 4 + 4);
  memcpy(out.data(), "GIMLP001", 8);
  uint32_t hdr[2] = {(uint32_t)kParams, (uint32_t)m->impl.step};
  memcpy(out.data() + 8, hdr, 8);
  memcpy(out.data() + 16, buf.data(), buf.size() * 4);
  uint32_t crc = crc32(out.data(), out.size() - 4);
  memcpy(out.data() + out.size() - 4, &crc, 4);
  FILE* f = fopen(path, "wb");
  if (!f) return fail(GI_ERR_IO, std::string("gi_mlp_save: cannot open ") + path);
  size_t w = fwrite(out.data(), 1, out.size(), f);
  fclose(f);
  return w == out.size() ? GI_OK : fail(GI_ERR_IO, "gi_mlp_save: short write");
}

extern "C" int gi_mlp_load(gi_mlp* m, const char* path) {
  GI_CHECK_ARG(m && path, "gi_mlp_load: bad arguments");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(GI_ERR_IO, std::string("gi_mlp_load: cannot open ") + path);
  std::vector<char> in(16 + (size_t)kParams * 12 + 4);
  size_t r = fread(in.data(), 1, in.size(), f);
  char extra;
  bool trailing = fread(&extra, 1, 1, f) == 1;
  fclose(f);
  if (r != in.size() || trailing) return fail(GI_ERR_IO, "gi_mlp_load: wrong file size");
  if (memcmp(in.data(), "GIMLP001", 8) != 0) return fail(GI_ERR_IO, "gi_mlp_load: bad magic");
  uint32_t hdr[2];
  memcpy(hdr, in.data() + 8, 8);
  if (hdr[0] != (uint32_t)kParams) return fail(GI_ERR_IO, "gi_mlp_load: parameter count mismatch");
  uint32_t crc;
  memcpy(&crc, in.data() + in.size() - 4, 4);
  if (crc != crc32(in.data(), in.size() - 4)) return fail(GI_ERR_IO, "gi_mlp_load: CRC mismatch");
  const float* p = reinterpret_cast<const float*>(in.data() + 16);
  int e = gi_mlp_set_params(m, p, kParams);
  e = e ? e : check_cuda(cudaMemcpy(m->impl.m, p + kParams, kParams * 4, cudaMemcpyHostToDevice), "gi_mlp_load");
  e = e ? e : check_cuda(cudaMemcpy(m->impl.v, p + 2 * kParams, kParams * 4, cudaMemcpyHostToDevice), "gi_mlp_load");
  if (e) return e;
  m->impl.step = (int)hdr[1];
  return GI_OK;
}

extern "C" int gi_features(int width, int height, int pattern_size, const float* depth_moments, const float* normal,
                           const float* albedo, const float* direct, const float* const* indirect_levels,
                           const float* filtered, const float* depth_blur_l2, void* out, float* scale,
                           const int* tiles, int num_tiles, void* stream) {
  GI_CHECK_ARG(width >= 16 && height >= 16 && pattern_size >= 1 && pattern_size <= 8, "gi_features: bad size");
  GI_CHECK_ARG(depth_moments && normal && albedo && direct && indirect_levels && filtered && depth_blur_l2 && out &&
                   scale,
               "gi_features: null argument");
  GI_CHECK_ARG(indirect_levels[0] && indirect_levels[1] && indirect_levels[2], "gi_features: null indirect level");
  GI_CHECK_ARG(aligned16(out) && aligned16(normal) && aligned16(albedo) && aligned16(direct) && aligned16(filtered),
               "gi_features: unaligned buffer");
  GI_CHECK_ARG(!tiles || num_tiles >= 0, "gi_features: bad tile count");
  FeatureArgs a{};
  a.width = width;
  a.height = height;
  a.pattern = pattern_size;
  a.moments = depth_moments;
  a.normal = normal;
  a.albedo = albedo;
  a.direct = direct;
  for (int k = 0; k < 3; k++) a.indirect[k] = indirect_levels[k];
  a.depth_l2 = depth_blur_l2;
  a.filtered = filtered;
  a.out = static_cast<__nv_bfloat16*>(out);
  a.scale = scale;
  a.tiles = tiles;
  return launch_features(a, num_tiles, (cudaStream_t)stream);
}

extern "C" int gi_mlp_reconstruct(const gi_mlp* m, int width, int height, int pattern_size,
                                  const float* depth_moments, const float* normal, const float* albedo,
                                  const float* direct, const float* const* indirect_levels, const float* filtered,
                                  const float* depth_blur_l2, float* out, void* stream) {
  GI_CHECK_ARG(m, "gi_mlp_reconstruct: null network");
  GI_CHECK_ARG(width >= 16 && height >= 16 && pattern_size >= 1 && pattern_size <= 8,
               "gi_mlp_reconstruct: bad size");
  GI_CHECK_ARG(depth_moments && normal && albedo && direct && indirect_levels && filtered && depth_blur_l2 && out,
               "gi_mlp_reconstruct: null argument");
  GI_CHECK_ARG(indirect_levels[0] && indirect_levels[1] && indirect_levels[2],
               "gi_mlp_reconstruct: null indirect level");
  GI_CHECK_ARG(aligned16(out) && aligned16(normal) && aligned16(albedo) && aligned16(direct) && aligned16(filtered),
               "gi_mlp_reconstruct: unaligned buffer");
  FeatureArgs a{};
  a.width = width;
  a.height = height;
  a.pattern = pattern_size;
  a.moments = depth_moments;
  a.normal = normal;
  a.albedo = albedo;
  a.direct = direct;
  for (int k = 0; k < 3; k++) a.indirect[k] = indirect_levels[k];
  a.depth_l2 = depth_blur_l2;
  a.filtered = filtered;
  return launch_reconstruct(a, m->impl.wb, m->impl.params, out, (cudaStream_t)stream);
}

extern "C" int gi_mlp_tensor_core_errors(int* count) {
  GI_CHECK_ARG(count, "gi_mlp_tensor_core_errors: null");
  return reconstruct_errors(count);
}

extern "C" int gi_debug_tensor_core_wait_limit(long long cycles) { return reconstruct_wait_limit(cycles); }

extern "C" int gi_gather_tiles(const float* image, int width, int height, int pattern_size, const int* tiles,
                               int num_tiles, float* out, void* stream) {
  GI_CHECK_ARG(image && tiles && out && num_tiles >= 0 && pattern_size >= 1 && pattern_size <= 8,
               "gi_gather_tiles: bad arguments");
  return launch_tiles_copy(image, out, width, height, pattern_size, tiles, num_tiles, false, (cudaStream_t)stream);
}

extern "C" int gi_scatter_tiles(const float* values, int width, int height, int pattern_size, const int* tiles,
                                int num_tiles, float* image, void* stream) {
  GI_CHECK_ARG(image && tiles && values && num_tiles >= 0 && pattern_size >= 1 && pattern_size <= 8,
               "gi_scatter_tiles: bad arguments");
  return launch_tiles_copy(values, image, width, height, pattern_size, tiles, num_tiles, true, (cudaStream_t)stream);
}

// Per-device set-up of the allocation-free entry point: the device address of
// the file-scope scratch array (host code cannot use the array's name as a
// device pointer) and the kernel's shared-memory limit.
static std::mutex g_noalloc_mutex;
static NoAllocScratch* g_noalloc_ptr[64] = {};

static int noalloc_setup(NoAllocScratch** out, cudaStream_t stream) {
  int dev = 0;
  int e = check_cuda(cudaGetDevice(&dev), "gi_mlp_gradients_noalloc: cudaGetDevice");
  if (e) return e;
  GI_CHECK_ARG(dev >= 0 && dev < 64, "gi_mlp_gradients_noalloc: device index above 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    // The set-up's runtime calls must not land inside a caller's stream capture.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = check_cuda(cudaStreamIsCapturing(stream, &cs), "gi_mlp_gradients_noalloc: capture status");
    if (e) return e;
    if (cs != cudaStreamCaptureStatusNone)
      return fail(GI_ERR_INVALID_ARGUMENT,
                  "gi_mlp_gradients_noalloc: the first call on a device sets it up and cannot run on a stream "
                  "in capture mode");
    void* ptr = nullptr;
    e = check_cuda(cudaGetSymbolAddress(&ptr, g_noalloc_scratch), "gi_mlp_gradients_noalloc: cudaGetSymbolAddress");
    if (e) return e;
    e = check_cuda(cudaFuncSetAttribute(mlp_grad_partials_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kSmemTrain),
                   "gi_mlp_gradients_noalloc: shared memory limit");
    if (e) return e;
    g_noalloc_ptr[dev] = static_cast<NoAllocScratch*>(ptr);
  }
  *out = g_noalloc_ptr[dev];
  return GI_OK;
}

extern "C" int gi_mlp_gradients_noalloc(const float* params, const void* features, const float* targets,
                                        const float* scale, int n, float* grads, float* loss, void* stream) {
  GI_CHECK_ARG(params && features && targets && grads && loss, "gi_mlp_gradients_noalloc: null argument");
  GI_CHECK_ARG(aligned16(features) && aligned16(targets), "gi_mlp_gradients_noalloc: unaligned buffer");
  GI_CHECK_ARG(n >= 1, "gi_mlp_gradients_noalloc: empty batch");
  if (n > kNoAllocMaxPixels)
    return fail(GI_ERR_INVALID_ARGUMENT, "gi_mlp_gradients_noalloc: batch of " + std::to_string(n) +
                                             " pixels exceeds the allocation-free maximum of " +
                                             std::to_string(kNoAllocMaxPixels));
  NoAllocScratch* scratch = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  int e = noalloc_setup(&scratch, s);
  if (e) return e;
  const int ctas = (n + kTileP - 1) / kTileP;
  sync_bf16_kernel<<<(kWbf + 255) / 256, 256, 0, s>>>(params, scratch->wb);
  GI_CHECK_LAUNCH("gi_mlp_gradients_noalloc: weight copy");
  mlp_grad_partials_kernel<<<ctas, kThreads, kSmemTrain, s>>>(static_cast<const bf16*>(features), targets, scale,
                                                               n, params, scratch);
  GI_CHECK_LAUNCH("gi_mlp_gradients_noalloc: partial sums");
  noalloc_reduce_kernel<<<(kParams + 1 + 255) / 256, 256, 0, s>>>(scratch, ctas, n, grads, loss);
  GI_CHECK_LAUNCH("gi_mlp_gradients_noalloc: reduction");
  count_launches(3);
  return GI_OK;
}
