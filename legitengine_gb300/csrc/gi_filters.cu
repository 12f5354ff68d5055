// gi_filters.cu -- the passes after the march: the 5x5 depth/normal bilateral
// filter, the least-squares denoiser (Common/denoiser.frag:72-184), the final
// gather (Common/finalGatherer.frag:42-59), and the deinterleave / interleave
// permutations (Common/deinterleave.frag, Common/interleave.frag).
#include "gi_device.cuh"
#include "gi_internal.h"
#include "gi_kernels.h"

namespace gi {
namespace {

using namespace dev;

constexpr int kTx = 32, kTy = 8;

template <int DCH> __device__ __forceinline__ float depth_at(const float* p, int idx) {
  if (DCH == 2) return __ldg(reinterpret_cast<const float2*>(p) + idx).x;
  return __ldg(p + idx);
}

// Bilateral: taps y outer, x inner over [-2, 2]; w = exp(-|d-d0|*10.5) *
// exp(-|n-n0|^2*20) (weights of denoiser.frag:103,105), evaluated as one
// exponential of the summed exponents; out = sum / (sumW + 1e-7).  The block's
// (32+4) x (16+4) halo of light, depth and normal is staged in shared memory
// (clamp-to-edge applied while staging), so every tap is a shared-memory read.
// Each thread filters kBilRows vertically adjacent pixels: their windows share
// tap rows, so a thread reads kBilRows + 4 rows of taps for kBilRows outputs
// instead of 5 kBilRows (the kernel is bound by the shared-memory reads); each
// output still sums its taps in the order above.  Two rows measured best at 1080p:
// 88.7 us against 96.9 (three) and 101.0 (four; larger halo tiles and registers).
constexpr int kBilRows = 2;
constexpr int kHx = kTx + 4, kHy = kTy * kBilRows + 4;

// FAST (the march's fast precision): the weights by the hardware exponential
// (__expf) and the sums by fused multiply-adds.
template <bool FAST>
__device__ __forceinline__ void bilateral_tap(const float4& col, const float4& n, const float4& c, float4& acc) {
  const float ndx = n.x - c.x, ndy = n.y - c.y, ndz = n.z - c.z;
  if (FAST) {
    const float wt = __expf(-fmaf(fabsf(n.w - c.w), 10.5f, fmaf(ndz, ndz, fmaf(ndy, ndy, ndx * ndx)) * 20.0f));
    acc.x = fmaf(col.x, wt, acc.x);
    acc.y = fmaf(col.y, wt, acc.y);
    acc.z = fmaf(col.z, wt, acc.z);
    acc.w = acc.w + wt;
  } else {
    const float wt = expf_(-(fabsf(n.w - c.w) * 10.5f + (ndx * ndx + ndy * ndy + ndz * ndz) * 20.0f));
    acc.x = acc.x + col.x * wt;
    acc.y = acc.y + col.y * wt;
    acc.z = acc.z + col.z * wt;
    acc.w = acc.w + wt;
  }
}

template <int DCH, bool FAST>
__global__ void __launch_bounds__(kTx* kTy) bilateral_kernel(const float* __restrict__ ind,
                                                             const float* __restrict__ depth,
                                                             const float* __restrict__ normal,
                                                             float* __restrict__ out, int w, int h) {
  __shared__ float4 s_col[kHy][kHx];
  __shared__ float4 s_nrm[kHy][kHx];  // xyz, w = depth
  const int x0 = blockIdx.x * kTx - 2, y0 = blockIdx.y * (kTy * kBilRows) - 2;
  for (int i = threadIdx.y * kTx + threadIdx.x; i < kHx * kHy; i += kTx * kTy) {
    const int hx = i % kHx, hy = i / kHx;
    const int q = iclamp(y0 + hy, 0, h - 1) * w + iclamp(x0 + hx, 0, w - 1);
    s_col[hy][hx] = ld4(ind, q);
    float4 n = ld4(normal, q);
    n.w = depth_at<DCH>(depth, q);
    s_nrm[hy][hx] = n;
  }
  __syncthreads();
  const int x = blockIdx.x * kTx + threadIdx.x;
  const int ty = threadIdx.y * kBilRows;  // first of the thread's rows within the tile
  const int y = blockIdx.y * (kTy * kBilRows) + ty;
  if (x >= w || y >= h) return;
  float4 c[kBilRows], acc[kBilRows];
#pragma unroll
  for (int k = 0; k < kBilRows; k++) {
    c[k] = s_nrm[ty + 2 + k][threadIdx.x + 2];
    acc[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
#pragma unroll
  for (int r = 0; r < 5 + kBilRows - 1; r++) {  // tap rows of the windows, top to bottom
#pragma unroll
    for (int dx = 0; dx < 5; dx++) {
      const float4 col = s_col[ty + r][threadIdx.x + dx];
      const float4 n = s_nrm[ty + r][threadIdx.x + dx];
#pragma unroll
      for (int k = 0; k < kBilRows; k++)  // output k's window holds tap rows k .. k + 4
        if (r >= k && r < k + 5) bilateral_tap<FAST>(col, n, c[k], acc[k]);
    }
  }
  float4* o = reinterpret_cast<float4*>(out);
#pragma unroll
  for (int k = 0; k < kBilRows; k++) {
    if (y + k < h) {
      const float d = acc[k].w + 1e-7f;
      o[(size_t)(y + k) * w + x] = make_float4(div_(acc[k].x, d), div_(acc[k].y, d), div_(acc[k].z, d), 1.0f);
    }
  }
}

// denoiser.frag:72-184 with radius 2: 16 equations [depth, 1] -> colour over
// the taps y, x in [-2, 2), Gramian + 1e-7 I, closed-form 2x2 inverse.
template <int DCH> __device__ __forceinline__ float depth_sample(const float* p, int w, int h, float s, float t) {
  Bilin B = bilin(s, t, w, h);
  return blend1(B, depth_at<DCH>(p, B.o00), depth_at<DCH>(p, B.o10), depth_at<DCH>(p, B.o01),
                depth_at<DCH>(p, B.o11));
}

template <int DCH>
__global__ void __launch_bounds__(kTx* kTy) denoise_kernel(const float* __restrict__ noisy,
                                                           const float* __restrict__ depth, float* __restrict__ out,
                                                           int w, int h, int radius) {
  const int x = blockIdx.x * kTx + threadIdx.x, y = blockIdx.y * kTy + threadIdx.y;
  if (x >= w || y >= h) return;
  const float W = (float)w, H = (float)h;
  const float cpx = (float)x + 0.5f, cpy = (float)y + 0.5f;
  if (radius == 0) {
    reinterpret_cast<float4*>(out)[y * w + x] = sample4(noisy, w, h, div_(cpx, W), div_(cpy, H));
    return;
  }
  float p0[16];
  float col[16][3];
  int i = 0;
#pragma unroll
  for (int dy = -2; dy < 2; dy++)
#pragma unroll
    for (int dx = -2; dx < 2; dx++) {
      const float sx = div_(cpx + (float)dx, W), sy = div_(cpy + (float)dy, H);
      p0[i] = depth_sample<DCH>(depth, w, h, sx, sy);
      float4 c = sample4(noisy, w, h, sx, sy);
      col[i][0] = c.x;
      col[i][1] = c.y;
      col[i][2] = c.z;
      i++;
    }
  float g00 = 0.0f, g01 = 0.0f, g10 = 0.0f, g11 = 0.0f;
#pragma unroll
  for (int k = 0; k < 16; k++) g00 = g00 + p0[k] * p0[k];
  g00 = g00 + 1e-7f;
#pragma unroll
  for (int k = 0; k < 16; k++) g01 = g01 + p0[k] * 1.0f;
  g01 = g01 + 0.0f;
#pragma unroll
  for (int k = 0; k < 16; k++) g10 = g10 + 1.0f * p0[k];
  g10 = g10 + 0.0f;
#pragma unroll
  for (int k = 0; k < 16; k++) g11 = g11 + 1.0f * 1.0f;
  g11 = g11 + 1e-7f;
  const float det = g00 * g11 - g01 * g10;
  const float inv00 = div_(g11, det), inv01 = div_(-g01, det), inv10 = div_(-g10, det), inv11 = div_(g00, det);
  const float cp0 = depth_sample<DCH>(depth, w, h, div_(cpx, W), div_(cpy, H));
  float res[3];
#pragma unroll
  for (int ch = 0; ch < 3; ch++) {
    float m0 = 0.0f, m1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 16; k++) m0 = m0 + p0[k] * col[k][ch];
#pragma unroll
    for (int k = 0; k < 16; k++) m1 = m1 + 1.0f * col[k][ch];
    float c0 = 0.0f, c1 = 0.0f;
    c0 = c0 + inv00 * m0;
    c0 = c0 + inv10 * m1;
    c1 = c1 + inv01 * m0;
    c1 = c1 + inv11 * m1;
    float v = 0.0f;
    v = v + c0 * cp0;
    v = v + c1 * 1.0f;
    res[ch] = v;
  }
  reinterpret_cast<float4*>(out)[y * w + x] = make_float4(res[0], res[1], res[2], 1.0f);
}

// finalGatherer.frag:42-59: direct + indirect * albedo (the :50-57 loop adds
// only zero-weighted terms).
// Rows per thread of the streaming kernels: every thread issues the loads of
// kRowsPerThread pixels (kTy rows apart) before it computes or stores any, which
// keeps enough bytes in flight per SM to stream at HBM speed.
constexpr int kRowsPerThread = 2;

__global__ void __launch_bounds__(kTx* kTy) final_gather_kernel(const float* __restrict__ direct,
                                                                const float* __restrict__ ind,
                                                                const float* __restrict__ albedo,
                                                                float* __restrict__ out, int w, int h) {
  const int x = blockIdx.x * kTx + threadIdx.x;
  const int y0 = blockIdx.y * (kTy * kRowsPerThread) + threadIdx.y;
  if (x >= w) return;
  float4 d[kRowsPerThread][4], i[kRowsPerThread][4], a[kRowsPerThread][4];
  Bilin B[kRowsPerThread];
#pragma unroll
  for (int r = 0; r < kRowsPerThread; r++) {
    const int y = min(y0 + r * kTy, h - 1);  // rows past the image repeat the last one; not stored
    const float s = div_((float)x + 0.5f, (float)w), t = div_((float)y + 0.5f, (float)h);
    B[r] = bilin(s, t, w, h);
    const int o[4] = {B[r].o00, B[r].o10, B[r].o01, B[r].o11};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      d[r][k] = ld4(direct, o[k]);
      i[r][k] = ld4(ind, o[k]);
      a[r][k] = ld4(albedo, o[k]);
    }
  }
#pragma unroll
  for (int r = 0; r < kRowsPerThread; r++) {
    const int y = y0 + r * kTy;
    if (y >= h) break;
    const float4 dd = blend4(B[r], d[r][0], d[r][1], d[r][2], d[r][3]);
    const float4 ii = blend4(B[r], i[r][0], i[r][1], i[r][2], i[r][3]);
    const float4 aa = blend4(B[r], a[r][0], a[r][1], a[r][2], a[r][3]);
    reinterpret_cast<float4*>(out)[y * w + x] =
        make_float4(dd.x + ii.x * aa.x, dd.y + ii.y * aa.y, dd.z + ii.z * aa.z, dd.w + ii.w * aa.w);
  }
}

// Permutations.  Each thread owns one pixel of the INTERLEAVED image, so reads
// (deinterleave) or writes (interleave) on that side are contiguous, and the
// other side is touched in runs of 32/grid_x consecutive texels per warp.
//   deinterleave.frag: dst[p] = src[InterleavePixel(p)]  ==  dst[DeinterleavePixel(q)] = src[q]
//   interleave.frag:   dst[q] = src[DeinterleavePixel(q)]
// Each thread moves kPermuteRows pixels (kTy rows apart), all loads first.
constexpr int kPermuteRows = 4;

template <int CH> struct Texel;
template <> struct Texel<4> { using T = float4; };
template <> struct Texel<2> { using T = float2; };
template <> struct Texel<1> { using T = float; };

template <int CH, bool INTERLEAVE>
__global__ void __launch_bounds__(kTx* kTy) permute_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                                           int w, int h, int gx, int gy) {
  using T = typename Texel<CH>::T;
  const int x = blockIdx.x * kTx + threadIdx.x;
  const int y0 = blockIdx.y * (kTy * kPermuteRows) + threadIdx.y;
  if (x >= w) return;
  const int dvx = w / gx, dvy = h / gy;
  const int dx = (x % gx) * dvx + x / gx;  // DeinterleavePixel, x part
  T v[kPermuteRows];
  size_t to[kPermuteRows];
#pragma unroll
  for (int r = 0; r < kPermuteRows; r++) {
    const int y = y0 + r * kTy;
    if (y < h) {
      const int dy = (y % gy) * dvy + y / gy;
      const size_t qi = (size_t)y * w + x, di = (size_t)dy * w + dx;
      to[r] = INTERLEAVE ? qi : di;
      v[r] = __ldg(reinterpret_cast<const T*>(src) + (INTERLEAVE ? di : qi));
    }
  }
#pragma unroll
  for (int r = 0; r < kPermuteRows; r++)
    if (y0 + r * kTy < h) reinterpret_cast<T*>(dst)[to[r]] = v[r];
}

dim3 grid2d(int w, int h) { return dim3((w + kTx - 1) / kTx, (h + kTy - 1) / kTy); }

}  // namespace

int launch_bilateral(const float* ind, const float* depth, int depth_ch, const float* normal, float* out, int w, int h,
                     cudaStream_t stream, bool fast) {
  const dim3 grid((w + kTx - 1) / kTx, (h + kTy * kBilRows - 1) / (kTy * kBilRows)), block(kTx, kTy);
  if (depth_ch == 2) {
    if (fast) bilateral_kernel<2, true><<<grid, block, 0, stream>>>(ind, depth, normal, out, w, h);
    else bilateral_kernel<2, false><<<grid, block, 0, stream>>>(ind, depth, normal, out, w, h);
  } else {
    if (fast) bilateral_kernel<1, true><<<grid, block, 0, stream>>>(ind, depth, normal, out, w, h);
    else bilateral_kernel<1, false><<<grid, block, 0, stream>>>(ind, depth, normal, out, w, h);
  }
  GI_CHECK_LAUNCH("bilateral_kernel");
  count_launches(1);
  return GI_OK;
}

int launch_final_gather(const float* direct, const float* ind, const float* albedo, float* out, int w, int h,
                        cudaStream_t stream) {
  const dim3 grid((w + kTx - 1) / kTx, (h + kTy * kRowsPerThread - 1) / (kTy * kRowsPerThread));
  final_gather_kernel<<<grid, dim3(kTx, kTy), 0, stream>>>(direct, ind, albedo, out, w, h);
  GI_CHECK_LAUNCH("final_gather_kernel");
  count_launches(1);
  return GI_OK;
}

int launch_deinterleave(const float* src, float* dst, int w, int h, int ch, int gx, int gy, bool inverse,
                        cudaStream_t stream) {
  dim3 g((w + kTx - 1) / kTx, (h + kTy * kPermuteRows - 1) / (kTy * kPermuteRows)), b(kTx, kTy);
  if (inverse) {
    if (ch == 4) permute_kernel<4, true><<<g, b, 0, stream>>>(src, dst, w, h, gx, gy);
    else if (ch == 2) permute_kernel<2, true><<<g, b, 0, stream>>>(src, dst, w, h, gx, gy);
    else permute_kernel<1, true><<<g, b, 0, stream>>>(src, dst, w, h, gx, gy);
  } else {
    if (ch == 4) permute_kernel<4, false><<<g, b, 0, stream>>>(src, dst, w, h, gx, gy);
    else if (ch == 2) permute_kernel<2, false><<<g, b, 0, stream>>>(src, dst, w, h, gx, gy);
    else permute_kernel<1, false><<<g, b, 0, stream>>>(src, dst, w, h, gx, gy);
  }
  GI_CHECK_LAUNCH("permute_kernel");
  count_launches(1);
  return GI_OK;
}

}  // namespace gi

using namespace gi;

extern "C" int gi_deinterleave(const float* src, float* dst, int width, int height, int channels, int grid_x,
                               int grid_y, void* stream) {
  GI_CHECK_ARG(src && dst && src != dst, "gi_deinterleave: null or aliased buffers");
  GI_CHECK_ARG(channels == 1 || channels == 2 || channels == 4, "gi_deinterleave: channels must be 1, 2 or 4");
  GI_CHECK_ARG(grid_x >= 1 && grid_y >= 1 && width >= grid_x && height >= grid_y && width % grid_x == 0 &&
                   height % grid_y == 0,
               "gi_deinterleave: size must be a multiple of the grid");
  GI_CHECK_ARG(aligned16(src) && aligned16(dst), "gi_deinterleave: unaligned buffer");
  return launch_deinterleave(src, dst, width, height, channels, grid_x, grid_y, false, (cudaStream_t)stream);
}

extern "C" int gi_interleave(const float* src, float* dst, int width, int height, int channels, int grid_x, int grid_y,
                             void* stream) {
  GI_CHECK_ARG(src && dst && src != dst, "gi_interleave: null or aliased buffers");
  GI_CHECK_ARG(channels == 1 || channels == 2 || channels == 4, "gi_interleave: channels must be 1, 2 or 4");
  GI_CHECK_ARG(grid_x >= 1 && grid_y >= 1 && width >= grid_x && height >= grid_y && width % grid_x == 0 &&
                   height % grid_y == 0,
               "gi_interleave: size must be a multiple of the grid");
  GI_CHECK_ARG(aligned16(src) && aligned16(dst), "gi_interleave: unaligned buffer");
  return launch_deinterleave(src, dst, width, height, channels, grid_x, grid_y, true, (cudaStream_t)stream);
}

extern "C" int gi_bilateral(const float* indirect, const float* depth_moments, const float* normal, float* out,
                            int width, int height, void* stream) {
  GI_CHECK_ARG(indirect && depth_moments && normal && out && width >= 1 && height >= 1, "gi_bilateral: bad arguments");
  GI_CHECK_ARG(out != indirect, "gi_bilateral: in-place filtering is not supported");
  GI_CHECK_ARG(aligned16(indirect) && aligned16(depth_moments) && aligned16(normal) && aligned16(out),
               "gi_bilateral: unaligned buffer");
  return launch_bilateral(indirect, depth_moments, 2, normal, out, width, height, (cudaStream_t)stream);
}

extern "C" int gi_denoise(const float* noisy, const float* depth_moments, const float* normal, float* out, int width,
                          int height, int radius, void* stream) {
  (void)normal;  // bound by the reference pass (SSVGIRenderer.h:293) but unused by its equations
  GI_CHECK_ARG(noisy && depth_moments && out && width >= 1 && height >= 1, "gi_denoise: bad arguments");
  GI_CHECK_ARG(radius == 0 || radius == 2, "gi_denoise: radius must be 0 or 2 (denoiser.frag:115)");
  GI_CHECK_ARG(out != noisy, "gi_denoise: in-place filtering is not supported");
  GI_CHECK_ARG(aligned16(noisy) && aligned16(depth_moments) && aligned16(out), "gi_denoise: unaligned buffer");
  denoise_kernel<2><<<grid2d(width, height), dim3(kTx, kTy), 0, (cudaStream_t)stream>>>(noisy, depth_moments, out,
                                                                                       width, height, radius);
  GI_CHECK_LAUNCH("denoise_kernel");
  count_launches(1);
  return GI_OK;
}

extern "C" int gi_final_gather(const float* direct, const float* indirect, const float* albedo, float* out, int width,
                               int height, void* stream) {
  GI_CHECK_ARG(direct && indirect && albedo && out && width >= 1 && height >= 1, "gi_final_gather: bad arguments");
  GI_CHECK_ARG(aligned16(direct) && aligned16(indirect) && aligned16(albedo) && aligned16(out),
               "gi_final_gather: unaligned buffer");
  return launch_final_gather(direct, indirect, albedo, out, width, height, (cudaStream_t)stream);
}
