// gi_features.cuh -- the 32 per-pixel input features of the learned
// reconstructor (channel layout documented in gi_mlp.cu), shared by the feature
// builder and the fused reconstruction kernel.
#pragma once

#include "gi_device.cuh"
#include "gi_kernels.h"
#include "gi_mlp.h"

namespace gi {

__device__ __forceinline__ float feat_lum(float4 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// Features of pixel (x, y), light-dependent channels already divided by the
// exposure scale, which is returned in `scale`; the pixel's own depth, normal,
// albedo, few-ray light and direct light are passed in (read from memory by the
// caller, global or staged), everything else is read here.
__device__ __forceinline__ void pixel_features_from(const FeatureArgs& a, int x, int y, float depth, float4 n4,
                                                    float4 al, float4 I0, float4 dl, float (&f)[GI_MLP_IN],
                                                    float& scale) {
  using namespace dev;
  const int P = a.pattern;
  const int W = a.width, H = a.height;
  const int c = y * W + x;
  f[0] = depth;
  f[1] = n4.x; f[2] = n4.y; f[3] = n4.z;
  f[4] = al.x; f[5] = al.y; f[6] = al.z;
  f[7] = I0.x; f[8] = I0.y; f[9] = I0.z;
  const float4 fl = ld4(a.filtered, c);
  f[10] = fl.x; f[11] = fl.y; f[12] = fl.z;
  {
    const int nx[6] = {-1, 1, 0, 0, -1, 1}, ny[6] = {0, 0, -1, 1, -1, 1};
#pragma unroll
    for (int k = 0; k < 6; k++)
      f[13 + k] = feat_lum(ld4(a.indirect[0], iclamp(y + ny[k], 0, H - 1) * W + iclamp(x + nx[k], 0, W - 1)));
  }
  const float s = ((float)x + 0.5f) / (float)W, t = ((float)y + 0.5f) / (float)H;
  const float4 i2 = sample4(a.indirect[1], W >> 2, H >> 2, s, t);
  const float4 i4 = sample4(a.indirect[2], W >> 4, H >> 4, s, t);
  f[19] = i2.x; f[20] = i2.y; f[21] = i2.z;
  f[22] = i4.x; f[23] = i4.y; f[24] = i4.z;
  {
    const int w2 = W >> 2, h2 = H >> 2;
    const float2 m = __ldg(reinterpret_cast<const float2*>(a.depth_l2) + iclamp(y >> 2, 0, h2 - 1) * w2 +
                           iclamp(x >> 2, 0, w2 - 1));
    f[25] = sqrtf(fmaxf(0.0f, m.y - m.x * m.x));
  }
  f[26] = dl.x; f[27] = dl.y; f[28] = dl.z;
  {
    const int pidx = (x % P) + (y % P) * P;
    uint32_t b = ((uint32_t)pidx << 16u) | ((uint32_t)pidx >> 16u);
    b = ((b & 0x55555555u) << 1u) | ((b & 0xAAAAAAAAu) >> 1u);
    b = ((b & 0x33333333u) << 2u) | ((b & 0xCCCCCCCCu) >> 2u);
    b = ((b & 0x0F0F0F0Fu) << 4u) | ((b & 0xF0F0F0F0u) >> 4u);
    b = ((b & 0x00FF00FFu) << 8u) | ((b & 0xFF00FF00u) >> 8u);
    f[29] = (float)pidx / (float)(P * P);
    f[30] = (float)b * 2.3283064365386963e-10f;
  }
  f[31] = fminf(fminf(s, 1.0f - s), fminf(t, 1.0f - t));
  // The indirect light can be slightly negative (light below the ambient term),
  // so the scale uses magnitudes, with a floor; the normalised values are clamped.
  scale = (fabsf(feat_lum(i2)) + fabsf(feat_lum(i4))) + 1e-3f;
  const float rs = 1.0f / scale;
  constexpr float lim = 32.0f;
#pragma unroll
  for (int i = 7; i <= 24; i++) f[i] = fminf(fmaxf(f[i] * rs, -lim), lim);
#pragma unroll
  for (int i = 26; i <= 28; i++) f[i] = fminf(fmaxf(f[i] * rs, -lim), lim);
}

// The same, reading the pixel's own inputs from global memory.
__device__ __forceinline__ void pixel_features(const FeatureArgs& a, int x, int y, float (&f)[GI_MLP_IN],
                                               float& scale) {
  using namespace dev;
  const int c = y * a.width + x;
  pixel_features_from(a, x, y, __ldg(reinterpret_cast<const float2*>(a.moments) + c).x, ld4(a.normal, c),
                      ld4(a.albedo, c), ld4(a.indirect[0], c), ld4(a.direct, c), f, scale);
}

}  // namespace gi
