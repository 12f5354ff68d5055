// gi_mlp_layout.h -- sizes and parameter layout of the 32 -> 64 -> 64 -> 64 -> 3
// reconstructor, shared by its training and inference kernels.
#pragma once

#include "../../include/legit_gi.h"

namespace gi {

constexpr int kIn = GI_MLP_IN, kHid = GI_MLP_HIDDEN, kOut = GI_MLP_OUT, kOutPad = 16;
// Output head: the 3 outputs are logits of a softmax whose weights blend three
// candidate estimates of the (exposure-normalised) indirect light taken from the
// network's own bf16 input row: the bilaterally filtered few-ray light (channels
// 10-12) and the few-ray light at mip levels 2 (19-21) and 4 (22-24).
constexpr int kCand0 = 10, kCand1 = 19, kCand2 = 22;

// FP32 master parameter offsets (floats): W1[32x64], b1, W2[64x64], b2, W3[64x64],
// b3, W4[64x3], b4, each weight row-major [in x out].
constexpr int oW1 = 0, ob1 = oW1 + kIn * kHid, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kHid * kHid, oW4 = ob3 + kHid, ob4 = oW4 + kHid * kOut, kParams = ob4 + kOut;
static_assert(kParams == GI_MLP_PARAMS, "parameter count");
// BF16 weight copy offsets (elements), same [in x out] order; W4 is padded to 16
// output columns (zeros).
constexpr int qW1 = 0, qW2 = qW1 + kIn * kHid, qW3 = qW2 + kHid * kHid, qW4 = qW3 + kHid * kHid,
              kWbf = qW4 + kHid * kOutPad;

#ifdef __CUDACC__
// Softmax weights w of the logits o and the blended estimate y = sum_k w_k c_k
// (c[k][ch]: candidate k, colour channel ch).
__device__ __forceinline__ void head_forward(const float (&o)[3], const float (&c)[3][3], float (&w)[3],
                                             float (&y)[3]) {
  const float m = fmaxf(fmaxf(o[0], o[1]), o[2]);
  const float e0 = expf(o[0] - m), e1 = expf(o[1] - m), e2 = expf(o[2] - m);
  const float inv = 1.0f / ((e0 + e1) + e2);
  w[0] = e0 * inv;
  w[1] = e1 * inv;
  w[2] = e2 * inv;
#pragma unroll
  for (int ch = 0; ch < 3; ch++) y[ch] = (w[0] * c[0][ch] + w[1] * c[1][ch]) + w[2] * c[2][ch];
}

// Gradient of the loss with respect to the logits, given its gradient g with
// respect to y: dL/do_k = w_k * sum_ch g_ch (c_k,ch - y_ch).
__device__ __forceinline__ void head_backward(const float (&w)[3], const float (&c)[3][3], const float (&y)[3],
                                              const float (&g)[3], float (&d)[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++)
    d[k] = w[k] * ((g[0] * (c[k][0] - y[0]) + g[1] * (c[k][1] - y[1])) + g[2] * (c[k][2] - y[2]));
}

// Loss term of one pixel and the gradient d of the summed weighted loss with
// respect to its 3 logits lo (bias included): y = the head's blend of the
// candidates c, e = y - T (T already divided by the exposure scale, T[3] the
// pixel's loss weight w), and per output
//   GI_MLP_LOSS_SQUARED   loss w e^2, gradient g = 2 w clip(e, -1, 1) (a
//                         Huber-style gradient: a target the few-ray signal
//                         cannot explain does not swamp the batch);
//   GI_MLP_LOSS_ABSOLUTE  loss w |e|, gradient g = w sign(e) (sign(0) = 0): the
//                         relative L1 error the learned method is judged by;
// d = the head's backward of g.
__device__ __forceinline__ float head_loss_grad_logits(const float (&lo)[3], const float (&c)[3][3], const float* T,
                                                       float (&d)[3], int loss_kind = GI_MLP_LOSS_SQUARED) {
  float w[3], y[3], g[3];
  head_forward(lo, c, w, y);
  const float wpx = T[3];
  float l = 0.0f;
#pragma unroll
  for (int ch = 0; ch < 3; ch++) {
    const float e = y[ch] - T[ch];
    if (loss_kind == GI_MLP_LOSS_ABSOLUTE) {
      l += wpx * fabsf(e);
      g[ch] = e > 0.0f ? wpx : (e < 0.0f ? -wpx : 0.0f);
    } else {
      l += wpx * (e * e);
      g[ch] = 2.0f * wpx * fminf(fmaxf(e, -1.0f), 1.0f);
    }
  }
  head_backward(w, c, y, g, d);
  return l;
}
#endif

}  // namespace gi
