// gi_mlp.h -- launch descriptors of the learned-reconstructor kernels.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/legit_gi.h"

namespace gi {

// Inputs of the feature builder (channel layout documented in gi_mlp.cu).
struct FeatureArgs {
  int width, height, pattern;
  const float* moments;      // 2 ch depth moments, level 0
  const float* normal;       // 4 ch
  const float* albedo;       // 4 ch
  const float* direct;       // 4 ch
  const float* indirect[3];  // few-ray indirect light at mip levels 0, 2 and 4 (4 ch)
  const float* filtered;     // the few-ray indirect light after the 5x5 bilateral (4 ch)
  const float* depth_l2;     // blurred depth moments, level 2 (2 ch)
  __nv_bfloat16* out;        // [pixels x 32]
  float* scale;              // [pixels]: the exposure scale s the light features were divided by
  const int* tiles;          // optional march-tile list (tile-major output)
  // The network on given rows (launch_forward_tc): bf16 [pixels x 32] features and
  // the optional [pixels] scale the output is multiplied by, instead of the images.
  const __nv_bfloat16* rows;
  const float* row_scale;
};

int launch_features(const FeatureArgs& a, int num_tiles, cudaStream_t stream);
// Fused features + network on the tensor cores (tcgen05) for a whole frame:
// out[p] = (network(features(p)) + skip) * scale, rgb + 1.  wb: the bf16 weight
// copy ([in x out] per layer, W4 padded to 16 columns); params: the FP32 masters
// (biases are read from them).  a.out, a.scale and a.tiles are not used.
int launch_reconstruct(const FeatureArgs& a, const __nv_bfloat16* wb, const float* params, float* out,
                       cudaStream_t stream);
// The same network on n given feature rows (bf16 [n x 32], the layout gi_features
// writes): out[i] = network(rows[i]) * (scale ? scale[i] : 1), rgb + 1.
int launch_forward_tc(const __nv_bfloat16* rows, const float* scale, int n, const __nv_bfloat16* wb,
                      const float* params, float* out, cudaStream_t stream);
// One training batch on the tensor cores (tcgen05): the forward with saved
// activations, the loss gradient and the backward of every tile of 128 pixels,
// gradient sums added to `grads` and the summed loss to `loss` (both FP32, the
// caller zeroes them).  feats: bf16 [n x 32]; targets [n x 4] (rgb, loss weight);
// scale: optional [n] exposure scale the rgb targets are divided by.
int launch_train_tc(const __nv_bfloat16* feats, const float* targets, const float* scale, int n,
                    const __nv_bfloat16* wb, const float* params, float* grads, float* loss, int loss_kind,
                    cudaStream_t stream);
// Number of tensor-core waits that ran out since the library was loaded.
int reconstruct_errors(int* count);
// Bound in SM cycles of each tile group's first MMA wait (<= 0: the default).
int reconstruct_wait_limit(long long cycles);
int launch_tiles_copy(const float* src, float* dst, int W, int H, int P, const int* tiles, int num_tiles,
                      bool scatter, cudaStream_t stream);

int launch_judge(float* learned, const float* plain, int W, int H, int P, const int* tiles, int num_tiles,
                 float threshold, int* counters, cudaStream_t stream);

}  // namespace gi
