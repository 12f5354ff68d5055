// gi_kernels.h -- launch descriptors shared between the kernel files and the
// renderer.  Each descriptor is passed by value as a __grid_constant__ kernel
// parameter, so a launch needs no device-side argument buffer.
#pragma once

#include <cuda_runtime.h>

#include "../../include/legit_gi.h"
#include "gi_device.cuh"

namespace gi {

constexpr int kMaxMipJobs = 16;
constexpr int kMaxBlurJobs = 32;

struct MipJob {
  float* levels[GI_MAX_LEVELS];  // levels[0] read, 1..num_levels-1 written
  int w, h, channels, num_levels, filter;
  int tiles_x, tile_begin;       // filled by launch_mips
};
struct MipJobs {
  MipJob job[kMaxMipJobs];
  int count;
};

struct BlurJob {
  const float* src;
  float* dst;
  int w, h, channels, radius;
  int tiles_x, tile_begin;       // filled by launch_blur
};
struct BlurJobs {
  BlurJob job[kMaxBlurJobs];
  int count;
};

int launch_mips(MipJobs& jobs, cudaStream_t stream);
int launch_blur(BlurJobs& jobs, cudaStream_t stream);

// The march's inputs in device-pointer form.
struct MarchArgs {
  dev::Mat4 inv_view_proj;
  dev::Mat4 inv_view;
  const float* light[GI_MAX_LEVELS];  // 4 ch
  const float* depth[GI_MAX_LEVELS];  // depth_ch ch, .x = linear depth
  const float* normal;                // 4 ch
  const float* ndc;                   // 1 ch
  float* out;                         // 4 ch
  int width, height, num_levels, depth_ch;
  int dirs, step_cap, pattern;
  int step_dirs;                      // direction count of the step/mip formulas (>= 1)
  int deinterleaved;                  // 1: A7' form (texelFetch centre, deinterleaved I/O)
  const int* tiles;                   // optional device list of tiles to march (nullptr: all)
  int num_tiles;
  int fast;                           // 1: GI_MARCH_FAST step loop (standard form, 2-ch depth)
  int soft;                           // 1: depth-variance horizon (exact contract, standard form, 2-ch depth)
  float ray[12];                      // fast step loop's view-ray basis (set_ray_basis)
  float ray_q[6];                     // |U|^2 of that ray as a quadratic form in (sx, sy) (set_ray_basis)
  // Recorded geometry of a march (standard form): per pixel and direction the
  // steps that raised the horizon, their horizon contributions and the initial
  // term -- all independent of the light pyramid -- so that a later bounce over
  // the same depth, normals and view re-lights them instead of marching again.
  float* rec_hc;                      // [direction][hit ordinal][record pixel]: hc of the k-th raising step
  unsigned long long* rec_mask;       // [direction][record pixel]: bit s set = step s raised the horizon
  float* rec_hc0;                     // [direction][record pixel]
  // (record pixel: the interleaved (pattern, sub-image row, column) index, so that a
  // warp's 32 pixels are consecutive)
  int rec;                            // 0: march; 1: march and record; 2: replay the record over `light`
  int rec_steps;                      // step stride of rec_hc, >= the step table size (<= 64)
  // Fast standard form only (GI_MARCH_TEXTURE): texture objects over the depth
  // pyramid's linear depth and the light pyramid (PyramidTexture) -- the step
  // loop's taps are then trilinear fetches by the texture units (the replay,
  // rec = 2, keeps software light taps from `light`).  0: software taps from
  // `depth` and `light`.
  unsigned long long depth_tex, light_tex;
};

// A mip pyramid as a CUDA mipmapped array (1 or 4 floats per texel, level k of
// size (width >> k) x (height >> k)) behind one texture object with bilinear
// filtering, linear mipmapping, clamp-to-edge addressing and normalised
// coordinates -- the sampler of the reference's textureLod.  Owned by a renderer
// or a batch view; Pack copies a pyramid's levels into it on a stream.
class PyramidTexture {
 public:
  PyramidTexture() = default;
  PyramidTexture(const PyramidTexture&) = delete;
  PyramidTexture& operator=(const PyramidTexture&) = delete;
  ~PyramidTexture() { Destroy(); }
  int Create(int width, int height, int num_levels, int channels);  // channels 1 or 4
  // sync: wait for the whole device first (the caller may instead have waited
  // for every launch that reads the objects).
  void Destroy(bool sync = true);
  // levels[k]: level k of the pyramid, `src_channels` floats per texel; the first
  // `channels` of each texel are copied.
  int Pack(const float* const* levels, int src_channels, cudaStream_t stream) const;
  unsigned long long Handle() const { return tex_; }

 private:
  cudaMipmappedArray_t mip_ = nullptr;
  unsigned long long tex_ = 0;
  unsigned long long surf_[GI_MAX_LEVELS] = {};
  int w_ = 0, h_ = 0, levels_ = 0, channels_ = 0;
};

constexpr int kMarchTileSubX = 32;  // sub-image pixels per march CTA along x (one warp row)
constexpr int kMarchTileSubY = 4;   // sub-image rows per march CTA

int launch_march(const MarchArgs& a, cudaStream_t stream);
// Bytes of the three record arrays of a march of this shape (0 if it cannot record:
// a table of more than 64 steps).
size_t march_record_bytes(const MarchArgs& a, size_t* hc_bytes, size_t* mask_bytes, size_t* hc0_bytes);
void set_ray_basis(MarchArgs& a);  // fills a.ray from a.inv_view_proj and a.inv_view
int autotune_march(const MarchArgs& a, cudaStream_t stream, int* best_rows, int* best_rays_per_warp,
                   float* best_ms);
int march_table_size(const MarchArgs& a);

// One view of a batched march: its arguments, step-table size and tile grid.
struct BatchView {
  MarchArgs a;
  int n_tab, tiles_x, tiles_total, pad;
};
// The views of one batched launch, passed by value as a kernel parameter (at
// most 32,764 bytes of parameters: 48 views).
constexpr int kBatchTableViews = 48;
struct BatchTable {
  BatchView v[kBatchTableViews];
};
static_assert(sizeof(BatchTable) + 64 <= 32764, "kernel parameter space");
// items[i] = (view index in the table, tile * 64 + pattern); the counter is
// device scratch reset by the launch; rows = CTA height (2, 4 or 8); every view
// of the table has the march precision `fast` and, with `tex`, both pyramid
// textures.
int launch_march_batch(const BatchTable& views, const int2* items, int num_items, int* counter, int rows, int grid,
                       bool fast, bool tex, cudaStream_t stream);
int march_batch_occupancy(int rows, bool fast, bool tex);

// fast: the hardware exponential and fused sums (the march's fast precision).
int launch_bilateral(const float* ind, const float* depth, int depth_ch, const float* normal, float* out, int w,
                     int h, cudaStream_t stream, bool fast = false);
int launch_final_gather(const float* direct, const float* ind, const float* albedo, float* out, int w, int h,
                        cudaStream_t stream);
int launch_deinterleave(const float* src, float* dst, int w, int h, int ch, int gx, int gy, bool inverse,
                        cudaStream_t stream);

}  // namespace gi
