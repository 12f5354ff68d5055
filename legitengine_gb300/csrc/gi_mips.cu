// gi_mips.cu -- mip chain (MipBuilder::BuildMips + Common/mipLevelBuilder.frag)
// and blur pyramid (BlurBuilder::ApplyBlur + Common/blurLayerBuilder.frag).
//
// The reference draws one full-screen pass per level (9 dependent passes per
// pyramid, SSVGIRenderer.h:207-208) and one per blurred level (20 passes,
// :209-221).  Here one launch builds levels 1..6 of every listed image: a CTA
// reads a 64x64 block of level 0 once (coalesced, vectorised by channel count)
// and reduces it through shared memory down to one level-6 texel.  A one-CTA
// tail launch finishes levels 7+ from level 6 (at 1920x1080 that is 480 texels).
// Every level >= 1 of every image is then blurred in one more launch.
//
// HBM per level-0 pixel (fp32, 4 ch): 16 B read + 16/3 B written by the chain;
// the blur reads and writes each level >= 1 once more (level 0 is aliased, its
// blur radius is 0).
#include "gi_device.cuh"
#include "gi_internal.h"
#include "gi_kernels.h"

namespace gi {
namespace {

constexpr int kTile1 = 32;     // level-1 tile edge per CTA
constexpr int kFusedTop = 6;   // deepest level built by the fused kernel
constexpr int kThreads = 256;

// Reduction of one 2x2 block (mipLevelBuilder.frag:19-42); t[i] are the texels
// at offsets (0,0), (1,0), (0,1), (1,1), channels padded to (0, 0, 0, 1).
__device__ __forceinline__ float4 reduce_block(const float4 t[4], int filter) {
  if (filter == GI_MIP_AVG) {
    float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      s.x = s.x + t[i].x;
      s.y = s.y + t[i].y;
      s.z = s.z + t[i].z;
      s.w = s.w + t[i].w;
    }
    return make_float4(div_(s.x, 4.0f), div_(s.y, 4.0f), div_(s.z, 4.0f), div_(s.w, 4.0f));
  }
  float mn = 1e5f, mx = -1e5f, mass = 0.0f;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    mn = dev::gmin(mn, t[i].x);
    mx = dev::gmax(mx, t[i].y);
    mass = mass + (t[i].y - t[i].x) * t[i].z;
  }
  return make_float4(mn, mx, div_(div_(mass, mx - mn), 4.0f), 0.0f);
}

template <int CH> __device__ __forceinline__ float4 load_texel(const float* p, size_t idx) {
  float4 r = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
  if (CH == 4) {
    r = __ldg(reinterpret_cast<const float4*>(p) + idx);
  } else if (CH == 2) {
    float2 v = __ldg(reinterpret_cast<const float2*>(p) + idx);
    r.x = v.x;
    r.y = v.y;
  } else {
    r.x = __ldg(p + idx);
  }
  return r;
}

// Loads texels idx and idx+1 of one row.  The pair is one vector load only
// when idx is even (the pair is then 2*CH*4-byte aligned); rows of odd-width
// images start at odd texel indices every other row, and those pairs are
// loaded texel by texel.
template <int CH> __device__ __forceinline__ void load_pair(const float* p, size_t idx, float4& a, float4& b) {
  if (CH == 4) {
    a = __ldg(reinterpret_cast<const float4*>(p) + idx);
    b = __ldg(reinterpret_cast<const float4*>(p) + idx + 1);
  } else if ((idx & 1) != 0) {
    a = load_texel<CH>(p, idx);
    b = load_texel<CH>(p, idx + 1);
  } else if (CH == 2) {
    float4 v = __ldg(reinterpret_cast<const float4*>(p + idx * 2));
    a = make_float4(v.x, v.y, 0.0f, 1.0f);
    b = make_float4(v.z, v.w, 0.0f, 1.0f);
  } else {
    float2 v = __ldg(reinterpret_cast<const float2*>(p + idx));
    a = make_float4(v.x, 0.0f, 0.0f, 1.0f);
    b = make_float4(v.y, 0.0f, 0.0f, 1.0f);
  }
}

template <int CH> __device__ __forceinline__ void store_texel(float* p, size_t idx, float4 v) {
  if (CH == 4) {
    reinterpret_cast<float4*>(p)[idx] = v;
  } else if (CH == 2) {
    reinterpret_cast<float2*>(p)[idx] = make_float2(v.x, v.y);
  } else {
    p[idx] = v.x;
  }
}

template <int CH> __device__ void fused_tile(const MipJob& J, int tile, float4* s_a, float4* s_b) {
  const int W1 = J.w >> 1, H1 = J.h >> 1;
  const int tx = tile % J.tiles_x, ty = tile / J.tiles_x;
  const float* l0 = J.levels[0];
  // Level 1 from level 0 (global -> registers -> global + shared).
  for (int i = threadIdx.x; i < kTile1 * kTile1; i += kThreads) {
    int lx = i % kTile1, ly = i / kTile1;
    int x = tx * kTile1 + lx, y = ty * kTile1 + ly;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (x < W1 && y < H1) {
      float4 t[4];
      load_pair<CH>(l0, (size_t)(2 * y) * J.w + 2 * x, t[0], t[1]);
      load_pair<CH>(l0, (size_t)(2 * y + 1) * J.w + 2 * x, t[2], t[3]);
      v = reduce_block(t, J.filter);
      if (CH < 4) v.w = 1.0f;
      if (CH < 3) v.z = 0.0f;
      if (CH < 2) v.y = 0.0f;
      store_texel<CH>(J.levels[1], (size_t)y * W1 + x, v);
    }
    s_a[i] = v;
  }
  __syncthreads();
  int size = kTile1;
  float4* src = s_a;
  float4* dst = s_b;
  for (int lev = 2; lev < J.num_levels && lev <= kFusedTop; lev++) {
    const int half = size >> 1;
    const int Wl = J.w >> lev, Hl = J.h >> lev;
    for (int i = threadIdx.x; i < half * half; i += kThreads) {
      int lx = i % half, ly = i / half;
      float4 t[4];
      t[0] = src[(2 * ly) * size + 2 * lx];
      t[1] = src[(2 * ly) * size + 2 * lx + 1];
      t[2] = src[(2 * ly + 1) * size + 2 * lx];
      t[3] = src[(2 * ly + 1) * size + 2 * lx + 1];
      float4 v = reduce_block(t, J.filter);
      if (CH < 4) v.w = 1.0f;
      if (CH < 3) v.z = 0.0f;
      if (CH < 2) v.y = 0.0f;
      dst[i] = v;
      int x = tx * half + lx, y = ty * half + ly;
      if (x < Wl && y < Hl) store_texel<CH>(J.levels[lev], (size_t)y * Wl + x, v);
    }
    __syncthreads();
    float4* t = src;
    src = dst;
    dst = t;
    size = half;
  }
}

__global__ void __launch_bounds__(kThreads) mip_fused_kernel(const __grid_constant__ MipJobs jobs) {
  __shared__ float4 s_a[kTile1 * kTile1];
  __shared__ float4 s_b[(kTile1 / 2) * (kTile1 / 2)];
  int b = blockIdx.x;
  int j = 0;
  while (j + 1 < jobs.count && b >= jobs.job[j + 1].tile_begin) j++;
  const MipJob& J = jobs.job[j];
  int tile = b - J.tile_begin;
  if (J.channels == 4) fused_tile<4>(J, tile, s_a, s_b);
  else if (J.channels == 2) fused_tile<2>(J, tile, s_a, s_b);
  else fused_tile<1>(J, tile, s_a, s_b);
}

// Levels kFusedTop+1 .. n-1, one CTA per job, level by level.  Reads use plain
// (coherent) loads: the previous level was written by this same CTA.
template <int CH> __device__ void tail_job(const MipJob& J) {
  for (int lev = kFusedTop + 1; lev < J.num_levels; lev++) {
    const int Ws = J.w >> (lev - 1);
    const int Wl = J.w >> lev, Hl = J.h >> lev;
    const float* src = J.levels[lev - 1];
    float* dst = J.levels[lev];
    for (int i = threadIdx.x; i < Wl * Hl; i += blockDim.x) {
      int x = i % Wl, y = i / Wl;
      float4 t[4];
      const int offs[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        size_t idx = (size_t)(2 * y + offs[k][1]) * Ws + (2 * x + offs[k][0]);
        float4 r = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        if (CH == 4) r = reinterpret_cast<const float4*>(src)[idx];
        else if (CH == 2) { float2 v = reinterpret_cast<const float2*>(src)[idx]; r.x = v.x; r.y = v.y; }
        else r.x = src[idx];
        t[k] = r;
      }
      store_texel<CH>(dst, (size_t)i, reduce_block(t, J.filter));
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) mip_tail_kernel(const __grid_constant__ MipJobs jobs) {
  const MipJob& J = jobs.job[blockIdx.x];
  if (J.channels == 4) tail_job<4>(J);
  else if (J.channels == 2) tail_job<2>(J);
  else tail_job<1>(J);
}

// ---------------------------------------------------------------------------
// Blur (blurLayerBuilder.frag:17-35): taps x outer, y inner, over [-r, r).
constexpr int kBlurTx = 32, kBlurTy = 8;

template <int CH> __device__ void blur_tile(const BlurJob& J, int tile) {
  const int tx = tile % J.tiles_x, ty = tile / J.tiles_x;
  const int x = tx * kBlurTx + (threadIdx.x % kBlurTx);
  const int y = ty * kBlurTy + (threadIdx.x / kBlurTx);
  if (x >= J.w || y >= J.h) return;
  const int r = J.radius;
  float4 out;
  if (r == 0) {
    out = load_texel<CH>(J.src, (size_t)y * J.w + x);
  } else {
    float4 s = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float tw = 0.0f;
    for (int dx = -r; dx < r; dx++) {
      int sx = dev::iclamp(x + dx, 0, J.w - 1);
      for (int dy = -r; dy < r; dy++) {
        int sy = dev::iclamp(y + dy, 0, J.h - 1);
        float4 t = load_texel<CH>(J.src, (size_t)sy * J.w + sx);
        s.x = s.x + t.x;
        s.y = s.y + t.y;
        s.z = s.z + t.z;
        s.w = s.w + t.w;
        tw = tw + 1.0f;
      }
    }
    out = make_float4(div_(s.x, tw), div_(s.y, tw), div_(s.z, tw), div_(s.w, tw));
  }
  store_texel<CH>(J.dst, (size_t)y * J.w + x, out);
}

__global__ void __launch_bounds__(kBlurTx * kBlurTy) blur_kernel(const __grid_constant__ BlurJobs jobs) {
  int b = blockIdx.x;
  int j = 0;
  while (j + 1 < jobs.count && b >= jobs.job[j + 1].tile_begin) j++;
  const BlurJob& J = jobs.job[j];
  int tile = b - J.tile_begin;
  if (J.channels == 4) blur_tile<4>(J, tile);
  else if (J.channels == 2) blur_tile<2>(J, tile);
  else blur_tile<1>(J, tile);
}

}  // namespace

int launch_mips(MipJobs& jobs, cudaStream_t stream) {
  int total = 0, tail = 0;
  for (int j = 0; j < jobs.count; j++) {
    MipJob& J = jobs.job[j];
    int W1 = J.w >> 1, H1 = J.h >> 1;
    J.tiles_x = (W1 + kTile1 - 1) / kTile1;
    int tiles_y = (H1 + kTile1 - 1) / kTile1;
    J.tile_begin = total;
    total += (J.num_levels > 1) ? J.tiles_x * tiles_y : 0;
    if (J.num_levels > kFusedTop + 1) tail++;
  }
  if (total == 0) return GI_OK;
  mip_fused_kernel<<<total, kThreads, 0, stream>>>(jobs);
  GI_CHECK_LAUNCH("mip_fused_kernel");
  count_launches(1);
  if (tail) {
    // Every job runs the tail loop; jobs without levels above 6 return at once.
    mip_tail_kernel<<<jobs.count, kThreads, 0, stream>>>(jobs);
    GI_CHECK_LAUNCH("mip_tail_kernel");
    count_launches(1);
  }
  return GI_OK;
}

int launch_blur(BlurJobs& jobs, cudaStream_t stream) {
  int total = 0;
  for (int j = 0; j < jobs.count; j++) {
    BlurJob& J = jobs.job[j];
    J.tiles_x = (J.w + kBlurTx - 1) / kBlurTx;
    int tiles_y = (J.h + kBlurTy - 1) / kBlurTy;
    J.tile_begin = total;
    total += J.tiles_x * tiles_y;
  }
  if (total == 0) return GI_OK;
  blur_kernel<<<total, kBlurTx * kBlurTy, 0, stream>>>(jobs);
  GI_CHECK_LAUNCH("blur_kernel");
  count_launches(1);
  return GI_OK;
}

}  // namespace gi

using namespace gi;

static int check_channels(int ch) { return ch == 1 || ch == 2 || ch == 4; }

extern "C" int gi_build_mips(float* const* levels, int width, int height, int channels, int num_levels, int filter,
                             void* stream) {
  GI_CHECK_ARG(levels && width >= 1 && height >= 1, "gi_build_mips: bad image");
  GI_CHECK_ARG(check_channels(channels), "gi_build_mips: channels must be 1, 2 or 4");
  GI_CHECK_ARG(filter == GI_MIP_AVG || filter == GI_MIP_DEPTH, "gi_build_mips: bad filter");
  GI_CHECK_ARG(num_levels >= 1 && num_levels <= gi_mip_level_count(width, height, GI_MAX_LEVELS),
               "gi_build_mips: num_levels exceeds the levels of this size");
  for (int k = 0; k < num_levels; k++)
    GI_CHECK_ARG(levels[k] && aligned16(levels[k]), "gi_build_mips: null or unaligned level");
  MipJobs jobs{};
  jobs.count = 1;
  MipJob& J = jobs.job[0];
  for (int k = 0; k < num_levels; k++) J.levels[k] = levels[k];
  J.w = width;
  J.h = height;
  J.channels = channels;
  J.num_levels = num_levels;
  J.filter = filter;
  return launch_mips(jobs, (cudaStream_t)stream);
}

extern "C" int gi_blur(const float* src, float* dst, int width, int height, int channels, int radius, void* stream) {
  GI_CHECK_ARG(src && dst && width >= 1 && height >= 1 && radius >= 0 && radius <= 64, "gi_blur: bad arguments");
  GI_CHECK_ARG(check_channels(channels), "gi_blur: channels must be 1, 2 or 4");
  GI_CHECK_ARG(aligned16(src) && aligned16(dst), "gi_blur: unaligned buffer");
  GI_CHECK_ARG(src != dst, "gi_blur: in-place blur is not supported");
  BlurJobs jobs{};
  jobs.count = 1;
  jobs.job[0] = BlurJob{src, dst, width, height, channels, radius, 0, 0};
  return launch_blur(jobs, (cudaStream_t)stream);
}

extern "C" int gi_blur_pyramid(const float* const* src_levels, float* const* dst_levels, int width, int height,
                               int channels, int num_levels, void* stream) {
  GI_CHECK_ARG(src_levels && dst_levels && width >= 1 && height >= 1, "gi_blur_pyramid: bad arguments");
  GI_CHECK_ARG(check_channels(channels), "gi_blur_pyramid: channels must be 1, 2 or 4");
  GI_CHECK_ARG(num_levels >= 1 && num_levels <= gi_mip_level_count(width, height, GI_MAX_LEVELS) &&
                   num_levels <= kMaxBlurJobs,
               "gi_blur_pyramid: bad level count");
  BlurJobs jobs{};
  for (int k = 0; k < num_levels; k++) {
    GI_CHECK_ARG(src_levels[k] && dst_levels[k] && aligned16(src_levels[k]) && aligned16(dst_levels[k]),
                 "gi_blur_pyramid: null or unaligned level");
    if (k == 0 && src_levels[0] == dst_levels[0]) continue;  // radius 0 onto itself
    GI_CHECK_ARG(src_levels[k] != dst_levels[k], "gi_blur_pyramid: only level 0 may alias");
    jobs.job[jobs.count++] =
        BlurJob{src_levels[k], dst_levels[k], width >> k, height >> k, channels, k == 0 ? 0 : 2, 0, 0};
  }
  return launch_blur(jobs, (cudaStream_t)stream);
}
