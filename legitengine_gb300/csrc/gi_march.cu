// gi_march.cu -- the screen-space GI march of SSVGI/indirectLighting.frag:114-271
// (pass SSVGIRenderer.h:224-263), generalised to R directions and a step cap.
//
// Work layout.  The reference draws one fragment per pixel; its pattern index
// (x mod 4, y mod 4) selects the Hammersley offsets (:155-164), and with them
// the directions and every step offset and mip level of the pixel.  Here a CTA
// takes pixels of ONE pattern (the interleaved form of LSGIRenderer.h:83-91
// without materialising deinterleaved copies): blockIdx.z is the pattern, and
// a warp covers 32 pixels of one row, 4 pixels apart.  All lanes of a warp then
// march the same directions with the same step offsets, so the per-step tables
// (offset, mip pair, blend weight) are warp-uniform shared-memory broadcasts,
// and the taps of neighbouring lanes land on neighbouring texels.
//
// Arithmetic mirrors the restatement exactly (see gi_device.cuh): the output is
// bit-identical to the fp32 oracle for the same inputs.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "gi_device.cuh"
#include "gi_internal.h"
#include "gi_kernels.h"

namespace gi {
namespace {

using namespace dev;

constexpr int kMarchTx = kMarchTileSubX;  // sub-image pixels per warp row
constexpr int kMarchTy = kMarchTileSubY;  // warps per CTA
constexpr float kPiRef = 3.1415f;  // indirectLighting.frag:169

struct StepEntry {
  float off;    // pixel offset of the step (:217)
  float delta;  // trilinear blend weight of the upper level
  int lo;       // mip level read first (Vulkan mipmap LINEAR selection)
  union {
    int hi;       // software taps: the second level read
    float level;  // texture taps: lo + delta, the fetch's level of detail
  };
};

__device__ __forceinline__ void hammersley(int i, int n, float& ax, float& ay) {
  uint32_t b = ((uint32_t)i << 16u) | ((uint32_t)i >> 16u);
  b = ((b & 0x55555555u) << 1u) | ((b & 0xAAAAAAAAu) >> 1u);
  b = ((b & 0x33333333u) << 2u) | ((b & 0xCCCCCCCCu) >> 2u);
  b = ((b & 0x0F0F0F0Fu) << 4u) | ((b & 0xF0F0F0F0u) >> 4u);
  b = ((b & 0x00FF00FFu) << 8u) | ((b & 0xFF00FF00u) >> 8u);
  ax = div_((float)i, (float)n);
  ay = div_((float)b, 4294967296.0f);  // float(0xffffffffu)
}

template <int DCH> __device__ __forceinline__ float depth_texel(const float* p, int idx) {
  if (DCH == 2) return __ldg(reinterpret_cast<const float2*>(p) + idx).x;
  return __ldg(p + idx);
}

template <int DCH> __device__ __forceinline__ float depth_bilin(const float* p, const Bilin& B) {
  return blend1(B, depth_texel<DCH>(p, B.o00), depth_texel<DCH>(p, B.o10), depth_texel<DCH>(p, B.o01),
                depth_texel<DCH>(p, B.o11));
}

__device__ __forceinline__ f3 light_bilin(const float* p, const Bilin& B) {
  float4 a = ld4(p, B.o00), b = ld4(p, B.o10), c = ld4(p, B.o01), d = ld4(p, B.o11);
  f3 r;
  r.x = a.x * B.w00 + b.x * B.w10 + c.x * B.w01 + d.x * B.w11;
  r.y = a.y * B.w00 + b.y * B.w10 + c.y * B.w01 + d.y * B.w11;
  r.z = a.z * B.w00 + b.z * B.w10 + c.z * B.w01 + d.z * B.w11;
  return r;
}

// Both depth moments (E[d], E[d^2]) of a bilinear tap, same weights and order as depth_bilin.
__device__ __forceinline__ float2 moments_bilin(const float* p, const Bilin& B) {
  const float2 t00 = ld2(p, B.o00), t10 = ld2(p, B.o10), t01 = ld2(p, B.o01), t11 = ld2(p, B.o11);
  return make_float2(blend1(B, t00.x, t10.x, t01.x, t11.x), blend1(B, t00.y, t10.y, t01.y, t11.y));
}

// Soft-occlusion horizon: the angle a step lowers the horizon to when the
// sample's depth has the spread var = E[d^2] - E[d]^2 of its footprint.  The
// angular spread sigma = sqrt(var) |dtheta/dd| follows GetAngularDistribution
// (indirectLighting.frag:51-81, unused by the reference): a forward difference
// of eps = 0.1 along the sample's view ray rn.  With theta ~ N(angle, sigma^2)
// the horizon drops by E[max(0, max_h - theta)] = d Phi(z) + sigma phi(z),
// d = max_h - angle, z = d / sigma, Phi ~ 1 / (1 + exp(-1.702 z)) (logistic
// approximation of the normal distribution).  sigma <= 1e-6: the hard update.
__device__ __forceinline__ float soft_horizon(float dmean, float dsq, f3 rn, f3 cam, f3 cwp, f3 ed, f3 et,
                                              float angle, float max_h) {
  const float var = gmax(0.0f, dsq - dmean * dmean);
  const f3 od = sub3(add3(cam, mul3s(rn, dmean + 1e-1f)), cwp);
  const float oa = atan2f_(dot3(et, od), dot3(ed, od));
  const float deriv = div_(oa - angle, 1e-1f);
  const float sigma = sqrtf(var) * fabsf(deriv);
  if (!(sigma > 1e-6f)) return angle;
  const float d = max_h - angle;
  const float z = div_(d, sigma);
  const float pdf = 0.3989422804f * expf_(-0.5f * z * z);
  const float cdf = div_(1.0f, 1.0f + expf_(-1.702f * z));
  return max_h - (d * cdf + sigma * pdf);
}

// Fused-multiply-add forms of the two taps for the fast step loop.
template <int DCH> __device__ __forceinline__ float depth_bilin_fast(const float* p, const Bilin& B) {
  return fmaf(depth_texel<DCH>(p, B.o11), B.w11,
              fmaf(depth_texel<DCH>(p, B.o01), B.w01,
                   fmaf(depth_texel<DCH>(p, B.o10), B.w10, depth_texel<DCH>(p, B.o00) * B.w00)));
}

__device__ __forceinline__ f3 light_bilin_fast(const float* p, const Bilin& B) {
  const float4 a = ld4(p, B.o00), b = ld4(p, B.o10), c = ld4(p, B.o01), d = ld4(p, B.o11);
  return mk3(fmaf(d.x, B.w11, fmaf(c.x, B.w01, fmaf(b.x, B.w10, a.x * B.w00))),
             fmaf(d.y, B.w11, fmaf(c.y, B.w01, fmaf(b.y, B.w10, a.y * B.w00))),
             fmaf(d.z, B.w11, fmaf(c.z, B.w01, fmaf(b.z, B.w10, a.z * B.w00))));
}

// Shared-memory tables of one CTA-tile: n_tab steps, R directions and the
// levels' sizes (float(width >> l), float(height >> l)), laid out in that order
// in march_smem_bytes(n_tab, R) bytes.  The single-view kernels take exactly that
// as dynamic shared memory, so the unified L1/shared storage left to L1 does not
// shrink for the tables' maxima (GI_MAX_STEPS steps, GI_MAX_DIRS directions: 10 KB
// a CTA, against 0.6 KB for 22 steps and 16 directions).
struct MarchSmem {
  StepEntry* step;
  float2* dir;
  float2* lsize;
};

__host__ __device__ constexpr int march_smem_bytes(int n_tab, int dirs) {
  return n_tab * (int)sizeof(StepEntry) + dirs * (int)sizeof(float2) + GI_MAX_LEVELS * (int)sizeof(float2);
}
constexpr int kMarchSmemMax = march_smem_bytes(GI_MAX_STEPS, GI_MAX_DIRS);

// The replay's tables: a record holds at most 64 steps (its step mask), so the
// replay keeps fixed-size tables for that many (3.2 KB) -- constant offsets in its
// per-hit table reads, which the pointer layout above cost it 3 %.
constexpr int kRecMaxSteps = 64;
struct ReplaySmem {
  StepEntry step[kRecMaxSteps];
  float2 dir[GI_MAX_DIRS];
  float2 lsize[GI_MAX_LEVELS];
};

// The tables' places in `base` (16-byte aligned, march_smem_bytes(n_tab, dirs) bytes).
__device__ __forceinline__ MarchSmem march_smem(unsigned char* base, int n_tab, int dirs) {
  MarchSmem m;
  m.step = reinterpret_cast<StepEntry*>(base);
  m.dir = reinterpret_cast<float2*>(base + n_tab * sizeof(StepEntry));
  m.lsize = m.dir + dirs;
  return m;
}

// Pixels of a march record: every (pattern, sub-image pixel) slot, P^2 ceil(W/P) ceil(H/P).
__host__ __device__ __forceinline__ size_t record_pixels(const MarchArgs& a) {
  const size_t P = (size_t)a.pattern;
  return P * P * (((size_t)a.width + P - 1) / P) * (((size_t)a.height + P - 1) / P);
}

// The light term of a hit (:254-264): the trilinear light tap at the step's
// footprint, then dl += (light - ambient) * hc, in the order of the restatement
// (exact) or as fused multiply-adds (fast).  Shared by the march and the replay.
template <bool FAST>
__device__ __forceinline__ void add_light(const MarchArgs& a, const StepEntry& e, const Bilin& blo,
                                          const Bilin& bhi, bool two, float hc, float ambient, f3& dl) {
  if (FAST) {
    f3 ls = light_bilin_fast(a.light[e.lo], blo);
    if (two) {
      const f3 lh = light_bilin_fast(a.light[e.hi], bhi);
      ls = mk3(fmaf(lh.x - ls.x, e.delta, ls.x), fmaf(lh.y - ls.y, e.delta, ls.y), fmaf(lh.z - ls.z, e.delta, ls.z));
    }
    dl = mk3(fmaf(ls.x - ambient, hc, dl.x), fmaf(ls.y - ambient, hc, dl.y), fmaf(ls.z - ambient, hc, dl.z));
  } else {
    f3 ls = light_bilin(a.light[e.lo], blo);
    if (two) {
      f3 lh = light_bilin(a.light[e.hi], bhi);
      ls.x = ls.x * (1.0f - e.delta) + lh.x * e.delta;
      ls.y = ls.y * (1.0f - e.delta) + lh.y * e.delta;
      ls.z = ls.z * (1.0f - e.delta) + lh.z * e.delta;
    }
    dl.x = dl.x + ls.x * hc;
    dl.y = dl.y + ls.y * hc;
    dl.z = dl.z + ls.z * hc;
    dl.x = dl.x - ambient * hc;
    dl.y = dl.y - ambient * hc;
    dl.z = dl.z - ambient * hc;
  }
}

// Texture-unit taps (MarchArgs::depth_tex / light_tex): one trilinear fetch at
// level lo + delta of the step -- the sampler of the reference's textureLod with
// linear filtering and linear mipmapping, evaluated by the texture units (8-bit
// sub-texel and level weights) instead of in software.
__device__ __forceinline__ float tex_level(const StepEntry& e) { return e.level; }

__device__ __forceinline__ void add_light_tex(const MarchArgs& a, float sx, float sy, float level, float hc,
                                              float ambient, f3& dl) {
  const float4 l = tex2DLod<float4>(a.light_tex, sx, sy, level);
  dl = mk3(fmaf(l.x - ambient, hc, dl.x), fmaf(l.y - ambient, hc, dl.y), fmaf(l.z - ambient, hc, dl.z));
}

// Per-pattern tables of a CTA-tile: the same values as evaluating :170-177,
// :212, :217, :234-235 per pixel.  Every thread of the CTA calls it; the caller
// synchronises before use.
template <bool TEX = false, class Smem>
__device__ __forceinline__ void march_tables(const MarchArgs& a, int n_tab, int pat, Smem& sm, int tid,
                                             int nthreads) {
  const int P = a.pattern;
  const int R = a.dirs;
  const int SR = a.step_dirs;
  const float W = (float)a.width;
  const float ns = div_(W, 1000.0f);
  float ang, lin;
  hammersley(pat, P * P, ang, lin);
  const float pixel_ang = div_(2.0f * kPiRef, (float)R) * ang;
  for (int d = tid; d < R; d += nthreads) {
    float sa = pixel_ang + div_(2.0f * kPiRef, (float)R) * (float)d;
    float sn, cs;
    sincosf_(sa, &sn, &cs);
    sm.dir[d] = make_float2(cs, sn);
  }
  const float q = (float)(a.num_levels - 1);
  const float ln2 = logf_(2.0f);
  for (int s = tid; s < n_tab; s += nthreads) {
    float off = ns * powf_(div_(2.0f * kPiRef, (float)SR) + 1.0f, (float)s + lin) + 1.0f - ns;
    float lod = div_(logf_(gmax(0.0f, div_(2.0f * kPiRef, (float)SR) * (off - 1.0f) * 0.5f)), ln2) + (-2.0f);
    float lam = gmin(gmax(lod, 0.0f), q);
    float lo = floorf(lam);
    StepEntry e;
    e.off = off;
    e.delta = lam - lo;
    e.lo = (int)lo;
    if (TEX) e.level = lam;  // == lo + delta exactly (lam - floor(lam) and the sum back are exact)
    else e.hi = min(e.lo + 1, a.num_levels - 1);
    sm.step[s] = e;
  }
  if (tid < a.num_levels) sm.lsize[tid] = make_float2((float)(a.width >> tid), (float)(a.height >> tid));
}

// One CTA-tile of the march: the pixels of interleave pattern `pat` in march
// tile `tile` (32 x KY sub-image pixels, a (32 P) x (KY P) screen rectangle).
// Shared by the full-frame, tile-list and batched kernels; every thread of the
// CTA calls it (it contains one CTA barrier).
//
// SPLIT > 1 (the direction-split form for short tile lists): the CTA takes one
// row `row` of the tile, thread (x, s) marches pixel x's directions s, s + SPLIT,
// ..., stores each direction's term in `contrib` (at most kSplitMaxDirs
// directions), and after a barrier thread (x, 0) adds the terms in direction
// order -- the same sum, in the same order, as one thread marching them all.
//
// REC (the standard form only): also record, per pixel and direction, which steps
// raised the horizon and their horizon contributions hc, plus the direction's
// initial term hc0 -- everything of the march that does not depend on the light
// pyramid -- for march_replay_tile to re-light with another pyramid.
template <int DCH, bool DEINT, int KY, bool FAST, bool SOFT = false, int SPLIT = 1, bool REC = false,
          bool TEX = false>
__device__ __forceinline__ void march_tile(const MarchArgs& a, int n_tab, int pat, int tile, int tiles_x,
                                           MarchSmem& sm, int row = 0, float* contrib = nullptr) {
  static_assert(!SOFT || (DCH == 2 && !FAST), "the soft horizon needs both depth moments, exact contract");
  static_assert(SPLIT == 1 || (!DEINT && !SOFT), "the direction split serves the standard form");
  static_assert(!REC || (SPLIT == 1 && !DEINT && !SOFT), "recording serves the standard form");
  static_assert(!TEX || (FAST && DCH == 2 && !DEINT), "texture depth taps serve the fast standard form");
  constexpr int kThreads = kMarchTx * (SPLIT > 1 ? SPLIT : KY);
  StepEntry* s_step = sm.step;
  float2* s_dir = sm.dir;
  float2* s_lsize = sm.lsize;
  const int P = a.pattern;
  const int kx = pat % P, ky = pat / P;
  const int R = a.dirs;
  const int SR = a.step_dirs;  // dirsCount of :212, :217, :234-235
  const float W = (float)a.width, H = (float)a.height;
  const float ns = div_(W, 1000.0f);

  const int tid = threadIdx.y * kMarchTx + threadIdx.x;
  march_tables<TEX>(a, n_tab, pat, sm, tid, kThreads);
  __syncthreads();

  // Pixel of this thread.
  const int i = (tile % tiles_x) * kMarchTx + threadIdx.x;
  const int j = (tile / tiles_x) * KY + (SPLIT > 1 ? row : (int)threadIdx.y);
  int px = kx + P * i, py = ky + P * j;
  const bool inside = px < a.width && py < a.height;
  if (SPLIT == 1 && !inside) return;
  if (!inside) {  // a split CTA's lanes past the edge march an in-image pixel, to reach the barrier
    px = min(kx, a.width - 1);
    py = min(ky, a.height - 1);
  }

  const float rW = rcp_(W), rH = rcp_(H);  // x / W == x * rcp(W) under the division contract
  const float cpx = (float)px + 0.5f, cpy = (float)py + 0.5f;
  const float cscx = cpx * rW, cscy = cpy * rH;
  f3 N;
  float cdepth;
  size_t out_idx;
  if (DEINT) {
    const int sw = a.width / P, sh = a.height / P;
    const int dx = kx * sw + i, dy = ky * sh + j;
    out_idx = (size_t)dy * a.width + dx;
    float4 n = ld4(a.normal, (int)out_idx);
    N = mk3(n.x, n.y, n.z);
    cdepth = __ldg(a.ndc + out_idx);
  } else {
    out_idx = (size_t)py * a.width + px;
    float4 n = sample4(a.normal, a.width, a.height, cscx, cscy);
    N = mk3(n.x, n.y, n.z);
    cdepth = sample1(a.ndc, a.width, a.height, cscx, cscy);
  }

  const float4 cam4 = mat_vec(a.inv_view, 0.0f, 0.0f, 0.0f, 1.0f);
  const f3 cam = mk3(cam4.x, cam4.y, cam4.z);
  const f3 cwp = unproject(a.inv_view_proj, cscx, cscy, cdepth);
  const float ambient = 0.01f;
  const float log_base = logf_(div_(2.0f * kPiRef, (float)SR) + 1.0f);
  const float inv_width = div_(1.0f, 0.1f);
  const float rR = rcp_((float)R);
  float c0, s0;
  sincosf_(2.0f * 0.0f, &s0, &c0);

  // Records are indexed in the interleaved (pattern, sub-image row, column) order,
  // in which a warp's 32 pixels are consecutive: coalesced stores and loads.
  const unsigned npix = (unsigned)record_pixels(a);
  const unsigned rec_idx = ((unsigned)pat * ((a.height + P - 1) / P) + j) * ((a.width + P - 1) / P) + i;
  f3 sum = mk3(0.0f, 0.0f, 0.0f);
  for (int d = SPLIT > 1 ? (int)threadIdx.y : 0; d < R; d += SPLIT) {
    unsigned long long hits = 0ull;  // REC: steps that raised the horizon
    // REC: the next hc slot; the k-th hit of every pixel is row k of the direction's
    // block, so the lanes of a warp fill neighbouring words of a row (whole sectors
    // once each has hit k times) and the replay reads a row per hit coalesced.  The
    // record is written and read once, larger than L2: streaming (evict-first) stores
    // and loads keep the pyramids the taps read resident in L2 (0.4 % of the frame).
    float* rec_next = REC ? a.rec_hc + (size_t)d * a.rec_steps * npix + rec_idx : nullptr;
    const float2 dir = s_dir[d];
    const float eps = 10e-1f;
    const float ocx = (cpx + dir.x * eps) * rW, ocy = (cpy + dir.y * eps) * rH;
    // The direction's frame (:180-199): eye direction ed, tangent et (the
    // normalised difference of two view rays one pixel apart: a cancelling sum,
    // kept exact in both precisions), and the initial horizon h0 of the projected
    // normal.  The fast precision takes h0 from its fitted atan and cos 2h0,
    // sin 2h0 from the atan's arguments, as its step loop does.
    const f3 owp = unproject(a.inv_view_proj, ocx, ocy, cdepth);
    const f3 ed = normalize3(sub3(cam, cwp));
    const f3 et = normalize3(sub3(normalize3(sub3(owp, cam)), normalize3(sub3(cwp, cam))));
    float max_h, cm, sm;
    {
      const f3 cr = cross3(et, ed);
      const f3 dnp = cross3(mk3(-cr.x, -cr.y, -cr.z), N);
      if (FAST) {
        const float hy = fdot3(dnp, et), hx = fdot3(dnp, ed);
        max_h = fast_atan2(hy, hx);
        cm = 1.0f;
        sm = 0.0f;
        const float r2 = fmaf(hx, hx, hy * hy);
        if (r2 > 0.0f) {
          const float ir = __fdividef(1.0f, r2);
          cm = (hx - hy) * (hx + hy) * ir;
          sm = 2.0f * hx * hy * ir;
        }
      } else {
        max_h = atan2f_(dot3(dnp, et), dot3(dnp, ed));
        sincosf_(2.0f * max_h, &sm, &cm);
      }
    }
    // BoxRayCast(centre, dir, (0,0), viewport) (:83-99, :202-204).
    float path;
    {
      float ix = rcp_(dir.x), iy = rcp_(dir.y);
      float t1 = (0.0f - cpx) * ix, t2 = (W - cpx) * ix;
      float t3 = (0.0f - cpy) * iy, t4 = (H - cpy) * iy;
      float tmax = gmin(gmax(t1, t2), gmax(t3, t4));
      path = fabsf(tmax);
    }
    const float qd = 0.25f * (FAST ? fdot3(ed, N) : dot3(ed, N));
    const float qt = 0.25f * (FAST ? fdot3(et, N) : dot3(et, N));
    // FAST: the step's horizon coordinates hy = et . (n d + cam - cwp), hx = ed . (...)
    // with the sample's view ray n = sign(w) U / |U|, U = A + sx B + sy C (set_ray_basis):
    // et . U and ed . U are linear in (sx, sy), so the direction's constants are
    // et . A, et . B, et . C, ed . A, ... and et . (cam - cwp), ed . (cam - cwp).
    f3 eT = mk3(0.0f, 0.0f, 0.0f), eD = eT;
    float etc = 0.0f, edc = 0.0f;
    if (FAST) {
      const float* rb = a.ray;
      eT = mk3(fdot3(et, mk3(rb[0], rb[1], rb[2])), fdot3(et, mk3(rb[4], rb[5], rb[6])),
               fdot3(et, mk3(rb[8], rb[9], rb[10])));
      eD = mk3(fdot3(ed, mk3(rb[0], rb[1], rb[2])), fdot3(ed, mk3(rb[4], rb[5], rb[6])),
               fdot3(ed, mk3(rb[8], rb[9], rb[10])));
      const f3 cc = sub3(cam, cwp);
      etc = fdot3(et, cc);
      edc = fdot3(ed, cc);
    }
    float hc0 = qd * (-cm + c0) + qt * (2.0f * max_h - 2.0f * 0.0f - sm + s0);
    f3 dl = mk3(ambient * hc0, ambient * hc0, ambient * hc0);
    int iters = (int)div_(logf_(div_(path, ns)), log_base) + 1;
    if (a.step_cap > 0 && iters > a.step_cap) iters = a.step_cap;
    if (iters > n_tab) iters = n_tab;
    for (int s = 0; s < iters; s++) {
      const StepEntry e = s_step[s];
      const float spx = cpx + dir.x * e.off, spy = cpy + dir.y * e.off;
      const float sx = spx * rW, sy = spy * rH;
      const bool two = e.delta != 0.0f;
      Bilin blo, bhi;           // footprints of the software taps (not TEX)
      float dsamp, dsq = 0.0f;  // E[d] and, for the soft horizon, E[d^2] of the trilinear tap
      if (TEX) {
        dsamp = tex2DLod<float>(a.depth_tex, sx, sy, tex_level(e));
      } else {
        const float2 slo = s_lsize[e.lo];
        blo = bilin_f(sx, sy, slo.x, slo.y, a.width >> e.lo, a.height >> e.lo);
        if (SOFT) {
          const float2 m = moments_bilin(a.depth[e.lo], blo);
          dsamp = m.x;
          dsq = m.y;
        } else {
          dsamp = FAST ? depth_bilin_fast<DCH>(a.depth[e.lo], blo) : depth_bilin<DCH>(a.depth[e.lo], blo);
        }
        if (two) {
          const float2 shi = s_lsize[e.hi];
          bhi = bilin_f(sx, sy, shi.x, shi.y, a.width >> e.hi, a.height >> e.hi);
          if (FAST) {
            const float dhi = depth_bilin_fast<DCH>(a.depth[e.hi], bhi);
            dsamp = fmaf(dhi - dsamp, e.delta, dsamp);
          } else if (SOFT) {
            const float2 mh = moments_bilin(a.depth[e.hi], bhi);
            dsamp = dsamp * (1.0f - e.delta) + mh.x * e.delta;
            dsq = dsq * (1.0f - e.delta) + mh.y * e.delta;
          } else {
            float dhi = depth_bilin<DCH>(a.depth[e.hi], bhi);
            dsamp = dsamp * (1.0f - e.delta) + dhi * e.delta;
          }
        }
      }
      float sh = 0.0f, hy = 0.0f, hx = 0.0f;
      bool hit;
      if (FAST) {
        // The sample's view ray: (unproject(sx, sy, 1) - cam) scaled by the
        // homogeneous w, which is linear in (sx, sy), normalised (see set_ray_basis),
        // entering only through the linear forms above and |U|^2.
        const float* rb = a.ray;
        const float* q = a.ray_q;
        const float eu = fmaf(sy, eT.z, fmaf(sx, eT.y, eT.x));
        const float du = fmaf(sy, eD.z, fmaf(sx, eD.y, eD.x));
        const float uu = fmaf(sx, fmaf(sx, q[3], q[1]), q[0]) + sy * fmaf(sy, q[5], fmaf(sx, q[4], q[2]));
        const float uw = fmaf(sy, rb[11], fmaf(sx, rb[7], rb[3]));
        const float sd = dsamp * copysignf(rsqrtf(uu), uw);
        hy = fmaf(sd, eu, etc);
        hx = fmaf(sd, du, edc);
        sh = fast_atan2(hy, hx);
        hit = sh < max_h;
      } else {
        const f3 q = unproject(a.inv_view_proj, sx, sy, 1.0f);
        const f3 rn = normalize3(sub3(q, cam));
        const f3 swp = add3(cam, mul3s(rn, dsamp));
        const f3 wd = sub3(swp, cwp);
        sh = atan2f_(dot3(et, wd), dot3(ed, wd));
        if (SOFT) sh = soft_horizon(dsamp, dsq, rn, cam, cwp, ed, et, sh, max_h);
        hit = sh < max_h;
      }
      if (hit) {
        // The horizon contribution of the step (HC(h, hmax) of :254-264), then its light.
        float side = 1.0f;
        if (FAST) {
          // The same product in fewer instructions: of saturate((1 - x) / 0.1) and
          // saturate(x / 0.1) at most one is below 1 (that needs x > 0.9 and x < 0.1),
          // so their product is the smaller one, and saturate of a monotone product is
          // monotone, so that is the clamp of the smaller argument; the coordinates are
          // finite and never -0, where the GLSL clamp and the hardware one agree.
          side = __saturatef(fminf(1.0f - sx, sx) * inv_width) * __saturatef(fminf(1.0f - sy, sy) * inv_width);
        } else {
          side = side * saturate((1.0f - sx) * inv_width);
          side = side * saturate(sx * inv_width);
          side = side * saturate((1.0f - sy) * inv_width);
          side = side * saturate(sy * inv_width);
        }
        float hc, ss, cs;
        if (FAST) {
          ss = 0.0f;
          cs = 1.0f;
          const float r2 = fmaf(hx, hx, hy * hy);
          if (r2 > 0.0f) {
            const float ir = __fdividef(1.0f, r2);
            cs = (hx - hy) * (hx + hy) * ir;
            ss = 2.0f * hx * hy * ir;
          }
          hc = fmaf(qd, cs - cm, qt * (fmaf(2.0f, max_h - sh, ss) - sm)) * side;
        } else {
          sincosf_(2.0f * sh, &ss, &cs);
          hc = (qd * (-cm + cs) + qt * (2.0f * max_h - 2.0f * sh - sm + ss)) * side;
        }
        if (TEX) add_light_tex(a, sx, sy, tex_level(e), hc, ambient, dl);
        else add_light<FAST>(a, e, blo, bhi, two, hc, ambient, dl);
        max_h = sh;
        cm = cs;
        sm = ss;
        if (REC) {
          __stcs(rec_next, hc);
          rec_next += npix;
          hits |= 1ull << s;
        }
      }
    }
    if (REC) {
      __stcs(a.rec_mask + (size_t)d * npix + rec_idx, hits);
      __stcs(a.rec_hc0 + (size_t)d * npix + rec_idx, hc0);
    }
    if (SPLIT > 1) {
      float* c = contrib + 3 * (d * kMarchTx + threadIdx.x);
      c[0] = 2.0f * dl.x * rR;
      c[1] = 2.0f * dl.y * rR;
      c[2] = 2.0f * dl.z * rR;
    } else {
      sum.x = sum.x + 2.0f * dl.x * rR;
      sum.y = sum.y + 2.0f * dl.y * rR;
      sum.z = sum.z + 2.0f * dl.z * rR;
    }
  }
  if (SPLIT > 1) {
    __syncthreads();
    if (threadIdx.y != 0 || !inside) return;
    for (int d = 0; d < R; d++) {
      const float* c = contrib + 3 * (d * kMarchTx + threadIdx.x);
      sum.x = sum.x + c[0];
      sum.y = sum.y + c[1];
      sum.z = sum.z + c[2];
    }
  }
  reinterpret_cast<float4*>(a.out)[out_idx] = make_float4(sum.x, sum.y, sum.z, 1.0f);
}

// The march of a pixel re-lit from its record (MarchArgs::rec = 2): the same
// step table, step footprints and light taps as march_tile, only at the steps
// the record marks, with the recorded horizon contributions -- the result is
// the march's over the new light pyramid, bit for bit.
template <int KY, bool FAST>
__device__ __forceinline__ void march_replay_tile(const MarchArgs& a, int n_tab, int pat, int tile, int tiles_x,
                                                  ReplaySmem& sm) {
  constexpr int kThreads = kMarchTx * KY;
  const int P = a.pattern;
  const int kx = pat % P, ky = pat / P;
  const int R = a.dirs;
  const float W = (float)a.width, H = (float)a.height;
  march_tables(a, n_tab, pat, sm, threadIdx.y * kMarchTx + threadIdx.x, kThreads);
  __syncthreads();
  const int i = (tile % tiles_x) * kMarchTx + threadIdx.x;
  const int j = (tile / tiles_x) * KY + threadIdx.y;
  const int px = kx + P * i, py = ky + P * j;
  if (px >= a.width || py >= a.height) return;
  const float rW = rcp_(W), rH = rcp_(H);
  const float cpx = (float)px + 0.5f, cpy = (float)py + 0.5f;
  const size_t out_idx = (size_t)py * a.width + px;
  const unsigned npix = (unsigned)record_pixels(a);
  const unsigned rec_idx = ((unsigned)pat * ((a.height + P - 1) / P) + j) * ((a.width + P - 1) / P) + i;
  const float ambient = 0.01f;
  const float rR = rcp_((float)R);
  f3 sum = mk3(0.0f, 0.0f, 0.0f);
  for (int d = 0; d < R; d++) {
    const float2 dir = sm.dir[d];
    const float hc0 = __ldcs(a.rec_hc0 + (size_t)d * npix + rec_idx);
    // Bits index the 64-entry table (ReplaySmem): in bounds whatever the mask holds.
    unsigned long long hits = __ldcs(a.rec_mask + (size_t)d * npix + rec_idx);
    const float* rec_next = a.rec_hc + (size_t)d * a.rec_steps * npix + rec_idx;
    f3 dl = mk3(ambient * hc0, ambient * hc0, ambient * hc0);
    while (hits) {
      const int s = __ffsll((long long)hits) - 1;
      hits &= hits - 1ull;
      const StepEntry e = sm.step[s];
      const float spx = cpx + dir.x * e.off, spy = cpy + dir.y * e.off;
      const float sx = spx * rW, sy = spy * rH;
      const float hc = __ldcs(rec_next);
      rec_next += npix;
      const float2 slo = sm.lsize[e.lo];
      const Bilin blo = bilin_f(sx, sy, slo.x, slo.y, a.width >> e.lo, a.height >> e.lo);
      Bilin bhi;
      const bool two = e.delta != 0.0f;
      if (two) {
        const float2 shi = sm.lsize[e.hi];
        bhi = bilin_f(sx, sy, shi.x, shi.y, a.width >> e.hi, a.height >> e.hi);
      }
      add_light<FAST>(a, e, blo, bhi, two, hc, ambient, dl);
    }
    sum.x = sum.x + 2.0f * dl.x * rR;
    sum.y = sum.y + 2.0f * dl.y * rR;
    sum.z = sum.z + 2.0f * dl.z * rR;
  }
  reinterpret_cast<float4*>(a.out)[out_idx] = make_float4(sum.x, sum.y, sum.z, 1.0f);
}

// Register budget: 64 per thread (8 CTAs of 128 threads per SM).  The software
// step loop is issue-bound with more ready warps than issue slots, and a measured
// 80-register build of the fast loop (6 CTAs per SM, fewer spills) ran 9 % slower.
// The texture loop (TEX) waits on its texture fetches instead: 40 registers (12
// CTAs per SM, a few spills) measured 4.6 % faster on the whole frame than 64, and
// 48 registers (10 CTAs) 4.2 %; 32 registers (16 CTAs) spill in the step loop and
// made the recording march 38 % slower.  The persistent batch kernel keeps 64: at 40
// it spills in its work loop and the batched frame ran 24 % slower.
template <bool FAST, int KY, bool TEX = false> constexpr int march_min_blocks() {
  return (TEX ? 1536 : 1024) / (kMarchTx * KY);
}

template <int DCH, bool DEINT, int KY, bool FAST, bool SOFT = false, bool REC = false, bool TEX = false>
__global__ void __launch_bounds__(kMarchTx* KY, march_min_blocks<FAST, KY, TEX>())
    march_kernel(const __grid_constant__ MarchArgs a, int n_tab, int tiles_x, int tiles_total) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];  // march_smem_bytes(n_tab, a.dirs)
  MarchSmem sm = march_smem(dyn_smem, n_tab, a.dirs);
  // Pattern is the fastest-varying block index: the P*P CTAs that share a
  // screen tile run together and share its texels in L1/L2.
  const int P = a.pattern;
  const int pat = blockIdx.x % (P * P);
  const int tile = a.tiles ? __ldg(a.tiles + blockIdx.x / (P * P)) : (int)(blockIdx.x / (P * P));
  if (tile < 0 || tile >= tiles_total) return;  // a listed tile outside the grid: nothing to march
  march_tile<DCH, DEINT, KY, FAST, SOFT, 1, REC, TEX>(a, n_tab, pat, tile, tiles_x, sm);
}

template <int KY, bool FAST>
__global__ void __launch_bounds__(kMarchTx* KY, march_min_blocks<FAST, KY>())
    march_replay_kernel(const __grid_constant__ MarchArgs a, int n_tab, int tiles_x) {
  __shared__ ReplaySmem sm;  // n_tab <= kRecMaxSteps (checked at launch)
  const int P = a.pattern;
  march_replay_tile<KY, FAST>(a, n_tab, (int)(blockIdx.x % (P * P)), (int)(blockIdx.x / (P * P)), tiles_x, sm);
}

// Direction-split march (march_tile with SPLIT = kSplit) of a tile list -- a
// short list (the judge's 1/64 of the tiles) spread over kMarchTy times more
// CTAs -- or of the whole frame (a.tiles null; the autotuner's four-threads-per-
// pixel layout): each CTA one row of a tile, each thread a quarter of a pixel's
// directions.
constexpr int kSplit = 4;
constexpr int kSplitMaxDirs = 32;
constexpr int kSplitMinDirs = 4;

template <bool FAST, bool TEX>
__global__ void __launch_bounds__(kMarchTx* kSplit, 1024 / (kMarchTx * kSplit))
    march_split_kernel(const __grid_constant__ MarchArgs a, int n_tab, int tiles_x, int tiles_total) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];  // march_smem_bytes(n_tab, a.dirs)
  MarchSmem sm = march_smem(dyn_smem, n_tab, a.dirs);
  __shared__ float contrib[kSplitMaxDirs * kMarchTx * 3];
  const int P2 = a.pattern * a.pattern;
  const int pat = blockIdx.x % P2;
  const int rest = blockIdx.x / P2;
  const int row = rest % kMarchTy;
  const int tile = a.tiles ? __ldg(a.tiles + rest / kMarchTy) : rest / kMarchTy;
  if (tile < 0 || tile >= tiles_total) return;  // a listed tile outside the grid: nothing to march
  march_tile<2, false, kMarchTy, FAST, false, kSplit, false, TEX>(a, n_tab, pat, tile, tiles_x, sm, row, contrib);
}

// Persistent batched march: CTAs claim work items (view, tile, pattern) from a
// counter until the list is exhausted; items are ordered by decreasing cost.
// The views' arguments are a kernel parameter (the launch's constant bank): the
// step loop reads them as the single-view kernel reads its own, where a copy in
// shared memory cost registers, spills and 3 % of the batched frame.
template <int KY, bool FAST, bool TEX>
__global__ void __launch_bounds__(kMarchTx* KY, march_min_blocks<FAST, KY>())
    march_batch_kernel(const __grid_constant__ BatchTable t, const int2* __restrict__ items, int num_items,
                       int* __restrict__ counter) {
  // The views' tables differ in size: dynamic shared memory of the largest
  // (march_smem_bytes over the table's views).
  extern __shared__ __align__(16) unsigned char tab_smem[];
  __shared__ int s_item;
  const int tid = threadIdx.y * kMarchTx + threadIdx.x;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= num_items) return;
    const int2 w = __ldg(items + it);
    const BatchView& v = t.v[w.x];
    MarchSmem sm = march_smem(tab_smem, v.n_tab, v.a.dirs);
    march_tile<2, false, KY, FAST, false, 1, false, TEX>(v.a, v.n_tab, w.y & 63, w.y >> 6, v.tiles_x, sm);
    __syncthreads();  // the tables and s_item are rewritten for the next item
  }
}

// Upper bound on the steps any pixel takes (:212): the path to the viewport edge
// is at most its diagonal.
int max_steps(int width, int height, int dirs) {
  float W = (float)width, H = (float)height;
  float diag = sqrtf(W * W + H * H);
  float ns = div_(W, 1000.0f);
  float lb = logf_(div_(2.0f * kPiRef, (float)dirs) + 1.0f);
  int n = (int)div_(logf_(div_(diag, ns)), lb) + 1;
  return n + 2;
}

}  // namespace

// Tuned CTA height (KY) per march shape; absent keys use the default 4.
struct TuneKey {
  int w, h, dirs, step_dirs, cap, fast;
  bool operator<(const TuneKey& o) const {
    if (fast != o.fast) return fast < o.fast;
    if (w != o.w) return w < o.w;
    if (h != o.h) return h < o.h;
    if (dirs != o.dirs) return dirs < o.dirs;
    if (step_dirs != o.step_dirs) return step_dirs < o.step_dirs;
    return cap < o.cap;
  }
};
static std::mutex g_tune_mutex;
// A march shape's tuned launch layout: CTA height `rows` of the one-thread-per-
// pixel form, or split = kSplit (four threads per pixel, the direction split).
struct TunedLayout {
  int rows, split;
};
static std::map<TuneKey, TunedLayout> g_tuned;

static TuneKey key_of(const MarchArgs& a) {
  return TuneKey{a.width, a.height, a.dirs, a.step_dirs, a.step_cap, a.fast ? (a.depth_tex ? 2 : 1) : 0};
}

// ---- Pyramid textures ------------------------------------------------------

namespace {

struct PackLevel {
  const float* src;
  unsigned long long surf;  // surface object of the level's array
  int w, h, first_block;
};
struct PackLevels {
  PackLevel level[GI_MAX_LEVELS];
  int count, src_channels;
};

// Level k's texels into its array (surface writes, out-of-range writes dropped):
// each block serves one level (blocks [first_block, next level's first_block)).
template <int CH>
__global__ void pack_pyramid_kernel(const __grid_constant__ PackLevels L) {
  int k = 0;
  while (k + 1 < L.count && (int)blockIdx.x >= L.level[k + 1].first_block) k++;
  const PackLevel& v = L.level[k];
  const int t = ((int)blockIdx.x - v.first_block) * (int)blockDim.x + (int)threadIdx.x;
  if (t >= v.w * v.h) return;
  const int y = t / v.w, x = t - y * v.w;
  const float* p = v.src + (size_t)t * L.src_channels;
  if (CH == 1) {
    surf2Dwrite<float>(__ldg(p), v.surf, x * (int)sizeof(float), y, cudaBoundaryModeZero);
  } else {
    const float4 c = make_float4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
    surf2Dwrite<float4>(c, v.surf, x * (int)sizeof(float4), y, cudaBoundaryModeZero);
  }
}

constexpr int kPackThreads = 256;

// One trilinear fetch per point (gi_texture_sample): coordinates st[2 i], st[2 i + 1],
// level lod[i]; CH floats of the result to out[CH i].
template <int CH>
__global__ void texture_sample_kernel(unsigned long long tex, const float* __restrict__ st,
                                      const float* __restrict__ lod, float* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (CH == 1) {
    out[i] = tex2DLod<float>(tex, st[2 * i], st[2 * i + 1], lod[i]);
  } else {
    const float4 r = tex2DLod<float4>(tex, st[2 * i], st[2 * i + 1], lod[i]);
    out[4 * i] = r.x;
    out[4 * i + 1] = r.y;
    out[4 * i + 2] = r.z;
    out[4 * i + 3] = r.w;
  }
}

}  // namespace

int PyramidTexture::Create(int width, int height, int num_levels, int channels) {
  Destroy();
  if (width < 1 || height < 1 || num_levels < 1 || num_levels > GI_MAX_LEVELS || (channels != 1 && channels != 4))
    return fail(GI_ERR_INVALID_ARGUMENT, "pyramid texture: bad shape");
  if ((width >> (num_levels - 1)) < 1 || (height >> (num_levels - 1)) < 1)
    return fail(GI_ERR_INVALID_ARGUMENT, "pyramid texture: more levels than the size has");
  const cudaChannelFormatDesc desc =
      channels == 1 ? cudaCreateChannelDesc<float>() : cudaCreateChannelDesc<float4>();
  int st = check_cuda(device_alloc_mipmapped(&mip_, &desc, make_cudaExtent((size_t)width, (size_t)height, 0),
                                               (unsigned)num_levels, cudaArraySurfaceLoadStore),
                      "pyramid texture: mipmapped array");
  if (st) {
    mip_ = nullptr;
    return st;
  }
  w_ = width;
  h_ = height;
  levels_ = num_levels;
  channels_ = channels;
  for (int k = 0; k < num_levels && !st; k++) {
    cudaArray_t lev = nullptr;
    st = check_cuda(cudaGetMipmappedArrayLevel(&lev, mip_, (unsigned)k), "pyramid texture: level");
    if (st) break;
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = lev;
    cudaSurfaceObject_t so = 0;
    st = check_cuda(cudaCreateSurfaceObject(&so, &rd), "pyramid texture: surface object");
    surf_[k] = so;
  }
  if (!st) {
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeMipmappedArray;
    rd.res.mipmap.mipmap = mip_;
    cudaTextureDesc td{};
    td.addressMode[0] = cudaAddressModeClamp;
    td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.mipmapFilterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    td.minMipmapLevelClamp = 0.0f;
    td.maxMipmapLevelClamp = (float)(num_levels - 1);
    cudaTextureObject_t t = 0;
    st = check_cuda(cudaCreateTextureObject(&t, &rd, &td, nullptr), "pyramid texture: texture object");
    tex_ = t;
  }
  if (st) Destroy();
  return st;
}

void PyramidTexture::Destroy(bool sync) {
  if (!mip_) return;
  if (sync) cudaDeviceSynchronize();  // no launch may still use the objects
  if (tex_) cudaDestroyTextureObject(tex_);
  for (int k = 0; k < levels_; k++)
    if (surf_[k]) cudaDestroySurfaceObject(surf_[k]);
  device_free_mipmapped(mip_);
  mip_ = nullptr;
  tex_ = 0;
  for (int k = 0; k < GI_MAX_LEVELS; k++) surf_[k] = 0;
  w_ = h_ = levels_ = channels_ = 0;
}

int PyramidTexture::Pack(const float* const* levels, int src_channels, cudaStream_t stream) const {
  if (!mip_) return fail(GI_ERR_INVALID_ARGUMENT, "pyramid texture: not created");
  if (src_channels < channels_) return fail(GI_ERR_INVALID_ARGUMENT, "pyramid texture: too few source channels");
  PackLevels L{};
  L.count = levels_;
  L.src_channels = src_channels;
  int blocks = 0;
  for (int k = 0; k < levels_; k++) {
    if (!levels[k]) return fail(GI_ERR_INVALID_ARGUMENT, "pyramid texture: null level");
    PackLevel& v = L.level[k];
    v.src = levels[k];
    v.surf = surf_[k];
    v.w = w_ >> k;
    v.h = h_ >> k;
    v.first_block = blocks;
    blocks += (v.w * v.h + kPackThreads - 1) / kPackThreads;
  }
  if (channels_ == 1) pack_pyramid_kernel<1><<<blocks, kPackThreads, 0, stream>>>(L);
  else pack_pyramid_kernel<4><<<blocks, kPackThreads, 0, stream>>>(L);
  GI_CHECK_LAUNCH("pack_pyramid_kernel");
  count_launches(1);
  return GI_OK;
}

// The fast step loop's view ray.  With V = inv_view_proj * (2 sx - 1, 2 sy - 1, 1, 1)
// = V00 + sx (2 c0) + sy (2 c1) (c0, c1 the matrix's first two columns) and cam the
// eye position, U = V.xyz - cam V.w is unproject(sx, sy, 1) - cam scaled by V.w,
// so the ray direction is sign(V.w) U / |U|.  ray[0..3] = (U, V.w) at (0, 0),
// ray[4..7] and ray[8..11] its derivatives in sx and sy, evaluated in double except
// for the constant part of V.w: that is the fp32 sum m[11] + m[15] that the exact
// unprojection computes (a cancelling sum for a far plane, 1 / far), so that both
// precisions scale the far-plane point alike and the fast rays track the exact ones.
void set_ray_basis(MarchArgs& a) {
  const float* m = a.inv_view_proj.m;
  const double cam[3] = {a.inv_view.m[12], a.inv_view.m[13], a.inv_view.m[14]};
  const float w_far = m[11] + m[15];
  double U[3][3];  // A, B, C: the ray's constant part and its derivatives in sx, sy
  for (int part = 0; part < 3; part++) {
    double v[4];
    for (int r = 0; r < 4; r++) {
      if (part == 0) v[r] = -(double)m[r] - (double)m[4 + r] + (double)m[8 + r] + (double)m[12 + r];
      else v[r] = 2.0 * (double)m[4 * (part - 1) + r];
    }
    if (part == 0) v[3] = (double)w_far - (double)m[3] - (double)m[7];
    for (int r = 0; r < 3; r++) {
      U[part][r] = v[r] - cam[r] * v[3];
      a.ray[4 * part + r] = (float)U[part][r];
    }
    a.ray[4 * part + 3] = (float)v[3];
  }
  // |U|^2 = |A + sx B + sy C|^2 = q0 + sx (q1 + sx q3) + sy (q2 + sx q4 + sy q5).
  auto dot = [&](int i, int j) { return U[i][0] * U[j][0] + U[i][1] * U[j][1] + U[i][2] * U[j][2]; };
  a.ray_q[0] = (float)dot(0, 0);
  a.ray_q[1] = (float)(2.0 * dot(0, 1));
  a.ray_q[2] = (float)(2.0 * dot(0, 2));
  a.ray_q[3] = (float)dot(1, 1);
  a.ray_q[4] = (float)(2.0 * dot(1, 2));
  a.ray_q[5] = (float)dot(2, 2);
}

// Rays a warp marches: 32 pixels x the directions of each thread.
static int rays_per_warp(int dirs, int split) { return kMarchTx * ((dirs + split - 1) / split); }

// Untuned shapes: 4 rows, or 8 for the texture-tap loop (at 1920x1080, R = 16 its
// recording march ran 1.8 % faster in 8-row CTAs and the two-bounce frame 0.8 %).
static TunedLayout tuned_layout(const MarchArgs& a) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tuned.find(key_of(a));
  const int rows = (a.fast && a.depth_tex) ? 8 : kMarchTy;
  return it == g_tuned.end() ? TunedLayout{rows, 1} : it->second;
}

int march_table_size(const MarchArgs& a) {
  int n_tab = max_steps(a.width, a.height, a.step_dirs);
  if (a.step_cap > 0 && a.step_cap < n_tab) n_tab = a.step_cap;
  return n_tab;
}

// Carveout of a march launch: the shared memory the kernel's register-limited
// occupancy needs (blocks x (static + dynamic + the 1 KB the CUDA driver reserves a
// block)), as a percentage of the SM's, so that the rest of the unified L1/shared
// storage stays L1.  The CUDA driver's default had sized the march's shared memory
// for 11 CTAs a SM where registers allow 6: the carveout alone made the recording
// march 1.9 % shorter, with the tables sized to the launch 3.4 % (replay 2.2 %).
// Given per launch (a launch attribute, part of a captured graph's kernel node), it
// changes no state of the kernel.
static unsigned carveout_pct(const void* kernel, dim3 block, int smem) {
  struct Attr {
    int regs, static_smem, per_sm;
  };
  static std::mutex mu;
  static std::map<const void*, Attr> attrs;  // kernel -> its registers and static shared memory
  Attr at{0, 0, 0};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = attrs.find(kernel);
    if (it == attrs.end()) {
      cudaFuncAttributes fa{};
      int dev = 0, per_sm = 0;
      if (cudaFuncGetAttributes(&fa, kernel) == cudaSuccess && cudaGetDevice(&dev) == cudaSuccess &&
          cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess)
        at = Attr{fa.numRegs, (int)fa.sharedSizeBytes, per_sm};
      else
        (void)cudaGetLastError();  // the query's own error: a hint, nothing to report
      attrs[kernel] = at;
    } else {
      at = it->second;
    }
  }
  if (at.regs <= 0 || at.per_sm <= 0) return 100;  // no figures: leave the choice to the driver's maximum
  const int threads = (int)(block.x * block.y * block.z);
  const int warp_regs = ((at.regs * 32 + 255) / 256) * 256;  // allocated per warp in units of 256
  const int blocks = 65536 / (warp_regs * ((threads + 31) / 32));
  const long long need = (long long)blocks * ((long long)at.static_smem + smem + 1024);
  const long long pct = (need * 100 + at.per_sm - 1) / at.per_sm + 1;
  return (unsigned)(pct > 100 ? 100 : pct);
}

// Launches a march kernel with its tables as dynamic shared memory (`smem` bytes)
// and its carveout; a failed launch is left for the caller's GI_CHECK_LAUNCH.
template <typename... P, typename... A>
static void launch_tables(void (*kernel)(P...), dim3 grid, dim3 block, int smem, cudaStream_t s, A&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePreferredSharedMemoryCarveout;
  attr[0].val.sharedMemCarveout = carveout_pct((const void*)kernel, block, smem);
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  (void)cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

// march_kernel over the standard form with 2-channel depth, by CTA height.
template <bool FAST, bool REC, bool TEX>
static void launch_standard(const MarchArgs& a, int rows, dim3 grid, int n_tab, int tiles_x, int total,
                            cudaStream_t s) {
  const int smem = march_smem_bytes(n_tab, a.dirs);
  if (rows == 2)
    launch_tables(march_kernel<2, false, 2, FAST, false, REC, TEX>, grid, dim3(kMarchTx, 2), smem, s, a, n_tab,
                  tiles_x, total);
  else if (rows == 8)
    launch_tables(march_kernel<2, false, 8, FAST, false, REC, TEX>, grid, dim3(kMarchTx, 8), smem, s, a, n_tab,
                  tiles_x, total);
  else
    launch_tables(march_kernel<2, false, 4, FAST, false, REC, TEX>, grid, dim3(kMarchTx, 4), smem, s, a, n_tab,
                  tiles_x, total);
}

template <bool FAST>
static void launch_replay(const MarchArgs& a, int rows, dim3 grid, int n_tab, int tiles_x, cudaStream_t s) {
  const int smem = 0;  // static tables (ReplaySmem)
  if (rows == 2) launch_tables(march_replay_kernel<2, FAST>, grid, dim3(kMarchTx, 2), smem, s, a, n_tab, tiles_x);
  else if (rows == 8) launch_tables(march_replay_kernel<8, FAST>, grid, dim3(kMarchTx, 8), smem, s, a, n_tab, tiles_x);
  else launch_tables(march_replay_kernel<4, FAST>, grid, dim3(kMarchTx, 4), smem, s, a, n_tab, tiles_x);
}

// Whether a march can take the direction-split form: the standard form with
// 2-channel moments, no record, kSplitMinDirs to kSplitMaxDirs directions.
static bool split_fits(const MarchArgs& a) {
  return !a.rec && !a.deinterleaved && a.depth_ch == 2 && !a.soft && a.dirs >= kSplitMinDirs &&
         a.dirs <= kSplitMaxDirs;
}

// Launches the march in the layout (rows, split): one thread per pixel in CTAs
// of `rows` = 2, 4 or 8 rows of 32 pixels, or split = kSplit, four threads per
// pixel (rows = 4), where split_fits allows it.  Tile lists always use the
// 4-row tile geometry of gi_march_tile_grid, and the direction-split form when
// they have at least 8 directions.
static int launch_march_rows(const MarchArgs& args, int rows, int split, cudaStream_t stream) {
  MarchArgs a = args;
  set_ray_basis(a);
  const int n_tab = march_table_size(a);
  if (n_tab > GI_MAX_STEPS) return fail(GI_ERR_UNSUPPORTED, "march: more steps per direction than GI_MAX_STEPS");
  const bool list_split = a.tiles && split_fits(a) && a.dirs >= 8;
  const bool frame_split = !a.tiles && split > 1 && split_fits(a);
  if (a.tiles || a.deinterleaved || a.depth_ch != 2 || a.soft || frame_split) rows = kMarchTy;
  const int P = a.pattern;
  const int sub_w = (a.width + P - 1) / P, sub_h = (a.height + P - 1) / P;
  const int tiles_x = (sub_w + kMarchTx - 1) / kMarchTx, tiles_y = (sub_h + rows - 1) / rows;
  const int n_tiles = a.tiles ? a.num_tiles : tiles_x * tiles_y;
  if (n_tiles == 0) return GI_OK;
  dim3 grid(n_tiles * P * P);
  const int total = tiles_x * tiles_y;
  const bool tex = a.depth_tex != 0;  // checked by the caller: fast standard form, both pyramids
  if (list_split || frame_split) {
    // The direction-split form (same result).
    grid.x *= kMarchTy;
    const dim3 block(kMarchTx, kSplit);
    const int smem = march_smem_bytes(n_tab, a.dirs);
    if (tex) launch_tables(march_split_kernel<true, true>, grid, block, smem, stream, a, n_tab, tiles_x, total);
    else if (a.fast) launch_tables(march_split_kernel<true, false>, grid, block, smem, stream, a, n_tab, tiles_x, total);
    else launch_tables(march_split_kernel<false, false>, grid, block, smem, stream, a, n_tab, tiles_x, total);
    GI_CHECK_LAUNCH("march_split_kernel");
    count_launches(1);
    return GI_OK;
  }
  if (a.rec) {  // record or replay: standard form, 2-channel moments, no tile list (checked by the caller)
    if (a.rec == 2) {
      if (n_tab > kRecMaxSteps) return fail(GI_ERR_INVALID_ARGUMENT, "march: replay of more steps than a record holds");
      // The replay re-lights with the fast loop's software light taps in the
      // texture precision too: its work is the light taps alone, and these loads
      // beat the four-channel trilinear fetch (measured, whole frame).
      if (a.fast) launch_replay<true>(a, rows, grid, n_tab, tiles_x, stream);
      else launch_replay<false>(a, rows, grid, n_tab, tiles_x, stream);
    } else if (tex) {
      launch_standard<true, true, true>(a, rows, grid, n_tab, tiles_x, total, stream);
    } else if (a.fast) {
      launch_standard<true, true, false>(a, rows, grid, n_tab, tiles_x, total, stream);
    } else {
      launch_standard<false, true, false>(a, rows, grid, n_tab, tiles_x, total, stream);
    }
    GI_CHECK_LAUNCH(a.rec == 2 ? "march_replay_kernel" : "march_kernel (recording)");
    count_launches(1);
    return GI_OK;
  }
  const int smem = march_smem_bytes(n_tab, a.dirs);
  const dim3 b4(kMarchTx, 4);
  if (a.soft) {  // exact contract, standard form, 2-channel moments (checked by the caller)
    launch_tables(march_kernel<2, false, 4, false, true>, grid, b4, smem, stream, a, n_tab, tiles_x, total);
  } else if (a.deinterleaved) {
    if (a.depth_ch == 2) launch_tables(march_kernel<2, true, 4, false>, grid, b4, smem, stream, a, n_tab, tiles_x, total);
    else launch_tables(march_kernel<1, true, 4, false>, grid, b4, smem, stream, a, n_tab, tiles_x, total);
  } else if (a.depth_ch != 2) {
    launch_tables(march_kernel<1, false, 4, false>, grid, b4, smem, stream, a, n_tab, tiles_x, total);
  } else if (tex) {
    launch_standard<true, false, true>(a, rows, grid, n_tab, tiles_x, total, stream);
  } else if (a.fast) {
    launch_standard<true, false, false>(a, rows, grid, n_tab, tiles_x, total, stream);
  } else {
    launch_standard<false, false, false>(a, rows, grid, n_tab, tiles_x, total, stream);
  }
  GI_CHECK_LAUNCH("march_kernel");
  count_launches(1);
  return GI_OK;
}

// Texture taps: the fast standard form, with both pyramids' textures.
static int check_textures(const MarchArgs& a, const char* what) {
  if (a.depth_tex == 0 && a.light_tex == 0) return GI_OK;
  if (!a.fast || a.soft || a.deinterleaved || a.depth_ch != 2)
    return fail(GI_ERR_INVALID_ARGUMENT, std::string(what) + ": texture taps need the fast standard form");
  if (a.depth_tex == 0 || a.light_tex == 0)
    return fail(GI_ERR_INVALID_ARGUMENT, std::string(what) + ": texture taps need both pyramids' textures");
  return GI_OK;
}

int launch_march(const MarchArgs& a, cudaStream_t stream) {
  if (int st = check_textures(a, "march")) return st;
  if (a.rec) {
    if (a.rec != 1 && a.rec != 2) return fail(GI_ERR_INVALID_ARGUMENT, "march: unknown record mode");
    if (a.tiles || a.deinterleaved || a.depth_ch != 2 || a.soft || !a.rec_hc || !a.rec_mask || !a.rec_hc0)
      return fail(GI_ERR_INVALID_ARGUMENT, "march: a record needs the standard form and its arrays");
    if (march_table_size(a) > a.rec_steps || a.rec_steps > 64)
      return fail(GI_ERR_INVALID_ARGUMENT, "march: record step stride");
    if (record_pixels(a) >= (1ull << 31) || (size_t)a.dirs * a.rec_steps >= (1ull << 31))
      return fail(GI_ERR_UNSUPPORTED, "march: record too large for 32-bit indices");
  }
  const TunedLayout t = tuned_layout(a);
  return launch_march_rows(a, t.rows, t.split, stream);
}

size_t march_record_bytes(const MarchArgs& a, size_t* hc_bytes, size_t* mask_bytes, size_t* hc0_bytes) {
  const int n_tab = march_table_size(a);
  if (n_tab > 64) return 0;
  const size_t npix = record_pixels(a), R = (size_t)a.dirs;
  *hc_bytes = R * (size_t)n_tab * npix * sizeof(float);
  *mask_bytes = R * npix * sizeof(unsigned long long);
  *hc0_bytes = R * npix * sizeof(float);
  return *hc_bytes + *mask_bytes + *hc0_bytes;
}

// Times each CTA height on the caller's inputs (one warm-up and three timed
// launches each, CUDA events on `stream`) and records the fastest for this
// march shape.
int autotune_march(const MarchArgs& a, cudaStream_t stream, int* best_rows, int* best_rays_per_warp,
                   float* best_ms) {
  // Layouts: one thread per pixel in CTAs of 2, 4 or 8 rows (a warp marches 32
  // pixels x R directions), and four threads per pixel (32 pixels x R/4).
  std::vector<TunedLayout> cand = {{2, 1}, {4, 1}, {8, 1}};
  if (split_fits(a) && !a.tiles) cand.push_back({kMarchTy, kSplit});
  float best = 1e30f;
  TunedLayout best_l{kMarchTy, 1};
  cudaEvent_t e0, e1;
  int st = check_cuda(cudaEventCreate(&e0), "autotune: event");
  if (st) return st;
  st = check_cuda(cudaEventCreate(&e1), "autotune: event");
  if (st) {
    cudaEventDestroy(e0);
    return st;
  }
  for (const TunedLayout& l : cand) {
    st = launch_march_rows(a, l.rows, l.split, stream);
    if (!st) st = check_cuda(cudaEventRecord(e0, stream), "autotune: record");
    for (int k = 0; k < 3 && !st; k++) st = launch_march_rows(a, l.rows, l.split, stream);
    if (!st) st = check_cuda(cudaEventRecord(e1, stream), "autotune: record");
    if (!st) st = check_cuda(cudaEventSynchronize(e1), "autotune: sync");
    float ms = 0.0f;
    if (!st) st = check_cuda(cudaEventElapsedTime(&ms, e0, e1), "autotune: elapsed");
    if (st) break;
    ms /= 3.0f;
    if (ms < best) {
      best = ms;
      best_l = l;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tuned[key_of(a)] = best_l;
  }
  if (best_rows) *best_rows = best_l.rows;
  if (best_rays_per_warp) *best_rays_per_warp = rays_per_warp(a.dirs, best_l.split);
  if (best_ms) *best_ms = best;
  return GI_OK;
}

int launch_march_batch(const BatchTable& views, const int2* items, int num_items, int* counter, int rows, int grid,
                       bool fast, bool tex, cudaStream_t stream) {
  if (num_items == 0) return GI_OK;
  if (tex && !fast) return fail(GI_ERR_INVALID_ARGUMENT, "march batch: texture depth taps need the fast precision");
  int st = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), stream), "march batch: counter reset");
  if (st) return st;
  const int ky = rows == 2 ? 2 : (rows == 8 ? 8 : 4);
  const dim3 block(kMarchTx, ky);
  int smem = 0;  // the largest view's tables (unused entries are zero)
  for (int v = 0; v < kBatchTableViews; v++) {
    const BatchView& bv = views.v[v];
    if (bv.n_tab < 0 || bv.n_tab > GI_MAX_STEPS || bv.a.dirs < 0 || bv.a.dirs > GI_MAX_DIRS)
      return fail(GI_ERR_INVALID_ARGUMENT, "march batch: view tables out of range");
    smem = std::max(smem, march_smem_bytes(bv.n_tab, bv.a.dirs));
  }
  auto go = [&](auto kernel) { launch_tables(kernel, dim3(grid), block, smem, stream, views, items, num_items, counter); };
  if (tex) {
    if (ky == 2) go(march_batch_kernel<2, true, true>);
    else if (ky == 8) go(march_batch_kernel<8, true, true>);
    else go(march_batch_kernel<4, true, true>);
  } else if (fast) {
    if (ky == 2) go(march_batch_kernel<2, true, false>);
    else if (ky == 8) go(march_batch_kernel<8, true, false>);
    else go(march_batch_kernel<4, true, false>);
  } else {
    if (ky == 2) go(march_batch_kernel<2, false, false>);
    else if (ky == 8) go(march_batch_kernel<8, false, false>);
    else go(march_batch_kernel<4, false, false>);
  }
  GI_CHECK_LAUNCH("march_batch_kernel");
  count_launches(1);
  return GI_OK;
}

int march_batch_occupancy(int rows, bool fast, bool tex) {
  int blocks = 0;
  const int ky = rows == 2 ? 2 : (rows == 8 ? 8 : 4);
  auto occ = [&](auto kernel) { cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, kMarchTx * ky, 0); };
  if (tex) {
    if (ky == 2) occ(march_batch_kernel<2, true, true>);
    else if (ky == 8) occ(march_batch_kernel<8, true, true>);
    else occ(march_batch_kernel<4, true, true>);
  } else if (fast) {
    if (ky == 2) occ(march_batch_kernel<2, true, false>);
    else if (ky == 8) occ(march_batch_kernel<8, true, false>);
    else occ(march_batch_kernel<4, true, false>);
  } else {
    if (ky == 2) occ(march_batch_kernel<2, false, false>);
    else if (ky == 8) occ(march_batch_kernel<8, false, false>);
    else occ(march_batch_kernel<4, false, false>);
  }
  return blocks > 0 ? blocks : 1;
}

static int fill_march(MarchArgs& a, const gi_view* view, const gi_march_params* p, const float* const* light,
                      const float* const* depth, int num_levels, const float* normal, const float* ndc, float* out) {
  GI_CHECK_ARG(view && p && light && depth && normal && ndc && out, "gi_march: null argument");
  GI_CHECK_ARG(view->width >= 1 && view->height >= 1, "gi_march: bad viewport");
  GI_CHECK_ARG(p->dirs >= 1 && p->dirs <= GI_MAX_DIRS, "gi_march: dirs out of range");
  GI_CHECK_ARG(p->step_cap >= 0, "gi_march: negative step cap");
  GI_CHECK_ARG(p->step_dirs >= 0 && p->step_dirs <= 4096, "gi_march: step_dirs out of range");
  GI_CHECK_ARG(p->pattern_size >= 1 && p->pattern_size <= 8, "gi_march: pattern size out of range");
  GI_CHECK_ARG(p->precision == GI_MARCH_EXACT || p->precision == GI_MARCH_FAST || p->precision == GI_MARCH_TEXTURE,
               "gi_march: unknown precision");
  GI_CHECK_ARG(p->occlusion == GI_OCCLUSION_HARD || p->occlusion == GI_OCCLUSION_SOFT, "gi_march: unknown occlusion");
  GI_CHECK_ARG(num_levels >= 1 && num_levels <= gi_mip_level_count(view->width, view->height, GI_MAX_LEVELS),
               "gi_march: bad level count");
  GI_CHECK_ARG(aligned16(normal) && aligned16(out), "gi_march: unaligned buffer");
  for (int k = 0; k < num_levels; k++) {
    GI_CHECK_ARG(light[k] && depth[k] && aligned16(light[k]) && aligned16(depth[k]),
                 "gi_march: null or unaligned pyramid level");
    a.light[k] = light[k];
    a.depth[k] = depth[k];
  }
  for (int k = 0; k < 16; k++) {
    a.inv_view_proj.m[k] = view->inv_view_proj[k];
    a.inv_view.m[k] = view->inv_view[k];
  }
  a.normal = normal;
  a.ndc = ndc;
  a.out = out;
  a.width = view->width;
  a.height = view->height;
  a.num_levels = num_levels;
  a.depth_ch = 2;
  a.dirs = p->dirs;
  a.step_cap = p->step_cap;
  a.pattern = p->pattern_size;
  a.step_dirs = p->step_dirs > 0 ? p->step_dirs : p->dirs;
  a.soft = p->occlusion == GI_OCCLUSION_SOFT ? 1 : 0;
  a.fast = (p->precision != GI_MARCH_EXACT && !a.soft) ? 1 : 0;  // the soft horizon runs in the exact contract
  return GI_OK;
}

// GI_MARCH_TEXTURE through the entry points that take caller-owned pyramids: the
// pyramids are copied into library-owned textures (one pair per device, kept for
// the last shape) before `run` launches on `stream`.  Calls are serialised on the
// host by a mutex and on the device by an event: a call on another stream waits
// for the previous call's launches before it overwrites the textures.
//
// Stream capture.  A call under capture bakes the pair's texture handles into
// the caller's graph, so from then on the pair is never freed: a later call of
// another shape retires it (kept until the process exits) and makes a new pair,
// and a replay of the old graph still reads valid objects.  Making a pair
// allocates device memory, which a capture forbids, so a captured call whose
// shape differs from the pair's returns GI_ERR_UNSUPPORTED (an eager call of that
// shape before the capture makes the pair).  A pair that no graph has seen is
// freed after the previous call's launches finish (an event wait; no device-wide
// synchronisation).
struct TexturePair {
  int w = 0, h = 0, levels = 0;
  bool captured = false;  // a captured graph may hold its handles
  PyramidTexture depth, light;
};
struct MarchTextureCache {
  std::mutex m;
  TexturePair* cur = nullptr;
  std::vector<TexturePair*> retired;  // pairs a graph may still read: never freed
  cudaEvent_t done = nullptr;
};
constexpr int kMaxCacheDevices = 64;
// Never destroyed: the process's exit releases the device objects.
static MarchTextureCache& march_texture_cache(int dev) {
  static MarchTextureCache* c = new MarchTextureCache[kMaxCacheDevices];
  return c[dev];
}

template <class Run>
static int with_march_textures(MarchArgs& a, const float* const* light, const float* const* depth,
                               cudaStream_t stream, Run run) {
  if (a.soft) return fail(GI_ERR_UNSUPPORTED, "gi_march: the soft horizon runs in the exact contract");
  int dev = 0;
  int st = check_cuda(cudaGetDevice(&dev), "gi_march: device");
  if (st) return st;
  if (dev < 0 || dev >= kMaxCacheDevices)
    return fail(GI_ERR_UNSUPPORTED, "gi_march: GI_MARCH_TEXTURE on a device index above 63");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  st = check_cuda(cudaStreamIsCapturing(stream, &cs), "gi_march: capture status");
  if (st) return st;
  const bool capturing = cs != cudaStreamCaptureStatusNone;
  MarchTextureCache& c = march_texture_cache(dev);
  std::lock_guard<std::mutex> lock(c.m);
  TexturePair* p = c.cur;
  if (!p || p->w != a.width || p->h != a.height || p->levels != a.num_levels) {
    if (capturing)
      return fail(GI_ERR_UNSUPPORTED,
                  "gi_march: GI_MARCH_TEXTURE under stream capture needs an earlier eager call of the same shape "
                  "(the library's pyramid textures are made outside the capture)");
    if (p) {
      if (p->captured) {
        c.retired.push_back(p);
      } else {
        if (c.done) {
          st = check_cuda(cudaEventSynchronize(c.done), "gi_march: texture order");
          if (st) return st;
        }
        p->depth.Destroy(false);  // the event wait above ordered every launch that read them
        p->light.Destroy(false);
        delete p;
      }
      c.cur = nullptr;
    }
    p = new TexturePair;
    st = p->depth.Create(a.width, a.height, a.num_levels, 1);
    st = st ? st : p->light.Create(a.width, a.height, a.num_levels, 4);
    if (st) {
      delete p;
      return st;
    }
    p->w = a.width;
    p->h = a.height;
    p->levels = a.num_levels;
    c.cur = p;
  }
  // Under stream capture the call joins no event outside the graph: the graph's
  // own order (one stream) is the caller's to keep.
  if (!c.done) {
    if (capturing)
      return fail(GI_ERR_UNSUPPORTED, "gi_march: GI_MARCH_TEXTURE under stream capture needs an earlier eager call");
    st = check_cuda(cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming), "gi_march: texture event");
    if (st) return st;
  } else if (!capturing) {
    st = check_cuda(cudaStreamWaitEvent(stream, c.done, 0), "gi_march: texture order");
    if (st) return st;
  }
  if (capturing) p->captured = true;
  st = p->depth.Pack(depth, a.depth_ch, stream);
  st = st ? st : p->light.Pack(light, 4, stream);
  if (st) return st;
  a.depth_tex = p->depth.Handle();
  a.light_tex = p->light.Handle();
  st = run(a);
  if (!st && !capturing) st = check_cuda(cudaEventRecord(c.done, stream), "gi_march: texture order");
  return st;
}

}  // namespace gi

using namespace gi;

extern "C" int gi_march(const gi_view* view, const gi_march_params* params, const float* const* light_levels,
                        const float* const* depth_levels, int num_levels, const float* normal, const float* ndc_depth,
                        float* out, void* stream) {
  MarchArgs a{};
  int st = fill_march(a, view, params, light_levels, depth_levels, num_levels, normal, ndc_depth, out);
  if (st) return st;
  a.deinterleaved = 0;
  if (params->precision == GI_MARCH_TEXTURE)
    return with_march_textures(a, light_levels, depth_levels, (cudaStream_t)stream,
                               [&](MarchArgs& m) { return launch_march(m, (cudaStream_t)stream); });
  return launch_march(a, (cudaStream_t)stream);
}

extern "C" int gi_march_tile_grid(int width, int height, int pattern_size, int* tiles_x, int* tiles_y, int* tile_w,
                                  int* tile_h) {
  GI_CHECK_ARG(width >= 1 && height >= 1 && pattern_size >= 1 && pattern_size <= 8 && tiles_x && tiles_y &&
                   tile_w && tile_h,
               "gi_march_tile_grid: bad arguments");
  const int sub_w = (width + pattern_size - 1) / pattern_size, sub_h = (height + pattern_size - 1) / pattern_size;
  *tiles_x = (sub_w + kMarchTx - 1) / kMarchTx;
  *tiles_y = (sub_h + kMarchTy - 1) / kMarchTy;
  *tile_w = kMarchTx * pattern_size;
  *tile_h = kMarchTy * pattern_size;
  return GI_OK;
}

extern "C" int gi_march_tiles(const gi_view* view, const gi_march_params* params, const float* const* light_levels,
                              const float* const* depth_levels, int num_levels, const float* normal,
                              const float* ndc_depth, float* out, const int* tiles, int num_tiles, void* stream) {
  MarchArgs a{};
  int st = fill_march(a, view, params, light_levels, depth_levels, num_levels, normal, ndc_depth, out);
  if (st) return st;
  GI_CHECK_ARG(tiles && num_tiles >= 0, "gi_march_tiles: null tile list");
  a.deinterleaved = 0;
  a.tiles = tiles;
  a.num_tiles = num_tiles;
  if (params->precision == GI_MARCH_TEXTURE)
    return with_march_textures(a, light_levels, depth_levels, (cudaStream_t)stream,
                               [&](MarchArgs& m) { return launch_march(m, (cudaStream_t)stream); });
  return launch_march(a, (cudaStream_t)stream);
}

extern "C" int gi_march_deinterleaved(const gi_view* view, const gi_march_params* params,
                                      const float* const* light_levels, const float* const* depth_levels,
                                      int num_levels, const float* normal_d, const float* ndc_depth_d, float* out_d,
                                      void* stream) {
  MarchArgs a{};
  int st = fill_march(a, view, params, light_levels, depth_levels, num_levels, normal_d, ndc_depth_d, out_d);
  if (st) return st;
  GI_CHECK_ARG(view->width % params->pattern_size == 0 && view->height % params->pattern_size == 0,
               "gi_march_deinterleaved: viewport must be a multiple of the pattern");
  if (a.soft) return fail(GI_ERR_UNSUPPORTED, "gi_march_deinterleaved: the soft horizon needs the standard form");
  if (params->precision == GI_MARCH_TEXTURE)
    return fail(GI_ERR_UNSUPPORTED, "gi_march_deinterleaved: GI_MARCH_TEXTURE needs the standard form");
  a.deinterleaved = 1;
  return launch_march(a, (cudaStream_t)stream);
}

extern "C" int gi_march_autotune(const gi_view* view, const gi_march_params* params, const float* const* light_levels,
                                 const float* const* depth_levels, int num_levels, const float* normal,
                                 const float* ndc_depth, float* out, int* best_rows, int* best_rays_per_warp,
                                 float* best_ms, void* stream) {
  MarchArgs a{};
  int st = fill_march(a, view, params, light_levels, depth_levels, num_levels, normal, ndc_depth, out);
  if (st) return st;
  if (params->precision == GI_MARCH_TEXTURE)
    return with_march_textures(a, light_levels, depth_levels, (cudaStream_t)stream, [&](MarchArgs& m) {
      return autotune_march(m, (cudaStream_t)stream, best_rows, best_rays_per_warp, best_ms);
    });
  return autotune_march(a, (cudaStream_t)stream, best_rows, best_rays_per_warp, best_ms);
}

// The tuned layout of a march shape, looked up as the march looks it up.
static bool tuned_lookup(int width, int height, int dirs, int step_dirs, int step_cap, int precision,
                         TunedLayout* out) {
  MarchArgs a{};
  a.width = width;
  a.height = height;
  a.dirs = dirs;
  a.step_dirs = step_dirs > 0 ? step_dirs : dirs;
  a.step_cap = step_cap;
  a.fast = precision != GI_MARCH_EXACT ? 1 : 0;
  a.depth_tex = precision == GI_MARCH_TEXTURE ? 1 : 0;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tuned.find(key_of(a));
  if (it == g_tuned.end()) return false;
  *out = it->second;
  return true;
}

extern "C" int gi_march_set_layout(int width, int height, int dirs, int step_dirs, int step_cap, int precision,
                                   int rows, int rays_per_warp_in) {
  GI_CHECK_ARG(width >= 1 && height >= 1 && dirs >= 1, "gi_march_set_layout: bad shape");
  GI_CHECK_ARG(precision >= GI_MARCH_EXACT && precision <= GI_MARCH_TEXTURE, "gi_march_set_layout: bad precision");
  MarchArgs a{};
  a.width = width;
  a.height = height;
  a.dirs = dirs;
  a.step_dirs = step_dirs > 0 ? step_dirs : dirs;
  a.step_cap = step_cap;
  a.fast = precision != GI_MARCH_EXACT ? 1 : 0;
  a.depth_tex = precision == GI_MARCH_TEXTURE ? 1 : 0;
  a.depth_ch = 2;
  TunedLayout l{};
  if (rays_per_warp_in == rays_per_warp(dirs, 1)) {
    GI_CHECK_ARG(rows == 2 || rows == 4 || rows == 8, "gi_march_set_layout: rows must be 2, 4 or 8");
    l = TunedLayout{rows, 1};
  } else if (rays_per_warp_in == rays_per_warp(dirs, kSplit)) {
    GI_CHECK_ARG(rows == kMarchTy, "gi_march_set_layout: the direction split has 4 rows");
    GI_CHECK_ARG(split_fits(a), "gi_march_set_layout: the direction split needs 4 to 32 directions");
    l = TunedLayout{kMarchTy, kSplit};
  } else {
    return fail(GI_ERR_INVALID_ARGUMENT, "gi_march_set_layout: rays per warp must be 32 x dirs or 32 x ceil(dirs / 4)");
  }
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tuned[key_of(a)] = l;
  return GI_OK;
}

extern "C" int gi_march_tuned_rows(int width, int height, int dirs, int step_dirs, int step_cap) {
  TunedLayout l{};
  return tuned_lookup(width, height, dirs, step_dirs, step_cap, GI_MARCH_EXACT, &l) ? l.rows : 0;
}

extern "C" int gi_march_tuned_layout(int width, int height, int dirs, int step_dirs, int step_cap, int precision,
                                     int* rows, int* rays_per_warp_out) {
  GI_CHECK_ARG(rows && rays_per_warp_out, "gi_march_tuned_layout: null argument");
  GI_CHECK_ARG(precision >= GI_MARCH_EXACT && precision <= GI_MARCH_TEXTURE, "gi_march_tuned_layout: bad precision");
  TunedLayout l{};
  if (!tuned_lookup(width, height, dirs, step_dirs, step_cap, precision, &l)) {
    *rows = 0;
    *rays_per_warp_out = 0;
    return GI_OK;
  }
  *rows = l.rows;
  *rays_per_warp_out = rays_per_warp(dirs, l.split);
  return GI_OK;
}

extern "C" int gi_texture_sample(const float* const* levels, int width, int height, int num_levels, int channels,
                                 int src_channels, const float* coords, const float* lods, int n, float* out,
                                 void* stream) {
  GI_CHECK_ARG(levels && coords && lods && out && n >= 0, "gi_texture_sample: null argument");
  GI_CHECK_ARG(channels == 1 || channels == 4, "gi_texture_sample: channels must be 1 or 4");
  GI_CHECK_ARG(src_channels >= channels && src_channels <= 4, "gi_texture_sample: bad source channel count");
  if (n == 0) return GI_OK;
  cudaStream_t s = (cudaStream_t)stream;
  PyramidTexture t;
  int st = t.Create(width, height, num_levels, channels);
  if (st) return st;
  st = t.Pack(levels, src_channels, s);
  if (st) return st;
  const int blocks = (n + 255) / 256;
  if (channels == 1) texture_sample_kernel<1><<<blocks, 256, 0, s>>>(t.Handle(), coords, lods, out, n);
  else texture_sample_kernel<4><<<blocks, 256, 0, s>>>(t.Handle(), coords, lods, out, n);
  GI_CHECK_LAUNCH("texture_sample_kernel");
  count_launches(1);
  st = check_cuda(cudaStreamSynchronize(s), "gi_texture_sample: sync");
  t.Destroy(false);  // the stream's launches are done
  return st;
}
