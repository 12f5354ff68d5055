// ref_runner.cpp -- runs the reference's fragment shaders, compiled as C++ by
// oracle/build_ref.py, once per pixel over fp32 images (test infrastructure).
//
// Each entry point binds images and uniforms the way the reference's pass does
// (the pass named beside it), sets gl_FragCoord to the pixel centre and the
// screen-quad varying to (pixel + 0.5) / viewport, calls the shader's main() and
// stores its output.  Images are fp32, row-major, channels interleaved; pyramids
// are their levels packed one after another (level k of size (w >> k) x (h >> k)).
// Matrices are column-major float[16], as glm and the library store them.
#include <omp.h>

#include "ref_shim.h"

namespace refglsl {

static int g_ref_dirs = 4;  // REF_DIRS of IndirectLightingDirs
#define REF_DIRS g_ref_dirs

#include "MipLevelBuilder.inc"
#include "BlurLayerBuilder.inc"
#include "Deinterleave.inc"
#include "Interleave.inc"
#include "IndirectLighting.inc"
#include "IndirectLightingDirs.inc"
#include "FinalGatherer.inc"
#include "DirectLighting.inc"
#include "Denoiser.inc"

static oracle::Pyr<float> pyramid(const float* base, int w, int h, int ch, int n) {
  oracle::Pyr<float> p;
  p.n = n;
  size_t off = 0;
  for (int k = 0; k < n; k++) {
    p.lv[k] = oracle::Img<float>(base + off, w, h, ch);
    off += (size_t)w * h * ch;
    w = w / 2 > 0 ? w / 2 : 1;
    h = h / 2 > 0 ? h / 2 : 1;
  }
  return p;
}
static sampler2D image(const float* p, int w, int h, int ch) {
  sampler2D s;
  s.pyr = pyramid(p, w, h, ch, 1);
  return s;
}
static mat4 load(const float* m) { return make_mat4(m); }
static void store(const vec4& v, float* dst, int ch) {
  for (int c = 0; c < ch; c++) dst[c] = v[c];
}
static void frag(FragmentShader& s, int x, int y) {
  s.gl_FragCoord.x = (float)x + 0.5f;
  s.gl_FragCoord.y = (float)y + 0.5f;
  s.gl_FragCoord.xy = vec2(s.gl_FragCoord.x, s.gl_FragCoord.y);
}
static vec2 quad(int x, int y, int w, int h) { return vec2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h); }

}  // namespace refglsl

using namespace refglsl;

extern "C" {

int ref_threads(void) { return omp_get_max_threads(); }

// inverse() of the shaders in double (1) or glm's float (0); see ref_shim.h.
void ref_set_inverse_in_double(int on) { g_inverse_in_double = on != 0; }

// MipBuilder::BuildMips, one level (MipBuilder.h:155-179): filter 0 average, 1 "Depth".
void ref_mip_level(const float* src, int sw, int sh, int ch, float* dst, int dw, int dh, int filter) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < dh; y++) {
    MipLevelBuilder s;
    s.filterType = (float)filter;
    s.prevLevelSampler = image(src, sw, sh, ch);
    for (int x = 0; x < dw; x++) {
      frag(s, x, y);
      s.fragScreenCoord = quad(x, y, dw, dh);
      s.main();
      store(s.outColor, dst + ((size_t)y * dw + x) * ch, ch);
    }
  }
}

// BlurBuilder::ApplyBlur (BlurBuilder.h:20-45): UBO {size, radius}.
void ref_blur(const float* src, float* dst, int w, int h, int ch, int radius) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++) {
    BlurLayerBuilder s;
    s.size = ivec4(w, h, 0, 0);
    s.radius = radius;
    s.srcSampler = image(src, w, h, ch);
    for (int x = 0; x < w; x++) {
      frag(s, x, y);
      s.fragScreenCoord = quad(x, y, w, h);
      s.main();
      store(s.outColor, dst + ((size_t)y * w + x) * ch, ch);
    }
  }
}

// InterleaveBuilder::Deinterleave / ::Interleave (InterleaveBuilder.h:14-80),
// each with its own shader (the reference's Interleave binds the deinterleave
// program by mistake, :60-62; the intended interleave.frag runs here).
void ref_permute(const float* src, float* dst, int w, int h, int ch, int gx, int gy, int inverse) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++) {
    Deinterleave d;
    Interleave i;
    d.gridSize = i.gridSize = ivec4(gx, gy, 0, 0);
    d.viewportSize = i.viewportSize = ivec4(w, h, 0, 0);
    d.interleavedSampler = image(src, w, h, ch);
    i.deinterleavedSampler = image(src, w, h, ch);
    for (int x = 0; x < w; x++) {
      vec4 r;
      if (inverse) {
        frag(i, x, y);
        i.fragScreenCoord = quad(x, y, w, h);
        i.main();
        r = i.resColor;
      } else {
        frag(d, x, y);
        d.fragScreenCoord = quad(x, y, w, h);
        d.main();
        r = d.resColor;
      }
      store(r, dst + ((size_t)y * w + x) * ch, ch);
    }
  }
}

// The indirect pass (SSVGIRenderer.h:224-263): UBO {view, proj, viewportSize},
// samplers blurredDirectLight (4 ch pyramid), blurredDepthMoments (2 ch pyramid),
// normal (4 ch), depthStencil (1 ch).  dirs 0 runs the shader as written
// (dirsCount = 4); dirs > 0 runs it with that dirsCount.  pix: optional (x, y)
// pairs; trace: optional 3 per pixel (count, sum and sum of squares of level + 1
// of the depth-moment taps' first mip level).
void ref_indirect(const float* view, const float* proj, int w, int h, int dirs, const float* light,
                  const float* depth, int nlev, const float* normal, const float* ndc, const int* pix, int npix,
                  float* out, long long* trace) {
  const long n = pix ? npix : (long)w * h;
  if (dirs > 0) g_ref_dirs = dirs;
#pragma omp parallel
  {
    IndirectLighting a;
    IndirectLightingDirs b;
    LodTrace tr;
    a.viewMatrix = b.viewMatrix = load(view);
    a.projMatrix = b.projMatrix = load(proj);
    a.viewportSize = b.viewportSize = vec4((float)w, (float)h, 0.0f, 0.0f);
    a.blurredDirectLightSampler.pyr = b.blurredDirectLightSampler.pyr = pyramid(light, w, h, 4, nlev);
    a.blurredDepthMomentsSampler.pyr = b.blurredDepthMomentsSampler.pyr = pyramid(depth, w, h, 2, nlev);
    a.normalSampler = b.normalSampler = image(normal, w, h, 4);
    a.depthStencilSampler = b.depthStencilSampler = image(ndc, w, h, 1);
    a.blurredDepthMomentsSampler.trace = b.blurredDepthMomentsSampler.trace = trace ? &tr : nullptr;
#pragma omp for schedule(dynamic, 64)
    for (long i = 0; i < n; i++) {
      const int x = pix ? pix[2 * i] : (int)(i % w), y = pix ? pix[2 * i + 1] : (int)(i / w);
      tr = LodTrace();
      vec4 r;
      if (dirs > 0) {
        frag(b, x, y);
        b.fragScreenCoord = quad(x, y, w, h);
        b.main();
        r = b.indirectLight;
      } else {
        frag(a, x, y);
        a.fragScreenCoord = quad(x, y, w, h);
        a.main();
        r = a.indirectLight;
      }
      store(r, out + (size_t)i * 4, 4);
      if (trace) {
        trace[3 * i] = tr.count;
        trace[3 * i + 1] = tr.sum;
        trace[3 * i + 2] = tr.sum2;
      }
    }
  }
}

// The gathering pass (SSVGIRenderer.h:305-342): direct, blurred direct (pyramid),
// albedo, (denoised) indirect light, all 4 ch.
void ref_final_gather(const float* direct, const float* blurred, int nlev, const float* albedo,
                      const float* indirect, int w, int h, float* out) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++) {
    FinalGatherer s;
    s.directLightSampler = image(direct, w, h, 4);
    s.blurredDirectLightSampler.pyr = pyramid(blurred, w, h, 4, nlev);
    s.albedoSampler = image(albedo, w, h, 4);
    s.indirectLightSampler = image(indirect, w, h, 4);
    for (int x = 0; x < w; x++) {
      frag(s, x, y);
      s.fragScreenCoord = quad(x, y, w, h);
      s.main();
      store(s.outColor, out + ((size_t)y * w + x) * 4, 4);
    }
  }
}

// The direct-lighting pass (SSVGIRenderer.h:161-205): albedo, emissive, normal
// (4 ch), hardware depth (1 ch), shadow map (1 ch, sw x sh) with a compare sampler.
void ref_direct(const float* view, const float* proj, const float* light_view, const float* light_proj,
                const float* albedo, const float* emissive, const float* normal, const float* ndc, const float* shadow,
                int sw, int sh, int w, int h, float* out) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++) {
    DirectLighting s;
    s.viewMatrix = load(view);
    s.projMatrix = load(proj);
    s.lightViewMatrix = load(light_view);
    s.lightProjMatrix = load(light_proj);
    s.time = 0.0f;
    s.albedoSampler = image(albedo, w, h, 4);
    s.emissiveSampler = image(emissive, w, h, 4);
    s.normalSampler = image(normal, w, h, 4);
    s.depthStencilSampler = image(ndc, w, h, 1);
    s.shadowmapSampler.img = oracle::Img<float>(shadow, sw, sh, 1);
    for (int x = 0; x < w; x++) {
      frag(s, x, y);
      s.fragScreenCoord = quad(x, y, w, h);
      s.main();
      store(s.outColor, out + ((size_t)y * w + x) * 4, 4);
    }
  }
}

// The denoiser pass (SSVGIRenderer.h:266-302): depthStencilSampler bound to the
// depth moments (2 ch), normal (4 ch), noisy indirect light (4 ch).
void ref_denoise(const float* view, const float* proj, const float* noisy, const float* moments, const float* normal,
                 int w, int h, int radius, float* out) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++) {
    Denoiser s;
    s.viewMatrix = load(view);
    s.projMatrix = load(proj);
    s.viewportSize = vec4((float)w, (float)h, 0.0f, 0.0f);
    s.radius = radius;
    s.noisySampler = image(noisy, w, h, 4);
    s.normalSampler = image(normal, w, h, 4);
    s.depthStencilSampler = image(moments, w, h, 2);
    for (int x = 0; x < w; x++) {
      frag(s, x, y);
      s.fragScreenCoord = quad(x, y, w, h);
      s.main();
      store(s.resColor, out + ((size_t)y * w + x) * 4, 4);
    }
  }
}

// The view and projection the reference's renderer builds with glm:
// view = inverse(Camera::GetTransformMatrix()) (Scene.h:30-33, SSVGIRenderer.h:54),
// proj = perspective(fovy, aspect, znear, zfar) * scale(1, -1, -1) (SSVGIRenderer.h:57),
// with main.cpp's GLM_FORCE_RADIANS and the [0, 1] depth range.
void ref_camera_matrices(const float* pos, float hor_angle, float vert_angle, float fovy, float aspect,
                         float znear, float zfar, float* view16, float* proj16) {
  const mat4 xf = glm::translate(glm::vec3(pos[0], pos[1], pos[2])) *
                  glm::rotate(hor_angle, glm::vec3(0.0f, 1.0f, 0.0f)) *
                  glm::rotate(vert_angle, glm::vec3(1.0f, 0.0f, 0.0f));
  const mat4 v = glm::inverse(xf);
  const mat4 p = glm::perspective(fovy, aspect, znear, zfar) * glm::scale(glm::vec3(1.0f, -1.0f, -1.0f));
  const float* a = glm::value_ptr(v);
  const float* b = glm::value_ptr(p);
  for (int k = 0; k < 16; k++) {
    view16[k] = a[k];
    proj16[k] = b[k];
  }
}

// The matrices the indirect pass's shader derives per pixel from its uniforms
// (indirectLighting.frag:123-126): inverse(proj * view) and inverse(view), with
// the current inverse() mode.
void ref_shader_inverses(const float* view16, const float* proj16, float* inv_view_proj16, float* inv_view16) {
  const mat4 v = load(view16), p = load(proj16);
  const mat4 ivp = refglsl::inverse(p * v), iv = refglsl::inverse(v);
  const float* a = glm::value_ptr(ivp);
  const float* b = glm::value_ptr(iv);
  for (int k = 0; k < 16; k++) {
    inv_view_proj16[k] = a[k];
    inv_view16[k] = b[k];
  }
}

}  // extern "C"
