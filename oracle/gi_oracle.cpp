// gi_oracle.cpp -- CPU restatement of LegitEngine's screen-space GI path.
//
// TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path: the
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the
// shipped library (legitengine_gb300) never links or calls it.
//
// Every pass is restated from the reference's GLSL (paths relative to
// bin/data/Shaders/glsl/) and host code (paths relative to src/), templated on
// the element type: float gives the FP32 parity oracle, double the FP64 error
// reference.  Evaluation order and the sampler arithmetic follow the contract
// written at the top of glsl.h and sampler.h.
//
// PARITY UNPINNED: the reference ships no tests, golden images or fixtures, and
// its Vulkan host (dependencies/LegitVulkan, an empty submodule) cannot be built
// or run, so no reference-produced output exists to check this restatement
// against.  It is pinned only by known-answer tables derived from the
// reference's formulas (tests/test_oracle_kat.py).
#include <omp.h>

#include <array>
#include <random>

#include <cstdio>
#include <cstring>
#include <limits>
#include <vector>

#include "../include/legit_gi.h"
#include "sampler.h"

namespace oracle {

template <typename T> static mat4<T> load_mat(const float* m) {
  mat4<T> r;
  for (int j = 0; j < 4; j++) r.c[j] = vec4<T>(T(m[4 * j + 0]), T(m[4 * j + 1]), T(m[4 * j + 2]), T(m[4 * j + 3]));
  return r;
}

template <typename T> static T gmin(T a, T b) { return b < a ? b : a; }  // GLSL min
template <typename T> static T gmax(T a, T b) { return a < b ? b : a; }  // GLSL max

// indirectLighting.frag:20-25 (also Common/projection.decl:2-7).
template <typename T> static vec3<T> Unproject(vec3<T> sp, const mat4<T>& inv) {
  vec4<T> vp = inv * vec4<T>(sp.x * T(2) - T(1), sp.y * T(2) - T(1), sp.z, T(1));
  T w = vp.w;
  return vec3<T>(gdiv(vp.x, w), gdiv(vp.y, w), gdiv(vp.z, w));
}

// indirectLighting.frag:27-34.
template <typename T> static vec3<T> Project(vec3<T> p, const mat4<T>& m) {
  vec4<T> n = m * vec4<T>(p, T(1));
  T w = n.w;
  n.x = gdiv(n.x, w);
  n.y = gdiv(n.y, w);
  n.z = gdiv(n.z, w);
  return vec3<T>(n.x * T(0.5) + T(0.5), n.y * T(0.5) + T(0.5), n.z);
}

// indirectLighting.frag:44-49.
template <typename T>
static T HorizonContribution(vec3<T> ed, vec3<T> et, vec3<T> n, T mn, T mx) {
  using M = Math<T>;
  T t1 = T(0.25) * dot(ed, n) * (-M::cos(T(2) * mx) + M::cos(T(2) * mn));
  T t2 = T(0.25) * dot(et, n) * (T(2) * mx - T(2) * mn - M::sin(T(2) * mx) + M::sin(T(2) * mn));
  return t1 + t2;
}

// indirectLighting.frag:83-99.
template <typename T>
static void BoxRayCast(vec2<T> s, vec2<T> d, vec2<T> bmin, vec2<T> bmax, T& pmin, T& pmax) {
  vec2<T> inv(gdiv(T(1), d.x), gdiv(T(1), d.y));
  T t1 = (bmin.x - s.x) * inv.x;
  T t2 = (bmax.x - s.x) * inv.x;
  T t3 = (bmin.y - s.y) * inv.y;
  T t4 = (bmax.y - s.y) * inv.y;
  pmin = gmax(gmin(t1, t2), gmin(t3, t4));
  pmax = gmin(gmax(t1, t2), gmax(t3, t4));
}

// indirectLighting.frag:102-112.
template <typename T> static vec2<T> HammersleyNorm(int i, int N) {
  uint32_t b = ((uint32_t)i << 16u) | ((uint32_t)i >> 16u);
  b = ((b & 0x55555555u) << 1u) | ((b & 0xAAAAAAAAu) >> 1u);
  b = ((b & 0x33333333u) << 2u) | ((b & 0xCCCCCCCCu) >> 2u);
  b = ((b & 0x0F0F0F0Fu) << 4u) | ((b & 0xF0F0F0F0u) >> 4u);
  b = ((b & 0x00FF00FFu) << 8u) | ((b & 0xFF00FF00u) >> 8u);
  return vec2<T>(gdiv(T(i), T(N)), gdiv(T(b), T(0xffffffffu)));
}

// indirectLighting.frag:201-212: steps of one direction, from the screen-space
// path to the viewport edge; capped at `cap` when cap > 0.
template <typename T>
static int IterationsCount(vec2<T> cpc, vec2<T> dir, vec2<T> vp, T nearStepSize, T pi, int dirsCount, int cap) {
  using M = Math<T>;
  T tmin, tmax;
  BoxRayCast(cpc, dir, vec2<T>(T(0), T(0)), vp, tmin, tmax);
  T totalPixelPath = std::abs(tmax);
  int iterationsCount =
      int(gdiv(M::log(gdiv(totalPixelPath, nearStepSize)), M::log(gdiv(T(2) * pi, T(dirsCount)) + T(1)))) + 1;
  if (cap > 0 && iterationsCount > cap) iterationsCount = cap;
  return iterationsCount;
}

template <typename T> struct MarchIn {
  int W = 0, H = 0;
  mat4<T> invVP, invView;
  Pyr<T> light, depth;  // blurred direct light (4 ch), blurred depth moments (2 ch)
  Img<T> normal, ndc;   // A7: full-resolution; A7': deinterleaved
  int R = 4, cap = 0, P = 4;
  int stepR = 0;  // direction count of the step/mip formulas; 0 = R
  int soft = 0;   // depth-variance (soft-occlusion) horizon update
  // Step taps through the texture units' fixed point (texture_lod_unit):
  // bit 0 the depth tap, bit 1 the light tap.  0: the exact sampler.
  int tex = 0;
};

// Soft-occlusion horizon (no counterpart in the reference's live code): the
// angle a step lowers the horizon to when the sample's depth is a distribution.
// The depth spread of the footprint is var = E[d^2] - E[d]^2 of the trilinear
// moments tap; GetAngularDistribution (indirectLighting.frag:51-81) turns it
// into an angular spread sigma = sqrt(var) |dtheta/dd| with the forward
// difference of eps = 0.1 along the sample's view ray (the angle taken in the
// march's own atan2(tangent, depth) form).  With theta ~ N(angle, sigma^2) the
// horizon drops by the expected positive part of (maxAngle - theta):
// (maxAngle - angle) Phi(z) + sigma phi(z), z = (maxAngle - angle) / sigma,
// phi the standard normal density and Phi its logistic approximation
// 1 / (1 + exp(-1.702 z)).  sigma <= 1e-6 keeps the hard update.
template <typename T>
static T SoftHorizon(vec4<T> depthSample, vec3<T> rayDir, vec3<T> camWorldPos, vec3<T> centerWorldPos,
                     vec3<T> eyeWorldDir, vec3<T> eyeWorldTangent, T angle, T maxAngle) {
  using M = Math<T>;
  T var = gmax(T(0), depthSample.y - depthSample.x * depthSample.x);
  T eps = T(1e-1);
  vec3<T> offsetDelta = camWorldPos + rayDir * (depthSample.x + eps) - centerWorldPos;
  T offsetAngle = M::atan2(dot(eyeWorldTangent, offsetDelta), dot(eyeWorldDir, offsetDelta));
  T derivative = gdiv(offsetAngle - angle, eps);
  T sigma = M::sqrt(var) * std::abs(derivative);
  if (!(sigma > T(1e-6))) return angle;
  T diff = maxAngle - angle;
  T z = gdiv(diff, sigma);
  T pdf = T(0.3989422804) * M::exp(T(-0.5) * z * z);
  T cdf = gdiv(T(1), T(1) + M::exp(T(-1.702) * z));
  return maxAngle - (diff * cdf + sigma * pdf);
}

// indirectLighting.frag:114-271 from the centre values on.  cpc is
// gl_FragCoord.xy of the full-resolution pixel, pidx its pattern index (:161).
template <typename T>
static vec4<T> march_core(const MarchIn<T>& A, vec2<T> cpc, int pidx, vec3<T> centerWorldNorm,
                          T centerDepth, int* steps_out, long long* lod_trace = nullptr) {
  using M = Math<T>;
  vec2<T> vp(T(A.W), T(A.H));
  vec2<T> csc = cpc / vp;
  vec3<T> camWorldPos = (A.invView * vec4<T>(T(0), T(0), T(0), T(1))).xyz();
  vec3<T> centerWorldPos = Unproject(vec3<T>(csc.x, csc.y, centerDepth), A.invVP);
  // :131 centerViewPos is computed and never used.
  vec3<T> ambientLight(T(0.01));
  vec2<T> distribution = HammersleyNorm<T>(pidx, A.P * A.P);
  T angOffset = distribution.x;
  T linOffset = distribution.y;
  const int dirsCount = A.R;
  const int stepDirs = A.stepR > 0 ? A.stepR : A.R;  // dirsCount of :212, :217, :234-235
  const T nearStepSize = gdiv(vp.x, T(1000));
  const T pi = T(3.1415);  // :169, kept as written
  T pixelAngOffset = gdiv(T(2) * pi, T(dirsCount)) * angOffset;
  vec3<T> sumLight(T(0));
  int steps = 0;
  for (int dirIndex = 0; dirIndex < dirsCount; dirIndex++) {
    T dirPixelOffset = linOffset;
    T screenAng = pixelAngOffset + gdiv(T(2) * pi, T(dirsCount)) * T(dirIndex);
    vec2<T> screenPixelDir(M::cos(screenAng), M::sin(screenAng));
    T eps = T(10e-1);
    vec2<T> oc = (cpc + screenPixelDir * eps) / vp;
    vec3<T> offsetWorldPos = Unproject(vec3<T>(oc.x, oc.y, centerDepth), A.invVP);
    vec3<T> eyeWorldDir = normalize(camWorldPos - centerWorldPos);
    vec3<T> eyeWorldTangent =
        normalize(normalize(offsetWorldPos - camWorldPos) - normalize(centerWorldPos - camWorldPos));
    T maxHorizonAngle;
    {
      vec3<T> dirNormalPoint = cross(-cross(eyeWorldTangent, eyeWorldDir), centerWorldNorm);
      vec2<T> projectedDirNormal(dot(dirNormalPoint, eyeWorldDir), dot(dirNormalPoint, eyeWorldTangent));
      maxHorizonAngle = M::atan2(projectedDirNormal.y, projectedDirNormal.x);
    }
    vec3<T> dirLight =
        ambientLight * HorizonContribution(eyeWorldDir, eyeWorldTangent, centerWorldNorm, T(0), maxHorizonAngle);
    int iterationsCount = IterationsCount(cpc, screenPixelDir, vp, nearStepSize, pi, stepDirs, A.cap);
    for (int offset = 0; offset < iterationsCount; offset++) {
      T pixelOffset =
          nearStepSize * M::pow(gdiv(T(2) * pi, T(stepDirs)) + T(1), T(offset) + dirPixelOffset) + T(1) - nearStepSize;
      vec2<T> samplePixelCoord = cpc + screenPixelDir * pixelOffset;
      vec2<T> sampleScreenCoord = samplePixelCoord / vp;
      T sideMult = T(1);
      {
        T width = T(0.1);
        T invWidth = gdiv(T(1), width);
        sideMult = sideMult * saturate((T(1) - sampleScreenCoord.x) * invWidth);
        sideMult = sideMult * saturate(sampleScreenCoord.x * invWidth);
        sideMult = sideMult * saturate((T(1) - sampleScreenCoord.y) * invWidth);
        sideMult = sideMult * saturate(sampleScreenCoord.y * invWidth);
      }
      T blurLodOffset = T(-2);
      T depthLodMult = T(0.5);
      T colorLodMult = T(0.5);
      T depthLod =
          gdiv(M::log(gmax(T(0), gdiv(T(2) * pi, T(stepDirs)) * (pixelOffset - T(1)) * depthLodMult)), M::log(T(2))) +
          blurLodOffset;
      T colorLod =
          gdiv(M::log(gmax(T(0), gdiv(T(2) * pi, T(stepDirs)) * (pixelOffset - T(1)) * colorLodMult)), M::log(T(2))) +
          blurLodOffset;
      vec4<T> depthSample = (A.tex & 1) ? texture_lod_unit(A.depth, sampleScreenCoord, depthLod)
                                        : texture_lod(A.depth, sampleScreenCoord, depthLod);
      if (lod_trace) {  // the first mip level the depth tap reads, as 1-based level
        const long long lv = (long long)std::floor(std::min(std::max(depthLod, T(0)), T(A.depth.n - 1))) + 1;
        lod_trace[0] += 1;
        lod_trace[1] += lv;
        lod_trace[2] += lv * lv;
      }
      vec3<T> rayDir =
          normalize(Unproject(vec3<T>(sampleScreenCoord.x, sampleScreenCoord.y, T(1)), A.invVP) - camWorldPos);
      vec3<T> sampleWorldPos = camWorldPos + rayDir * depthSample.x;
      vec3<T> worldDelta = sampleWorldPos - centerWorldPos;
      vec2<T> horizonPoint(dot(eyeWorldDir, worldDelta), dot(eyeWorldTangent, worldDelta));
      T sampleHorizonAngle = M::atan2(horizonPoint.y, horizonPoint.x);
      T newAngle = sampleHorizonAngle;
      if (A.soft) newAngle = SoftHorizon(depthSample, rayDir, camWorldPos, centerWorldPos, eyeWorldDir,
                                         eyeWorldTangent, sampleHorizonAngle, maxHorizonAngle);
      if (newAngle < maxHorizonAngle) {
        vec4<T> lightSample = (A.tex & 2) ? texture_lod_unit(A.light, sampleScreenCoord, colorLod)
                                          : texture_lod(A.light, sampleScreenCoord, colorLod);
        T horizonContribution =
            HorizonContribution(eyeWorldDir, eyeWorldTangent, centerWorldNorm, newAngle, maxHorizonAngle) *
            sideMult;
        dirLight = dirLight + lightSample.rgb() * horizonContribution;
        dirLight = dirLight - ambientLight * horizonContribution;
        maxHorizonAngle = newAngle;
      }
      steps++;
    }
    sumLight = sumLight + vec3<T>(T(2)) * dirLight / T(dirsCount);
  }
  if (steps_out) *steps_out = steps;
  return vec4<T>(sumLight, T(1));
}

// A7: indirectLighting.frag:116-121, centre values through the linear sampler.
template <typename T>
static vec4<T> march_pixel(const MarchIn<T>& A, int px, int py, int* steps, long long* lod_trace = nullptr) {
  vec2<T> cpc(T(px) + T(0.5), T(py) + T(0.5));
  vec2<T> csc = cpc / vec2<T>(T(A.W), T(A.H));
  vec4<T> n = texture_lod0(A.normal, csc);
  vec4<T> d = texture_lod0(A.ndc, csc);
  int pidx = (px % A.P) + (py % A.P) * A.P;
  return march_core(A, cpc, pidx, n.xyz(), d.x, steps, lod_trace);
}

// A7': deinterleaved pixel (dx, dy) of the sub-image grid; centre values by
// texelFetch from deinterleaved inputs (the compute-shader form of
// LSGIRenderer.h:83-91), result stored at the same deinterleaved pixel.
template <typename T> static vec4<T> march_pixel_deint(const MarchIn<T>& A, int dx, int dy) {
  int sw = A.W / A.P, sh = A.H / A.P;
  int kx = dx / sw, ky = dy / sh;
  int fx = (dx % sw) * A.P + kx, fy = (dy % sh) * A.P + ky;  // deinterleave.frag:16-21
  vec2<T> cpc(T(fx) + T(0.5), T(fy) + T(0.5));
  vec4<T> n = A.normal.fetch(dx, dy);
  vec4<T> d = A.ndc.fetch(dx, dy);
  int pidx = kx + ky * A.P;
  return march_core(A, cpc, pidx, n.xyz(), d.x, nullptr);
}

// ---------------------------------------------------------------------------
// Analytic ray cast of the procedural scene (stands in for rasterising the
// G-buffer and shadow-map meshes; SSVGIRenderer.h:61-158).
template <typename T> struct Hit {
  T t;
  vec3<T> n;
  int prim;      // analytic primitive, or -1
  int tri, obj;  // triangle and its object (prim == -1), or -1
  T u, v;
};

// Triangle meshes of a loaded scene (world space, grouped by object).
struct MeshSet {
  const gi_mesh_object* objects;
  const gi_triangle* tris;
  int num_objects;
  int cull;  // GI_CULL_BACK: only front faces (right-hand winding towards the ray)
};

template <typename T> static vec3<T> load3(const float* p) { return vec3<T>(T(p[0]), T(p[1]), T(p[2])); }

// Mesh part of the ray cast: object bounds by the slab test (entry clamped at
// 0, exit at the nearest hit so far), then Moller-Trumbore on its triangles
// (both faces, or front faces only), t > 0 and nearer than the hit so far.
template <typename T>
static void cast_mesh(const MeshSet& m, vec3<T> o, vec3<T> d, vec3<T> inv, Hit<T>& h) {
  const T ov[3] = {o.x, o.y, o.z}, iv[3] = {inv.x, inv.y, inv.z};
  for (int k = 0; k < m.num_objects; k++) {
    const gi_mesh_object& ob = m.objects[k];
    T tn = T(0), tf = h.t;
    for (int c = 0; c < 3; c++) {
      T a = (T(ob.lo[c]) - ov[c]) * iv[c];
      T b = (T(ob.hi[c]) - ov[c]) * iv[c];
      tn = gmax(tn, gmin(a, b));
      tf = gmin(tf, gmax(a, b));
    }
    if (!(tn <= tf)) continue;
    for (int i = ob.first; i < ob.first + ob.count; i++) {
      const gi_triangle& tr = m.tris[i];
      vec3<T> p0 = load3<T>(tr.p[0]);
      vec3<T> e1 = load3<T>(tr.p[1]) - p0, e2 = load3<T>(tr.p[2]) - p0;
      vec3<T> pv = cross(d, e2);
      T det = dot(e1, pv);  // -d . (e1 x e2)
      if (m.cull ? !(det > T(0)) : det == T(0)) continue;
      T invdet = gdiv(T(1), det);
      vec3<T> tv = o - p0;
      T u = dot(tv, pv) * invdet;
      if (u < T(0) || u > T(1)) continue;
      vec3<T> qv = cross(tv, e1);
      T v = dot(d, qv) * invdet;
      if (v < T(0) || u + v > T(1)) continue;
      T t = dot(e2, qv) * invdet;
      if (t > T(0) && t < h.t) {
        h.t = t;
        h.prim = -1;
        h.tri = i;
        h.obj = k;
        h.u = u;
        h.v = v;
      }
    }
  }
}

template <typename T>
static void cast_ray(const gi_prim* prims, int np, const MeshSet& mesh, vec3<T> o, vec3<T> d, Hit<T>& h) {
  h.t = std::numeric_limits<T>::infinity();
  h.prim = -1;
  h.tri = h.obj = -1;
  h.u = h.v = T(0);
  h.n = vec3<T>(T(0));
  vec3<T> inv(gdiv(T(1), d.x), gdiv(T(1), d.y), gdiv(T(1), d.z));
  for (int i = 0; i < np; i++) {
    const gi_prim& p = prims[i];
    if (p.kind == GI_PRIM_ROOM || p.kind == GI_PRIM_BOX) {
      T t1[3], t2[3];
      T ov[3] = {o.x, o.y, o.z}, iv[3] = {inv.x, inv.y, inv.z}, dv[3] = {d.x, d.y, d.z};
      for (int k = 0; k < 3; k++) {
        T a = (T(p.a[k]) - ov[k]) * iv[k];
        T b = (T(p.b[k]) - ov[k]) * iv[k];
        t1[k] = gmin(a, b);
        t2[k] = gmax(a, b);
      }
      if (p.kind == GI_PRIM_ROOM) {
        int ax = 0;
        T tf = t2[0];
        if (t2[1] < tf) { ax = 1; tf = t2[1]; }
        if (t2[2] < tf) { ax = 2; tf = t2[2]; }
        if (tf > T(0) && tf < h.t) {
          h.t = tf;
          h.prim = i;
          T nv[3] = {T(0), T(0), T(0)};
          nv[ax] = dv[ax] > T(0) ? T(-1) : T(1);
          h.n = vec3<T>(nv[0], nv[1], nv[2]);
        }
      } else {
        int ax = 0;
        T tn = t1[0];
        if (t1[1] > tn) { ax = 1; tn = t1[1]; }
        if (t1[2] > tn) { ax = 2; tn = t1[2]; }
        T tf = gmin(gmin(t2[0], t2[1]), t2[2]);
        if (tn <= tf && tn > T(0) && tn < h.t) {
          h.t = tn;
          h.prim = i;
          T nv[3] = {T(0), T(0), T(0)};
          nv[ax] = dv[ax] > T(0) ? T(-1) : T(1);
          h.n = vec3<T>(nv[0], nv[1], nv[2]);
        }
      }
    } else if (p.kind == GI_PRIM_SPHERE) {
      vec3<T> c(T(p.a[0]), T(p.a[1]), T(p.a[2]));
      T r = T(p.b[0]);
      vec3<T> oc = o - c;
      T b = dot(oc, d);
      T cc = dot(oc, oc) - r * r;
      T disc = b * b - cc;
      if (disc >= T(0)) {
        T t = -b - Math<T>::sqrt(disc);
        if (t > T(0) && t < h.t) {
          h.t = t;
          h.prim = i;
          h.n = normalize((o + d * t) - c);
        }
      }
    }
  }
  if (mesh.num_objects > 0) cast_mesh(mesh, o, d, inv, h);
}

// Common/gBufferBuilder.frag:28-38 for the primary hit of the pixel-centre ray.
template <typename T>
static void gbuffer_pixel(const gi_view& v, const gi_prim* prims, int np, const MeshSet& mesh, int x, int y,
                          T* albedo, T* emissive, T* normal, T* moments, T* ndc) {
  mat4<T> invVP = load_mat<T>(v.inv_view_proj), invV = load_mat<T>(v.inv_view), VP = load_mat<T>(v.view_proj);
  vec2<T> sc(gdiv(T(x) + T(0.5), T(v.width)), gdiv(T(y) + T(0.5), T(v.height)));
  vec3<T> cam = (invV * vec4<T>(T(0), T(0), T(0), T(1))).xyz();
  vec3<T> farp = Unproject(vec3<T>(sc.x, sc.y, T(1)), invVP);
  vec3<T> dir = normalize(farp - cam);
  Hit<T> h;
  cast_ray(prims, np, mesh, cam, dir, h);
  if (h.prim < 0 && h.tri < 0) {
    for (int c = 0; c < 4; c++) albedo[c] = emissive[c] = normal[c] = T(0);
    moments[0] = moments[1] = T(0);
    ndc[0] = T(1);
    return;
  }
  vec3<T> hit = cam + dir * h.t;
  T deltaLen = length(hit - cam);
  const float* src_al;
  const float* src_em;
  if (h.prim >= 0) {
    src_al = prims[h.prim].albedo;
    src_em = prims[h.prim].emissive;
  } else {
    // gBufferBuilder.vert:38 carries modelMatrix * (normal, 0) to the fragment;
    // the rasteriser blends it with the barycentric weights of the hit point.
    src_al = mesh.objects[h.obj].albedo;
    src_em = mesh.objects[h.obj].emissive;
    const gi_triangle& tr = mesh.tris[h.tri];
    T w0 = T(1) - h.u - h.v;
    h.n = load3<T>(tr.n[0]) * w0 + load3<T>(tr.n[1]) * h.u + load3<T>(tr.n[2]) * h.v;
  }
  for (int c = 0; c < 4; c++) {
    albedo[c] = Math<T>::pow(T(src_al[c]), T(2.2));
    emissive[c] = Math<T>::pow(T(src_em[c]), T(2.2));
  }
  normal[0] = h.n.x;
  normal[1] = h.n.y;
  normal[2] = h.n.z;
  normal[3] = T(1);
  moments[0] = deltaLen;
  moments[1] = deltaLen * deltaLen;
  ndc[0] = Project(hit, VP).z;
}

// Shadow map texel: depth of the nearest surface seen from the light.
template <typename T>
static T shadow_texel(const gi_view& lv, const gi_prim* prims, int np, const MeshSet& mesh, int x, int y) {
  mat4<T> invVP = load_mat<T>(lv.inv_view_proj), invV = load_mat<T>(lv.inv_view), VP = load_mat<T>(lv.view_proj);
  vec2<T> sc(gdiv(T(x) + T(0.5), T(lv.width)), gdiv(T(y) + T(0.5), T(lv.height)));
  vec3<T> org = (invV * vec4<T>(T(0), T(0), T(0), T(1))).xyz();
  vec3<T> farp = Unproject(vec3<T>(sc.x, sc.y, T(1)), invVP);
  vec3<T> dir = normalize(farp - org);
  Hit<T> h;
  cast_ray(prims, np, mesh, org, dir, h);
  if (h.prim < 0 && h.tri < 0) return T(1);
  vec3<T> hit = org + dir * h.t;
  return Project(hit, VP).z;
}

// Common/directLighting.frag:45-79.
template <typename T>
static vec4<T> direct_pixel(const gi_view& v, const gi_view& lv, const Img<T>& albedo, const Img<T>& emissive,
                            const Img<T>& normal, const Img<T>& depth, const Img<T>& shadow, int x, int y) {
  vec2<T> fsc(gdiv(T(x) + T(0.5), T(v.width)), gdiv(T(y) + T(0.5), T(v.height)));
  vec4<T> depthSample = bilinear(depth, fsc);
  vec4<T> normalSample = bilinear(normal, fsc);
  vec3<T> worldNormal = normalSample.xyz();
  mat4<T> invViewProj = load_mat<T>(v.inv_view_proj);
  mat4<T> invLightView = load_mat<T>(lv.inv_view);
  mat4<T> lightView = load_mat<T>(lv.view);
  mat4<T> lightViewProj = load_mat<T>(lv.view_proj);
  vec3<T> lightPos = (invLightView * vec4<T>(T(0), T(0), T(0), T(1))).xyz();
  vec3<T> worldPos = Unproject(vec3<T>(fsc.x, fsc.y, depthSample.x), invViewProj);
  vec3<T> lightVec = worldPos - lightPos;
  T diffuse = gmax(T(0), -dot(normalize(lightVec), worldNormal));
  vec3<T> shadowmapCoord = Project(worldPos, lightViewProj);
  vec3<T> lightViewPos = (lightView * vec4<T>(worldPos, T(1))).xyz();
  vec3<T> lightIntensity(T(5));
  T radius = length(vec2<T>(shadowmapCoord.x, shadowmapCoord.y) - vec2<T>(T(0.5))) * T(2);
  T penumbra = smoothstep(T(0), T(1), T(1) - saturate(gdiv(radius - T(0.6), T(1) - T(0.6)))) *
               (lightViewPos.z > T(0) ? T(1) : T(0));
  lightIntensity = lightIntensity * penumbra;
  T bias = T(2e-4);
  shadowmapCoord.z = shadowmapCoord.z - bias;
  lightIntensity = lightIntensity * Math<T>::pow(texture_shadow(shadow, shadowmapCoord), T(2.2));
  vec4<T> albedoColor = bilinear(albedo, fsc);
  vec4<T> emissiveColor = bilinear(emissive, fsc);
  vec3<T> c = diffuse * albedoColor.rgb() * lightIntensity + emissiveColor.rgb();
  return vec4<T>(c, T(1));
}

// Common/mipLevelBuilder.frag:17-43, one destination pixel.
template <typename T> static vec4<T> mip_texel(const Img<T>& src, int x, int y, int filter) {
  static const int off[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
  if (filter == GI_MIP_AVG) {
    vec4<T> sum(T(0));
    for (int i = 0; i < 4; i++) sum = sum + src.fetch(x * 2 + off[i][0], y * 2 + off[i][1]);
    return sum / T(4);
  }
  T minDepth = T(1e5), maxDepth = T(-1e5), totalMass = T(0);
  for (int i = 0; i < 4; i++) {
    vec4<T> s = src.fetch(x * 2 + off[i][0], y * 2 + off[i][1]);
    minDepth = gmin(minDepth, s.x);
    maxDepth = gmax(maxDepth, s.y);
    totalMass = totalMass + (s.y - s.x) * s.z;
  }
  return vec4<T>(minDepth, maxDepth, gdiv(gdiv(totalMass, maxDepth - minDepth), T(4)), T(0));
}

// Common/blurLayerBuilder.frag:17-35, one pixel (x outer, y inner).
template <typename T> static vec4<T> blur_texel(const Img<T>& src, int px, int py, int radius) {
  vec4<T> sum(T(0));
  T totalWeight = T(0);
  for (int x = -radius; x < radius; x++)
    for (int y = -radius; y < radius; y++) {
      sum = sum + src.fetch_clamped(px + x, py + y);
      totalWeight = totalWeight + T(1);
    }
  if (radius == 0) return src.fetch(px, py);
  return sum / totalWeight;
}

// Project-defined 5x5 bilateral (weights of Common/denoiser.frag:102-105).
template <typename T>
static vec4<T> bilateral_pixel(const Img<T>& ind, const Img<T>& depth, const Img<T>& normal, int px, int py) {
  T cd = depth.fetch(px, py).x;
  vec3<T> cn = normal.fetch(px, py).xyz();
  vec3<T> sum(T(0));
  T sumW = T(0);
  for (int y = -2; y <= 2; y++)
    for (int x = -2; x <= 2; x++) {
      vec3<T> c = ind.fetch_clamped(px + x, py + y).rgb();
      T d = depth.fetch_clamped(px + x, py + y).x;
      vec3<T> n = normal.fetch_clamped(px + x, py + y).xyz();
      // exp(-|dd| 10.5) * exp(-|dn|^2 20), evaluated as one exponential of the summed exponents
      vec3<T> nd = n - cn;
      T weight = Math<T>::exp(-(std::abs(d - cd) * T(10.5) + dot(nd, nd) * T(20)));
      sum = sum + c * weight;
      sumW = sumW + weight;
    }
  return vec4<T>(sum / (sumW + T(1e-7)), T(1));
}

// Common/denoiser.frag:72-184 with radius 2 (radius 0 returns the input).
template <typename T>
static vec4<T> denoise_pixel(const Img<T>& noisy, const Img<T>& depth, int W, int H, int px, int py, int radius) {
  vec2<T> vp{T(W), T(H)};
  vec2<T> cpc{T(px) + T(0.5), T(py) + T(0.5)};
  if (radius == 0) return bilinear(noisy, cpc / vp);
  T params[16][2];
  vec3<T> color[16];
  int i = 0;
  for (int y = -2; y < 2; y++)
    for (int x = -2; x < 2; x++) {
      vec2<T> sc = (cpc + vec2<T>(T(x), T(y))) / vp;
      params[i][0] = bilinear(depth, sc).x;
      params[i][1] = T(1);
      color[i] = bilinear(noisy, sc).rgb();
      i++;
    }
  T G[2][2];
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      T sum = T(0);
      for (int k = 0; k < 16; k++) sum = sum + params[k][a] * params[k][b];
      sum = sum + ((a == b) ? T(1e-7) : T(0));
      G[a][b] = sum;
    }
  // inverse of the 2x2 block (the rest of the 4x4 Gramian is the identity).
  T det = G[0][0] * G[1][1] - G[0][1] * G[1][0];
  T inv[2][2] = {{gdiv(G[1][1], det), gdiv(-G[0][1], det)}, {gdiv(-G[1][0], det), gdiv(G[0][0], det)}};
  T cparams[2] = {bilinear(depth, cpc / vp).x, T(1)};
  vec4<T> res(T(0), T(0), T(0), T(1));
  for (int ch = 0; ch < 3; ch++) {
    T mom[2];
    for (int a = 0; a < 2; a++) {
      T m = T(0);
      for (int k = 0; k < 16; k++) m = m + params[k][a] * color[k][ch];
      mom[a] = m;
    }
    T coeff[2];
    for (int a = 0; a < 2; a++) {
      T c = T(0);
      for (int b = 0; b < 2; b++) c = c + inv[b][a] * mom[b];  // transpose(inverse(G))[a][b]
      coeff[a] = c;
    }
    T v = T(0);
    for (int a = 0; a < 2; a++) v = v + coeff[a] * cparams[a];
    res[ch] = v;
  }
  return res;
}

}  // namespace oracle

using namespace oracle;

// ===========================================================================
// C API (ctypes).  Suffix _f32 / _f64 selects the element type.

extern "C" int go_threads(void) { return omp_get_max_threads(); }
// fp32 transcendentals and division from the C library (1) or the evaluation
// contract (0, the default); see Math<float> in glsl.h.
extern "C" void go_set_libm(int on) { glsl::Math<float>::libm = on != 0; }
extern "C" void go_set_threads(int n) { omp_set_num_threads(n); }

extern "C" float go_logf(float x) { return gi::logf_(x); }
extern "C" float go_log2f(float x) { return gi::log2f_(x); }
extern "C" float go_expf(float x) { return gi::expf_(x); }
extern "C" float go_exp2f(float x) { return gi::exp2f_(x); }
extern "C" float go_powf(float b, float e) { return gi::powf_(b, e); }
extern "C" float go_atan2f(float y, float x) { return gi::atan2f_(y, x); }
extern "C" float go_sinf(float x) { return gi::sinf_(x); }
extern "C" float go_cosf(float x) { return gi::cosf_(x); }
extern "C" void go_math_batch(int fn, const float* a, const float* b, float* out, int n) {
  for (int i = 0; i < n; i++) {
    switch (fn) {
      case 0: out[i] = gi::logf_(a[i]); break;
      case 1: out[i] = gi::log2f_(a[i]); break;
      case 2: out[i] = gi::expf_(a[i]); break;
      case 3: out[i] = gi::exp2f_(a[i]); break;
      case 4: out[i] = gi::powf_(a[i], b[i]); break;
      case 5: out[i] = gi::atan2f_(a[i], b[i]); break;
      case 6: out[i] = gi::sinf_(a[i]); break;
      default: out[i] = gi::cosf_(a[i]); break;
    }
  }
}

extern "C" int go_iterations_f32(int W, int H, int R, int cap, float cx, float cy, float dx, float dy) {
  return IterationsCount<float>(vec2<float>(cx, cy), vec2<float>(dx, dy), vec2<float>(float(W), float(H)),
                                gdiv(float(W), 1000.0f), 3.1415f, R, cap);
}

extern "C" double go_horizon_contribution_f64(const double* ed, const double* et, const double* n, double mn,
                                              double mx) {
  return HorizonContribution<double>(vec3<double>(ed[0], ed[1], ed[2]), vec3<double>(et[0], et[1], et[2]),
                                     vec3<double>(n[0], n[1], n[2]), mn, mx);
}

extern "C" void go_hammersley(int i, int n, float* out2) {
  vec2<float> v = HammersleyNorm<float>(i, n);
  out2[0] = v.x;
  out2[1] = v.y;
}

extern "C" int go_mip_level_count(int w, int h, int req) {
  int m = std::min(w, h), n = 0;
  while (m >= 1) { n++; m >>= 1; }
  return std::min(req, n);
}

template <typename T>
static void mip_level_t(const T* src, int sw, int sh, int ch, T* dst, int dw, int dh, int filter) {
  Img<T> s(src, sw, sh, ch);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < dh; y++)
    for (int x = 0; x < dw; x++) {
      vec4<T> v = mip_texel(s, x, y, filter);
      for (int c = 0; c < ch; c++) dst[((size_t)y * dw + x) * ch + c] = v[c];
    }
}
extern "C" void go_mip_level_f32(const float* s, int sw, int sh, int ch, float* d, int dw, int dh, int f) { mip_level_t(s, sw, sh, ch, d, dw, dh, f); }
extern "C" void go_mip_level_f64(const double* s, int sw, int sh, int ch, double* d, int dw, int dh, int f) { mip_level_t(s, sw, sh, ch, d, dw, dh, f); }

template <typename T> static void blur_t(const T* src, T* dst, int w, int h, int ch, int r) {
  Img<T> s(src, w, h, ch);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      vec4<T> v = blur_texel(s, x, y, r);
      for (int c = 0; c < ch; c++) dst[((size_t)y * w + x) * ch + c] = v[c];
    }
}
extern "C" void go_blur_f32(const float* s, float* d, int w, int h, int ch, int r) { blur_t(s, d, w, h, ch, r); }
extern "C" void go_blur_f64(const double* s, double* d, int w, int h, int ch, int r) { blur_t(s, d, w, h, ch, r); }

// deinterleave.frag:16-28 / interleave.frag:15-27 (integer maps; payload copied).
extern "C" void go_deinterleave_map(int w, int h, int gx, int gy, int* src_index) {
  int dvx = w / gx, dvy = h / gy;
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      int px = x / dvx, py = y / dvy;
      int sx = (x % dvx) * gx + px, sy = (y % dvy) * gy + py;
      src_index[(size_t)y * w + x] = sy * w + sx;
    }
}
extern "C" void go_interleave_map(int w, int h, int gx, int gy, int* src_index) {
  int dvx = w / gx, dvy = h / gy;
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      int px = x % gx, py = y % gy;
      int sx = px * dvx + x / gx, sy = py * dvy + y / gy;
      src_index[(size_t)y * w + x] = sy * w + sx;
    }
}
extern "C" void go_permute_f32(const float* src, float* dst, const int* map, int n, int ch) {
  for (int i = 0; i < n; i++)
    for (int c = 0; c < ch; c++) dst[(size_t)i * ch + c] = src[(size_t)map[i] * ch + c];
}

// Pyramid arguments: level k of width >> k etc. packed back to back.
template <typename T> static Pyr<T> make_pyr(const T* base, int w, int h, int ch, int n) {
  Pyr<T> p;
  p.n = n;
  size_t off = 0;
  int lw = w, lh = h;
  for (int k = 0; k < n; k++) {
    p.lv[k] = Img<T>(base + off, lw, lh, ch);
    off += (size_t)lw * lh * ch;
    lw /= 2;
    lh /= 2;
  }
  return p;
}

template <typename T>
static void march_t(const gi_view* v, int R, int cap, int P, const T* light, const T* depth, int nlev,
                    const T* normal, const T* ndc, const int* pix, int npix, T* out, int* steps, int deint,
                    int stepR, int soft = 0, int tex = 0, long long* lod_trace = nullptr) {
  MarchIn<T> A;
  A.W = v->width;
  A.H = v->height;
  A.invVP = load_mat<T>(v->inv_view_proj);
  A.invView = load_mat<T>(v->inv_view);
  A.light = make_pyr(light, A.W, A.H, 4, nlev);
  A.depth = make_pyr(depth, A.W, A.H, 2, nlev);
  A.normal = Img<T>(normal, A.W, A.H, 4);
  A.ndc = Img<T>(ndc, A.W, A.H, 1);
  A.R = R;
  A.cap = cap;
  A.P = P;
  A.stepR = stepR;
  A.soft = soft;
  A.tex = tex;
  long n = pix ? npix : (long)A.W * A.H;
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < n; i++) {
    int x, y;
    if (pix) { x = pix[2 * i]; y = pix[2 * i + 1]; }
    else { x = (int)(i % A.W); y = (int)(i / A.W); }
    int st = 0;
    long long* tr = lod_trace ? lod_trace + 3 * i : nullptr;
    if (tr) tr[0] = tr[1] = tr[2] = 0;
    vec4<T> r = deint ? march_pixel_deint(A, x, y) : march_pixel(A, x, y, &st, tr);
    for (int c = 0; c < 4; c++) out[i * 4 + c] = r[c];
    if (steps) steps[i] = st;
  }
}
extern "C" void go_march_f32(const gi_view* v, int R, int cap, int P, const float* light, const float* depth, int nlev,
                  const float* normal, const float* ndc, const int* pix, int npix, float* out, int* steps, int stepR,
                  int soft, int tex, long long* lod_trace) {
  march_t(v, R, cap, P, light, depth, nlev, normal, ndc, pix, npix, out, steps, 0, stepR, soft, tex, lod_trace);
}
extern "C" void go_march_f64(const gi_view* v, int R, int cap, int P, const double* light, const double* depth, int nlev,
                  const double* normal, const double* ndc, const int* pix, int npix, double* out, int* steps,
                  int stepR, int soft) {
  march_t(v, R, cap, P, light, depth, nlev, normal, ndc, pix, npix, out, steps, 0, stepR, soft);
}
// textureLod at n points: unit = 1 the texture units' fixed-point trilinear fetch
// (texture_lod_unit), unit = 0 the exact sampler (texture_lod).
extern "C" void go_texture_lod_f32(const float* levels, int w, int h, int ch, int nlev, const float* st,
                                   const float* lod, int n, int out_ch, float* out, int unit) {
  Pyr<float> py = make_pyr(levels, w, h, ch, nlev);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    const vec2<float> c(st[2 * i], st[2 * i + 1]);
    vec4<float> r = unit ? texture_lod_unit(py, c, lod[i]) : texture_lod(py, c, lod[i]);
    for (int c = 0; c < out_ch; c++) out[(size_t)i * out_ch + c] = r[c];
  }
}

extern "C" void go_march_deint_f32(const gi_view* v, int R, int cap, int P, const float* light, const float* depth, int nlev,
                        const float* normal_d, const float* ndc_d, float* out_d) {
  march_t(v, R, cap, P, light, depth, nlev, normal_d, ndc_d, (const int*)nullptr, 0, out_d, (int*)nullptr, 1, 0);
}

template <typename T>
static void bilateral_t(const T* ind, const T* mom, const T* nrm, T* out, int w, int h) {
  Img<T> I(ind, w, h, 4), D(mom, w, h, 2), N(nrm, w, h, 4);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      vec4<T> r = bilateral_pixel(I, D, N, x, y);
      for (int c = 0; c < 4; c++) out[((size_t)y * w + x) * 4 + c] = r[c];
    }
}
extern "C" void go_bilateral_f32(const float* i, const float* m, const float* n, float* o, int w, int h) { bilateral_t(i, m, n, o, w, h); }
extern "C" void go_bilateral_f64(const double* i, const double* m, const double* n, double* o, int w, int h) { bilateral_t(i, m, n, o, w, h); }

template <typename T>
static void denoise_t(const T* noisy, const T* mom, T* out, int w, int h, int radius) {
  Img<T> I(noisy, w, h, 4), D(mom, w, h, 2);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      vec4<T> r = denoise_pixel(I, D, w, h, x, y, radius);
      for (int c = 0; c < 4; c++) out[((size_t)y * w + x) * 4 + c] = r[c];
    }
}
extern "C" void go_denoise_f32(const float* i, const float* m, float* o, int w, int h, int r) { denoise_t(i, m, o, w, h, r); }
extern "C" void go_denoise_f64(const double* i, const double* m, double* o, int w, int h, int r) { denoise_t(i, m, o, w, h, r); }

// Common/finalGatherer.frag:42-59.  The loop at :50-57 multiplies every term by
// currWeight = 0 (:54) and leaves totalWeight = 1, so it contributes nothing
// for finite inputs and is not evaluated.
template <typename T>
static void final_gather_t(const T* direct, const T* ind, const T* alb, T* out, int w, int h) {
  Img<T> Dl(direct, w, h, 4), In(ind, w, h, 4), Al(alb, w, h, 4);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      vec2<T> fsc(gdiv(T(x) + T(0.5), T(w)), gdiv(T(y) + T(0.5), T(h)));
      vec4<T> r = bilinear(Dl, fsc) + bilinear(In, fsc) * bilinear(Al, fsc);
      for (int c = 0; c < 4; c++) out[((size_t)y * w + x) * 4 + c] = r[c];
    }
}
extern "C" void go_final_gather_f32(const float* d, const float* i, const float* a, float* o, int w, int h) { final_gather_t(d, i, a, o, w, h); }
extern "C" void go_final_gather_f64(const double* d, const double* i, const double* a, double* o, int w, int h) { final_gather_t(d, i, a, o, w, h); }

template <typename T>
static void gbuffer_t(const gi_view* v, const gi_prim* prims, int np, const MeshSet& mesh, T* albedo, T* emissive,
                      T* normal, T* moments, T* ndc) {
  int W = v->width, H = v->height;
#pragma omp parallel for schedule(dynamic, 16)
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      size_t i = (size_t)y * W + x;
      gbuffer_pixel<T>(*v, prims, np, mesh, x, y, albedo + 4 * i, emissive + 4 * i, normal + 4 * i, moments + 2 * i,
                       ndc + i);
    }
}
static const MeshSet kNoMesh = {nullptr, nullptr, 0, 0};
extern "C" void go_gbuffer_f32(const gi_view* v, const gi_prim* p, int np, float* a, float* e, float* n, float* m, float* z) { gbuffer_t(v, p, np, kNoMesh, a, e, n, m, z); }
extern "C" void go_gbuffer_f64(const gi_view* v, const gi_prim* p, int np, double* a, double* e, double* n, double* m, double* z) { gbuffer_t(v, p, np, kNoMesh, a, e, n, m, z); }
extern "C" void go_gbuffer_mesh_f32(const gi_view* v, const gi_prim* p, int np, const gi_mesh_object* ob, int nob, const gi_triangle* tr, int cull, float* a, float* e, float* n, float* m, float* z) { gbuffer_t(v, p, np, MeshSet{ob, tr, nob, cull}, a, e, n, m, z); }
extern "C" void go_gbuffer_mesh_f64(const gi_view* v, const gi_prim* p, int np, const gi_mesh_object* ob, int nob, const gi_triangle* tr, int cull, double* a, double* e, double* n, double* m, double* z) { gbuffer_t(v, p, np, MeshSet{ob, tr, nob, cull}, a, e, n, m, z); }

template <typename T> static void shadow_t(const gi_view* lv, const gi_prim* prims, int np, const MeshSet& mesh, T* out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int y = 0; y < lv->height; y++)
    for (int x = 0; x < lv->width; x++) out[(size_t)y * lv->width + x] = shadow_texel<T>(*lv, prims, np, mesh, x, y);
}
extern "C" void go_shadow_f32(const gi_view* lv, const gi_prim* p, int np, float* o) { shadow_t(lv, p, np, kNoMesh, o); }
extern "C" void go_shadow_f64(const gi_view* lv, const gi_prim* p, int np, double* o) { shadow_t(lv, p, np, kNoMesh, o); }
extern "C" void go_shadow_mesh_f32(const gi_view* lv, const gi_prim* p, int np, const gi_mesh_object* ob, int nob, const gi_triangle* tr, int cull, float* o) { shadow_t(lv, p, np, MeshSet{ob, tr, nob, cull}, o); }
extern "C" void go_shadow_mesh_f64(const gi_view* lv, const gi_prim* p, int np, const gi_mesh_object* ob, int nob, const gi_triangle* tr, int cull, double* o) { shadow_t(lv, p, np, MeshSet{ob, tr, nob, cull}, o); }

template <typename T>
static void direct_t(const gi_view* v, const gi_view* lv, const T* alb, const T* em, const T* nrm, const T* ndc,
                     const T* shadow, int ssize, T* out) {
  int W = v->width, H = v->height;
  Img<T> A(alb, W, H, 4), E(em, W, H, 4), N(nrm, W, H, 4), Z(ndc, W, H, 1), S(shadow, ssize, ssize, 1);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      vec4<T> r = direct_pixel(*v, *lv, A, E, N, Z, S, x, y);
      for (int c = 0; c < 4; c++) out[((size_t)y * W + x) * 4 + c] = r[c];
    }
}
extern "C" void go_direct_f32(const gi_view* v, const gi_view* lv, const float* a, const float* e, const float* n, const float* z,
                   const float* s, int ss, float* o) { direct_t(v, lv, a, e, n, z, s, ss, o); }
extern "C" void go_direct_f64(const gi_view* v, const gi_view* lv, const double* a, const double* e, const double* n,
                   const double* z, const double* s, int ss, double* o) { direct_t(v, lv, a, e, n, z, s, ss, o); }


// ---------------------------------------------------------------------------
// The benchmark's frames restated: the seeded room, the light camera, the camera
// spline and the view matrices, as the library defines them (the room and the
// spline are the benchmark configurations' own definitions; the matrices follow
// Scene.h:30-33 and SSVGIRenderer.h:54-59 in double, rounded once to float), so
// that the CPU reference arm builds its frames without the CUDA library.  The
// inverses here are the adjugate over the determinant, an independent evaluation
// from the library's elimination: the two agree to a float ulp.
namespace scene_oracle {

using D4 = std::array<std::array<double, 4>, 4>;  // [column][row], glm's layout

static D4 ident4() {
  D4 r{};
  for (int i = 0; i < 4; i++) r[i][i] = 1.0;
  return r;
}
static D4 mul4(const D4& a, const D4& b) {
  D4 r{};
  for (int c = 0; c < 4; c++)
    for (int row = 0; row < 4; row++) {
      double s = 0.0;
      for (int k = 0; k < 4; k++) s += a[k][row] * b[c][k];
      r[c][row] = s;
    }
  return r;
}
static double det3(const D4& m, int r0, int r1, int r2, int c0, int c1, int c2) {
  return m[c0][r0] * (m[c1][r1] * m[c2][r2] - m[c2][r1] * m[c1][r2]) -
         m[c1][r0] * (m[c0][r1] * m[c2][r2] - m[c2][r1] * m[c0][r2]) +
         m[c2][r0] * (m[c0][r1] * m[c1][r2] - m[c1][r1] * m[c0][r2]);
}
static bool inverse4(const D4& m, D4* out) {
  D4 cof{};
  for (int c = 0; c < 4; c++)
    for (int row = 0; row < 4; row++) {
      int rs[3], cs[3], nr = 0, nc = 0;
      for (int k = 0; k < 4; k++) {
        if (k != row) rs[nr++] = k;
        if (k != c) cs[nc++] = k;
      }
      const double minor = det3(m, rs[0], rs[1], rs[2], cs[0], cs[1], cs[2]);
      cof[c][row] = ((c + row) % 2 ? -1.0 : 1.0) * minor;
    }
  double det = 0.0;
  for (int c = 0; c < 4; c++) det += m[c][0] * cof[c][0];
  if (det == 0.0) return false;
  for (int c = 0; c < 4; c++)
    for (int row = 0; row < 4; row++) (*out)[c][row] = cof[row][c] / det;  // adjugate = cofactor transpose
  return true;
}
static void to_float(const D4& a, float* dst) {
  for (int c = 0; c < 4; c++)
    for (int row = 0; row < 4; row++) dst[4 * c + row] = (float)a[c][row];
}

// Uniform double in [0, 1) from the top 53 bits of one mt19937_64 draw.
static double unit(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
// An 8-bit colour channel in [0.2, 0.9]: RGBA8 / 255.
static float channel8(std::mt19937_64& g) { return (float)(int)std::lround((0.2 + 0.7 * unit(g)) * 255.0) / 255.0f; }

}  // namespace scene_oracle

// The seeded room: the unit-cube interior, boxes with edges U[0.05, 0.3] and
// spheres with radii U[0.05, 0.2] inside it and below y = 0.85, RGBA8 albedo in
// [0.2, 0.9]; draws in the order room colour, then per box (size, position) per
// axis and colour, then per sphere radius, centre and colour.
extern "C" int go_scene_generate(uint64_t seed, int boxes, int spheres, gi_prim* out, int max_prims, int* count) {
  using namespace scene_oracle;
  const int n = 1 + boxes + spheres;
  if (boxes < 0 || spheres < 0 || n > max_prims) return -1;
  std::mt19937_64 g(seed);
  std::memset(out, 0, sizeof(gi_prim) * (size_t)n);
  out[0].kind = GI_PRIM_ROOM;
  for (int k = 0; k < 3; k++) out[0].b[k] = 1.0f;
  for (int c = 0; c < 4; c++) out[0].albedo[c] = channel8(g);
  for (int i = 1; i <= boxes; i++) {
    out[i].kind = GI_PRIM_BOX;
    for (int k = 0; k < 3; k++) {
      const double size = 0.05 + 0.25 * unit(g);
      const double lo = unit(g) * ((k == 1 ? 0.85 : 1.0) - size);
      out[i].a[k] = (float)lo;
      out[i].b[k] = (float)(lo + size);
    }
    for (int c = 0; c < 4; c++) out[i].albedo[c] = channel8(g);
  }
  for (int i = 1 + boxes; i < n; i++) {
    out[i].kind = GI_PRIM_SPHERE;
    const double r = 0.05 + 0.15 * unit(g);
    for (int k = 0; k < 3; k++) out[i].a[k] = (float)(r + unit(g) * ((k == 1 ? 0.85 : 1.0) - 2.0 * r));
    out[i].b[0] = (float)r;
    for (int c = 0; c < 4; c++) out[i].albedo[c] = channel8(g);
  }
  *count = n;
  return 0;
}

// The light camera: the reference's light looks straight down (main.cpp:166-169),
// placed inside the room.
extern "C" void go_scene_light(gi_camera* c) {
  c->pos[0] = 0.5f;
  c->pos[1] = 0.93f;
  c->pos[2] = 0.5f;
  c->hor_angle = 0.0f;
  c->vert_angle = 3.1415f / 2.0f;
  c->fovy = 1.6f;
  c->znear = 0.02f;
  c->zfar = 10.0f;
}

// The camera spline: 8 seeded control positions (kept 0.08 clear of every
// primitive when a scene is given, up to 2000 draws each) and 8 look-at targets,
// a closed Catmull-Rom curve through both, frame f at parameter 8 f / frames;
// the camera looks from the position toward the target (Scene.h:20-34 angles),
// with the reference's projection fovy 1, near 0.01, far 1000 (SSVGIRenderer.h:57).
extern "C" void go_camera_spline(uint64_t seed, const gi_prim* prims, int n, int frame, int frames, gi_camera* cam) {
  using namespace scene_oracle;
  std::mt19937_64 g(seed);
  constexpr int K = 8;
  double P[K][3], Q[K][3];
  auto clear_of = [&](const double* p) {
    for (int j = 0; prims && j < n; j++) {
      const gi_prim& q = prims[j];
      double d = 1e30;
      if (q.kind == GI_PRIM_SPHERE) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (p[k] - q.a[k]) * (p[k] - q.a[k]);
        d = std::sqrt(s) - q.b[0];
      } else if (q.kind == GI_PRIM_BOX) {
        double out2 = 0.0, in = -1e30;
        for (int k = 0; k < 3; k++) {
          const double e = std::max(q.a[k] - p[k], p[k] - q.b[k]);
          if (e > 0.0) out2 += e * e;
          in = std::max(in, e);
        }
        d = out2 > 0.0 ? std::sqrt(out2) : in;
      }
      if (d < 0.08) return false;
    }
    return true;
  };
  for (int i = 0; i < K; i++) {
    for (int attempt = 0; attempt < 2000; attempt++) {
      P[i][0] = 0.2 + 0.6 * unit(g);
      P[i][1] = 0.3 + 0.4 * unit(g);
      P[i][2] = 0.2 + 0.6 * unit(g);
      if (clear_of(P[i])) break;
    }
    Q[i][0] = 0.1 + 0.8 * unit(g);
    Q[i][1] = 0.05 + 0.5 * unit(g);
    Q[i][2] = 0.1 + 0.8 * unit(g);
  }
  const int f = ((frame % frames) + frames) % frames;
  const double u = (double)f / (double)frames * K;
  const int s = (int)std::floor(u);
  const double t = u - s;
  auto curve = [&](double (*X)[3], int k) {
    const double p0 = X[(s + K - 1) % K][k], p1 = X[s % K][k], p2 = X[(s + 1) % K][k], p3 = X[(s + 2) % K][k];
    return 0.5 * ((2.0 * p1) + (-p0 + p2) * t + (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3) * t * t +
                  (-p0 + 3.0 * p1 - 3.0 * p2 + p3) * t * t * t);
  };
  double pos[3], dir[3];
  for (int k = 0; k < 3; k++) {
    pos[k] = curve(P, k);
    dir[k] = curve(Q, k) - pos[k];
  }
  double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
  if (len < 1e-6) {
    dir[0] = 0.0; dir[1] = 0.0; dir[2] = 1.0; len = 1.0;
  }
  for (int k = 0; k < 3; k++) {
    dir[k] /= len;
    cam->pos[k] = (float)pos[k];
  }
  cam->hor_angle = (float)std::atan2(dir[0], dir[2]);
  cam->vert_angle = (float)std::asin(-dir[1]);
  cam->fovy = 1.0f;
  cam->znear = 0.01f;
  cam->zfar = 1000.0f;
}

// View matrices of a camera: view = inverse(translate(pos) rotY(hor) rotX(vert))
// (Scene.h:30-33), proj = perspectiveRH_ZO(fovy, W / H, near, far) scale(1, -1, -1)
// (SSVGIRenderer.h:57), products and inverses in double, each rounded once.
extern "C" int go_view_from_camera(const gi_camera* cam, int width, int height, gi_view* out) {
  using namespace scene_oracle;
  D4 T = ident4(), RY = ident4(), RX = ident4();
  for (int k = 0; k < 3; k++) T[3][k] = cam->pos[k];
  const double ch = std::cos((double)cam->hor_angle), sh = std::sin((double)cam->hor_angle);
  RY[0][0] = ch; RY[0][2] = -sh; RY[2][0] = sh; RY[2][2] = ch;
  const double cv = std::cos((double)cam->vert_angle), sv = std::sin((double)cam->vert_angle);
  RX[1][1] = cv; RX[1][2] = sv; RX[2][1] = -sv; RX[2][2] = cv;
  const D4 xf = mul4(mul4(T, RY), RX);
  D4 view{};
  if (!inverse4(xf, &view)) return -1;
  const double th = std::tan((double)cam->fovy / 2.0), aspect = (double)width / (double)height;
  const double zn = cam->znear, zf = cam->zfar;
  D4 P{}, S = ident4();
  P[0][0] = 1.0 / (aspect * th);
  P[1][1] = 1.0 / th;
  P[2][2] = zf / (zn - zf);
  P[2][3] = -1.0;
  P[3][2] = -(zf * zn) / (zf - zn);
  S[1][1] = -1.0;
  S[2][2] = -1.0;
  const D4 proj = mul4(P, S), vp = mul4(proj, view);
  D4 inv_proj{}, inv_vp{};
  if (!inverse4(proj, &inv_proj) || !inverse4(vp, &inv_vp)) return -1;
  out->width = width;
  out->height = height;
  to_float(view, out->view);
  to_float(proj, out->proj);
  to_float(vp, out->view_proj);
  to_float(xf, out->inv_view);
  to_float(inv_proj, out->inv_proj);
  to_float(inv_vp, out->inv_view_proj);
  return 0;
}
