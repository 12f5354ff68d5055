// gi_inputs.cu -- the passes that feed the GI path (SSVGIRenderer.h:61-205):
// G-buffer, shadow map and direct light.  The reference rasterises meshes; here
// the scene is ray cast through the pixel centres, one thread per pixel: the
// procedural primitives (boxes and spheres inside a room) staged in shared
// memory, then the triangle meshes of a loaded scene, object by object behind a
// bounds test.
#include "gi_device.cuh"
#include "gi_internal.h"
#include "gi_kernels.h"

namespace gi {
namespace {

using namespace dev;

constexpr int kTx = 32, kTy = 4;
constexpr int kPrimStage = 256;  // primitives staged per shared-memory batch

struct ViewArgs {
  Mat4 inv_view_proj, inv_view, view_proj, view;
  int width, height;
};

ViewArgs view_args(const gi_view& v) {
  ViewArgs a;
  for (int k = 0; k < 16; k++) {
    a.inv_view_proj.m[k] = v.inv_view_proj[k];
    a.inv_view.m[k] = v.inv_view[k];
    a.view_proj.m[k] = v.view_proj[k];
    a.view.m[k] = v.view[k];
  }
  a.width = v.width;
  a.height = v.height;
  return a;
}

struct Hit {
  float t;
  f3 n;
  int prim;  // analytic primitive hit, or -1
  int tri;   // triangle hit (when prim == -1), or -1
  int obj;   // the triangle's object
  float u, v;
};

// Triangle meshes of a loaded scene (num_objects == 0: none).
struct MeshSet {
  const gi_mesh_object* objects;
  const gi_triangle* tris;
  int num_objects;
  int cull;  // GI_CULL_BACK: only triangles whose right-hand winding faces the ray (det > 0)
};

__device__ __forceinline__ f3 ld3(const float (&p)[3]) { return mk3(__ldg(p + 0), __ldg(p + 1), __ldg(p + 2)); }

// The mesh part of the ray cast: each object's bounds (slab test), then its
// triangles (Moller-Trumbore, t > 0, nearer than the hit so far).
__device__ void cast_mesh(const MeshSet& m, f3 o, f3 d, const float (&iv)[3], Hit& h) {
  const float ov[3] = {o.x, o.y, o.z};
  for (int k = 0; k < m.num_objects; k++) {
    const gi_mesh_object& ob = m.objects[k];
    float tn = 0.0f, tf = h.t;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float a = (__ldg(ob.lo + c) - ov[c]) * iv[c];
      const float b = (__ldg(ob.hi + c) - ov[c]) * iv[c];
      tn = gmax(tn, gmin(a, b));
      tf = gmin(tf, gmax(a, b));
    }
    if (!(tn <= tf)) continue;
    const int first = __ldg(&ob.first), count = __ldg(&ob.count);
    for (int i = first; i < first + count; i++) {
      const gi_triangle& tr = m.tris[i];
      const f3 p0 = ld3(tr.p[0]);
      const f3 e1 = sub3(ld3(tr.p[1]), p0), e2 = sub3(ld3(tr.p[2]), p0);
      const f3 pv = cross3(d, e2);
      const float det = dot3(e1, pv);  // -d . (e1 x e2): > 0 when the ray meets the front face
      if (m.cull ? !(det > 0.0f) : det == 0.0f) continue;
      const float inv = rcp_(det);
      const f3 tv = sub3(o, p0);
      const float u = dot3(tv, pv) * inv;
      if (u < 0.0f || u > 1.0f) continue;
      const f3 qv = cross3(tv, e1);
      const float v = dot3(d, qv) * inv;
      if (v < 0.0f || u + v > 1.0f) continue;
      const float t = dot3(e2, qv) * inv;
      if (t > 0.0f && t < h.t) {
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

// Nearest hit: room interior (exit face), box exterior (entry face), sphere
// (near root), ties kept by the earlier primitive.
__device__ void cast_ray(const gi_prim* __restrict__ prims, int np, const MeshSet& mesh, f3 o, f3 d, Hit& h,
                         gi_prim* s_prims) {
  h.t = __int_as_float(0x7f800000);
  h.prim = -1;
  h.tri = -1;
  h.obj = -1;
  h.u = h.v = 0.0f;
  h.n = mk3(0.0f, 0.0f, 0.0f);
  const float iv[3] = {rcp_(d.x), rcp_(d.y), rcp_(d.z)};
  const float ov[3] = {o.x, o.y, o.z};
  const float dv[3] = {d.x, d.y, d.z};
  for (int base = 0; base < np; base += kPrimStage) {
    const int cnt = min(kPrimStage, np - base);
    __syncthreads();
    for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < cnt; i += blockDim.x * blockDim.y)
      s_prims[i] = prims[base + i];
    __syncthreads();
    for (int ii = 0; ii < cnt; ii++) {
      const gi_prim& p = s_prims[ii];
      const int i = base + ii;
      if (p.kind == GI_PRIM_ROOM || p.kind == GI_PRIM_BOX) {
        float t1[3], t2[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
          float a = (p.a[k] - ov[k]) * iv[k];
          float b = (p.b[k] - ov[k]) * iv[k];
          t1[k] = gmin(a, b);
          t2[k] = gmax(a, b);
        }
        if (p.kind == GI_PRIM_ROOM) {
          int ax = 0;
          float tf = t2[0];
          if (t2[1] < tf) { ax = 1; tf = t2[1]; }
          if (t2[2] < tf) { ax = 2; tf = t2[2]; }
          if (tf > 0.0f && tf < h.t) {
            h.t = tf;
            h.prim = i;
            float nv[3] = {0.0f, 0.0f, 0.0f};
            nv[ax] = dv[ax] > 0.0f ? -1.0f : 1.0f;
            h.n = mk3(nv[0], nv[1], nv[2]);
          }
        } else {
          int ax = 0;
          float tn = t1[0];
          if (t1[1] > tn) { ax = 1; tn = t1[1]; }
          if (t1[2] > tn) { ax = 2; tn = t1[2]; }
          float tf = gmin(gmin(t2[0], t2[1]), t2[2]);
          if (tn <= tf && tn > 0.0f && tn < h.t) {
            h.t = tn;
            h.prim = i;
            float nv[3] = {0.0f, 0.0f, 0.0f};
            nv[ax] = dv[ax] > 0.0f ? -1.0f : 1.0f;
            h.n = mk3(nv[0], nv[1], nv[2]);
          }
        }
      } else if (p.kind == GI_PRIM_SPHERE) {
        const f3 c = mk3(p.a[0], p.a[1], p.a[2]);
        const float r = p.b[0];
        const f3 oc = sub3(o, c);
        const float b = dot3(oc, d);
        const float cc = dot3(oc, oc) - r * r;
        const float disc = b * b - cc;
        if (disc >= 0.0f) {
          const float t = -b - sqrtf(disc);
          if (t > 0.0f && t < h.t) {
            h.t = t;
            h.prim = i;
            h.n = normalize3(sub3(add3(o, mul3s(d, t)), c));
          }
        }
      }
    }
  }
  if (mesh.num_objects > 0) cast_mesh(mesh, o, d, iv, h);
}

// gBufferBuilder.frag:28-38 at the primary hit.
__global__ void __launch_bounds__(kTx* kTy) gbuffer_kernel(const __grid_constant__ ViewArgs v,
                                                           const gi_prim* __restrict__ prims, int np, MeshSet mesh,
                                                           float* __restrict__ albedo, float* __restrict__ emissive,
                                                           float* __restrict__ normal, float* __restrict__ moments,
                                                           float* __restrict__ ndc) {
  __shared__ gi_prim s_prims[kPrimStage];
  const int x = blockIdx.x * kTx + threadIdx.x, y = blockIdx.y * kTy + threadIdx.y;
  const bool live = x < v.width && y < v.height;
  const int xc = live ? x : 0, yc = live ? y : 0;
  const float sx = div_((float)xc + 0.5f, (float)v.width), sy = div_((float)yc + 0.5f, (float)v.height);
  const float4 cam4 = mat_vec(v.inv_view, 0.0f, 0.0f, 0.0f, 1.0f);
  const f3 cam = mk3(cam4.x, cam4.y, cam4.z);
  const f3 farp = unproject(v.inv_view_proj, sx, sy, 1.0f);
  const f3 dir = normalize3(sub3(farp, cam));
  Hit h;
  cast_ray(prims, np, mesh, cam, dir, h, s_prims);  // every thread joins the staging barriers
  if (!live) return;
  const size_t i = (size_t)y * v.width + x;
  if (h.prim < 0 && h.tri < 0) {
    reinterpret_cast<float4*>(albedo)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    reinterpret_cast<float4*>(emissive)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    reinterpret_cast<float4*>(normal)[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    reinterpret_cast<float2*>(moments)[i] = make_float2(0.0f, 0.0f);
    ndc[i] = 1.0f;
    return;
  }
  const f3 hit = add3(cam, mul3s(dir, h.t));
  const f3 dl = sub3(hit, cam);
  const float delta_len = sqrtf(dot3(dl, dl));
  const float* src_al;
  const float* src_em;
  if (h.prim >= 0) {
    src_al = prims[h.prim].albedo;
    src_em = prims[h.prim].emissive;
  } else {
    src_al = mesh.objects[h.obj].albedo;
    src_em = mesh.objects[h.obj].emissive;
    // Barycentric blend of the vertex normals, (1 - u - v) n0 + u n1 + v n2.
    const gi_triangle& tr = mesh.tris[h.tri];
    const float w0 = 1.0f - h.u - h.v;
    const f3 n0 = ld3(tr.n[0]), n1 = ld3(tr.n[1]), n2 = ld3(tr.n[2]);
    h.n = add3(add3(mul3s(n0, w0), mul3s(n1, h.u)), mul3s(n2, h.v));
  }
  float4 al, em;
  al.x = powf_(src_al[0], 2.2f);
  al.y = powf_(src_al[1], 2.2f);
  al.z = powf_(src_al[2], 2.2f);
  al.w = powf_(src_al[3], 2.2f);
  em.x = powf_(src_em[0], 2.2f);
  em.y = powf_(src_em[1], 2.2f);
  em.z = powf_(src_em[2], 2.2f);
  em.w = powf_(src_em[3], 2.2f);
  reinterpret_cast<float4*>(albedo)[i] = al;
  reinterpret_cast<float4*>(emissive)[i] = em;
  reinterpret_cast<float4*>(normal)[i] = make_float4(h.n.x, h.n.y, h.n.z, 1.0f);
  reinterpret_cast<float2*>(moments)[i] = make_float2(delta_len, delta_len * delta_len);
  ndc[i] = project(v.view_proj, hit).z;
}

__global__ void __launch_bounds__(kTx* kTy) shadow_kernel(const __grid_constant__ ViewArgs v,
                                                          const gi_prim* __restrict__ prims, int np, MeshSet mesh,
                                                          float* __restrict__ out) {
  __shared__ gi_prim s_prims[kPrimStage];
  const int x = blockIdx.x * kTx + threadIdx.x, y = blockIdx.y * kTy + threadIdx.y;
  const bool live = x < v.width && y < v.height;
  const int xc = live ? x : 0, yc = live ? y : 0;
  const float sx = div_((float)xc + 0.5f, (float)v.width), sy = div_((float)yc + 0.5f, (float)v.height);
  const float4 o4 = mat_vec(v.inv_view, 0.0f, 0.0f, 0.0f, 1.0f);
  const f3 org = mk3(o4.x, o4.y, o4.z);
  const f3 farp = unproject(v.inv_view_proj, sx, sy, 1.0f);
  const f3 dir = normalize3(sub3(farp, org));
  Hit h;
  cast_ray(prims, np, mesh, org, dir, h, s_prims);
  if (!live) return;
  float z = 1.0f;
  if (h.prim >= 0 || h.tri >= 0) z = project(v.view_proj, add3(org, mul3s(dir, h.t))).z;
  out[(size_t)y * v.width + x] = z;
}

// directLighting.frag:45-79.
__global__ void __launch_bounds__(kTx* kTy) direct_kernel(const __grid_constant__ ViewArgs v,
                                                          const __grid_constant__ ViewArgs lv,
                                                          const float* __restrict__ albedo,
                                                          const float* __restrict__ emissive,
                                                          const float* __restrict__ normal,
                                                          const float* __restrict__ ndc,
                                                          const float* __restrict__ shadow, int ssize,
                                                          float* __restrict__ out) {
  const int x = blockIdx.x * kTx + threadIdx.x, y = blockIdx.y * kTy + threadIdx.y;
  if (x >= v.width || y >= v.height) return;
  const int W = v.width, H = v.height;
  const float fx = div_((float)x + 0.5f, (float)W), fy = div_((float)y + 0.5f, (float)H);
  const float depth = sample1(ndc, W, H, fx, fy);
  const float4 n4 = sample4(normal, W, H, fx, fy);
  const f3 wn = mk3(n4.x, n4.y, n4.z);
  const float4 lp4 = mat_vec(lv.inv_view, 0.0f, 0.0f, 0.0f, 1.0f);
  const f3 light_pos = mk3(lp4.x, lp4.y, lp4.z);
  const f3 wp = unproject(v.inv_view_proj, fx, fy, depth);
  const f3 lvec = sub3(wp, light_pos);
  const float diffuse = gmax(0.0f, -dot3(normalize3(lvec), wn));
  f3 sc = project(lv.view_proj, wp);
  const float4 lvp = mat_vec(lv.view, wp.x, wp.y, wp.z, 1.0f);
  f3 li = mk3(5.0f, 5.0f, 5.0f);
  const float rx = sc.x - 0.5f, ry = sc.y - 0.5f;
  const float radius = sqrtf(rx * rx + ry * ry) * 2.0f;
  float t = div_(1.0f - saturate(div_(radius - 0.6f, 1.0f - 0.6f)) - 0.0f, 1.0f - 0.0f);
  t = gmin(gmax(t, 0.0f), 1.0f);
  const float penumbra = t * t * (3.0f - 2.0f * t) * (lvp.z > 0.0f ? 1.0f : 0.0f);
  li = mul3s(li, penumbra);
  const float bias = 2e-4f;
  sc.z = sc.z - bias;
  // sampler2DShadow, linear, compare LESS_OR_EQUAL.
  float pcf;
  {
    const Bilin B = bilin(sc.x, sc.y, ssize, ssize);
    const float r = sc.z;
    const float p00 = r <= __ldg(shadow + B.o00) ? 1.0f : 0.0f;
    const float p10 = r <= __ldg(shadow + B.o10) ? 1.0f : 0.0f;
    const float p01 = r <= __ldg(shadow + B.o01) ? 1.0f : 0.0f;
    const float p11 = r <= __ldg(shadow + B.o11) ? 1.0f : 0.0f;
    pcf = blend1(B, p00, p10, p01, p11);
  }
  li = mul3s(li, powf_(pcf, 2.2f));
  const float4 al = sample4(albedo, W, H, fx, fy);
  const float4 em = sample4(emissive, W, H, fx, fy);
  float4 o;
  o.x = diffuse * al.x * li.x + em.x;
  o.y = diffuse * al.y * li.y + em.y;
  o.z = diffuse * al.z * li.z + em.z;
  o.w = 1.0f;
  reinterpret_cast<float4*>(out)[(size_t)y * W + x] = o;
}

dim3 grid2d(int w, int h) { return dim3((w + kTx - 1) / kTx, (h + kTy - 1) / kTy); }

}  // namespace
}  // namespace gi

using namespace gi;

extern "C" int gi_gbuffer(const gi_view* view, const gi_prim* prims, int num_prims, float* albedo, float* emissive,
                          float* normal, float* depth_moments, float* ndc_depth, void* stream) {
  GI_CHECK_ARG(view && prims && albedo && emissive && normal && depth_moments && ndc_depth, "gi_gbuffer: null");
  GI_CHECK_ARG(num_prims >= 1 && num_prims <= GI_MAX_PRIMS, "gi_gbuffer: bad primitive count");
  GI_CHECK_ARG(view->width >= 1 && view->height >= 1, "gi_gbuffer: bad viewport");
  GI_CHECK_ARG(aligned16(albedo) && aligned16(emissive) && aligned16(normal) && aligned16(depth_moments),
               "gi_gbuffer: unaligned buffer");
  ViewArgs v = view_args(*view);
  gbuffer_kernel<<<grid2d(v.width, v.height), dim3(kTx, kTy), 0, (cudaStream_t)stream>>>(
      v, prims, num_prims, MeshSet{nullptr, nullptr, 0, 0}, albedo, emissive, normal, depth_moments, ndc_depth);
  GI_CHECK_LAUNCH("gbuffer_kernel");
  count_launches(1);
  return GI_OK;
}

static int check_mesh(const gi_prim* prims, int num_prims, const gi_mesh_object* objects, int num_objects,
                      const gi_triangle* tris, int num_tris, const char* who) {
  GI_CHECK_ARG(num_prims >= 0 && num_prims <= GI_MAX_PRIMS && (num_prims == 0 || prims), who);
  GI_CHECK_ARG(num_objects >= 0 && num_objects <= GI_MAX_MESH_OBJECTS && (num_objects == 0 || (objects && tris)),
               who);
  GI_CHECK_ARG(num_tris >= 0 && num_tris <= GI_MAX_TRIANGLES, who);
  GI_CHECK_ARG(num_prims + num_objects >= 1, who);
  return GI_OK;
}

extern "C" int gi_gbuffer_mesh(const gi_view* view, const gi_prim* prims, int num_prims,
                               const gi_mesh_object* objects, int num_objects, const gi_triangle* tris, int num_tris,
                               int cull, float* albedo, float* emissive, float* normal, float* depth_moments, float* ndc_depth,
                               void* stream) {
  GI_CHECK_ARG(view && albedo && emissive && normal && depth_moments && ndc_depth, "gi_gbuffer_mesh: null");
  int st = check_mesh(prims, num_prims, objects, num_objects, tris, num_tris, "gi_gbuffer_mesh: bad scene arrays");
  if (st) return st;
  GI_CHECK_ARG(cull == GI_CULL_NONE || cull == GI_CULL_BACK, "gi_gbuffer_mesh: unknown cull mode");
  GI_CHECK_ARG(view->width >= 1 && view->height >= 1, "gi_gbuffer_mesh: bad viewport");
  GI_CHECK_ARG(aligned16(albedo) && aligned16(emissive) && aligned16(normal) && aligned16(depth_moments),
               "gi_gbuffer_mesh: unaligned buffer");
  ViewArgs v = view_args(*view);
  gbuffer_kernel<<<grid2d(v.width, v.height), dim3(kTx, kTy), 0, (cudaStream_t)stream>>>(
      v, prims, num_prims, MeshSet{objects, tris, num_objects, cull}, albedo, emissive, normal, depth_moments, ndc_depth);
  GI_CHECK_LAUNCH("gbuffer_kernel");
  count_launches(1);
  return GI_OK;
}

extern "C" int gi_shadow_map_mesh(const gi_view* light_view, const gi_prim* prims, int num_prims,
                                  const gi_mesh_object* objects, int num_objects, const gi_triangle* tris,
                                  int num_tris, int cull, float* shadow, void* stream) {
  GI_CHECK_ARG(light_view && shadow, "gi_shadow_map_mesh: null");
  int st = check_mesh(prims, num_prims, objects, num_objects, tris, num_tris, "gi_shadow_map_mesh: bad scene arrays");
  if (st) return st;
  GI_CHECK_ARG(cull == GI_CULL_NONE || cull == GI_CULL_BACK, "gi_shadow_map_mesh: unknown cull mode");
  ViewArgs v = view_args(*light_view);
  shadow_kernel<<<grid2d(v.width, v.height), dim3(kTx, kTy), 0, (cudaStream_t)stream>>>(
      v, prims, num_prims, MeshSet{objects, tris, num_objects, cull}, shadow);
  GI_CHECK_LAUNCH("shadow_kernel");
  count_launches(1);
  return GI_OK;
}

extern "C" int gi_shadow_map(const gi_view* light_view, const gi_prim* prims, int num_prims, float* shadow,
                             void* stream) {
  GI_CHECK_ARG(light_view && prims && shadow, "gi_shadow_map: null");
  GI_CHECK_ARG(num_prims >= 1 && num_prims <= GI_MAX_PRIMS, "gi_shadow_map: bad primitive count");
  ViewArgs v = view_args(*light_view);
  shadow_kernel<<<grid2d(v.width, v.height), dim3(kTx, kTy), 0, (cudaStream_t)stream>>>(
      v, prims, num_prims, MeshSet{nullptr, nullptr, 0, 0}, shadow);
  GI_CHECK_LAUNCH("shadow_kernel");
  count_launches(1);
  return GI_OK;
}

extern "C" int gi_direct_light(const gi_view* view, const gi_view* light_view, const float* albedo,
                               const float* emissive, const float* normal, const float* ndc_depth, const float* shadow,
                               int shadow_size, float* out, void* stream) {
  GI_CHECK_ARG(view && light_view && albedo && emissive && normal && ndc_depth && shadow && out,
               "gi_direct_light: null");
  GI_CHECK_ARG(shadow_size >= 1, "gi_direct_light: bad shadow size");
  GI_CHECK_ARG(aligned16(albedo) && aligned16(emissive) && aligned16(normal) && aligned16(out),
               "gi_direct_light: unaligned buffer");
  ViewArgs v = view_args(*view), lv = view_args(*light_view);
  direct_kernel<<<grid2d(v.width, v.height), dim3(kTx, kTy), 0, (cudaStream_t)stream>>>(
      v, lv, albedo, emissive, normal, ndc_depth, shadow, shadow_size, out);
  GI_CHECK_LAUNCH("direct_kernel");
  count_launches(1);
  return GI_OK;
}
