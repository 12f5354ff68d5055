// gi_host.cpp -- host-side parts of the C ABI: status strings, error reporting,
// mip geometry, view matrices, the procedural scene and the camera spline.
#include <cmath>
#include <cstring>
#include <random>
#include <string>

#include "gi_internal.h"

namespace gi {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return GI_OK;
  int st = (e == cudaErrorMemoryAllocation) ? GI_ERR_OUT_OF_MEMORY : GI_ERR_CUDA;
  return fail(st, std::string(what) + ": " + cudaGetErrorString(e));
}

void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static std::atomic<long long> g_live_allocations{0};
static std::atomic<int> g_allocs_before_failure{-1};  // -1: no failures injected

// True if the test hook says this allocation fails (the count of allocations
// still allowed reached 0; it stays there until the hook is reset).
static bool injected_failure() {
  int left = g_allocs_before_failure.load();
  while (left > 0 && !g_allocs_before_failure.compare_exchange_weak(left, left - 1)) {
  }
  return left == 0;
}

cudaError_t device_alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (injected_failure()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) g_live_allocations.fetch_add(1);
  return e;
}

void device_free(void* p) {
  if (p && cudaFree(p) == cudaSuccess) g_live_allocations.fetch_sub(1);
}

cudaError_t device_alloc_mipmapped(cudaMipmappedArray_t* a, const cudaChannelFormatDesc* desc, cudaExtent extent,
                                   unsigned levels, unsigned flags) {
  *a = nullptr;
  if (injected_failure()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMallocMipmappedArray(a, desc, extent, levels, flags);
  if (e == cudaSuccess) g_live_allocations.fetch_add(1);
  return e;
}

void device_free_mipmapped(cudaMipmappedArray_t a) {
  if (a && cudaFreeMipmappedArray(a) == cudaSuccess) g_live_allocations.fetch_sub(1);
}

// ---------------------------------------------------------------------------
// Double-precision 4x4 helpers, column-major m[c][r] (glm's layout).
struct M4 {
  double m[4][4];
};

static M4 ident() {
  M4 r{};
  for (int i = 0; i < 4; i++) r.m[i][i] = 1.0;
  return r;
}

static M4 mul(const M4& a, const M4& b) {
  M4 r{};
  for (int c = 0; c < 4; c++)
    for (int rr = 0; rr < 4; rr++) {
      double s = 0.0;
      for (int k = 0; k < 4; k++) s += a.m[k][rr] * b.m[c][k];
      r.m[c][rr] = s;
    }
  return r;
}

// Gauss-Jordan with partial pivoting; returns false for a singular matrix.
static bool inverse(const M4& a, M4* out) {
  double w[4][8];
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) {
      w[r][c] = a.m[c][r];
      w[r][c + 4] = (r == c) ? 1.0 : 0.0;
    }
  for (int col = 0; col < 4; col++) {
    int piv = col;
    for (int r = col + 1; r < 4; r++)
      if (std::fabs(w[r][col]) > std::fabs(w[piv][col])) piv = r;
    if (w[piv][col] == 0.0) return false;
    if (piv != col)
      for (int c = 0; c < 8; c++) std::swap(w[piv][c], w[col][c]);
    double d = w[col][col];
    for (int c = 0; c < 8; c++) w[col][c] /= d;
    for (int r = 0; r < 4; r++) {
      if (r == col) continue;
      double f = w[r][col];
      if (f == 0.0) continue;
      for (int c = 0; c < 8; c++) w[r][c] -= f * w[col][c];
    }
  }
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) out->m[c][r] = w[r][c + 4];
  return true;
}

static void store(const M4& a, float* dst) {
  for (int c = 0; c < 4; c++)
    for (int r = 0; r < 4; r++) dst[4 * c + r] = (float)a.m[c][r];
}

static M4 translate(double x, double y, double z) {
  M4 r = ident();
  r.m[3][0] = x;
  r.m[3][1] = y;
  r.m[3][2] = z;
  return r;
}

// glm::rotate(angle, axis) for the unit axes used by Camera (Scene.h:32).
static M4 rot_y(double a) {
  M4 r = ident();
  double c = std::cos(a), s = std::sin(a);
  r.m[0][0] = c;  r.m[0][2] = -s;
  r.m[2][0] = s;  r.m[2][2] = c;
  return r;
}
static M4 rot_x(double a) {
  M4 r = ident();
  double c = std::cos(a), s = std::sin(a);
  r.m[1][1] = c;  r.m[1][2] = s;
  r.m[2][1] = -s; r.m[2][2] = c;
  return r;
}

// glm 0.9.9 perspectiveRH_ZO (ext/matrix_clip_space.inl) times scale(1, -1, -1).
static M4 projection(double fovy, double aspect, double zn, double zf) {
  double th = std::tan(fovy / 2.0);
  M4 p{};
  p.m[0][0] = 1.0 / (aspect * th);
  p.m[1][1] = 1.0 / th;
  p.m[2][2] = zf / (zn - zf);
  p.m[2][3] = -1.0;
  p.m[3][2] = -(zf * zn) / (zf - zn);
  M4 s = ident();
  s.m[1][1] = -1.0;
  s.m[2][2] = -1.0;
  return mul(p, s);
}

// Uniform double in [0, 1) from the top 53 bits of one mt19937_64 output.
static double u01(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

static float rgba8(std::mt19937_64& g) {
  double v = 0.2 + 0.7 * u01(g);
  int q = (int)std::lround(v * 255.0);
  return (float)q / 255.0f;
}

}  // namespace gi

using namespace gi;

extern "C" {

int gi_abi_version(void) { return GI_ABI_VERSION; }

const char* gi_status_string(int s) {
  switch (s) {
    case GI_OK: return "ok";
    case GI_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GI_ERR_CUDA: return "CUDA error";
    case GI_ERR_OUT_OF_MEMORY: return "out of memory";
    case GI_ERR_UNSUPPORTED: return "unsupported";
    case GI_ERR_TIMEOUT: return "timeout";
    case GI_ERR_IO: return "I/O error";
    default: return "unknown status";
  }
}

const char* gi_last_error(void) { return g_last_error.c_str(); }

uint64_t gi_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int gi_debug_fail_allocations(int after) {
  GI_CHECK_ARG(after >= -1, "gi_debug_fail_allocations: after must be >= -1");
  g_allocs_before_failure.store(after);
  return GI_OK;
}

int gi_debug_live_allocations(long long* count) {
  GI_CHECK_ARG(count, "gi_debug_live_allocations: null");
  *count = g_live_allocations.load();
  return GI_OK;
}

int gi_mip_level_count(int width, int height, int requested) {
  if (width < 1 || height < 1 || requested < 1) return 0;
  int m = width < height ? width : height;
  int n = 0;
  while (m >= 1) {
    n++;
    m >>= 1;
  }
  if (requested > GI_MAX_LEVELS) requested = GI_MAX_LEVELS;
  return requested < n ? requested : n;
}

int gi_mip_level_size(int width, int height, int level, int* lw, int* lh) {
  GI_CHECK_ARG(width >= 1 && height >= 1 && level >= 0 && level < GI_MAX_LEVELS && lw && lh,
               "gi_mip_level_size: bad arguments");
  *lw = width >> level;
  *lh = height >> level;
  return GI_OK;
}

int gi_view_from_camera(const gi_camera* cam, int width, int height, gi_view* out) {
  GI_CHECK_ARG(cam && out && width > 0 && height > 0, "gi_view_from_camera: bad arguments");
  GI_CHECK_ARG(cam->znear > 0.0f && cam->zfar > cam->znear && cam->fovy > 0.0f,
               "gi_view_from_camera: bad projection");
  M4 xf = mul(mul(translate(cam->pos[0], cam->pos[1], cam->pos[2]), rot_y(cam->hor_angle)), rot_x(cam->vert_angle));
  M4 view, inv_view = xf;
  if (!inverse(xf, &view)) return fail(GI_ERR_INVALID_ARGUMENT, "gi_view_from_camera: singular camera");
  double aspect = (double)width / (double)height;
  M4 proj = projection(cam->fovy, aspect, cam->znear, cam->zfar);
  M4 vp = mul(proj, view), inv_proj, inv_vp;
  if (!inverse(proj, &inv_proj) || !inverse(vp, &inv_vp))
    return fail(GI_ERR_INVALID_ARGUMENT, "gi_view_from_camera: singular projection");
  out->width = width;
  out->height = height;
  store(view, out->view);
  store(proj, out->proj);
  store(vp, out->view_proj);
  store(inv_view, out->inv_view);
  store(inv_proj, out->inv_proj);
  store(inv_vp, out->inv_view_proj);
  return GI_OK;
}

int gi_scene_generate(uint64_t seed, int num_boxes, int num_spheres, gi_prim* prims, int max_prims, int* count) {
  GI_CHECK_ARG(prims && count && num_boxes >= 0 && num_spheres >= 0, "gi_scene_generate: bad arguments");
  int n = 1 + num_boxes + num_spheres;
  GI_CHECK_ARG(n <= max_prims && n <= GI_MAX_PRIMS, "gi_scene_generate: too many primitives");
  std::mt19937_64 g(seed);
  std::memset(prims, 0, sizeof(gi_prim) * (size_t)n);
  gi_prim& room = prims[0];
  room.kind = GI_PRIM_ROOM;
  for (int k = 0; k < 3; k++) {
    room.a[k] = 0.0f;
    room.b[k] = 1.0f;
  }
  for (int c = 0; c < 4; c++) room.albedo[c] = rgba8(g);
  // Objects stay below y = 0.85 so that the light at y = 0.93 is never inside one.
  const double top = 0.85;
  for (int i = 0; i < num_boxes; i++) {
    gi_prim& p = prims[1 + i];
    p.kind = GI_PRIM_BOX;
    for (int k = 0; k < 3; k++) {
      double s = 0.05 + 0.25 * u01(g);
      double lim = (k == 1) ? top : 1.0;
      double lo = u01(g) * (lim - s);
      p.a[k] = (float)lo;
      p.b[k] = (float)(lo + s);
    }
    for (int c = 0; c < 4; c++) p.albedo[c] = rgba8(g);
  }
  for (int i = 0; i < num_spheres; i++) {
    gi_prim& p = prims[1 + num_boxes + i];
    p.kind = GI_PRIM_SPHERE;
    double r = 0.05 + 0.15 * u01(g);
    for (int k = 0; k < 3; k++) {
      double lim = (k == 1) ? top : 1.0;
      p.a[k] = (float)(r + u01(g) * (lim - 2.0 * r));
    }
    p.b[0] = (float)r;
    for (int c = 0; c < 4; c++) p.albedo[c] = rgba8(g);
  }
  *count = n;
  return GI_OK;
}

int gi_scene_light(gi_camera* light) {
  GI_CHECK_ARG(light, "gi_scene_light: null");
  light->pos[0] = 0.5f;
  light->pos[1] = 0.93f;
  light->pos[2] = 0.5f;
  light->hor_angle = 0.0f;
  light->vert_angle = 3.1415f / 2.0f;  // main.cpp:168
  light->fovy = 1.6f;
  light->znear = 0.02f;
  light->zfar = 10.0f;
  return GI_OK;
}

// Distance from p to the primitive's surface, negative inside (boxes, spheres).
static double clearance(const gi_prim& q, const double* p) {
  if (q.kind == GI_PRIM_SPHERE) {
    double d2 = 0.0;
    for (int k = 0; k < 3; k++) d2 += (p[k] - q.a[k]) * (p[k] - q.a[k]);
    return std::sqrt(d2) - q.b[0];
  }
  if (q.kind == GI_PRIM_BOX) {
    double out2 = 0.0, in = -1e30;
    for (int k = 0; k < 3; k++) {
      double lo = q.a[k] - p[k], hi = p[k] - q.b[k];
      double e = std::max(lo, hi);
      if (e > 0.0) out2 += e * e;
      in = std::max(in, e);
    }
    return out2 > 0.0 ? std::sqrt(out2) : in;
  }
  return 1e30;
}

static int camera_spline_impl(uint64_t seed, const gi_prim* prims, int n, int frame, int num_frames,
                              gi_camera* cam) {
  std::mt19937_64 g(seed);
  const int K = 8;
  const double margin = 0.08;
  double P[K][3], Q[K][3];
  for (int i = 0; i < K; i++) {
    for (int attempt = 0; attempt < 2000; attempt++) {
      P[i][0] = 0.2 + 0.6 * u01(g);
      P[i][1] = 0.3 + 0.4 * u01(g);
      P[i][2] = 0.2 + 0.6 * u01(g);
      bool ok = true;
      for (int j = 0; prims && j < n && ok; j++) ok = clearance(prims[j], P[i]) >= margin;
      if (ok) break;
    }
    Q[i][0] = 0.1 + 0.8 * u01(g);
    Q[i][1] = 0.05 + 0.5 * u01(g);
    Q[i][2] = 0.1 + 0.8 * u01(g);
  }
  int f = ((frame % num_frames) + num_frames) % num_frames;
  double u = (double)f / (double)num_frames * K;
  int s = (int)std::floor(u);
  double t = u - s;
  auto cr = [&](double (*X)[3], int k) {
    double p0 = X[(s + K - 1) % K][k], p1 = X[s % K][k], p2 = X[(s + 1) % K][k], p3 = X[(s + 2) % K][k];
    return 0.5 * ((2.0 * p1) + (-p0 + p2) * t + (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3) * t * t +
                  (-p0 + 3.0 * p1 - 3.0 * p2 + p3) * t * t * t);
  };
  double pos[3], tgt[3];
  for (int k = 0; k < 3; k++) {
    pos[k] = cr(P, k);
    tgt[k] = cr(Q, k);
  }
  double fx = tgt[0] - pos[0], fy = tgt[1] - pos[1], fz = tgt[2] - pos[2];
  double l = std::sqrt(fx * fx + fy * fy + fz * fz);
  if (l < 1e-6) {
    fx = 0.0; fy = 0.0; fz = 1.0; l = 1.0;
  }
  fx /= l; fy /= l; fz /= l;
  // Camera forward is rotY(hor) * rotX(vert) * (0, 0, 1) = (cos v sin h, -sin v, cos v cos h).
  cam->pos[0] = (float)pos[0];
  cam->pos[1] = (float)pos[1];
  cam->pos[2] = (float)pos[2];
  cam->hor_angle = (float)std::atan2(fx, fz);
  cam->vert_angle = (float)std::asin(-fy);
  cam->fovy = 1.0f;  // SSVGIRenderer.h:57
  cam->znear = 0.01f;
  cam->zfar = 1000.0f;
  return GI_OK;
}

int gi_camera_spline(uint64_t seed, int frame, int num_frames, gi_camera* cam) {
  GI_CHECK_ARG(cam && num_frames > 0, "gi_camera_spline: bad arguments");
  return camera_spline_impl(seed, nullptr, 0, frame, num_frames, cam);
}

int gi_camera_spline_in_scene(uint64_t seed, const gi_prim* prims, int num_prims, int frame, int num_frames,
                              gi_camera* cam) {
  GI_CHECK_ARG(cam && num_frames > 0 && prims && num_prims >= 0, "gi_camera_spline_in_scene: bad arguments");
  return camera_spline_impl(seed, prims, num_prims, frame, num_frames, cam);
}

}  // extern "C"
