// gi_render_scene.cpp -- headless renderer of a scene file, the GB300 stand-in
// for the reference application's main loop (main.cpp:120-172 loads the scene,
// places the camera and the light and renders with SSVGIRenderer): one frame
// through the C ABI only -- gi_scene_load, the mesh G-buffer and shadow map, the
// direct light, the GI renderer (plain or learned) -- written as a PFM image.
//
//   gi_render_scene SCENE.json OUT.pfm [--width W] [--height H] [--dirs R]
//       [--cap C] [--bounces B] [--exact | --texture] [--learned WEIGHTS] [--two-sided]
//
// Prints one JSON line with the counts and the GPU times.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "legit_gi.h"

namespace {

struct Failure {
  std::string what;
};

void check(int status, const char* what) {
  if (status != GI_OK) throw Failure{std::string(what) + ": " + gi_last_error()};
}

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Failure{std::string(what) + ": " + cudaGetErrorString(e)};
}

struct DeviceBuffer {
  void* p = nullptr;
  explicit DeviceBuffer(size_t bytes) { check_cuda(cudaMalloc(&p, bytes ? bytes : 16), "cudaMalloc"); }
  ~DeviceBuffer() { cudaFree(p); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  float* f() const { return static_cast<float*>(p); }
};

// main.cpp:164-172 with the projections of SSVGIRenderer.h:57-59.
gi_camera camera() {
  gi_camera c{};
  c.pos[1] = 0.5f;
  c.pos[2] = -2.0f;
  c.fovy = 1.0f;
  c.znear = 0.01f;
  c.zfar = 1000.0f;
  return c;
}

gi_camera light() {
  gi_camera c{};
  c.pos[1] = 5.0f;
  c.vert_angle = 3.1415f / 2.0f;
  c.fovy = 0.8f;
  c.znear = 0.1f;
  c.zfar = 100.0f;
  return c;
}

// PFM: "PF", size, -1 (little endian), float RGB rows from the bottom up.
void write_pfm(const char* path, const std::vector<float>& rgba, int w, int h) {
  FILE* f = std::fopen(path, "wb");
  if (!f) throw Failure{std::string("cannot write ") + path};
  std::fprintf(f, "PF\n%d %d\n-1.0\n", w, h);
  std::vector<float> row(3 * (size_t)w);
  for (int y = h - 1; y >= 0; y--) {
    for (int x = 0; x < w; x++)
      for (int c = 0; c < 3; c++) row[3 * (size_t)x + c] = rgba[4 * ((size_t)y * w + x) + c];
    std::fwrite(row.data(), sizeof(float), row.size(), f);
  }
  std::fclose(f);
}

int run(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr,
                 "usage: %s SCENE.json OUT.pfm [--width W] [--height H] [--dirs R] [--cap C] [--bounces B] "
                 "[--exact | --texture] [--learned WEIGHTS] [--two-sided]\n",
                 argv[0]);
    return 2;
  }
  const char* scene_path = argv[1];
  const char* out_path = argv[2];
  int W = 1280, H = 720, dirs = 16, cap = 64, bounces = 2, precision = GI_MARCH_FAST, cull = GI_CULL_BACK;
  const char* weights = nullptr;
  for (int i = 3; i < argc; i++) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) throw Failure{"missing value after " + a};
      return argv[++i];
    };
    if (a == "--width") W = std::atoi(next());
    else if (a == "--height") H = std::atoi(next());
    else if (a == "--dirs") dirs = std::atoi(next());
    else if (a == "--cap") cap = std::atoi(next());
    else if (a == "--bounces") bounces = std::atoi(next());
    else if (a == "--exact") precision = GI_MARCH_EXACT;
    else if (a == "--texture") precision = GI_MARCH_TEXTURE;
    else if (a == "--learned") weights = next();
    else if (a == "--two-sided") cull = GI_CULL_NONE;
    else throw Failure{"unknown option " + a};
  }

  gi_scene* scene = nullptr;
  check(gi_scene_load(scene_path, &scene), "gi_scene_load");
  int nobj = 0, ntri = 0, ssize = 0;
  check(gi_scene_info(scene, &nobj, &ntri, &ssize), "gi_scene_info");
  std::vector<gi_mesh_object> objects((size_t)nobj);
  std::vector<gi_triangle> tris((size_t)ntri);
  check(gi_scene_copy(scene, objects.data(), tris.data()), "gi_scene_copy");
  gi_scene_destroy(scene);

  const size_t px = (size_t)W * H;
  DeviceBuffer d_obj(objects.size() * sizeof(gi_mesh_object)), d_tri(tris.size() * sizeof(gi_triangle));
  check_cuda(cudaMemcpy(d_obj.p, objects.data(), objects.size() * sizeof(gi_mesh_object), cudaMemcpyHostToDevice),
             "objects H2D");
  check_cuda(cudaMemcpy(d_tri.p, tris.data(), tris.size() * sizeof(gi_triangle), cudaMemcpyHostToDevice),
             "triangles H2D");
  DeviceBuffer albedo(px * 16), emissive(px * 16), normal(px * 16), moments(px * 8), ndc(px * 4), direct(px * 16),
      lit(px * 16), shadow((size_t)ssize * ssize * 4);

  gi_view view, light_view;
  const gi_camera cam = camera(), lcam = light();
  check(gi_view_from_camera(&cam, W, H, &view), "gi_view_from_camera");
  check(gi_view_from_camera(&lcam, ssize, ssize, &light_view), "gi_view_from_camera");

  gi_frame_params fp{};
  fp.march.dirs = dirs;
  fp.march.step_cap = cap;
  fp.march.pattern_size = 4;
  fp.march.precision = precision;
  fp.bounces = bounces;
  fp.bilateral = 1;
  fp.mip_levels = 10;
  gi_renderer* r = nullptr;
  check(gi_renderer_create(W, H, &fp, &r), "gi_renderer_create");
  gi_mlp* net = nullptr;
  if (weights) {
    check(gi_mlp_create(&net), "gi_mlp_create");
    check(gi_mlp_load(net, weights), "gi_mlp_load");
    check(gi_renderer_set_learned(r, net, 1, 32, 64, 0.25f), "gi_renderer_set_learned");
  }

  cudaStream_t s;
  check_cuda(cudaStreamCreate(&s), "cudaStreamCreate");
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  cudaEventRecord(e0, s);
  check(gi_gbuffer_mesh(&view, nullptr, 0, static_cast<gi_mesh_object*>(d_obj.p), nobj,
                        static_cast<gi_triangle*>(d_tri.p), ntri, cull, albedo.f(), emissive.f(), normal.f(),
                        moments.f(), ndc.f(), s),
        "gi_gbuffer_mesh");
  check(gi_shadow_map_mesh(&light_view, nullptr, 0, static_cast<gi_mesh_object*>(d_obj.p), nobj,
                           static_cast<gi_triangle*>(d_tri.p), ntri, cull, shadow.f(), s),
        "gi_shadow_map_mesh");
  check(gi_direct_light(&view, &light_view, albedo.f(), emissive.f(), normal.f(), ndc.f(), shadow.f(), ssize,
                        direct.f(), s),
        "gi_direct_light");
  cudaEventRecord(e1, s);
  const gi_frame_inputs in{albedo.f(), normal.f(), moments.f(), ndc.f(), direct.f()};
  check(gi_renderer_render(r, &view, &in, lit.f(), nullptr, s), "gi_renderer_render");
  cudaEventRecord(e2, s);
  std::vector<float> host(px * 4);
  check_cuda(cudaMemcpyAsync(host.data(), lit.p, px * 16, cudaMemcpyDeviceToHost, s), "lit D2H");
  check_cuda(cudaStreamSynchronize(s), "render");
  float t_in = 0.0f, t_gi = 0.0f;
  cudaEventElapsedTime(&t_in, e0, e1);
  cudaEventElapsedTime(&t_gi, e1, e2);
  write_pfm(out_path, host, W, H);
  std::printf(
      "{\"scene\": \"%s\", \"out\": \"%s\", \"width\": %d, \"height\": %d, \"objects\": %d, \"triangles\": %d, "
      "\"method\": \"%s\", \"dirs\": %d, \"bounces\": %d, \"precision\": \"%s\", \"inputs_ms\": %.4f, "
      "\"gi_ms\": %.4f}\n",
      scene_path, out_path, W, H, nobj, ntri, weights ? "learned" : "plain", dirs, bounces,
      precision == GI_MARCH_FAST ? "fast" : (precision == GI_MARCH_TEXTURE ? "texture" : "exact"), t_in, t_gi);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaStreamDestroy(s);
  gi_renderer_destroy(r);
  if (net) gi_mlp_destroy(net);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const Failure& f) {
    std::fprintf(stderr, "gi_render_scene: %s\n", f.what.c_str());
    return 1;
  }
}
