/*
 * legit_gi.h -- C ABI of the GB300 screen-space global-illumination path.
 *
 * The reference (LegitEngine, src/Render) drives this path through C++ pass
 * builders that record full-screen draws into a Vulkan render graph.  Each entry
 * point below replaces one of those builders or shader passes; the citation in
 * front of it names the reference code it stands in for.  A C++ render-graph
 * shim with the reference's AddPass/RenderPassDesc/record-function surface sits
 * on top (legitengine_gb300/csrc/legit_render_graph.h).
 *
 * Conventions
 *  - Every function returns int: 0 (GI_OK) or a gi_status code; nothing throws
 *    across this boundary.  gi_last_error() returns a message for the calling
 *    thread's last failure.
 *  - Image buffers are caller-owned CUDA device memory, fp32, row-major, channels
 *    interleaved (1, 2 or 4 floats per pixel), tightly packed: the element of
 *    pixel (x, y), channel c is at ((y * width + x) * channels + c).  Buffers must
 *    be 16-byte aligned.
 *  - A pyramid is passed as a host array of device pointers, one per mip level;
 *    level k has size gi_mip_level_size(width, height, k).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    asynchronous with respect to the host and ordered on that stream.
 *  - Matrices are column-major float[16], as glm stores them.
 */
#ifndef LEGIT_GI_H
#define LEGIT_GI_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GI_API __attribute__((visibility("default")))
#else
#define GI_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GI_ABI_VERSION 1
#define GI_MAX_LEVELS 16
#define GI_MAX_DIRS 256         /* directions per pixel accepted by the GPU march */
#define GI_MAX_STEPS 512        /* steps per direction accepted by the GPU march */
#define GI_MAX_PRIMS 1024

typedef enum gi_status {
  GI_OK = 0,
  GI_ERR_INVALID_ARGUMENT = 1,
  GI_ERR_CUDA = 2,
  GI_ERR_OUT_OF_MEMORY = 3,
  GI_ERR_UNSUPPORTED = 4,
  GI_ERR_TIMEOUT = 5,
  GI_ERR_IO = 6
} gi_status;

/* Library identity and error reporting. */
GI_API int gi_abi_version(void);
GI_API const char* gi_status_string(int status);
GI_API const char* gi_last_error(void);
/* Number of CUDA kernel launches this library has issued in this process. */
GI_API uint64_t gi_launch_count(void);
/* Test hooks of allocation failure (no counterpart in the reference; the
 * reference's only recovery path is its swapchain reset, main.cpp:314-318).
 * Every device allocation of the library (images of the render graph, pyramid
 * textures, staging and record buffers, networks, batches) goes through one
 * allocator.  gi_debug_fail_allocations(after): the next `after` allocations
 * succeed and every later one fails as out of memory (GI_ERR_OUT_OF_MEMORY)
 * until the hook is called again; after = -1 turns failures off (the default).
 * gi_debug_live_allocations: how many of those allocations are live. */
GI_API int gi_debug_fail_allocations(int after);
GI_API int gi_debug_live_allocations(long long* count);

/* ---------------------------------------------------------------------------
 * Mip pyramid geometry.
 * Replaces MippedProxy's fixed `mipsCount = 10` (src/Render/Common/MipBuilder.h:21)
 * and the level loop of MipBuilder::BuildMips (MipBuilder.h:146-152): level k
 * is floor(size_{k-1} / 2) in each axis.  The count is min(requested,
 * floor(log2(min(w, h))) + 1), so that no level has a zero extent (the
 * reference requests 10 levels even where fewer exist).
 */
GI_API int gi_mip_level_count(int width, int height, int requested);
GI_API int gi_mip_level_size(int width, int height, int level, int* level_width, int* level_height);

typedef enum gi_mip_filter {
  GI_MIP_AVG = 0,   /* 2x2 mean (mipLevelBuilder.frag:22-28) */
  GI_MIP_DEPTH = 1  /* (min .x, max .y, mass .z, 0) (mipLevelBuilder.frag:29-42) */
} gi_mip_filter;

/* Replaces MipBuilder::BuildMips (MipBuilder.h:142-181) with
 * Common/mipLevelBuilder.frag:17-43: levels[0] is read, levels[1..n-1] written.
 * All levels are built by one fused launch plus one tail launch. */
GI_API int gi_build_mips(float* const* levels, int width, int height, int channels, int num_levels,
                  int filter, void* stream);

/* Replaces BlurBuilder::ApplyBlur (src/Render/Common/BlurBuilder.h:14-46) with
 * Common/blurLayerBuilder.frag:17-35: box mean over taps [-r, r) x [-r, r),
 * clamp-to-edge; radius 0 copies. */
GI_API int gi_blur(const float* src, float* dst, int width, int height, int channels, int radius,
            void* stream);

/* Replaces the two blur loops of SSVGIRenderer::RenderFrame
 * (src/Render/Renderers/SSVGIRenderer.h:209-221): every level of a pyramid,
 * radius 0 at level 0 and 2 above, in one launch.  dst_levels[0] may equal
 * src_levels[0] (the radius-0 copy is then skipped). */
GI_API int gi_blur_pyramid(const float* const* src_levels, float* const* dst_levels, int width, int height,
                    int channels, int num_levels, void* stream);

/* Replace InterleaveBuilder::Deinterleave / ::Interleave
 * (src/Render/Common/InterleaveBuilder.h:14-46, :48-80) with
 * Common/deinterleave.frag:16-28 and Common/interleave.frag:15-27.  The image is
 * split into grid_x * grid_y sub-images of (width / grid_x) x (height / grid_y);
 * width and height must be multiples of the grid. */
GI_API int gi_deinterleave(const float* src, float* dst, int width, int height, int channels, int grid_x,
                    int grid_y, void* stream);
GI_API int gi_interleave(const float* src, float* dst, int width, int height, int channels, int grid_x,
                  int grid_y, void* stream);

/* ---------------------------------------------------------------------------
 * Views.  The UBO of the indirect pass is {view, proj, viewportSize}
 * (SSVGI/indirectLighting.frag:4-9, SSVGIRenderer.h:473-487).  The shader
 * inverts the matrices per pixel (indirectLighting.frag:123-126); here the host
 * computes them once, in double precision rounded to float.
 */
typedef struct gi_view {
  int width, height;
  float view[16];           /* world -> camera */
  float proj[16];           /* camera -> clip */
  float view_proj[16];      /* proj * view */
  float inv_view[16];
  float inv_proj[16];
  float inv_view_proj[16];
} gi_view;

/* Scene.h:20-34 Camera {pos, vertAngle, horAngle} and the projection of
 * SSVGIRenderer.h:57: perspective(fovy, aspect, znear, zfar) * scale(1, -1, -1),
 * right-handed, depth range [0, 1]. */
typedef struct gi_camera {
  float pos[3];
  float hor_angle, vert_angle;
  float fovy, znear, zfar;
} gi_camera;

GI_API int gi_view_from_camera(const gi_camera* cam, int width, int height, gi_view* out);

/* ---------------------------------------------------------------------------
 * The indirect march: SSVGI/indirectLighting.frag:114-271, pass
 * SSVGIRenderer.h:224-263.
 */
typedef struct gi_march_params {
  int dirs;          /* directions per pixel; the reference's dirsCount = 4 (:166) */
  int step_cap;      /* upper bound on steps per direction; 0 = none */
  int pattern_size;  /* interleaved pattern edge; the reference's 4 (:141) */
  int step_dirs;     /* the direction count of the step growth, step count and mip
                        level formulas (:212, :217, :234-235); 0 = dirs, as in the
                        reference.  With dirs = 2 and step_dirs = 32 each pixel takes 2
                        of the 32 directions of its 4x4 pattern block, stepped at the
                        block's angular density. */
  int precision;     /* GI_MARCH_EXACT (0): the fixed-order fp32 evaluation contract,
                        bit-identical to the CPU restatement.  GI_MARCH_FAST (1): the
                        step loop uses the hardware reciprocal square root and
                        reciprocal, a fitted atan polynomial and fused multiply-adds --
                        within 1e-3 relative per pixel of the exact result; step
                        counts, mip selection and texel indices stay exact.  FAST
                        applies to the standard form with 2-channel depth moments;
                        other forms run exact.  The renderer and the batch also run
                        their bilateral filters with the hardware exponential when
                        FAST.  GI_MARCH_TEXTURE (2): the FAST step loop with its depth
                        and light taps fetched by the texture units (one trilinear
                        fetch at the step's level, 8-bit sub-texel and level weights,
                        as the reference's textureLod on its GPU; later bounces re-light
                        their recorded march with software taps).  The renderer and the
                        batch keep the pyramids as textures; gi_march, gi_march_tiles
                        and gi_march_autotune copy the caller's pyramids into a
                        library-owned pair per device first (calls ordered across
                        streams by an event, except under stream capture).  Under
                        stream capture the pair must already exist for the call's
                        shape (width, height, level count): make it with an eager call
                        of that shape before capturing, else the call returns
                        GI_ERR_UNSUPPORTED; a pair a captured graph has used is never
                        freed, so replaying that graph after calls of other shapes
                        stays valid.  gi_march_deinterleaved returns
                        GI_ERR_UNSUPPORTED for it. */
  int occlusion;     /* GI_OCCLUSION_HARD (0): the reference's horizon test.
                        GI_OCCLUSION_SOFT (1): a step lowers the horizon by the
                        expected drop of a Gaussian horizon angle whose spread comes
                        from the depth moments' variance through the reference's
                        unused GetAngularDistribution (:51-81); no counterpart in the
                        reference's live code.  Runs in the exact contract; standard
                        form with 2-channel depth moments only. */
} gi_march_params;

#define GI_MARCH_EXACT 0
#define GI_MARCH_FAST 1
#define GI_MARCH_TEXTURE 2
#define GI_OCCLUSION_HARD 0
#define GI_OCCLUSION_SOFT 1

/* light_levels: blurred direct-light pyramid (4 ch); depth_levels: blurred depth
 * moments pyramid (2 ch); normal: 4 ch; ndc_depth: 1 ch (hardware depth);
 * out: 4 ch (rgb, 1). */
GI_API int gi_march(const gi_view* view, const gi_march_params* params, const float* const* light_levels,
             const float* const* depth_levels, int num_levels, const float* normal,
             const float* ndc_depth, float* out, void* stream);

/* The same march in the explicit interleaved form (LSGIRenderer.h:83-91,
 * SSShiftGIRenderer.h:294-385): normal_d and ndc_depth_d are deinterleaved
 * (gi_deinterleave with the pattern grid), the centre values are read with
 * texelFetch, and out_d is written deinterleaved. */
GI_API int gi_march_deinterleaved(const gi_view* view, const gi_march_params* params,
                           const float* const* light_levels, const float* const* depth_levels,
                           int num_levels, const float* normal_d, const float* ndc_depth_d,
                           float* out_d, void* stream);

/* The march restricted to a list of screen tiles (the same arithmetic; pixels
 * outside the listed tiles are not written).  A tile is the pixel footprint of
 * one CTA of one interleave pattern: tile_w x tile_h pixels from
 * gi_march_tile_grid; tile t covers pixels [tx*tile_w, (tx+1)*tile_w) x
 * [ty*tile_h, (ty+1)*tile_h) with tx = t % tiles_x, ty = t / tiles_x.  `tiles` is
 * a device array of tile indices.  Used for the 256-ray training targets and for
 * judging the learned reconstructor on a subset of tiles. */
GI_API int gi_march_tile_grid(int width, int height, int pattern_size, int* tiles_x, int* tiles_y,
                              int* tile_w, int* tile_h);
GI_API int gi_march_tiles(const gi_view* view, const gi_march_params* params,
                          const float* const* light_levels, const float* const* depth_levels,
                          int num_levels, const float* normal, const float* ndc_depth, float* out,
                          const int* tiles, int num_tiles, void* stream);

/* Autotuner: times the march in each launch layout on these inputs (it writes
 * `out`) and records the fastest for this march shape (width, height, dirs,
 * step_dirs, step_cap, precision); later gi_march calls of the same shape use it.
 * The layouts, all with the same result bit for bit:
 *   one thread per pixel, CTAs of 2, 4 or 8 rows of 32 pixels (the tile shape
 *     of the launch): a warp marches 32 pixels x all `dirs` directions;
 *   four threads per pixel (the direction split; 4 <= dirs <= 32): each thread
 *     marches every fourth direction of its pixel, a warp 32 pixels x
 *     ceil(dirs / 4) directions, CTAs of one 32-pixel row.
 * best_rows, best_rays_per_warp (32 x the directions a thread marches) and
 * best_ms (optional, host) receive the choice and its time per launch. */
GI_API int gi_march_autotune(const gi_view* view, const gi_march_params* params,
                             const float* const* light_levels, const float* const* depth_levels,
                             int num_levels, const float* normal, const float* ndc_depth, float* out,
                             int* best_rows, int* best_rays_per_warp, float* best_ms, void* stream);
/* The recorded CTA height for a march shape of the GI_MARCH_EXACT precision, or
 * 0 if it was never tuned. */
GI_API int gi_march_tuned_rows(int width, int height, int dirs, int step_dirs, int step_cap);
/* The recorded layout of a march shape (precision: GI_MARCH_*): CTA rows and
 * rays per warp, both 0 if the shape was never tuned. */
GI_API int gi_march_tuned_layout(int width, int height, int dirs, int step_dirs, int step_cap, int precision,
                                 int* rows, int* rays_per_warp);
/* Records a layout for a march shape without timing (for instance one an
 * earlier process tuned): rows 2, 4 or 8 with rays_per_warp = 32 x dirs, or rows
 * 4 with rays_per_warp = 32 x ceil(dirs / 4) (the direction split, 4 <= dirs <=
 * 32).  Anything else is GI_ERR_INVALID_ARGUMENT. */
GI_API int gi_march_set_layout(int width, int height, int dirs, int step_dirs, int step_cap, int precision,
                               int rows, int rays_per_warp);

/* Diagnostic: n trilinear fetches through the texture units, as GI_MARCH_TEXTURE
 * takes the march's taps -- the pyramid `levels` (src_channels floats per texel,
 * the first `channels` (1 or 4) used) copied into a mipmapped array behind a
 * texture object with the reference's screenspaceSampler state (linear filter,
 * linear mipmapping, clamp-to-edge; SSVGIRenderer.h:17), fetched at normalised
 * coordinates coords[2i], coords[2i+1] and level lods[i]; `channels` floats per
 * fetch to out.  All device memory.  Allocates the array, synchronises `stream`
 * and frees it: for tests of the sampler arithmetic, not for the frame loop. */
GI_API int gi_texture_sample(const float* const* levels, int width, int height, int num_levels, int channels,
                             int src_channels, const float* coords, const float* lods, int n, float* out,
                             void* stream);

/* 5x5 depth/normal-weighted bilateral filter of the indirect light.  The
 * reference has only its weights, commented out in Common/denoiser.frag:102-105:
 * w = exp(-|d - d0| * 10.5) * exp(-|n - n0|^2 * 20), taps x, y in [-2, 2],
 * clamp-to-edge.  depth: 2-ch depth moments level 0 (.x = linear depth). */
GI_API int gi_bilateral(const float* indirect, const float* depth_moments, const float* normal,
                 float* out, int width, int height, void* stream);

/* Common/denoiser.frag:72-184 (per-pixel least-squares fit of colour on
 * [depth, 1] over a 4x4 window); radius 0 copies (:82-86). */
GI_API int gi_denoise(const float* noisy, const float* depth_moments, const float* normal, float* out,
               int width, int height, int radius, void* stream);

/* Common/finalGatherer.frag:42-59: out = direct + indirect * albedo. */
GI_API int gi_final_gather(const float* direct, const float* indirect, const float* albedo, float* out,
                    int width, int height, void* stream);

/* ---------------------------------------------------------------------------
 * Input stages (the passes that feed the path in SSVGIRenderer.h:61-205),
 * restated as analytic ray casts over a procedural scene of axis-aligned boxes
 * and spheres inside a room.
 */
typedef enum gi_prim_kind { GI_PRIM_ROOM = 0, GI_PRIM_BOX = 1, GI_PRIM_SPHERE = 2 } gi_prim_kind;

typedef struct gi_prim {
  int32_t kind;         /* gi_prim_kind */
  float a[3];           /* room, box: min corner; sphere: centre */
  float b[3];           /* room, box: max corner; sphere: b[0] = radius */
  float albedo[4];      /* RGBA in [0, 1]; generated as RGBA8 / 255 */
  float emissive[4];
  float pad;
} gi_prim;

/* Seeded procedural room: the unit-cube interior, num_boxes axis-aligned boxes
 * with edges U[0.05, 0.3], num_spheres spheres with radii U[0.05, 0.2], albedo
 * RGBA8 in [0.2, 0.9].  Seeds std::mt19937_64 with `seed`.  Writes the room first.
 * Returns the primitive count in *count. */
GI_API int gi_scene_generate(uint64_t seed, int num_boxes, int num_spheres, gi_prim* prims, int max_prims,
                      int* count);
/* Point light of the scene: Camera at (0.5, 0.93, 0.5) looking down
 * (main.cpp:166-169 places the reference's light the same way). */
GI_API int gi_scene_light(gi_camera* light);
/* Camera on a seeded closed Catmull-Rom spline through 8 control points,
 * sampled at frame / num_frames. */
GI_API int gi_camera_spline(uint64_t seed, int frame, int num_frames, gi_camera* cam);
/* The same spline with its control points kept at least 0.08 from every box and
 * sphere of `prims` (host array), so that the camera looks from free space. */
GI_API int gi_camera_spline_in_scene(uint64_t seed, const gi_prim* prims, int num_prims, int frame,
                                     int num_frames, gi_camera* cam);

/* Triangle meshes of a JSON scene (bin/data/Scenes/*.json as Scene.h:55-117
 * loads it): an object is one mesh placed by translate(pos) * rotate(angle),
 * with albedoColor and emissiveColor (alpha 1, as SSVGIRenderer.h:142-143 sets
 * them).  Triangles are in world space, grouped by object; legitengine_gb300/scene.py
 * builds these arrays from a scene file. */
typedef struct gi_mesh_object {
  float lo[3], hi[3];     /* world-space bounds of the object's triangles */
  int32_t first, count;   /* its triangles: tris[first, first + count) */
  float albedo[4];
  float emissive[4];
  int32_t pad[4];
} gi_mesh_object;         /* 80 bytes */

typedef struct gi_triangle {
  float p[3][3];          /* world-space vertices */
  float n[3][3];          /* world-space vertex normals: modelMatrix * (n, 0) (gBufferBuilder.vert:38) */
  float pad[2];
} gi_triangle;            /* 80 bytes */

#define GI_MAX_MESH_OBJECTS 4096
#define GI_MAX_TRIANGLES (1 << 24)

/* A scene file loaded into host memory (Scene.h:55-117 with Mesh.h:14-57:
 * OBJ meshes triangulated as the reference's tinyobjloader 1.4 does, placed by
 * translate(pos) * rotate(angle), ReadJsonVec3f defaults of main.cpp:24-27;
 * objects with an undeclared mesh skipped).  Mesh paths are tried as given,
 * next to the scene file, and one and two folders up from it. */
typedef struct gi_scene gi_scene;
GI_API int gi_scene_load(const char* path, gi_scene** out);
/* Object and triangle counts, and the "renderer" section's shadowmapSize[0]
 * (1024 when absent). */
GI_API int gi_scene_info(const gi_scene* scene, int* num_objects, int* num_triangles, int* shadow_size);
/* Copies the objects and their world-space triangles into caller arrays of
 * num_objects and num_triangles entries (host memory). */
GI_API int gi_scene_copy(const gi_scene* scene, gi_mesh_object* objects, gi_triangle* triangles);
/* Name of the mesh object i was built from (NULL out of range). */
GI_API const char* gi_scene_object_mesh(const gi_scene* scene, int i);
GI_API int gi_scene_destroy(gi_scene* scene);

/* G-buffer (Common/gBufferBuilder.frag:28-38): albedo^2.2 (4 ch), emissive^2.2
 * (4 ch), normal (n, 1) (4 ch), depth moments (d, d^2) with d the distance to
 * the camera (2 ch), hardware depth (1 ch).  prims: device array. */
GI_API int gi_gbuffer(const gi_view* view, const gi_prim* prims, int num_prims, float* albedo,
               float* emissive, float* normal, float* depth_moments, float* ndc_depth, void* stream);
/* Shadow map (Common/shadowmapBuilder.vert:30-38): light-space depth, 1 ch. */
GI_API int gi_shadow_map(const gi_view* light_view, const gi_prim* prims, int num_prims, float* shadow,
                  void* stream);
/* The same two passes over analytic primitives (num_prims >= 0) and triangle
 * meshes (device arrays).  A ray takes the nearest hit, the earlier primitive on
 * a tie (analytic primitives before meshes, objects and triangles in order); a
 * triangle hit (Moller-Trumbore) writes its object's colours and the barycentric
 * blend of its vertex normals, unnormalised, as the rasteriser's interpolation of
 * vertWorldNormal does.  Objects whose bounds the ray misses are skipped.
 * cull: GI_CULL_NONE hits both faces; GI_CULL_BACK skips a triangle whose
 * counter-clockwise (right-hand) winding faces away from the ray, so that an
 * inward-facing room lets the light through its ceiling as the reference's
 * scenes expect (their light sits above the room, main.cpp:164-166). */
#define GI_CULL_NONE 0
#define GI_CULL_BACK 1
GI_API int gi_gbuffer_mesh(const gi_view* view, const gi_prim* prims, int num_prims,
                           const gi_mesh_object* objects, int num_objects, const gi_triangle* tris,
                           int num_tris, int cull, float* albedo, float* emissive, float* normal,
                           float* depth_moments, float* ndc_depth, void* stream);
GI_API int gi_shadow_map_mesh(const gi_view* light_view, const gi_prim* prims, int num_prims,
                              const gi_mesh_object* objects, int num_objects,
                              const gi_triangle* tris, int num_tris, int cull, float* shadow,
                              void* stream);
/* Direct light (Common/directLighting.frag:45-79), 4 ch. */
GI_API int gi_direct_light(const gi_view* view, const gi_view* light_view, const float* albedo,
                    const float* emissive, const float* normal, const float* ndc_depth,
                    const float* shadow, int shadow_size, float* out, void* stream);

/* ---------------------------------------------------------------------------
 * Batched views: the GI segment (mips, blur pyramids, march, bilateral, gather;
 * one bounce) of many independent views of uneven resolution per frame.  The
 * marches of all views run as ONE persistent launch over a work list of
 * (view, tile, pattern) items ordered by decreasing cost; the whole frame is
 * captured once into a CUDA graph that gi_batch_render replays.  Buffers are
 * fixed at creation: refresh their contents between frames.
 */
typedef struct gi_batch_view {
  gi_view view;
  gi_march_params march;
  const float* albedo;         /* device inputs, view size (4 / 4 / 2 / 1 / 4 ch) */
  const float* normal;
  const float* depth_moments;
  const float* ndc_depth;
  const float* direct;
  float* out_lit;              /* device output, 4 ch */
  float* out_indirect;         /* optional: filtered indirect light, 4 ch */
} gi_batch_view;

typedef struct gi_batch gi_batch;

/* tile_rows: CTA height of the batched march (2, 4, 8), or 0 to let the
 * autotuner time each and keep the fastest. */
GI_API int gi_batch_create(const gi_batch_view* views, int num_views, int tile_rows, gi_batch** out);
GI_API int gi_batch_render(gi_batch* b, void* stream);
GI_API int gi_batch_info(const gi_batch* b, int* work_items, int* grid, int* tile_rows, float* tuned_ms);
GI_API int gi_batch_destroy(gi_batch* b);

/* ---------------------------------------------------------------------------
 * Learned reconstructor (no counterpart in the reference): a 32 -> 64 -> 64 ->
 * 64 -> 3 ReLU MLP that maps a few-ray gather plus G-buffer features to the
 * many-ray indirect light.  BF16 weights/activations on the tensor cores with
 * FP32 accumulation; FP32 master weights and Adam state.
 */
#define GI_MLP_IN 32
#define GI_MLP_HIDDEN 64
#define GI_MLP_OUT 3
#define GI_MLP_PARAMS 10627

typedef struct gi_mlp gi_mlp;

GI_API int gi_mlp_param_count(void);
GI_API int gi_mlp_create(gi_mlp** out);
GI_API int gi_mlp_destroy(gi_mlp* m);
/* He-uniform weights, zero biases, Adam state cleared (std::mt19937_64(seed)). */
GI_API int gi_mlp_init(gi_mlp* m, uint64_t seed);
/* FP32 masters in the order W1[32x64], b1, W2[64x64], b2, W3[64x64], b3, W4[64x3], b4,
 * each weight row-major [in x out] (y = x W + b). */
GI_API int gi_mlp_set_params(gi_mlp* m, const float* host, int count);
GI_API int gi_mlp_get_params(const gi_mlp* m, float* host, int count);
/* features: device bf16 [n x 32]; the network's 3 outputs are softmax logits whose
 * weights blend three candidate estimates from the row itself: input channels
 * 10-12 (the bilaterally filtered few-ray light), 19-21 (its mip level 2) and
 * 22-24 (mip level 4); scale (optional, device [n]): the blend is multiplied by it
 * (the exposure scale written by gi_features); out: device fp32 [n x 4] (rgb, 1). */
GI_API int gi_mlp_forward(const gi_mlp* m, const void* features, const float* scale, int n, float* out,
                          void* stream);
/* Training loss of gi_mlp_train_step and gi_mlp_gradients (default
 * GI_MLP_LOSS_SQUARED; not part of a checkpoint). */
#define GI_MLP_LOSS_SQUARED 0  /* sum_i w_i |y_i - t_i|^2 / (3 n); per-output error clipped to [-1, 1] in the gradient */
#define GI_MLP_LOSS_ABSOLUTE 1 /* sum_i w_i |y_i - t_i|_1 / (3 n): the relative L1 error of the evaluation */
GI_API int gi_mlp_set_loss(gi_mlp* m, int loss);
/* One Adam step (lr, beta 0.9/0.999, eps 1e-8) on the network's loss (above)
 * against targets [n x 4]: rgb t_i (divided by scale[i] when scale, device [n],
 * is given) and the pixel's loss weight w_i in channel 3 (a march output carries
 * 1 there).  loss_out (host, optional) receives the batch loss and makes the call
 * synchronous. */
GI_API int gi_mlp_train_step(gi_mlp* m, const void* features, const float* targets, const float* scale, int n,
                             float lr, float* loss_out, void* stream);
/* Gradient of the batch loss of gi_mlp_train_step with respect to the FP32 parameters (same order as
 * gi_mlp_set_params) into grads_host, without updating; synchronous. */
GI_API int gi_mlp_gradients(gi_mlp* m, const void* features, const float* targets, const float* scale, int n,
                            float* grads_host, float* loss_host, void* stream);
/* Allocation-free gradients (this entry point has no counterpart in the
 * reference).  Same result as gi_mlp_gradients, for callers that cannot call
 * cudaMalloc: a host whose device memory is all handed out by its own arena
 * allocator, or a process at its memory cap.
 * The caller passes everything the call reads and writes, all device memory:
 * params (the 10,627 FP32 weights in the gi_mlp_set_params order), features
 * (bf16 [n x 32]), targets ([n x 4], rgb + loss weight), scale (optional, [n]), and
 * receives grads (10,627 floats: the gradient of gi_mlp_train_step's batch loss
 * with GI_MLP_LOSS_SQUARED) and loss (one float).  Nothing is allocated: the scratch (a bf16 copy of the weights and one
 * slot of gradient sums per 64 pixels, summed in a fixed order, so repeated calls
 * return the same bits) is a 5.2 MiB array compiled into the library, which every
 * GPU that loads the library keeps until the process exits.  n is limited to 8192
 * pixels; larger batches return GI_ERR_INVALID_ARGUMENT.  The first call on a
 * device looks up the array's device address and sets the kernel's shared-memory
 * limit (a first call on a stream in capture mode returns
 * GI_ERR_INVALID_ARGUMENT).  All calls share the one array: calls that can run
 * at the same time on the GPU (different streams) overwrite each other's scratch
 * and must be ordered by the caller.  Asynchronous on `stream`. */
GI_API int gi_mlp_gradients_noalloc(const float* params, const void* features, const float* targets,
                                    const float* scale, int n, float* grads, float* loss, void* stream);
/* Checkpoint: FP32 weights + Adam moments + step, with a CRC-32. */
GI_API int gi_mlp_save(const gi_mlp* m, const char* path);
GI_API int gi_mlp_load(gi_mlp* m, const char* path);
/* The 32 per-pixel features (bf16) for the whole frame (tiles == NULL, pixel-major)
 * or for a list of march tiles (tile-major, tile_w*tile_h pixels per tile).
 * indirect_levels: the few-ray indirect light (4 ch) at mip levels 0, 2 and 4;
 * filtered: the few-ray indirect light after gi_bilateral (4 ch; the network's
 * output is added to it); depth_blur_l2: level 2 of the blurred depth-moments
 * pyramid.  The light-dependent
 * features are divided by a per-pixel exposure scale written to scale (device,
 * one float per output row). */
GI_API int gi_features(int width, int height, int pattern_size, const float* depth_moments,
                       const float* normal, const float* albedo, const float* direct,
                       const float* const* indirect_levels, const float* filtered,
                       const float* depth_blur_l2, void* out, float* scale, const int* tiles,
                       int num_tiles, void* stream);
/* Fused reconstruction of a whole frame (no counterpart in the reference): the
 * gi_features inputs in, the network's blended estimate x exposure scale out
 * (device fp32 [height x width x 4], rgb + 1) -- the result of gi_features
 * followed by gi_mlp_forward, without the feature buffer, on the tcgen05 tensor
 * cores (accumulation order differs from gi_mlp_forward, so the two agree to
 * FP32 rounding of the accumulators, not bit for bit). */
GI_API int gi_mlp_reconstruct(const gi_mlp* m, int width, int height, int pattern_size,
                              const float* depth_moments, const float* normal, const float* albedo,
                              const float* direct, const float* const* indirect_levels, const float* filtered,
                              const float* depth_blur_l2, float* out, void* stream);
/* Count of tensor-core completion waits in gi_mlp_reconstruct that ran out (each
 * abandons its launch's remaining tiles); 0 in normal operation. */
GI_API int gi_mlp_tensor_core_errors(int* count);
/* Test hook of the failure path above (no counterpart in the reference):
 * bounds the FIRST tensor-core completion wait of each 128-pixel tile group in
 * later gi_mlp_reconstruct launches to `cycles` SM clock cycles, so that a short
 * bound makes the wait run out: the group records an error
 * (gi_mlp_tensor_core_errors), stops, waits with the full bound for its MMAs in
 * flight, frees its tensor memory and the launch returns.  cycles <= 0 restores
 * the default (about 2^31 cycles).  For the current device. */
GI_API int gi_debug_tensor_core_wait_limit(long long cycles);
/* 4-channel pixels of listed march tiles, image <-> tile-major arrays. */
GI_API int gi_gather_tiles(const float* image, int width, int height, int pattern_size, const int* tiles,
                           int num_tiles, float* out, void* stream);
GI_API int gi_scatter_tiles(const float* values, int width, int height, int pattern_size,
                            const int* tiles, int num_tiles, float* image, void* stream);

/* Learned mode of a batch (no counterpart in the reference): every view's
 * indirect light comes from a few_dirs gather (steps spaced for few_step_dirs
 * directions; 0 = few_dirs) marched for all views in the one persistent launch,
 * its mip levels and 5x5 bilateral, and the reconstructor m (gi_mlp_reconstruct);
 * a judge marches the view's own directions on a rotating 1/judge_every of its
 * march tiles (the same tiles gi_renderer_set_learned judges in the same frame)
 * and a tile whose learned light differs from that march by more than threshold
 * (relative L1) takes the march's result.  The rotation runs on the device, so the
 * frame stays one captured graph.  m = NULL returns to the plain method.  The
 * batch keeps the pointer: m must outlive its use. */
GI_API int gi_batch_set_learned(gi_batch* b, const gi_mlp* m, int few_dirs, int few_step_dirs, int judge_every,
                                float threshold);
/* Online fine-tuning of a learned batch (no counterpart in the reference): for
 * every view, marches target_dirs directions without a step cap on the tiles
 * judged in the last rendered frame, builds their features and takes one Adam
 * step of m (lr; pixel loss weights as in training) on all views' tiles together.
 * sampled_error_out (optional) receives the relative L1 error of the last frame's
 * result on those tiles against that march; loss_out or sampled_error_out makes
 * the call synchronous. */
GI_API int gi_batch_finetune(gi_batch* b, gi_mlp* m, int target_dirs, float lr, float* loss_out,
                             float* sampled_error_out, void* stream);
/* Tiles judged and tiles that fell back, since gi_batch_set_learned. */
GI_API int gi_batch_stats(const gi_batch* b, int* judged_tiles, int* fallback_tiles);

/* ---------------------------------------------------------------------------
 * Whole-frame renderer: the GI segment of SSVGIRenderer::RenderFrame
 * (SSVGIRenderer.h:207-342) on resident G-buffer images.  Owns its pyramids
 * and intermediate images; records the passes through the render-graph shim
 * and replays them as one CUDA graph.
 */
typedef struct gi_renderer gi_renderer;

typedef struct gi_frame_params {
  gi_march_params march;
  int bounces;        /* >= 1; bounce k > 1 marches over the lit result of bounce k-1 */
  int bilateral;      /* 1: 5x5 bilateral on each bounce's indirect light */
  int denoise_radius; /* Common/denoiser.frag radius (0 = passthrough, the default) */
  int mip_levels;     /* requested levels (the reference's 10) */
  int feedback;       /* 1 (with bounces = 1): temporal feedback -- each frame's light
                         pyramid is built from the previous frame's gathered image
                         (finalGatherer output, SSVGIRenderer.h:305-342) instead of the
                         direct light, so bounces accumulate over frames at one march
                         per frame; the first frame after creation uses the direct
                         light.  0: bounces within the frame. */
} gi_frame_params;

typedef struct gi_frame_inputs {   /* device pointers, width x height */
  const float* albedo;        /* 4 ch */
  const float* normal;        /* 4 ch */
  const float* depth_moments; /* 2 ch */
  const float* ndc_depth;     /* 1 ch */
  const float* direct;        /* 4 ch */
} gi_frame_inputs;

GI_API int gi_renderer_create(int width, int height, const gi_frame_params* params, gi_renderer** out);
GI_API int gi_renderer_destroy(gi_renderer* r);
/* Learned mode: the indirect light of each bounce comes from a few_dirs-direction
 * march (stepped for few_step_dirs directions; 0 = few_dirs) reconstructed by
 * `mlp` (which must outlive the renderer's use of it);
 * every frame the plain march (params.march.dirs) is run on 1/judge_every of the
 * tiles, and a judged tile whose learned result differs from it by more than
 * judge_threshold (relative L1, rgb) uses the plain result.  mlp == NULL returns
 * to the plain method.  The renderer's mip count must be >= 5. */
GI_API int gi_renderer_set_learned(gi_renderer* r, const gi_mlp* mlp, int few_dirs, int few_step_dirs,
                                   int judge_every, float judge_threshold);
/* Tiles judged and tiles that fell back since creation (synchronous). */
GI_API int gi_renderer_stats(gi_renderer* r, int* judged_tiles, int* fallback_tiles);
/* GPU profiling of the frame's passes, as the reference's GPU profiler shows them
 * (each pass's SetProfilerInfo name; main.cpp:273-285): while enabled, every
 * frame records a timing event before each pass and after the last (event-record
 * nodes of the captured graph). */
GI_API int gi_renderer_set_profiling(gi_renderer* r, int enable);
/* The last profiled frame's passes (waits for it): *num_passes = their count; the
 * first max_passes get their name (valid until the next render), start and end in
 * milliseconds from the start of the first pass.  Passes on the frame's stream;
 * work a pass forks onto another stream ends within the pass that joins it. */
GI_API int gi_renderer_pass_times(gi_renderer* r, int max_passes, const char** names, float* start_ms,
                                  float* end_ms, int* num_passes);
/* out_lit: 4 ch final image; out_indirect (optional): last bounce's filtered
 * indirect light, 4 ch. */
GI_API int gi_renderer_render(gi_renderer* r, const gi_view* view, const gi_frame_inputs* in,
                       float* out_lit, float* out_indirect, void* stream);
/* Same, from host buffers: copies the inputs in and the lit image out on `stream`
 * and waits for it. */
GI_API int gi_renderer_render_host(gi_renderer* r, const gi_view* view, const float* albedo,
                            const float* normal, const float* depth_moments,
                            const float* ndc_depth, const float* direct, float* out_lit,
                            void* stream);
/* Pipelined form of gi_renderer_render_host for a sequence of frames: frame k's
 * inputs are copied in on the renderer's own copy stream while frame k - 1 renders
 * on `stream`, and its lit image is copied out to out_lit on a second copy stream
 * while frame k + 1 renders (two device staging sets).  Returns without waiting.
 * Frame k's host buffers (inputs and out_lit) must stay valid and its inputs
 * unchanged until the call for frame k + 2 returns or gi_renderer_host_wait
 * returns; out_lit holds frame k's image from then on.  (Host memory should be
 * pinned for the copies to overlap the rendering.) */
GI_API int gi_renderer_render_host_async(gi_renderer* r, const gi_view* view, const float* albedo,
                                  const float* normal, const float* depth_moments,
                                  const float* ndc_depth, const float* direct, float* out_lit,
                                  void* stream);
/* Waits until every frame submitted by gi_renderer_render_host_async is on the host. */
GI_API int gi_renderer_host_wait(gi_renderer* r);

#ifdef __cplusplus
}
#endif

#endif /* LEGIT_GI_H */
