// gi_batch.cu -- many independent views of uneven resolution in one frame: the
// GI segment (mip chains, blur pyramids, march, bilateral, gather; one bounce)
// of every view, with the marches of all views in ONE persistent launch, and
// the whole frame captured once into a CUDA graph that gi_batch_render replays.
//
// Work list: one item per (view, march tile, interleave pattern), ordered by
// decreasing estimated cost (directions x steps), claimed by CTAs from a device
// counter (longest-first list scheduling).  The CTA height (tile shape) is
// chosen by timing the batched launch with each candidate (the autotuner) unless
// the caller fixes it.
#include <algorithm>
#include <memory>
#include <vector>

#include "gi_internal.h"
#include "gi_kernels.h"
#include "legit_render_graph.h"

namespace gi {

class Batch {
 public:
  struct ViewRes {
    gi_batch_view in;
    int levels;
    std::unique_ptr<legit::MippedProxy> light, light_blur, depth, depth_blur;
    std::unique_ptr<legit::UnmippedProxy> indirect, filtered;
  };

  ~Batch() {
    if (exec_) cudaGraphExecDestroy(exec_);
    cudaFree(d_views_);
    cudaFree(d_items_);
    cudaFree(d_counter_);
    if (stream_) cudaStreamDestroy(stream_);
  }

  int Create(const gi_batch_view* views, int n, int rows) {
    // The creation marches the views' current inputs (to time the tile shapes),
    // on a stream of its own: wait for whatever is producing them.
    int e = check_cuda(cudaDeviceSynchronize(), "gi_batch_create: sync");
    if (e) return e;
    e = check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "gi_batch_create: stream");
    if (e) return e;
    std::vector<BatchView> bv(n);
    std::vector<std::pair<double, int2>> work;
    for (int v = 0; v < n; v++) {
      ViewRes r;
      r.in = views[v];
      const int W = r.in.view.width, H = r.in.view.height;
      r.levels = gi_mip_level_count(W, H, 10);
      legit::uvec2 size((uint32_t)W, (uint32_t)H);
      try {
        r.light.reset(new legit::MippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size, 0, 10));
        r.light_blur.reset(new legit::MippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size, 0, 10));
        r.depth.reset(new legit::MippedProxy(&rg_, legit::Format::R32G32Sfloat, size, 0, 10));
        r.depth_blur.reset(new legit::MippedProxy(&rg_, legit::Format::R32G32Sfloat, size, 0, 10));
        r.indirect.reset(new legit::UnmippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size));
        r.filtered.reset(new legit::UnmippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size));
      } catch (const legit::GiError& err) {
        return fail(err.status, err.what());
      }
      MarchArgs& a = bv[v].a;
      a = MarchArgs{};
      for (int k = 0; k < 16; k++) {
        a.inv_view_proj.m[k] = r.in.view.inv_view_proj[k];
        a.inv_view.m[k] = r.in.view.inv_view[k];
      }
      std::vector<float*> lb = Levels(*r.light_blur), db = Levels(*r.depth_blur);
      lb[0] = const_cast<float*>(r.in.direct);
      db[0] = const_cast<float*>(r.in.depth_moments);
      for (int k = 0; k < r.levels; k++) {
        a.light[k] = lb[k];
        a.depth[k] = db[k];
      }
      a.normal = r.in.normal;
      a.ndc = r.in.ndc_depth;
      a.out = Level0(*r.indirect);
      a.width = W;
      a.height = H;
      a.num_levels = r.levels;
      a.depth_ch = 2;
      a.dirs = r.in.march.dirs;
      a.step_cap = r.in.march.step_cap;
      a.pattern = r.in.march.pattern_size;
      a.step_dirs = r.in.march.step_dirs > 0 ? r.in.march.step_dirs : r.in.march.dirs;
      a.tiles = nullptr;
      a.num_tiles = 0;
      bv[v].n_tab = march_table_size(a);
      if (bv[v].n_tab > GI_MAX_STEPS) return fail(GI_ERR_UNSUPPORTED, "gi_batch_create: too many steps per direction");
      res_.push_back(std::move(r));
    }
    views_ = bv;
    rows_ = rows;
    e = BuildWork(rows == 0 ? 4 : rows);
    if (e) return e;
    e = check_cuda(cudaMalloc(&d_counter_, sizeof(int)), "gi_batch_create: counter");
    if (e) return e;
    // Pyramids first (the autotuner marches real inputs), then choose the tile
    // shape, then capture the frame.
    e = RecordFrame(stream_, /*capture=*/false);
    if (e) return e;
    if (rows == 0) {
      e = Autotune();
      if (e) return e;
    }
    return Capture();
  }

  int Render(cudaStream_t s) {
    int e = check_cuda(cudaGraphLaunch(exec_, s), "gi_batch_render");
    if (!e) count_launches(launches_per_frame_);
    return e;
  }

  int rows_ = 4, grid_ = 0, num_items_ = 0;

 private:
  std::vector<float*> Levels(const legit::MippedProxy& p) { return rg_.ResolveView(p.imageViewProxy->Id()).levels; }
  float* Level0(const legit::UnmippedProxy& p) { return rg_.ResolveView(p.imageViewProxy->Id()).level(0); }

  // Work items for CTA height `rows`, longest first; uploads views and items.
  int BuildWork(int rows) {
    std::vector<std::pair<double, int2>> work;
    for (size_t v = 0; v < views_.size(); v++) {
      MarchArgs& a = views_[v].a;
      const int P = a.pattern;
      const int sub_w = (a.width + P - 1) / P, sub_h = (a.height + P - 1) / P;
      const int tx = (sub_w + 31) / 32, ty = (sub_h + rows - 1) / rows;
      views_[v].tiles_x = tx;
      views_[v].tiles_total = tx * ty;
      const double cost = (double)a.dirs * views_[v].n_tab;
      for (int t = 0; t < tx * ty; t++)
        for (int p = 0; p < P * P; p++) work.push_back({cost, make_int2((int)v, t * 64 + p)});
    }
    std::stable_sort(work.begin(), work.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
    std::vector<int2> items(work.size());
    for (size_t i = 0; i < work.size(); i++) items[i] = work[i].second;
    num_items_ = (int)items.size();
    cudaFree(d_items_);
    cudaFree(d_views_);
    d_items_ = nullptr;
    d_views_ = nullptr;
    int e = check_cuda(cudaMalloc(&d_items_, std::max<size_t>(1, items.size()) * sizeof(int2)), "gi_batch: items");
    e = e ? e : check_cuda(cudaMalloc(&d_views_, views_.size() * sizeof(BatchView)), "gi_batch: views");
    e = e ? e : check_cuda(cudaMemcpy(d_items_, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice),
                           "gi_batch: items");
    e = e ? e : check_cuda(cudaMemcpy(d_views_, views_.data(), views_.size() * sizeof(BatchView),
                                      cudaMemcpyHostToDevice),
                           "gi_batch: views");
    if (e) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_ = std::max(1, std::min(num_items_, sms * march_batch_occupancy(rows)));
    rows_ = rows;
    return GI_OK;
  }

  int Autotune() {
    const int cand[3] = {2, 4, 8};
    float best = 1e30f;
    int best_r = 4;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int st = GI_OK;
    for (int r : cand) {
      st = BuildWork(r);
      if (st) break;
      st = launch_march_batch(d_views_, d_items_, num_items_, d_counter_, rows_, grid_, stream_);
      if (!st) st = check_cuda(cudaEventRecord(e0, stream_), "gi_batch autotune");
      for (int k = 0; k < 3 && !st; k++)
        st = launch_march_batch(d_views_, d_items_, num_items_, d_counter_, rows_, grid_, stream_);
      if (!st) st = check_cuda(cudaEventRecord(e1, stream_), "gi_batch autotune");
      if (!st) st = check_cuda(cudaEventSynchronize(e1), "gi_batch autotune");
      float ms = 0.0f;
      if (!st) cudaEventElapsedTime(&ms, e0, e1);
      if (st) break;
      if (ms < best) {
        best = ms;
        best_r = r;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    tuned_ms_ = best / 3.0f;
    return BuildWork(best_r);
  }

  // Records the frame's passes (mips and blur of every view, the batched march,
  // per-view bilateral and gather) on `s`.
  int RecordFrame(cudaStream_t s, bool capture) {
    (void)capture;
    std::vector<MipJob> mips;
    std::vector<BlurJob> blurs;
    for (auto& r : res_) {
      const int W = r.in.view.width, H = r.in.view.height, L = r.levels;
      std::vector<float*> ll = Levels(*r.light), lb = Levels(*r.light_blur), dl = Levels(*r.depth),
                          db = Levels(*r.depth_blur);
      ll[0] = lb[0] = const_cast<float*>(r.in.direct);
      dl[0] = db[0] = const_cast<float*>(r.in.depth_moments);
      for (int c = 0; c < 2; c++) {
        MipJob J{};
        const std::vector<float*>& lv = c == 0 ? ll : dl;
        for (int k = 0; k < L; k++) J.levels[k] = lv[k];
        J.w = W;
        J.h = H;
        J.channels = c == 0 ? 4 : 2;
        J.num_levels = L;
        J.filter = GI_MIP_AVG;
        mips.push_back(J);
      }
      for (int k = 1; k < L; k++) {
        blurs.push_back(BlurJob{ll[k], lb[k], W >> k, H >> k, 4, 2, 0, 0});
        blurs.push_back(BlurJob{dl[k], db[k], W >> k, H >> k, 2, 2, 0, 0});
      }
    }
    int launches = 0;
    for (size_t i = 0; i < mips.size(); i += kMaxMipJobs) {
      MipJobs jobs{};
      for (size_t j = i; j < std::min(mips.size(), i + kMaxMipJobs); j++) jobs.job[jobs.count++] = mips[j];
      int e = launch_mips(jobs, s);
      if (e) return e;
      launches += 2;
    }
    for (size_t i = 0; i < blurs.size(); i += kMaxBlurJobs) {
      BlurJobs jobs{};
      for (size_t j = i; j < std::min(blurs.size(), i + kMaxBlurJobs); j++) jobs.job[jobs.count++] = blurs[j];
      int e = launch_blur(jobs, s);
      if (e) return e;
      launches++;
    }
    int e = launch_march_batch(d_views_, d_items_, num_items_, d_counter_, rows_, grid_, s);
    if (e) return e;
    launches++;
    for (auto& r : res_) {
      const int W = r.in.view.width, H = r.in.view.height;
      float* ind = Level0(*r.indirect);
      float* filt = Level0(*r.filtered);
      e = launch_bilateral(ind, r.in.depth_moments, 2, r.in.normal, filt, W, H, s);
      if (!e) e = launch_final_gather(r.in.direct, filt, r.in.albedo, r.in.out_lit, W, H, s);
      if (!e && r.in.out_indirect)
        e = check_cuda(cudaMemcpyAsync(r.in.out_indirect, filt, (size_t)W * H * 16, cudaMemcpyDeviceToDevice, s),
                       "gi_batch: indirect copy");
      if (e) return e;
      launches += 2;
    }
    launches_per_frame_ = launches;
    return GI_OK;
  }

  int Capture() {
    int e = check_cuda(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "gi_batch: capture");
    if (e) return e;
    e = RecordFrame(stream_, true);
    cudaGraph_t g = nullptr;
    int e2 = check_cuda(cudaStreamEndCapture(stream_, &g), "gi_batch: end capture");
    if (e || e2) {
      if (g) cudaGraphDestroy(g);
      return e ? e : e2;
    }
    e = check_cuda(cudaGraphInstantiate(&exec_, g, 0), "gi_batch: instantiate");
    cudaGraphDestroy(g);
    if (e) return e;
    return check_cuda(cudaStreamSynchronize(stream_), "gi_batch: sync");
  }

  legit::RenderGraph rg_;
  std::vector<ViewRes> res_;
  std::vector<BatchView> views_;
  BatchView* d_views_ = nullptr;
  int2* d_items_ = nullptr;
  int* d_counter_ = nullptr;
  cudaStream_t stream_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  int launches_per_frame_ = 0;

 public:
  float tuned_ms_ = 0.0f;
};

}  // namespace gi

struct gi_batch {
  std::unique_ptr<gi::Batch> impl;
};

using namespace gi;

extern "C" int gi_batch_create(const gi_batch_view* views, int num_views, int tile_rows, gi_batch** out) {
  GI_CHECK_ARG(views && out && num_views >= 1 && num_views <= 4096, "gi_batch_create: bad arguments");
  GI_CHECK_ARG(tile_rows == 0 || tile_rows == 2 || tile_rows == 4 || tile_rows == 8,
               "gi_batch_create: tile_rows must be 0 (tune), 2, 4 or 8");
  *out = nullptr;
  for (int v = 0; v < num_views; v++) {
    const gi_batch_view& b = views[v];
    GI_CHECK_ARG(b.view.width >= 16 && b.view.height >= 16, "gi_batch_create: viewport smaller than 16x16");
    GI_CHECK_ARG(b.albedo && b.normal && b.depth_moments && b.ndc_depth && b.direct && b.out_lit,
                 "gi_batch_create: null view buffer");
    GI_CHECK_ARG(aligned16(b.albedo) && aligned16(b.normal) && aligned16(b.depth_moments) && aligned16(b.direct) &&
                     aligned16(b.out_lit),
                 "gi_batch_create: unaligned view buffer");
    GI_CHECK_ARG(b.march.dirs >= 1 && b.march.dirs <= GI_MAX_DIRS && b.march.step_cap >= 0 &&
                     b.march.pattern_size >= 1 && b.march.pattern_size <= 8 && b.march.step_dirs >= 0,
                 "gi_batch_create: bad march parameters");
  }
  std::unique_ptr<gi_batch> b(new gi_batch);
  b->impl.reset(new Batch);
  int e = b->impl->Create(views, num_views, tile_rows);
  if (e) return e;
  *out = b.release();
  return GI_OK;
}

extern "C" int gi_batch_render(gi_batch* b, void* stream) {
  GI_CHECK_ARG(b, "gi_batch_render: null batch");
  return b->impl->Render((cudaStream_t)stream);
}

extern "C" int gi_batch_info(const gi_batch* b, int* work_items, int* grid, int* tile_rows, float* tuned_ms) {
  GI_CHECK_ARG(b && work_items && grid && tile_rows, "gi_batch_info: null argument");
  *work_items = b->impl->num_items_;
  *grid = b->impl->grid_;
  *tile_rows = b->impl->rows_;
  if (tuned_ms) *tuned_ms = b->impl->tuned_ms_;
  return GI_OK;
}

extern "C" int gi_batch_destroy(gi_batch* b) {
  delete b;
  return GI_OK;
}
