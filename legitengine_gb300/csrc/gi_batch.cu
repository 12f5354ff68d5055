// gi_batch.cu -- many independent views of uneven resolution in one frame: the
// GI segment (mip chains, blur pyramids, march, bilateral, gather; one bounce)
// of every view, with the marches of all views in ONE persistent launch (one per
// march precision present), and
// the whole frame captured once into a CUDA graph that gi_batch_render replays.
//
// Work list: one item per (view, march tile, interleave pattern), ordered by
// decreasing estimated cost (directions x steps), claimed by CTAs from a device
// counter (longest-first list scheduling).  The CTA height (tile shape) is
// chosen by timing the batched launch with each candidate (the autotuner) unless
// the caller fixes it.
//
// Learned mode (gi_batch_set_learned): the persistent launch marches every view
// with few directions; per view the few-ray mip levels, the 5x5 bilateral and the
// fused feature + network kernel follow; a judge marches the view's own
// directions on a rotating 1/judge_every of its tiles and lets tiles whose learned
// result is off by more than the threshold fall back to that march.  The rotation
// lives on the device (a frame counter and a table of tile lists), so the one
// captured graph serves every frame.  gi_batch_finetune trains the network on the
// tiles judged in the last frame against a many-direction march of them.
#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "gi_internal.h"
#include "gi_kernels.h"
#include "gi_mlp.h"
#define LEGIT_RG_DEVICE_ALLOC(p, bytes) ::gi::dmalloc(p, bytes)
#define LEGIT_RG_DEVICE_FREE(p) ::gi::dfree(p)
#include "legit_render_graph.h"

namespace gi {
namespace {

// cur[v * max_count + i] = table[(v * every + frame % every) * max_count + i]
__global__ void select_judge_kernel(const int* __restrict__ table, int* __restrict__ cur, int views, int max_count,
                                    int every, const unsigned* __restrict__ frame) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= views * max_count) return;
  const int v = i / max_count, k = i % max_count;
  const int phase = (int)(*frame % (unsigned)every);
  cur[i] = table[((size_t)v * every + phase) * max_count + k];
}

__global__ void frame_tick_kernel(unsigned* frame) { *frame += 1u; }

// T[i].w *= S[i] / mean(S) over the n rows (one block).
__global__ void loss_weights_kernel(float* __restrict__ T, const float* __restrict__ S, int n) {
  __shared__ float part[32];
  float s = 0.0f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += S[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += part[k];
    part[0] = t / (float)n;
  }
  __syncthreads();
  const float inv_mean = 1.0f / fmaxf(part[0], 1e-20f);
  for (int i = threadIdx.x; i < n; i += blockDim.x) T[(size_t)i * 4 + 3] *= S[i] * inv_mean;
}

// sums[0] += sum |a - b| (rgb), sums[1] += sum |b| over tile-major rows with b.w != 0.
__global__ void tile_error_kernel(const float* __restrict__ a, const float* __restrict__ b, int n,
                                  float* __restrict__ sums) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float num = 0.0f, den = 0.0f;
  if (i < n) {
    const float4 x = reinterpret_cast<const float4*>(a)[i], y = reinterpret_cast<const float4*>(b)[i];
    if (y.w != 0.0f) {
      num = fabsf(x.x - y.x) + fabsf(x.y - y.y) + fabsf(x.z - y.z);
      den = fabsf(y.x) + fabsf(y.y) + fabsf(y.z);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    num += __shfl_xor_sync(0xffffffffu, num, o);
    den += __shfl_xor_sync(0xffffffffu, den, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums + 0, num);
    atomicAdd(sums + 1, den);
  }
}

}  // namespace

// One persistent-march work list: the views of one march precision in chunks of
// at most kBatchTableViews (the views of one launch travel as its parameter),
// each chunk with its items (longest first) and grid.
struct WorkList {
  std::vector<BatchView> views;  // all of one march precision
  std::vector<int> owner;        // index of each view in the batch
  bool fast = false, tex = false;  // GI_MARCH_FAST step loop; tex: taps by the texture units
  struct Chunk {
    std::unique_ptr<BatchTable> table;
    int2* d_items = nullptr;
    int num_items = 0, grid = 0;
  };
  std::vector<Chunk> chunks;
  int num_items = 0, grid = 0;  // over all chunks: items, largest grid
  ~WorkList() { Free(); }
  void Free() {
    for (Chunk& c : chunks) dfree(c.d_items);
    chunks.clear();
    num_items = grid = 0;
  }
  int Build(int rows) {
    Free();
    for (const BatchView& v : views)
      if (tex != (v.a.depth_tex != 0 && v.a.light_tex != 0))
        return fail(GI_ERR_INVALID_ARGUMENT, "gi_batch: view in the wrong work list");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = march_batch_occupancy(rows, fast, tex);
    for (size_t c0 = 0; c0 < views.size(); c0 += kBatchTableViews) {
      const size_t c1 = std::min(views.size(), c0 + (size_t)kBatchTableViews);
      chunks.emplace_back();
      Chunk& ch = chunks.back();
      ch.table.reset(new BatchTable());
      std::vector<std::pair<double, int2>> work;
      for (size_t v = c0; v < c1; v++) {
        MarchArgs& a = views[v].a;
        const int P = a.pattern;
        const int sub_w = (a.width + P - 1) / P, sub_h = (a.height + P - 1) / P;
        const int tx = (sub_w + 31) / 32, ty = (sub_h + rows - 1) / rows;
        views[v].tiles_x = tx;
        views[v].tiles_total = tx * ty;
        ch.table->v[v - c0] = views[v];
        const double cost = (double)a.dirs * views[v].n_tab;
        for (int t = 0; t < tx * ty; t++)
          for (int p = 0; p < P * P; p++) work.push_back({cost, make_int2((int)(v - c0), t * 64 + p)});
      }
      std::stable_sort(work.begin(), work.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
      std::vector<int2> items(work.size());
      for (size_t i = 0; i < work.size(); i++) items[i] = work[i].second;
      ch.num_items = (int)items.size();
      int e = check_cuda(dmalloc(&ch.d_items, std::max<size_t>(1, items.size()) * sizeof(int2)), "gi_batch: items");
      e = e ? e : check_cuda(cudaMemcpy(ch.d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice),
                             "gi_batch: items");
      if (e) return e;
      ch.grid = std::max(1, std::min(ch.num_items, sms * per_sm));
      num_items += ch.num_items;
      grid = std::max(grid, ch.grid);
    }
    return GI_OK;
  }
  // One persistent launch per chunk, in order on `s` (each resets the counter).
  int Launch(int* counter, int rows, cudaStream_t s, int& launches) {
    for (Chunk& ch : chunks) {
      if (ch.num_items == 0) continue;
      launches++;
      int e = launch_march_batch(*ch.table, ch.d_items, ch.num_items, counter, rows, ch.grid, fast, tex, s);
      if (e) return e;
    }
    return GI_OK;
  }
};

// The views of a batch split by march precision (exact, fast, texture): one
// persistent launch each.
constexpr int kPrecisions = 3;
inline int precision_of(const MarchArgs& a) { return a.fast ? (a.depth_tex ? 2 : 1) : 0; }

struct WorkLists {
  WorkList list[kPrecisions];
  void Reset() {
    for (int k = 0; k < kPrecisions; k++) {
      list[k].views.clear();
      list[k].owner.clear();
      list[k].fast = k >= 1;
      list[k].tex = k == 2;
    }
  }
  void Add(int owner, const BatchView& v) {
    WorkList& w = list[precision_of(v.a)];
    w.views.push_back(v);
    w.owner.push_back(owner);
  }
  int Build(int rows) {
    int e = GI_OK;
    for (int k = 0; k < kPrecisions && !e; k++) e = list[k].Build(rows);
    return e;
  }
  int Launch(int* counter, int rows, cudaStream_t s, int& launches) {
    int e = GI_OK;
    for (int k = 0; k < kPrecisions && !e; k++) e = list[k].Launch(counter, rows, s, launches);
    return e;
  }
  int Items() const { return list[0].num_items + list[1].num_items + list[2].num_items; }
  int Grid() const { return std::max(list[0].grid, std::max(list[1].grid, list[2].grid)); }
};

class Batch {
 public:
  struct ViewRes {
    gi_batch_view in;
    int levels;
    std::unique_ptr<legit::MippedProxy> light, light_blur, depth, depth_blur, few;
    std::unique_ptr<legit::UnmippedProxy> indirect, filtered, few_f, learned, plain;
    std::vector<int> judge_count;  // valid tile ids per judge phase
    std::unique_ptr<PyramidTexture> dtex, ltex;  // GI_MARCH_TEXTURE: the pyramids for the texture units
  };

  ~Batch() {
    if (exec_) cudaGraphExecDestroy(exec_);
    dfree(d_counter_);
    dfree(d_judge_table_);
    dfree(d_judge_cur_);
    dfree(d_target_items_);
    dfree(d_target_counter_);
    dfree(d_frame_);
    dfree(d_stats_);
    dfree(d_sums_);
    dfree(d_x_);
    dfree(d_t_);
    dfree(d_s_);
    dfree(d_learned_rows_);
    if (stream_) cudaStreamDestroy(stream_);
  }

  int Create(const gi_batch_view* views, int n, int rows) {
    // The creation marches the views' current inputs (to time the tile shapes),
    // on a stream of its own: wait for whatever is producing them.
    int e = check_cuda(cudaDeviceSynchronize(), "gi_batch_create: sync");
    if (e) return e;
    e = check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "gi_batch_create: stream");
    if (e) return e;
    plain_.Reset();
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
      if (r.in.march.precision == GI_MARCH_TEXTURE) {
        r.dtex.reset(new PyramidTexture);
        r.ltex.reset(new PyramidTexture);
        e = r.dtex->Create(W, H, r.levels, 1);
        e = e ? e : r.ltex->Create(W, H, r.levels, 4);
        if (e) return e;
      }
      res_.push_back(std::move(r));
      BatchView bv{};
      FillArgs(res_.back(), res_.back().in.march.dirs, res_.back().in.march.step_dirs,
               Level0(*res_.back().indirect), bv.a);
      bv.n_tab = march_table_size(bv.a);
      if (bv.n_tab > GI_MAX_STEPS) return fail(GI_ERR_UNSUPPORTED, "gi_batch_create: too many steps per direction");
      plain_.Add(v, bv);
    }
    rows_ = rows == 0 ? 4 : rows;
    e = plain_.Build(rows_);
    if (e) return e;
    grid_ = plain_.Grid();
    e = check_cuda(dmalloc(&d_counter_, sizeof(int)), "gi_batch_create: counter");
    if (e) return e;
    // Pyramids first (the autotuner marches real inputs), then choose the tile
    // shape, then capture the frame.
    e = RecordFrame(stream_);
    if (e) return e;
    if (rows == 0) {
      e = Autotune();
      if (e) return e;
    }
    return Capture();
  }

  // Switches to the learned method (mlp != nullptr) or back; re-captures the frame.
  int SetLearned(const gi_mlp* mlp, int few_dirs, int few_step_dirs, int judge_every, float threshold) {
    mlp_ = mlp;
    if (mlp) {
      few_dirs_ = few_dirs;
      few_step_dirs_ = few_step_dirs;
      judge_every_ = judge_every;
      threshold_ = threshold;
      int e = PrepareLearned();
      if (e) return e;
    }
    return Capture();
  }

  int Render(cudaStream_t s) {
    int e = check_cuda(cudaGraphLaunch(exec_, s), "gi_batch_render");
    if (!e) {
      count_launches(launches_per_frame_);
      frames_++;
    }
    return e;
  }

  int Stats(int* judged, int* fell) {
    int h[2] = {0, 0};
    if (d_stats_) {
      int e = check_cuda(cudaMemcpy(h, d_stats_, sizeof(h), cudaMemcpyDeviceToHost), "gi_batch_stats");
      if (e) return e;
    }
    *judged = h[0];
    *fell = h[1];
    return GI_OK;
  }

  // One Adam step on the tiles judged in the last rendered frame of every view.
  int Finetune(gi_mlp* mlp, int target_dirs, float lr, float* loss_out, float* err_out, cudaStream_t s) {
    if (!mlp_) return fail(GI_ERR_INVALID_ARGUMENT, "gi_batch_finetune: the batch is not in learned mode");
    if (frames_ == 0) return fail(GI_ERR_INVALID_ARGUMENT, "gi_batch_finetune: no frame rendered yet");
    const int phase = (int)((frames_ - 1) % (uint64_t)judge_every_);
    if (target_dirs < 1 || target_dirs > GI_MAX_DIRS)
      return fail(GI_ERR_INVALID_ARGUMENT, "gi_batch_finetune: target_dirs out of range");
    int e = GI_OK;
    if (target_dirs != target_dirs_) {
      // Target views: an uncapped march with target_dirs directions into each
      // view's plain image (launch parameters: no launch in flight reads them).
      target_dirs_ = 0;  // until every table is filled
      for (TargetChunk& c : target_chunks_)
        for (size_t i = 0; i < c.views.size(); i++) {
          ViewRes& r = res_[c.views[i]];
          BatchView& tv = c.table->v[i];
          tv = BatchView{};
          FillArgs(r, target_dirs, target_dirs, Level0(*r.plain), tv.a);
          tv.a.step_cap = 0;
          tv.n_tab = march_table_size(tv.a);
          if (tv.n_tab > GI_MAX_STEPS)
            return fail(GI_ERR_UNSUPPORTED, "gi_batch_finetune: more steps per direction than GI_MAX_STEPS");
          int tx, ty, tw, th;
          gi_march_tile_grid(r.in.view.width, r.in.view.height, r.in.march.pattern_size, &tx, &ty, &tw, &th);
          tv.tiles_x = tx;
          tv.tiles_total = tx * ty;
        }
      target_dirs_ = target_dirs;
    }
    // The target march of every view's judged tiles: one persistent launch per
    // chunk of views of one march precision (a launch per view leaves most of a
    // wave idle).
    const size_t nc = target_chunks_.size();
    for (size_t c = 0; c < nc && !e; c++) {
      const int cnt = target_cnt_[phase * nc + c];
      if (cnt == 0) continue;
      const int k = target_chunks_[c].precision;
      e = launch_march_batch(*target_chunks_[c].table, d_target_items_ + target_off_[phase * nc + c], cnt,
                             d_target_counter_, kMarchTileSubY, std::min(cnt, target_grid_[k]), k >= 1, k == 2, s);
    }
    size_t row = 0;
    e = e ? e : check_cuda(cudaMemsetAsync(d_sums_, 0, 2 * sizeof(float), s), "gi_batch_finetune");
    for (size_t v = 0; v < res_.size() && !e; v++) {
      ViewRes& r = res_[v];
      const int cnt = r.judge_count[phase];
      if (cnt == 0) continue;
      const int* tiles = d_judge_table_ + ((size_t)v * judge_every_ + phase) * max_count_;
      const int W = r.in.view.width, H = r.in.view.height, P = r.in.march.pattern_size;
      const size_t tp = (size_t)kMarchTileSubX * kMarchTileSubY * P * P;  // pixels per tile
      float* target = Level0(*r.plain);
      e = launch_tiles_copy(target, d_t_ + row * 4, W, H, P, tiles, cnt, false, s);
      e = e ? e : launch_tiles_copy(Level0(*r.learned), d_learned_rows_ + row * 4, W, H, P, tiles, cnt, false, s);
      FeatureArgs fa = Features(r);
      fa.out = d_x_ + row * GI_MLP_IN;
      fa.scale = d_s_ + row;
      fa.tiles = tiles;
      e = e ? e : launch_features(fa, cnt, s);
      row += (size_t)cnt * tp;
    }
    if (e) return e;
    if (row == 0) return GI_OK;
    const int n = (int)row;
    tile_error_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_learned_rows_, d_t_, n, d_sums_);
    e = check_cuda(cudaGetLastError(), "tile_error_kernel");
    loss_weights_kernel<<<1, 1024, 0, s>>>(d_t_, d_s_, n);
    e = e ? e : check_cuda(cudaGetLastError(), "loss_weights_kernel");
    count_launches(2);
    if (e) return e;
    e = gi_mlp_train_step(mlp, d_x_, d_t_, d_s_, n, lr, loss_out, s);
    if (e) return e;
    if (err_out) {
      float h[2];
      e = check_cuda(cudaMemcpyAsync(h, d_sums_, sizeof(h), cudaMemcpyDeviceToHost, s), "gi_batch_finetune");
      e = e ? e : check_cuda(cudaStreamSynchronize(s), "gi_batch_finetune");
      if (e) return e;
      *err_out = h[0] / std::max(h[1], 1e-20f);
    }
    return GI_OK;
  }

  int rows_ = 4, grid_ = 0;
  int NumItems() const { return plain_.Items(); }
  float tuned_ms_ = 0.0f;

 private:
  std::vector<float*> Levels(const legit::MippedProxy& p) { return rg_.ResolveView(p.imageViewProxy->Id()).levels; }
  float* Level0(const legit::UnmippedProxy& p) { return rg_.ResolveView(p.imageViewProxy->Id()).level(0); }

  // March arguments of view r over its blurred pyramids (level 0 = its inputs).
  void FillArgs(ViewRes& r, int dirs, int step_dirs, float* out, MarchArgs& a) {
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
    a.out = out;
    a.width = r.in.view.width;
    a.height = r.in.view.height;
    a.num_levels = r.levels;
    a.depth_ch = 2;
    a.dirs = dirs;
    a.step_cap = r.in.march.step_cap;
    a.pattern = r.in.march.pattern_size;
    a.step_dirs = step_dirs > 0 ? step_dirs : dirs;
    a.tiles = nullptr;
    a.num_tiles = 0;
    a.fast = r.in.march.precision != GI_MARCH_EXACT ? 1 : 0;
    if (a.fast && r.dtex && r.ltex) {
      a.depth_tex = r.dtex->Handle();
      a.light_tex = r.ltex->Handle();
    }
    set_ray_basis(a);
  }

  FeatureArgs Features(ViewRes& r) {
    std::vector<float*> few = Levels(*r.few), db = Levels(*r.depth_blur);
    FeatureArgs fa{};
    fa.width = r.in.view.width;
    fa.height = r.in.view.height;
    fa.pattern = r.in.march.pattern_size;
    fa.moments = r.in.depth_moments;
    fa.normal = r.in.normal;
    fa.albedo = r.in.albedo;
    fa.direct = r.in.direct;
    fa.indirect[0] = few[0];
    fa.indirect[1] = few[2];
    fa.indirect[2] = few[4];
    fa.filtered = Level0(*r.few_f);
    fa.depth_l2 = db[2];
    return fa;
  }

  // Buffers, the few-ray work list and the judge tables of the learned mode.
  int PrepareLearned() {
    max_count_ = 0;
    size_t rows_total = 0;
    few_.Reset();
    for (size_t v = 0; v < res_.size(); v++) {
      ViewRes& r = res_[v];
      const int W = r.in.view.width, H = r.in.view.height;
      if (!r.few) {
        legit::uvec2 size((uint32_t)W, (uint32_t)H);
        try {
          r.few.reset(new legit::MippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size, 0, 5));
          r.few_f.reset(new legit::UnmippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size));
          r.learned.reset(new legit::UnmippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size));
          r.plain.reset(new legit::UnmippedProxy(&rg_, legit::Format::R32G32B32A32Sfloat, size));
        } catch (const legit::GiError& err) {
          return fail(err.status, err.what());
        }
      }
      BatchView bv{};
      FillArgs(r, few_dirs_, few_step_dirs_, Levels(*r.few)[0], bv.a);
      bv.n_tab = march_table_size(bv.a);
      if (bv.n_tab > GI_MAX_STEPS) return fail(GI_ERR_UNSUPPORTED, "gi_batch_set_learned: too many steps per direction");
      few_.Add((int)v, bv);
      int tx, ty, tw, th;
      gi_march_tile_grid(W, H, r.in.march.pattern_size, &tx, &ty, &tw, &th);
      max_count_ = std::max(max_count_, (tx * ty + judge_every_ - 1) / judge_every_);
    }
    int e = few_.Build(rows_);
    if (e) return e;
    std::vector<int> table(res_.size() * (size_t)judge_every_ * max_count_, -1);
    for (size_t v = 0; v < res_.size(); v++) {
      ViewRes& r = res_[v];
      int tx, ty, tw, th;
      gi_march_tile_grid(r.in.view.width, r.in.view.height, r.in.march.pattern_size, &tx, &ty, &tw, &th);
      r.judge_count.assign(judge_every_, 0);
      for (int f = 0; f < judge_every_; f++) {
        int k = 0;
        for (int t = f; t < tx * ty; t += judge_every_) table[((size_t)v * judge_every_ + f) * max_count_ + k++] = t;
        r.judge_count[f] = k;
      }
      rows_total += (size_t)max_count_ * tw * th;
    }
    // Target-march chunks and items: per march precision, the views with the
    // longest diagonals (most steps uncapped) first, in chunks of at most
    // kBatchTableViews; per judge phase and chunk the items (index in the chunk,
    // tile * 64 + pattern), so that each persistent launch ends evenly.
    std::vector<int> order(res_.size());
    for (size_t v = 0; v < order.size(); v++) order[v] = (int)v;
    auto diag = [&](int v) {
      const double W = res_[v].in.view.width, H = res_[v].in.view.height;
      return W * W + H * H;
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return diag(x) > diag(y); });
    target_chunks_.clear();
    for (int k = 0; k < kPrecisions; k++) {  // GI_MARCH_EXACT, _FAST, _TEXTURE = 0, 1, 2
      std::vector<int> of_k;
      for (int v : order)
        if (res_[v].in.march.precision == k) of_k.push_back(v);
      for (size_t c0 = 0; c0 < of_k.size(); c0 += kBatchTableViews) {
        target_chunks_.emplace_back();
        TargetChunk& c = target_chunks_.back();
        c.precision = k;
        c.views.assign(of_k.begin() + c0, of_k.begin() + std::min(of_k.size(), c0 + (size_t)kBatchTableViews));
        c.table.reset(new BatchTable());
      }
    }
    const size_t nc = target_chunks_.size();
    std::vector<int2> titems;
    target_off_.assign(nc * (size_t)judge_every_, 0);
    target_cnt_.assign(nc * (size_t)judge_every_, 0);
    for (int f = 0; f < judge_every_; f++)
      for (size_t c = 0; c < nc; c++) {
        target_off_[f * nc + c] = titems.size();
        const std::vector<int>& vs = target_chunks_[c].views;
        for (size_t i = 0; i < vs.size(); i++) {
          const ViewRes& r = res_[vs[i]];
          const int P2 = r.in.march.pattern_size * r.in.march.pattern_size;
          for (int j = 0; j < r.judge_count[f]; j++) {
            const int t = table[((size_t)vs[i] * judge_every_ + f) * max_count_ + j];
            for (int p = 0; p < P2; p++) titems.push_back(make_int2((int)i, t * 64 + p));
          }
        }
        target_cnt_[f * nc + c] = (int)(titems.size() - target_off_[f * nc + c]);
      }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int k = 0; k < kPrecisions; k++)
      target_grid_[k] = sms * march_batch_occupancy(kMarchTileSubY, k >= 1, k == 2);
    target_dirs_ = 0;  // target views are filled by the first finetune
    dfree(d_target_items_);
    d_target_items_ = nullptr;
    e = check_cuda(dmalloc(&d_target_items_, std::max<size_t>(1, titems.size()) * sizeof(int2)),
                   "gi_batch_set_learned");
    e = e ? e : check_cuda(cudaMemcpy(d_target_items_, titems.data(), titems.size() * sizeof(int2),
                                      cudaMemcpyHostToDevice), "gi_batch_set_learned");
    if (!d_target_counter_) e = e ? e : check_cuda(dmalloc(&d_target_counter_, sizeof(int)), "gi_batch_set_learned");
    if (e) return e;
    dfree(d_judge_table_);
    dfree(d_judge_cur_);
    dfree(d_x_);
    dfree(d_t_);
    dfree(d_s_);
    dfree(d_learned_rows_);
    d_judge_table_ = d_judge_cur_ = nullptr;
    d_x_ = nullptr;
    d_t_ = d_s_ = d_learned_rows_ = nullptr;
    e = check_cuda(dmalloc(&d_judge_table_, table.size() * sizeof(int)), "gi_batch_set_learned");
    e = e ? e : check_cuda(cudaMemcpy(d_judge_table_, table.data(), table.size() * sizeof(int),
                                      cudaMemcpyHostToDevice), "gi_batch_set_learned");
    e = e ? e : check_cuda(dmalloc(&d_judge_cur_, res_.size() * (size_t)max_count_ * sizeof(int)),
                           "gi_batch_set_learned");
    if (!d_frame_) e = e ? e : check_cuda(dmalloc(&d_frame_, sizeof(unsigned)), "gi_batch_set_learned");
    if (!d_stats_) e = e ? e : check_cuda(dmalloc(&d_stats_, 2 * sizeof(int)), "gi_batch_set_learned");
    if (!d_sums_) e = e ? e : check_cuda(dmalloc(&d_sums_, 2 * sizeof(float)), "gi_batch_set_learned");
    e = e ? e : check_cuda(dmalloc(&d_x_, rows_total * GI_MLP_IN * sizeof(__nv_bfloat16)), "gi_batch_set_learned");
    e = e ? e : check_cuda(dmalloc(&d_t_, rows_total * 4 * sizeof(float)), "gi_batch_set_learned");
    e = e ? e : check_cuda(dmalloc(&d_s_, rows_total * sizeof(float)), "gi_batch_set_learned");
    e = e ? e : check_cuda(dmalloc(&d_learned_rows_, rows_total * 4 * sizeof(float)), "gi_batch_set_learned");
    e = e ? e : check_cuda(cudaMemset(d_frame_, 0, sizeof(unsigned)), "gi_batch_set_learned");
    e = e ? e : check_cuda(cudaMemset(d_stats_, 0, 2 * sizeof(int)), "gi_batch_set_learned");
    frames_ = 0;
    return e;
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
      st = plain_.Build(r);
      if (st) break;
      int unused = 0;
      st = plain_.Launch(d_counter_, r, stream_, unused);
      if (!st) st = check_cuda(cudaEventRecord(e0, stream_), "gi_batch autotune");
      for (int k = 0; k < 3 && !st; k++) st = plain_.Launch(d_counter_, r, stream_, unused);
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
    rows_ = best_r;
    st = plain_.Build(best_r);
    grid_ = plain_.Grid();
    return st;
  }

  // Records the frame's passes on `s`: mips and blur of every view, the batched
  // march, then per view the plain (bilateral) or learned tail and the gather.
  int RecordFrame(cudaStream_t s) {
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
    int e = LaunchMips(mips, s, launches);
    if (e) return e;
    for (size_t i = 0; i < blurs.size(); i += kMaxBlurJobs) {
      BlurJobs jobs{};
      for (size_t j = i; j < std::min(blurs.size(), i + kMaxBlurJobs); j++) jobs.job[jobs.count++] = blurs[j];
      e = launch_blur(jobs, s);
      if (e) return e;
      launches++;
    }
    for (auto& r : res_) {
      if (!r.dtex) continue;
      std::vector<float*> db = Levels(*r.depth_blur), lb = Levels(*r.light_blur);
      db[0] = const_cast<float*>(r.in.depth_moments);
      lb[0] = const_cast<float*>(r.in.direct);
      e = r.dtex->Pack(db.data(), 2, s);
      e = e ? e : r.ltex->Pack(lb.data(), 4, s);
      if (e) return e;
      launches += 2;
    }
    e = mlp_ ? RecordLearnedTail(s, launches) : RecordPlainTail(s, launches);
    if (e) return e;
    launches_per_frame_ = launches;
    return GI_OK;
  }

  int LaunchMips(const std::vector<MipJob>& mips, cudaStream_t s, int& launches) {
    for (size_t i = 0; i < mips.size(); i += kMaxMipJobs) {
      MipJobs jobs{};
      for (size_t j = i; j < std::min(mips.size(), i + kMaxMipJobs); j++) jobs.job[jobs.count++] = mips[j];
      int e = launch_mips(jobs, s);
      if (e) return e;
      launches += 2;
    }
    return GI_OK;
  }

  int RecordPlainTail(cudaStream_t s, int& launches) {
    int e = plain_.Launch(d_counter_, rows_, s, launches);
    if (e) return e;
    for (auto& r : res_) {
      const int W = r.in.view.width, H = r.in.view.height;
      float* ind = Level0(*r.indirect);
      float* filt = Level0(*r.filtered);
      e = launch_bilateral(ind, r.in.depth_moments, 2, r.in.normal, filt, W, H, s,
                           r.in.march.precision != GI_MARCH_EXACT);
      if (!e) e = launch_final_gather(r.in.direct, filt, r.in.albedo, r.in.out_lit, W, H, s);
      if (!e && r.in.out_indirect)
        e = check_cuda(cudaMemcpyAsync(r.in.out_indirect, filt, (size_t)W * H * 16, cudaMemcpyDeviceToDevice, s),
                       "gi_batch: indirect copy");
      if (e) return e;
      launches += 2;
    }
    return GI_OK;
  }

  int RecordLearnedTail(cudaStream_t s, int& launches) {
    int e = few_.Launch(d_counter_, rows_, s, launches);
    if (e) return e;
    std::vector<MipJob> mips;
    for (auto& r : res_) {
      MipJob J{};
      std::vector<float*> few = Levels(*r.few);
      for (int k = 0; k < 5; k++) J.levels[k] = few[k];
      J.w = r.in.view.width;
      J.h = r.in.view.height;
      J.channels = 4;
      J.num_levels = 5;
      J.filter = GI_MIP_AVG;
      mips.push_back(J);
    }
    e = LaunchMips(mips, s, launches);
    if (e) return e;
    const int nv = (int)res_.size();
    select_judge_kernel<<<(nv * max_count_ + 255) / 256, 256, 0, s>>>(d_judge_table_, d_judge_cur_, nv, max_count_,
                                                                     judge_every_, d_frame_);
    e = check_cuda(cudaGetLastError(), "select_judge_kernel");
    if (e) return e;
    launches++;
    for (int v = 0; v < nv; v++) {
      ViewRes& r = res_[v];
      const int W = r.in.view.width, H = r.in.view.height, P = r.in.march.pattern_size;
      std::vector<float*> few = Levels(*r.few);
      float* few_f = Level0(*r.few_f);
      float* learned = Level0(*r.learned);
      float* plain = Level0(*r.plain);
      e = launch_bilateral(few[0], r.in.depth_moments, 2, r.in.normal, few_f, W, H, s,
                           r.in.march.precision != GI_MARCH_EXACT);
      if (e) return e;
      FeatureArgs fa = Features(r);
      const float* lv[3] = {fa.indirect[0], fa.indirect[1], fa.indirect[2]};
      e = gi_mlp_reconstruct(mlp_, W, H, P, fa.moments, fa.normal, fa.albedo, fa.direct, lv, fa.filtered,
                             fa.depth_l2, learned, s);
      if (e) return e;
      const int* cur = d_judge_cur_ + (size_t)v * max_count_;
      MarchArgs a{};
      FillArgs(r, r.in.march.dirs, r.in.march.step_dirs, plain, a);
      a.tiles = cur;
      a.num_tiles = max_count_;
      e = launch_march(a, s);
      e = e ? e : launch_judge(learned, plain, W, H, P, cur, max_count_, threshold_, d_stats_, s);
      e = e ? e : launch_final_gather(r.in.direct, learned, r.in.albedo, r.in.out_lit, W, H, s);
      if (!e && r.in.out_indirect)
        e = check_cuda(cudaMemcpyAsync(r.in.out_indirect, learned, (size_t)W * H * 16, cudaMemcpyDeviceToDevice, s),
                       "gi_batch: indirect copy");
      if (e) return e;
      launches += 5;
    }
    frame_tick_kernel<<<1, 1, 0, s>>>(d_frame_);
    e = check_cuda(cudaGetLastError(), "frame_tick_kernel");
    launches++;
    return e;
  }

  int Capture() {
    if (exec_) {
      cudaGraphExecDestroy(exec_);
      exec_ = nullptr;
    }
    int e = check_cuda(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "gi_batch: capture");
    if (e) return e;
    e = RecordFrame(stream_);
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
  WorkLists plain_, few_;
  int* d_counter_ = nullptr;
  cudaStream_t stream_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  int launches_per_frame_ = 0;
  // learned mode
  const gi_mlp* mlp_ = nullptr;
  int few_dirs_ = 2, few_step_dirs_ = 0, judge_every_ = 64, max_count_ = 0;
  float threshold_ = 0.25f;
  int* d_judge_table_ = nullptr;
  int* d_judge_cur_ = nullptr;
  // finetune target march: the views of each march precision in chunks of at
  // most kBatchTableViews (one persistent launch each, the views of the last
  // target_dirs_ as its parameter), items per (judge phase, chunk), the launch's
  // work counter (its own: finetunes may run on another stream than the frames)
  struct TargetChunk {
    int precision = 0;
    std::vector<int> views;  // batch view index of each table entry
    std::unique_ptr<BatchTable> table;
  };
  std::vector<TargetChunk> target_chunks_;
  std::vector<size_t> target_off_;
  std::vector<int> target_cnt_;
  int target_grid_[kPrecisions] = {0, 0, 0};
  int target_dirs_ = 0;
  int2* d_target_items_ = nullptr;
  int* d_target_counter_ = nullptr;
  unsigned* d_frame_ = nullptr;
  int* d_stats_ = nullptr;
  float* d_sums_ = nullptr;
  __nv_bfloat16* d_x_ = nullptr;
  float* d_t_ = nullptr;
  float* d_s_ = nullptr;
  float* d_learned_rows_ = nullptr;
  uint64_t frames_ = 0;
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
                     b.march.pattern_size >= 1 && b.march.pattern_size <= 8 && b.march.step_dirs >= 0 &&
                     (b.march.precision == GI_MARCH_EXACT || b.march.precision == GI_MARCH_FAST ||
                      b.march.precision == GI_MARCH_TEXTURE),
                 "gi_batch_create: bad march parameters");
    if (b.march.occlusion != GI_OCCLUSION_HARD)
      return fail(GI_ERR_UNSUPPORTED, "gi_batch_create: the soft horizon is not batched");
  }
  try {
    std::unique_ptr<gi_batch> b(new gi_batch);
    b->impl.reset(new Batch);
    int e = b->impl->Create(views, num_views, tile_rows);
    if (e) return e;
    *out = b.release();
    return GI_OK;
  } catch (const std::exception& err) {
    return fail(GI_ERR_CUDA, std::string("gi_batch_create: ") + err.what());
  }
}

extern "C" int gi_batch_render(gi_batch* b, void* stream) {
  GI_CHECK_ARG(b, "gi_batch_render: null batch");
  return b->impl->Render((cudaStream_t)stream);
}

extern "C" int gi_batch_info(const gi_batch* b, int* work_items, int* grid, int* tile_rows, float* tuned_ms) {
  GI_CHECK_ARG(b && work_items && grid && tile_rows, "gi_batch_info: null argument");
  *work_items = b->impl->NumItems();
  *grid = b->impl->grid_;
  *tile_rows = b->impl->rows_;
  if (tuned_ms) *tuned_ms = b->impl->tuned_ms_;
  return GI_OK;
}

extern "C" int gi_batch_set_learned(gi_batch* b, const gi_mlp* mlp, int few_dirs, int few_step_dirs, int judge_every,
                                    float threshold) {
  GI_CHECK_ARG(b, "gi_batch_set_learned: null batch");
  GI_CHECK_ARG(!mlp || (few_dirs >= 1 && few_dirs <= GI_MAX_DIRS && few_step_dirs >= 0 && few_step_dirs <= 4096 &&
                        judge_every >= 1 && judge_every <= 4096 && threshold >= 0.0f),
               "gi_batch_set_learned: bad arguments");
  try {
    return b->impl->SetLearned(mlp, few_dirs, few_step_dirs, judge_every, threshold);
  } catch (const std::exception& err) {
    return fail(GI_ERR_CUDA, std::string("gi_batch_set_learned: ") + err.what());
  }
}

extern "C" int gi_batch_finetune(gi_batch* b, gi_mlp* mlp, int target_dirs, float lr, float* loss_out,
                                 float* sampled_error_out, void* stream) {
  GI_CHECK_ARG(b && mlp && target_dirs >= 1 && target_dirs <= GI_MAX_DIRS && lr >= 0.0f,
               "gi_batch_finetune: bad arguments");
  try {
    return b->impl->Finetune(mlp, target_dirs, lr, loss_out, sampled_error_out, (cudaStream_t)stream);
  } catch (const std::exception& err) {
    return fail(GI_ERR_CUDA, std::string("gi_batch_finetune: ") + err.what());
  }
}

extern "C" int gi_batch_stats(const gi_batch* b, int* judged_tiles, int* fallback_tiles) {
  GI_CHECK_ARG(b && judged_tiles && fallback_tiles, "gi_batch_stats: null argument");
  return b->impl->Stats(judged_tiles, fallback_tiles);
}

extern "C" int gi_batch_destroy(gi_batch* b) {
  delete b;
  return GI_OK;
}
