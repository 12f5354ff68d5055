// gi_renderer.cu -- the GI segment of SSVGIRenderer::RenderFrame
// (src/Render/Renderers/SSVGIRenderer.h:207-342) on resident G-buffer images,
// recorded through the render-graph shim and replayed as one CUDA graph.
//
// Per bounce:  MipBuilderPass (light, and on the first bounce depth moments; one
// fused launch + tail)  ->  BlurPass (every level >= 1 of both pyramids, one
// launch; level 0 aliased; with GI_MARCH_TEXTURE it also copies the light pyramid,
// and on the first bounce the depth pyramid, into the march's textures)  ->  IndirectLightPass (march)  ->  BilateralPass
// ->  [DenoiserPass]  ->  GatheringPass (direct + indirect * albedo).
// Bounce k > 1 builds its light pyramid from bounce k-1's gathered image; with
// temporal feedback (one bounce per frame) the light pyramid of frame t is built
// from frame t-1's gathered image.
//
// Learned mode (gi_renderer_set_learned) replaces IndirectLightPass by:
// FewRayPass (the march with few directions) -> FewRayMipPass (its levels 1-4)
// -> FewRayFilterPass (5x5 bilateral) -> ReconstructPass (features + MLP in one
// tensor-core kernel: a softmax blend of the filtered few-ray light and its mip
// averages; replaces BilateralPass) -> JudgePass (a tile whose learned result
// differs from the plain march by more than the threshold (relative L1) takes the
// plain result).  The judge's plain march of a rotating 1/judge_every of the
// tiles is forked onto a side stream in FewRayPass and joined in JudgePass, so it
// runs beside the few-ray march and the reconstruction (a parallel branch of the
// captured graph).
//
// Host-buffer frames (gi_renderer_render_host_async) pipeline their copies on
// two more streams: frame k's inputs go in while frame k - 1 renders and its
// image comes out while frame k + 1 renders.
#include <memory>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "gi_internal.h"
#include "gi_kernels.h"
#include "gi_mlp.h"
#define LEGIT_RG_DEVICE_ALLOC(p, bytes) ::gi::dmalloc(p, bytes)
#define LEGIT_RG_DEVICE_FREE(p) ::gi::dfree(p)
#include "legit_render_graph.h"

namespace gi {

class Renderer {
 public:
  Renderer(int w, int h, const gi_frame_params& p) : w_(w), h_(h), p_(p) {
    using legit::Format;
    using legit::uvec2;
    levels_ = gi_mip_level_count(w, h, p.mip_levels);
    uvec2 size((uint32_t)w, (uint32_t)h);
    depth_pyr_.reset(new legit::MippedProxy(&rg_, Format::R32G32Sfloat, size, 0, (uint32_t)levels_));
    depth_blur_.reset(new legit::MippedProxy(&rg_, Format::R32G32Sfloat, size, 0, (uint32_t)levels_));
    light_pyr_.reset(new legit::MippedProxy(&rg_, Format::R32G32B32A32Sfloat, size, 0, (uint32_t)levels_));
    light_blur_.reset(new legit::MippedProxy(&rg_, Format::R32G32B32A32Sfloat, size, 0, (uint32_t)levels_));
    indirect_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
    filtered_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
    denoised_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
    lit_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
    if (p.feedback) prev_lit_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
    // GI_MARCH_TEXTURE: the march fetches its depth and light taps through the
    // texture units, from copies of the pyramids in mipmapped arrays.
    if (p.march.precision == GI_MARCH_TEXTURE && p.march.occlusion != GI_OCCLUSION_SOFT) {
      tex_status_ = depth_tex_.Create(w, h, levels_, 1);
      if (!tex_status_) tex_status_ = light_tex_.Create(w, h, levels_, 4);
    }
  }

  ~Renderer() {
    HostWait();
    for (float* p : staging_) dfree(p);
    for (int* p : judge_lists_) dfree(p);
    dfree(counters_);
    if (judge_fork_) cudaEventDestroy(judge_fork_);
    if (judge_join_) cudaEventDestroy(judge_join_);
    if (judge_stream_) cudaStreamDestroy(judge_stream_);
    for (int k = 0; k < 2; k++) {
      if (in_ready_[k]) cudaEventDestroy(in_ready_[k]);
      if (rendered_[k]) cudaEventDestroy(rendered_[k]);
      if (done_[k]) cudaEventDestroy(done_[k]);
    }
    if (h2d_) cudaStreamDestroy(h2d_);
    if (d2h_) cudaStreamDestroy(d2h_);
  }

  // Pipelined host-buffer frames: frame k's inputs go in on a copy stream into
  // staging set k % 2 while frame k - 1 renders on `s`; its lit image comes out on
  // a second copy stream while frame k + 1 renders.  Before reusing a staging set
  // the host waits for the frame that last used it (k - 2) to be fully copied out.
  void RenderHostAsync(const gi_view& view, const float* const host_in[5], float* out_lit, cudaStream_t s) {
    auto ok = [](cudaError_t e, const char* what) {
      if (e != cudaSuccess) throw legit::GiError(GI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    if (!h2d_) {
      ok(cudaStreamCreateWithFlags(&h2d_, cudaStreamNonBlocking), "render_host_async: stream");
      ok(cudaStreamCreateWithFlags(&d2h_, cudaStreamNonBlocking), "render_host_async: stream");
      for (int k = 0; k < 2; k++) {
        ok(cudaEventCreateWithFlags(&in_ready_[k], cudaEventDisableTiming), "render_host_async: event");
        ok(cudaEventCreateWithFlags(&rendered_[k], cudaEventDisableTiming), "render_host_async: event");
        ok(cudaEventCreateWithFlags(&done_[k], cudaEventDisableTiming), "render_host_async: event");
      }
    }
    const int slot = (int)(host_frames_ & 1);
    if (pending_[slot]) {
      ok(cudaEventSynchronize(done_[slot]), "render_host_async: wait for frame k - 2");
      pending_[slot] = false;
    }
    const size_t px = (size_t)w_ * h_;
    const size_t bytes[5] = {px * 16, px * 16, px * 8, px * 4, px * 16};  // albedo, normal, moments, ndc, direct
    float* d[5];
    for (int j = 0; j < 5; j++) {
      d[j] = Staging(kAsyncStaging + 6 * slot + j, bytes[j]);
      ok(cudaMemcpyAsync(d[j], host_in[j], bytes[j], cudaMemcpyHostToDevice, h2d_), "render_host_async: H2D");
    }
    float* d_out = Staging(kAsyncStaging + 6 * slot + 5, px * 16);
    ok(cudaEventRecord(in_ready_[slot], h2d_), "render_host_async: record");
    ok(cudaStreamWaitEvent(s, in_ready_[slot], 0), "render_host_async: wait");
    gi_frame_inputs in{d[0], d[1], d[2], d[3], d[4]};
    Render(view, in, d_out, nullptr, s);
    ok(cudaEventRecord(rendered_[slot], s), "render_host_async: record");
    ok(cudaStreamWaitEvent(d2h_, rendered_[slot], 0), "render_host_async: wait");
    ok(cudaMemcpyAsync(out_lit, d_out, px * 16, cudaMemcpyDeviceToHost, d2h_), "render_host_async: D2H");
    ok(cudaEventRecord(done_[slot], d2h_), "render_host_async: record");
    pending_[slot] = true;
    host_frames_++;
  }

  // Waits until every pipelined frame's lit image is on the host.
  int HostWait() {
    int e = GI_OK;
    for (int k = 0; k < 2; k++) {
      if (!pending_[k]) continue;
      const int ek = check_cuda(cudaEventSynchronize(done_[k]), "gi_renderer_host_wait");
      pending_[k] = false;
      if (!e) e = ek;
    }
    return e;
  }

  // Enables (mlp != nullptr) or disables the learned reconstructor.
  void SetLearned(const gi_mlp* mlp, int few_dirs, int few_step_dirs, int judge_every, float threshold) {
    using legit::Format;
    using legit::uvec2;
    mlp_ = mlp;
    if (!mlp) return;
    few_dirs_ = few_dirs;
    few_step_dirs_ = few_step_dirs;
    threshold_ = threshold;
    if (!few_pyr_) {
      uvec2 size((uint32_t)w_, (uint32_t)h_);
      few_pyr_.reset(new legit::MippedProxy(&rg_, Format::R32G32B32A32Sfloat, size, 0, 5));
      learned_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
      plain_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
      few_f_.reset(new legit::UnmippedProxy(&rg_, Format::R32G32B32A32Sfloat, size));
      if (dmalloc(&counters_, 2 * sizeof(int)) != cudaSuccess ||
          cudaMemset(counters_, 0, 2 * sizeof(int)) != cudaSuccess)
        throw legit::GiError(GI_ERR_OUT_OF_MEMORY, "SetLearned: device allocation");
      // The judge's march runs beside the few-ray march and the reconstruction:
      // forked onto its own stream, joined before the judge compares.
      if (cudaStreamCreateWithFlags(&judge_stream_, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&judge_fork_, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&judge_join_, cudaEventDisableTiming) != cudaSuccess)
        throw legit::GiError(GI_ERR_CUDA, "SetLearned: judge stream");
    }
    // One tile list per phase: phase f judges the tiles t with t % judge_every == f.
    for (int* p : judge_lists_) dfree(p);
    judge_lists_.clear();
    judge_counts_.clear();
    judge_every_ = judge_every;
    int tx, ty, tw, th;
    gi_march_tile_grid(w_, h_, p_.march.pattern_size, &tx, &ty, &tw, &th);
    for (int f = 0; f < judge_every; f++) {
      std::vector<int> list;
      for (int t = f; t < tx * ty; t += judge_every) list.push_back(t);
      int* d = nullptr;
      if (!list.empty()) {
        if (dmalloc(&d, list.size() * sizeof(int)) != cudaSuccess ||
            cudaMemcpy(d, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
          throw legit::GiError(GI_ERR_OUT_OF_MEMORY, "SetLearned: tile lists");
      }
      judge_lists_.push_back(d);
      judge_counts_.push_back((int)list.size());
    }
  }

  void SetProfiling(bool on) { rg_.SetProfiling(on); }
  const std::vector<legit::RenderGraph::ProfilerTask>& PassTimes() { return rg_.GetLastFrameGpuProfilerData(); }

  void Stats(int* judged, int* fell_back) {
    int h[2] = {0, 0};
    if (counters_) cudaMemcpy(h, counters_, sizeof(h), cudaMemcpyDeviceToHost);
    *judged = h[0];
    *fell_back = h[1];
  }

  // Records and executes one frame.  Level 0 of the depth and light pyramids is
  // the caller's image (no copy): the owned level-0 storage stays unused.
  void Render(const gi_view& view, const gi_frame_inputs& in, float* out_lit, float* out_ind, cudaStream_t s) {
    rg_.DiscardPasses();  // a previous frame whose recording threw (e.g. out of memory) left its passes
    const int L = levels_;
    auto levels_of = [](const legit::MippedProxy& p, legit::RenderGraph& rg) {
      return rg.ResolveView(p.imageViewProxy->Id()).levels;
    };
    std::vector<float*> dl = levels_of(*depth_pyr_, rg_), db = levels_of(*depth_blur_, rg_);
    std::vector<float*> ll = levels_of(*light_pyr_, rg_), lb = levels_of(*light_blur_, rg_);
    dl[0] = const_cast<float*>(in.depth_moments);
    db[0] = dl[0];
    float* ind = rg_.ResolveView(indirect_->imageViewProxy->Id()).level(0);
    float* filt = rg_.ResolveView(filtered_->imageViewProxy->Id()).level(0);
    float* den = rg_.ResolveView(denoised_->imageViewProxy->Id()).level(0);
    float* lit_tmp = rg_.ResolveView(lit_->imageViewProxy->Id()).level(0);
    const int w = w_, h = h_;
    const gi_frame_params p = p_;
    const int plain_sd = p.march.step_dirs > 0 ? p.march.step_dirs : p.march.dirs;
    const int few_sd = few_step_dirs_ > 0 ? few_step_dirs_ : few_dirs_;
    legit::Check(tex_status_, "pyramid textures");
    const PyramidTexture* dtex = depth_tex_.Handle() ? &depth_tex_ : nullptr;
    const PyramidTexture* ltex = light_tex_.Handle() ? &light_tex_ : nullptr;

    // Temporal feedback: the previous frame's gathered image is this frame's light.
    float* prev = prev_lit_ ? rg_.ResolveView(prev_lit_->imageViewProxy->Id()).level(0) : nullptr;
    const bool from_prev = prev && have_prev_;
    for (int b = 0; b < p.bounces; b++) {
      const bool first = b == 0, last = b + 1 == p.bounces;
      std::vector<float*> lvl = ll, lbl = lb;
      lvl[0] = first ? (from_prev ? prev : const_cast<float*>(in.direct)) : lit_tmp;
      lbl[0] = lvl[0];
      rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                      .SetProfilerInfo(legit::Colors::nephritis, "MipBuilderPass")
                      .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                        MipJobs jobs{};
                        auto add = [&](const std::vector<float*>& lv, int ch) {
                          MipJob& J = jobs.job[jobs.count++];
                          for (int k = 0; k < L; k++) J.levels[k] = lv[k];
                          J.w = w;
                          J.h = h;
                          J.channels = ch;
                          J.num_levels = L;
                          J.filter = GI_MIP_AVG;
                        };
                        add(lvl, 4);
                        if (first) add(dl, 2);
                        legit::Check(launch_mips(jobs, ctx.GetCommandBuffer()), "MipBuilderPass");
                      }));
      const bool fast_filters = p.march.precision != GI_MARCH_EXACT;
      auto march_args = [=](int dirs, int step_dirs, float* out) {
        MarchArgs a{};
        for (int k = 0; k < 16; k++) {
          a.inv_view_proj.m[k] = view.inv_view_proj[k];
          a.inv_view.m[k] = view.inv_view[k];
        }
        for (int k = 0; k < L; k++) {
          a.light[k] = lbl[k];
          a.depth[k] = db[k];
        }
        a.normal = in.normal;
        a.ndc = in.ndc_depth;
        a.out = out;
        a.width = w;
        a.height = h;
        a.num_levels = L;
        a.depth_ch = 2;
        a.dirs = dirs;
        a.step_cap = p.march.step_cap;
        a.pattern = p.march.pattern_size;
        a.step_dirs = step_dirs;
        a.deinterleaved = 0;
        a.soft = p.march.occlusion == GI_OCCLUSION_SOFT ? 1 : 0;
        a.fast = (p.march.precision != GI_MARCH_EXACT && !a.soft) ? 1 : 0;
        if (a.fast && dtex && ltex) {
          a.depth_tex = dtex->Handle();
          a.light_tex = ltex->Handle();
        }
        return a;
      };
      // Within a frame every bounce marches the same depth, normals and view; only
      // the light differs.  So the first bounce also records the light-independent
      // part of its march and later bounces re-light the record (bit-identical to
      // marching again, at a fraction of the cost).
      const bool multi = p.bounces > 1;
      auto with_record = [=](MarchArgs a, int slot) {
        if (!multi) return a;
        size_t hb = 0, mb = 0, zb = 0;
        if (march_record_bytes(a, &hb, &mb, &zb) == 0) return a;  // more than 64 steps: march every bounce
        a.rec = first ? 1 : 2;
        a.rec_hc = Staging(kRecordStaging + 3 * slot, hb);
        a.rec_mask = reinterpret_cast<unsigned long long*>(Staging(kRecordStaging + 3 * slot + 1, mb));
        a.rec_hc0 = Staging(kRecordStaging + 3 * slot + 2, zb);
        a.rec_steps = march_table_size(a);
        return a;
      };
      // The light pyramid goes into its texture for the marches that tap it: not
      // for a plain bounce that re-lights the first one's record (the replay
      // takes software light taps).
      const MarchArgs plain_args =
          mlp_ ? MarchArgs{} : with_record(march_args(p.march.dirs, plain_sd, ind), 0);
      const bool pack_light = ltex && (mlp_ || plain_args.rec != 2);
      rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                      .SetProfilerInfo(legit::Colors::wisteria, "BlurPass")
                      .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                        BlurJobs jobs{};
                        for (int k = 1; k < L; k++) {
                          jobs.job[jobs.count++] = BlurJob{lvl[k], lbl[k], w >> k, h >> k, 4, 2, 0, 0};
                          if (first) jobs.job[jobs.count++] = BlurJob{dl[k], db[k], w >> k, h >> k, 2, 2, 0, 0};
                        }
                        legit::Check(launch_blur(jobs, ctx.GetCommandBuffer()), "BlurPass");
                        if (first && dtex) legit::Check(dtex->Pack(db.data(), 2, ctx.GetCommandBuffer()), "BlurPass");
                        if (pack_light) legit::Check(ltex->Pack(lbl.data(), 4, ctx.GetCommandBuffer()), "BlurPass");
                      }));
      const float* cur = ind;
      if (!mlp_) {
        const MarchArgs ma = plain_args;
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::sunFlower, "IndirectLightPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          legit::Check(launch_march(ma, ctx.GetCommandBuffer()), "IndirectLightPass");
                        }));
      } else {
        std::vector<float*> few = levels_of(*few_pyr_, rg_);
        float* learned = rg_.ResolveView(learned_->imageViewProxy->Id()).level(0);
        float* plain = rg_.ResolveView(plain_->imageViewProxy->Id()).level(0);
        float* few_f = rg_.ResolveView(few_f_->imageViewProxy->Id()).level(0);
        const gi_mlp* mlp = mlp_;
        int* counters = counters_;
        const int phase = (int)(frame_ % (uint64_t)judge_every_);
        const int* jl = judge_lists_[phase];
        const int jn = judge_counts_[phase];
        const int few_dirs = few_dirs_;
        const float thr = threshold_;
        const float* dl2 = db[2];
        cudaStream_t js = judge_stream_;
        cudaEvent_t fork = judge_fork_, join = judge_join_;
        const MarchArgs few_args = with_record(march_args(few_dirs, few_sd, few[0]), 1);
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::sunFlower, "FewRayPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          cudaStream_t s = ctx.GetCommandBuffer();
                          if (jn > 0) {  // the judge's plain march of this phase's tiles, on the side stream
                            MarchArgs a = march_args(p.march.dirs, plain_sd, plain);
                            a.tiles = jl;
                            a.num_tiles = jn;
                            legit::Check(check_cuda(cudaEventRecord(fork, s), "judge fork"), "FewRayPass");
                            legit::Check(check_cuda(cudaStreamWaitEvent(js, fork, 0), "judge fork"), "FewRayPass");
                            legit::Check(launch_march(a, js), "JudgePass");
                            legit::Check(check_cuda(cudaEventRecord(join, js), "judge join"), "FewRayPass");
                          }
                          legit::Check(launch_march(few_args, s), "FewRayPass");
                        }));
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::nephritis, "FewRayMipPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          MipJobs jobs{};
                          MipJob& J = jobs.job[jobs.count++];
                          for (int k = 0; k < 5; k++) J.levels[k] = few[k];
                          J.w = w;
                          J.h = h;
                          J.channels = 4;
                          J.num_levels = 5;
                          J.filter = GI_MIP_AVG;
                          legit::Check(launch_mips(jobs, ctx.GetCommandBuffer()), "FewRayMipPass");
                        }));
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::greenSea, "FewRayFilterPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          legit::Check(launch_bilateral(few[0], in.depth_moments, 2, in.normal, few_f, w, h,
                                                        ctx.GetCommandBuffer(), fast_filters),
                                       "FewRayFilterPass");
                        }));
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::orange, "ReconstructPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          const float* lv[3] = {few[0], few[2], few[4]};
                          legit::Check(gi_mlp_reconstruct(mlp, w, h, p.march.pattern_size, in.depth_moments,
                                                          in.normal, in.albedo, lvl[0], lv, few_f, dl2, learned,
                                                          ctx.GetCommandBuffer()),
                                       "ReconstructPass");
                        }));
        if (jn > 0) {
          rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                          .SetProfilerInfo(legit::Colors::pomegranate, "JudgePass")
                          .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                            legit::Check(check_cuda(cudaStreamWaitEvent(ctx.GetCommandBuffer(), join, 0),
                                                    "judge join"),
                                         "JudgePass");
                            legit::Check(launch_judge(learned, plain, w, h, p.march.pattern_size, jl, jn, thr,
                                                      counters, ctx.GetCommandBuffer()),
                                         "JudgePass");
                          }));
        }
        cur = learned;
      }
      // The learned result is already a filtered estimate (residual over the
      // bilaterally filtered few-ray light), so it is not filtered again.
      if (p.bilateral && !mlp_) {
        const float* src = cur;
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::greenSea, "BilateralPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          legit::Check(launch_bilateral(src, in.depth_moments, 2, in.normal, filt, w, h,
                                                        ctx.GetCommandBuffer(), fast_filters),
                                       "BilateralPass");
                        }));
        cur = filt;
      }
      if (p.denoise_radius > 0) {
        const float* src = cur;
        const int r = p.denoise_radius;
        rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                        .SetProfilerInfo(legit::Colors::greenSea, "DenoiserPass")
                        .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                          legit::Check(gi_denoise(src, in.depth_moments, in.normal, den, w, h, r,
                                                  ctx.GetCommandBuffer()),
                                       "DenoiserPass");
                        }));
        cur = den;
      }
      float* dst = last ? out_lit : lit_tmp;
      const float* fin = cur;
      const bool copy_ind = last && out_ind;
      rg_.AddPass(legit::RenderGraph::RenderPassDesc()
                      .SetProfilerInfo(legit::Colors::pomegranate, "GatheringPass")
                      .SetRecordFunc([=](legit::RenderGraph::RenderPassContext ctx) {
                        legit::Check(launch_final_gather(in.direct, fin, in.albedo, dst, w, h,
                                                         ctx.GetCommandBuffer()),
                                     "GatheringPass");
                        if (last && prev) {  // the next frame's light
                          cudaError_t e = cudaMemcpyAsync(prev, dst, (size_t)w * h * 16, cudaMemcpyDeviceToDevice,
                                                          ctx.GetCommandBuffer());
                          if (e != cudaSuccess) throw legit::GiError(GI_ERR_CUDA, "GatheringPass: feedback copy");
                        }
                        if (copy_ind) {
                          cudaError_t e = cudaMemcpyAsync(out_ind, fin, (size_t)w * h * 16, cudaMemcpyDeviceToDevice,
                                                          ctx.GetCommandBuffer());
                          if (e != cudaSuccess) throw legit::GiError(GI_ERR_CUDA, "GatheringPass: copy");
                        }
                      }));
    }
    rg_.Execute(s, s != nullptr);
    frame_++;
    if (prev) have_prev_ = true;
  }

  // Device staging buffers for the host-input entry point.
  float* Staging(int i, size_t bytes) {
    if (staging_.size() <= (size_t)i) staging_.resize(i + 1, nullptr), staging_bytes_.resize(i + 1, 0);
    if (staging_bytes_[i] < bytes) {
      if (staging_[i]) dfree(staging_[i]);
      staging_[i] = nullptr;
      if (dmalloc(&staging_[i], bytes) != cudaSuccess) throw legit::GiError(GI_ERR_OUT_OF_MEMORY, "staging");
      staging_bytes_[i] = bytes;
    }
    return staging_[i];
  }

  int w_, h_, levels_;
  gi_frame_params p_;
  legit::RenderGraph rg_;
  std::unique_ptr<legit::MippedProxy> depth_pyr_, depth_blur_, light_pyr_, light_blur_;
  std::unique_ptr<legit::UnmippedProxy> indirect_, filtered_, denoised_, lit_, prev_lit_;
  PyramidTexture depth_tex_, light_tex_;  // GI_MARCH_TEXTURE: the pyramids for the texture units
  int tex_status_ = GI_OK;
  bool have_prev_ = false;
  std::vector<float*> staging_;
  std::vector<size_t> staging_bytes_;
  // Learned mode.
  const gi_mlp* mlp_ = nullptr;
  int few_dirs_ = 2, few_step_dirs_ = 0, judge_every_ = 64;
  float threshold_ = 0.25f;
  std::unique_ptr<legit::MippedProxy> few_pyr_;
  std::unique_ptr<legit::UnmippedProxy> learned_, plain_, few_f_;
  int* counters_ = nullptr;
  cudaStream_t judge_stream_ = nullptr;
  cudaEvent_t judge_fork_ = nullptr, judge_join_ = nullptr;
  // Pipelined host frames.
  static constexpr int kAsyncStaging = 6;  // staging 0-5: the synchronous host path
  static constexpr int kRecordStaging = 18;  // after the two pipelined sets: the march records (plain, few-ray)
  cudaStream_t h2d_ = nullptr, d2h_ = nullptr;
  cudaEvent_t in_ready_[2] = {nullptr, nullptr}, rendered_[2] = {nullptr, nullptr}, done_[2] = {nullptr, nullptr};
  bool pending_[2] = {false, false};
  uint64_t host_frames_ = 0;
  std::vector<int*> judge_lists_;
  std::vector<int> judge_counts_;
  uint64_t frame_ = 0;
};

}  // namespace gi

struct gi_renderer {
  std::unique_ptr<gi::Renderer> impl;
};

using namespace gi;

extern "C" int gi_renderer_create(int width, int height, const gi_frame_params* params, gi_renderer** out) {
  GI_CHECK_ARG(params && out && width >= 1 && height >= 1, "gi_renderer_create: bad arguments");
  GI_CHECK_ARG(params->bounces >= 1 && params->bounces <= 8, "gi_renderer_create: bounces must be 1..8");
  GI_CHECK_ARG(params->march.dirs >= 1 && params->march.dirs <= GI_MAX_DIRS, "gi_renderer_create: dirs out of range");
  GI_CHECK_ARG(params->march.step_dirs >= 0 && params->march.step_dirs <= 4096,
               "gi_renderer_create: step_dirs out of range");
  GI_CHECK_ARG(params->march.pattern_size >= 1 && params->march.pattern_size <= 8,
               "gi_renderer_create: pattern size out of range");
  GI_CHECK_ARG(params->denoise_radius == 0 || params->denoise_radius == 2, "gi_renderer_create: denoise radius");
  GI_CHECK_ARG(params->march.precision == GI_MARCH_EXACT || params->march.precision == GI_MARCH_FAST ||
                   params->march.precision == GI_MARCH_TEXTURE,
               "gi_renderer_create: unknown precision");
  GI_CHECK_ARG(params->march.occlusion == GI_OCCLUSION_HARD || params->march.occlusion == GI_OCCLUSION_SOFT,
               "gi_renderer_create: unknown occlusion");
  GI_CHECK_ARG(params->mip_levels >= 1, "gi_renderer_create: mip levels");
  GI_CHECK_ARG(params->feedback == 0 || (params->feedback == 1 && params->bounces == 1),
               "gi_renderer_create: temporal feedback takes bounces = 1");
  *out = nullptr;
  try {
    std::unique_ptr<gi_renderer> r(new gi_renderer);
    r->impl.reset(new Renderer(width, height, *params));
    if (r->impl->tex_status_) return r->impl->tex_status_;
    *out = r.release();
    return GI_OK;
  } catch (const legit::GiError& e) {
    return fail(e.status, e.what());
  } catch (const std::exception& e) {
    return fail(GI_ERR_OUT_OF_MEMORY, e.what());
  }
}

extern "C" int gi_renderer_set_learned(gi_renderer* r, const gi_mlp* mlp, int few_dirs, int few_step_dirs,
                                      int judge_every, float judge_threshold) {
  GI_CHECK_ARG(r, "gi_renderer_set_learned: null renderer");
  GI_CHECK_ARG(!mlp || (few_dirs >= 1 && few_dirs <= GI_MAX_DIRS && few_step_dirs >= 0 && few_step_dirs <= 4096 &&
                        judge_every >= 1 && judge_threshold >= 0.0f),
               "gi_renderer_set_learned: bad parameters");
  GI_CHECK_ARG(!mlp || gi_mip_level_count(r->impl->w_, r->impl->h_, 10) >= 5,
               "gi_renderer_set_learned: the viewport needs at least 5 mip levels");
  try {
    r->impl->SetLearned(mlp, few_dirs, few_step_dirs, judge_every, judge_threshold);
  } catch (const legit::GiError& e) {
    return fail(e.status, e.what());
  } catch (const std::exception& e) {
    return fail(GI_ERR_CUDA, e.what());
  }
  return GI_OK;
}

extern "C" int gi_renderer_stats(gi_renderer* r, int* judged_tiles, int* fallback_tiles) {
  GI_CHECK_ARG(r && judged_tiles && fallback_tiles, "gi_renderer_stats: null argument");
  r->impl->Stats(judged_tiles, fallback_tiles);
  return GI_OK;
}

extern "C" int gi_renderer_set_profiling(gi_renderer* r, int enable) {
  GI_CHECK_ARG(r, "gi_renderer_set_profiling: null renderer");
  r->impl->SetProfiling(enable != 0);
  return GI_OK;
}

extern "C" int gi_renderer_pass_times(gi_renderer* r, int max_passes, const char** names, float* start_ms,
                                      float* end_ms, int* num_passes) {
  GI_CHECK_ARG(r && num_passes && max_passes >= 0 && (max_passes == 0 || (names && start_ms && end_ms)),
               "gi_renderer_pass_times: bad arguments");
  try {
    const auto& t = r->impl->PassTimes();
    *num_passes = (int)t.size();
    for (int i = 0; i < max_passes && (size_t)i < t.size(); i++) {
      names[i] = t[(size_t)i].name.c_str();
      start_ms[i] = t[(size_t)i].startMs;
      end_ms[i] = t[(size_t)i].endMs;
    }
  } catch (const legit::GiError& e) {
    return fail(e.status, e.what());
  } catch (const std::exception& e) {
    return fail(GI_ERR_CUDA, e.what());
  }
  return GI_OK;
}

extern "C" int gi_renderer_destroy(gi_renderer* r) {
  delete r;
  return GI_OK;
}

static int check_inputs(const gi_renderer* r, const gi_view* view, const gi_frame_inputs* in) {
  GI_CHECK_ARG(r && view && in, "gi_renderer_render: null argument");
  GI_CHECK_ARG(view->width == r->impl->w_ && view->height == r->impl->h_, "gi_renderer_render: view size mismatch");
  GI_CHECK_ARG(in->albedo && in->normal && in->depth_moments && in->ndc_depth && in->direct,
               "gi_renderer_render: null input");
  GI_CHECK_ARG(aligned16(in->albedo) && aligned16(in->normal) && aligned16(in->depth_moments) &&
                   aligned16(in->direct),
               "gi_renderer_render: unaligned input");
  return GI_OK;
}

extern "C" int gi_renderer_render(gi_renderer* r, const gi_view* view, const gi_frame_inputs* in, float* out_lit,
                                  float* out_indirect, void* stream) {
  int st = check_inputs(r, view, in);
  if (st) return st;
  GI_CHECK_ARG(out_lit && aligned16(out_lit), "gi_renderer_render: bad output");
  try {
    r->impl->Render(*view, *in, out_lit, out_indirect, (cudaStream_t)stream);
  } catch (const legit::GiError& e) {
    return fail(e.status, e.what());
  } catch (const std::exception& e) {
    return fail(GI_ERR_CUDA, e.what());
  }
  return GI_OK;
}

extern "C" int gi_renderer_render_host(gi_renderer* r, const gi_view* view, const float* albedo, const float* normal,
                                       const float* depth_moments, const float* ndc_depth, const float* direct,
                                       float* out_lit, void* stream) {
  GI_CHECK_ARG(r && view && albedo && normal && depth_moments && ndc_depth && direct && out_lit,
               "gi_renderer_render_host: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t px = (size_t)r->impl->w_ * r->impl->h_;
  try {
    float* d_alb = r->impl->Staging(0, px * 16);
    float* d_nrm = r->impl->Staging(1, px * 16);
    float* d_mom = r->impl->Staging(2, px * 8);
    float* d_ndc = r->impl->Staging(3, px * 4);
    float* d_dir = r->impl->Staging(4, px * 16);
    float* d_out = r->impl->Staging(5, px * 16);
    struct Cp {
      float* d;
      const float* h;
      size_t n;
    } cps[5] = {{d_alb, albedo, px * 16}, {d_nrm, normal, px * 16}, {d_mom, depth_moments, px * 8},
                {d_ndc, ndc_depth, px * 4}, {d_dir, direct, px * 16}};
    for (auto& c : cps) {
      int e = check_cuda(cudaMemcpyAsync(c.d, c.h, c.n, cudaMemcpyHostToDevice, s), "gi_renderer_render_host: H2D");
      if (e) return e;
    }
    gi_frame_inputs in{d_alb, d_nrm, d_mom, d_ndc, d_dir};
    int st = gi_renderer_render(r, view, &in, d_out, nullptr, stream);
    if (st) return st;
    int e = check_cuda(cudaMemcpyAsync(out_lit, d_out, px * 16, cudaMemcpyDeviceToHost, s),
                       "gi_renderer_render_host: D2H");
    if (e) return e;
    return check_cuda(cudaStreamSynchronize(s), "gi_renderer_render_host: sync");
  } catch (const legit::GiError& e) {
    return fail(e.status, e.what());
  } catch (const std::exception& e) {
    return fail(GI_ERR_CUDA, e.what());
  }
}

extern "C" int gi_renderer_render_host_async(gi_renderer* r, const gi_view* view, const float* albedo,
                                             const float* normal, const float* depth_moments, const float* ndc_depth,
                                             const float* direct, float* out_lit, void* stream) {
  GI_CHECK_ARG(r && view && albedo && normal && depth_moments && ndc_depth && direct && out_lit,
               "gi_renderer_render_host_async: null argument");
  GI_CHECK_ARG(view->width == r->impl->w_ && view->height == r->impl->h_,
               "gi_renderer_render_host_async: view size mismatch");
  const float* in[5] = {albedo, normal, depth_moments, ndc_depth, direct};
  try {
    r->impl->RenderHostAsync(*view, in, out_lit, (cudaStream_t)stream);
  } catch (const legit::GiError& e) {
    return fail(e.status, e.what());
  } catch (const std::exception& e) {
    return fail(GI_ERR_CUDA, e.what());
  }
  return GI_OK;
}

extern "C" int gi_renderer_host_wait(gi_renderer* r) {
  GI_CHECK_ARG(r, "gi_renderer_host_wait: null argument");
  return r->impl->HostWait();
}
