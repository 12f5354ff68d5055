// legit_render_graph.h -- a CUDA render graph with the call surface of
// LegitEngine's legit::RenderGraph (dependencies/LegitVulkan, an absent
// submodule; the surface below is the one its call sites use):
//
//   renderGraph->AddImage(format, mips, layers, size, usage)      MipBuilder.h:8,22
//   renderGraph->AddImageView(imageId, baseMip, mipCount, ...)    MipBuilder.h:9,23,26
//   renderGraph->GetMipSize(viewId, mip)                          BlurBuilder.h:16
//   renderGraph->AddPass(RenderPassDesc()
//       .SetColorAttachments({dst}).SetInputImages({src})
//       .SetRenderAreaExtent(extent).SetProfilerInfo(color, name)
//       .SetRecordFunc([=](RenderPassContext ctx) { ... }))        MipBuilder.h:155-179
//   ctx.GetCommandBuffer(), ctx.GetImageView(id)                  MipBuilder.h:162,173
//
// Passes are recorded during the frame and executed, in order, by Execute()
// (the reference's InFlightQueue::EndFrame, main.cpp:312).  A record function
// receives the CUDA stream as its "command buffer" and resolves image-view ids
// to device pointers; it launches kernels through the C ABI (legit_gi.h).
// Execute() can capture the frame into a CUDA graph and, when the pass list has
// the same shape as the previous frame's, update the instantiated graph in place
// (cudaGraphExecUpdate) instead of re-instantiating it.
//
// There are no layout transitions or barriers to insert: CUDA stream order
// already serialises the passes.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/legit_gi.h"

// Device memory of the graph's images.  A host program gets cudaMalloc and
// cudaFree; the library's own translation units define these first, to its
// allocator (which counts live allocations and honours the allocation-failure
// test hook).
#ifndef LEGIT_RG_DEVICE_ALLOC
#define LEGIT_RG_DEVICE_ALLOC(p, bytes) cudaMalloc(p, bytes)
#define LEGIT_RG_DEVICE_FREE(p) cudaFree(p)
#endif

namespace legit {

enum class Format { R32Sfloat = 1, R32G32Sfloat = 2, R32G32B32A32Sfloat = 4 };
inline int Channels(Format f) { return (int)f; }

struct uvec2 {
  uint32_t x = 0, y = 0;
  uvec2() {}
  uvec2(uint32_t a, uint32_t b) : x(a), y(b) {}
  bool operator==(const uvec2& o) const { return x == o.x && y == o.y; }
};
struct Extent2D {
  uint32_t width = 0, height = 0;
  Extent2D() {}
  Extent2D(uint32_t w, uint32_t h) : width(w), height(h) {}
};

// The reference passes a per-frame uniform pool to every builder
// (MipBuilder.h:142, BlurBuilder.h:14).  Pass parameters here travel by value
// inside the record function and the kernel arguments, so the pool carries
// nothing; the type keeps the builders' signatures.
struct ShaderMemoryPool {};

namespace Colors {
constexpr uint32_t nephritis = 0xff27ae60, wisteria = 0xff8e44ad, sunFlower = 0xfff1c40f, greenSea = 0xff16a085,
                   pomegranate = 0xffc0392b, orange = 0xfff39c12;
}

class GiError : public std::runtime_error {
 public:
  GiError(int status, const std::string& what) : std::runtime_error(what), status(status) {}
  int status;
};

inline void Check(int status, const char* what) {
  if (status != GI_OK) throw GiError(status, std::string(what) + ": " + gi_last_error());
}

class RenderGraph {
 public:
  struct ImageProxyId {
    int id = -1;
  };
  struct ImageViewProxyId {
    int id = -1;
    bool operator<(const ImageViewProxyId& o) const { return id < o.id; }
  };

  // A resolved view: device pointer of each mip level of the view and its size.
  struct ImageView {
    std::vector<float*> levels;
    uvec2 size;  // size of the view's first level
    int channels = 0;
    float* level(int k) const { return levels.at(k); }
  };

  class ImageProxy {
   public:
    ImageProxyId Id() const { return id; }
    ImageProxyId id;
  };
  class ImageViewProxy {
   public:
    ImageViewProxyId Id() const { return id; }
    ImageViewProxyId id;
  };
  struct ProxyDeleter {
    RenderGraph* graph;
    void operator()(ImageProxy* p) const;
    void operator()(ImageViewProxy* p) const;
  };
  using ImageProxyUnique = std::unique_ptr<ImageProxy, ProxyDeleter>;
  using ImageViewProxyUnique = std::unique_ptr<ImageViewProxy, ProxyDeleter>;

  struct PassContext {
    cudaStream_t GetCommandBuffer() const { return stream; }
    const ImageView& GetImageView(ImageViewProxyId id) const { return graph->ResolveView(id); }
    cudaStream_t stream;
    const RenderGraph* graph;
  };
  using RenderPassContext = PassContext;

  struct PassDescBase {
    std::vector<ImageViewProxyId> colorAttachments, inputImages, storageImages;
    Extent2D renderArea;
    uint32_t profilerColor = 0;
    std::string profilerName;
    std::function<void(PassContext)> recordFunc;
  };
  struct RenderPassDesc : PassDescBase {
    RenderPassDesc& SetColorAttachments(std::vector<ImageViewProxyId> ids) {
      colorAttachments = std::move(ids);
      return *this;
    }
    RenderPassDesc& SetInputImages(std::vector<ImageViewProxyId> ids) {
      inputImages = std::move(ids);
      return *this;
    }
    RenderPassDesc& SetRenderAreaExtent(Extent2D e) {
      renderArea = e;
      return *this;
    }
    RenderPassDesc& SetProfilerInfo(uint32_t color, std::string name) {
      profilerColor = color;
      profilerName = std::move(name);
      return *this;
    }
    RenderPassDesc& SetRecordFunc(std::function<void(RenderPassContext)> f) {
      recordFunc = std::move(f);
      return *this;
    }
  };
  struct ComputePassDesc : PassDescBase {
    ComputePassDesc& SetStorageImages(std::vector<ImageViewProxyId> ids) {
      storageImages = std::move(ids);
      return *this;
    }
    ComputePassDesc& SetInputImages(std::vector<ImageViewProxyId> ids) {
      inputImages = std::move(ids);
      return *this;
    }
    ComputePassDesc& SetProfilerInfo(uint32_t color, std::string name) {
      profilerColor = color;
      profilerName = std::move(name);
      return *this;
    }
    ComputePassDesc& SetRecordFunc(std::function<void(PassContext)> f) {
      recordFunc = std::move(f);
      return *this;
    }
  };

  RenderGraph() = default;
  ~RenderGraph() { Release(); }
  RenderGraph(const RenderGraph&) = delete;
  RenderGraph& operator=(const RenderGraph&) = delete;

  // Allocates an image of `mips` levels (level k: size >> k) in one device
  // allocation, levels 256-byte aligned.
  ImageProxyUnique AddImage(Format format, uint32_t mips, uint32_t layers, uvec2 size, uint32_t usage = 0) {
    (void)usage;
    if (layers != 1) throw GiError(GI_ERR_UNSUPPORTED, "AddImage: only single-layer images");
    Image img;
    img.format = format;
    img.size = size;
    size_t off = 0;
    for (uint32_t k = 0; k < mips; k++) {
      img.offsets.push_back(off);
      size_t bytes = (size_t)(size.x >> k) * (size.y >> k) * Channels(format) * sizeof(float);
      off += (bytes + 255) / 256 * 256;
    }
    if (off == 0) off = 256;
    cudaError_t e = LEGIT_RG_DEVICE_ALLOC(&img.base, off);
    if (e != cudaSuccess) throw GiError(GI_ERR_OUT_OF_MEMORY, "AddImage: cudaMalloc failed");
    img.bytes = off;
    int id = next_image_++;
    images_[id] = img;
    ImageProxyUnique p(new ImageProxy, ProxyDeleter{this});
    p->id.id = id;
    return p;
  }

  ImageViewProxyUnique AddImageView(ImageProxyId image, uint32_t baseMip, uint32_t mipCount, uint32_t baseLayer,
                                    uint32_t layerCount) {
    (void)baseLayer;
    (void)layerCount;
    const Image& img = images_.at(image.id);
    View v;
    v.image = image.id;
    v.view.channels = Channels(img.format);
    v.view.size = uvec2(img.size.x >> baseMip, img.size.y >> baseMip);
    for (uint32_t k = 0; k < mipCount; k++)
      v.view.levels.push_back(reinterpret_cast<float*>(img.base + img.offsets.at(baseMip + k)));
    return MakeView(std::move(v));
  }

  // A view over caller-owned device memory (the reference's
  // AddExternalImageView, MipBuilder.h:65); `levels` may be rebound each frame
  // with RebindExternalView.
  ImageViewProxyUnique AddExternalImageView(std::vector<float*> levels, uvec2 size, Format format) {
    View v;
    v.image = -1;
    v.view.channels = Channels(format);
    v.view.size = size;
    v.view.levels = std::move(levels);
    return MakeView(std::move(v));
  }
  void RebindExternalView(ImageViewProxyId id, std::vector<float*> levels) {
    View& v = views_.at(id.id);
    v.view.levels = std::move(levels);
  }

  uvec2 GetMipSize(ImageViewProxyId id, uint32_t mip) const {
    const ImageView& v = ResolveView(id);
    return uvec2(v.size.x >> mip, v.size.y >> mip);
  }

  // Drops passes recorded but not executed (a frame whose recording failed).
  void DiscardPasses() { passes_.clear(); }
  void AddPass(RenderPassDesc& desc) { passes_.push_back(desc); }
  void AddPass(RenderPassDesc&& desc) { passes_.push_back(std::move(desc)); }
  void AddPass(ComputePassDesc& desc) { passes_.push_back(desc); }
  void AddPass(ComputePassDesc&& desc) { passes_.push_back(std::move(desc)); }

  // GPU profiling of the passes (what the reference's GPU profiler shows from
  // each pass's SetProfilerInfo): while enabled, Execute records a timing event
  // on the stream before every pass and after the last one (in a captured graph
  // as event-record nodes), and GetLastFrameGpuProfilerData() turns the last
  // executed frame's events into per-pass intervals.
  struct ProfilerTask {
    std::string name;
    uint32_t color;
    float startMs, endMs;  // from the start of the frame's first pass
  };
  void SetProfiling(bool on) { profiling_ = on; }
  bool Profiling() const { return profiling_; }
  // Waits for the last profiled frame's final event.
  const std::vector<ProfilerTask>& GetLastFrameGpuProfilerData() {
    if (profiled_passes_ > 0) {
      if (cudaEventSynchronize(events_[profiled_passes_]) != cudaSuccess)
        throw GiError(GI_ERR_CUDA, "GetLastFrameGpuProfilerData: event wait failed");
      for (size_t i = 0; i < profiled_passes_; i++) {
        float a = 0.0f, b = 0.0f;
        cudaEventElapsedTime(&a, events_[0], events_[i]);
        cudaEventElapsedTime(&b, events_[0], events_[i + 1]);
        tasks_[i].startMs = a;
        tasks_[i].endMs = b;
      }
    }
    return tasks_;
  }

  // Runs every recorded pass on `stream` and clears the list.  With use_graph,
  // the passes are captured into a CUDA graph that is launched once.
  void Execute(cudaStream_t stream, bool use_graph) {
    std::vector<PassDescBase> passes;
    passes.swap(passes_);
    if (profiling_) PrepareProfiler(passes);
    else profiled_passes_ = 0;
    auto run = [&](bool captured) {
      for (size_t i = 0; i < passes.size(); i++) {
        if (profiling_) Mark(i, stream, captured);
        passes[i].recordFunc(PassContext{stream, this});
      }
      if (profiling_) Mark(passes.size(), stream, captured);
    };
    if (!use_graph) {
      run(false);
      return;
    }
    cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    if (cudaStreamBeginCapture(stream, mode) != cudaSuccess)
      throw GiError(GI_ERR_CUDA, "Execute: cudaStreamBeginCapture failed");
    try {
      run(true);
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    cudaGraph_t graph = nullptr;
    if (cudaStreamEndCapture(stream, &graph) != cudaSuccess)
      throw GiError(GI_ERR_CUDA, "Execute: cudaStreamEndCapture failed");
    bool updated = false;
    if (exec_) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(exec_, graph, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
      }
    }
    if (!updated && cudaGraphInstantiate(&exec_, graph, 0) != cudaSuccess) {
      cudaGraphDestroy(graph);
      exec_ = nullptr;
      throw GiError(GI_ERR_CUDA, "Execute: cudaGraphInstantiate failed");
    }
    cudaGraphDestroy(graph);
    if (cudaGraphLaunch(exec_, stream) != cudaSuccess) throw GiError(GI_ERR_CUDA, "Execute: cudaGraphLaunch failed");
    graph_launches_++;
  }

  const ImageView& ResolveView(ImageViewProxyId id) const { return views_.at(id.id).view; }
  uint64_t GraphLaunches() const { return graph_launches_; }

 private:
  struct Image {
    Format format;
    uvec2 size;
    std::vector<size_t> offsets;
    char* base = nullptr;
    size_t bytes = 0;
  };
  struct View {
    int image;
    ImageView view;
  };

  ImageViewProxyUnique MakeView(View v) {
    int id = next_view_++;
    views_[id] = std::move(v);
    ImageViewProxyUnique p(new ImageViewProxy, ProxyDeleter{this});
    p->id.id = id;
    return p;
  }
  void FreeImage(int id) {
    auto it = images_.find(id);
    if (it == images_.end()) return;
    LEGIT_RG_DEVICE_FREE(it->second.base);
    images_.erase(it);
  }
  void FreeView(int id) { views_.erase(id); }
  void Release() {
    for (auto& kv : images_) LEGIT_RG_DEVICE_FREE(kv.second.base);
    images_.clear();
    views_.clear();
    if (exec_) cudaGraphExecDestroy(exec_);
    exec_ = nullptr;
    for (cudaEvent_t e : events_) cudaEventDestroy(e);
    events_.clear();
  }

  void PrepareProfiler(const std::vector<PassDescBase>& passes) {
    while (events_.size() < passes.size() + 1) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) throw GiError(GI_ERR_CUDA, "profiler: cudaEventCreate failed");
      events_.push_back(e);
    }
    tasks_.clear();
    for (const auto& p : passes) tasks_.push_back(ProfilerTask{p.profilerName, p.profilerColor, 0.0f, 0.0f});
    profiled_passes_ = passes.size();
  }

  // Timing event i on the stream; inside a capture it becomes an event-record node.
  void Mark(size_t i, cudaStream_t stream, bool captured) {
    const cudaError_t e = captured ? cudaEventRecordWithFlags(events_[i], stream, cudaEventRecordExternal)
                                   : cudaEventRecord(events_[i], stream);
    if (e != cudaSuccess) throw GiError(GI_ERR_CUDA, "profiler: event record failed");
  }

  std::map<int, Image> images_;
  std::map<int, View> views_;
  std::vector<PassDescBase> passes_;
  int next_image_ = 0, next_view_ = 0;
  cudaGraphExec_t exec_ = nullptr;
  bool profiling_ = false;
  std::vector<cudaEvent_t> events_;
  std::vector<ProfilerTask> tasks_;
  size_t profiled_passes_ = 0;
  uint64_t graph_launches_ = 0;
};

inline void RenderGraph::ProxyDeleter::operator()(ImageProxy* p) const {
  if (graph) graph->FreeImage(p->id.id);
  delete p;
}
inline void RenderGraph::ProxyDeleter::operator()(ImageViewProxy* p) const {
  if (graph) graph->FreeView(p->id.id);
  delete p;
}

// MipBuilder.h:3-14.
struct UnmippedProxy {
  UnmippedProxy(RenderGraph* rg, Format format, uvec2 baseSize, uint32_t usage = 0) : baseSize(baseSize) {
    imageProxy = rg->AddImage(format, 1, 1, baseSize, usage);
    imageViewProxy = rg->AddImageView(imageProxy->Id(), 0, 1, 0, 1);
  }
  RenderGraph::ImageProxyUnique imageProxy;
  RenderGraph::ImageViewProxyUnique imageViewProxy;
  uvec2 baseSize;
};

// MipBuilder.h:16-33, with the level count clamped to the levels the size has
// (gi_mip_level_count).
struct MippedProxy {
  MippedProxy(RenderGraph* rg, Format format, uvec2 baseSize, uint32_t usage = 0, uint32_t requestedMips = 10)
      : baseSize(baseSize) {
    mipsCount = (uint32_t)gi_mip_level_count((int)baseSize.x, (int)baseSize.y, (int)requestedMips);
    imageProxy = rg->AddImage(format, mipsCount, 1, baseSize, usage);
    imageViewProxy = rg->AddImageView(imageProxy->Id(), 0, mipsCount, 0, 1);
    for (uint32_t m = 0; m < mipsCount; m++) mipImageViewProxies.push_back(rg->AddImageView(imageProxy->Id(), m, 1, 0, 1));
  }
  RenderGraph::ImageProxyUnique imageProxy;
  RenderGraph::ImageViewProxyUnique imageViewProxy;
  std::vector<RenderGraph::ImageViewProxyUnique> mipImageViewProxies;
  uvec2 baseSize;
  uint32_t mipsCount;
};

// MipBuilder::BuildMips (MipBuilder.h:142-181): the per-level passes of the
// reference become one pass whose record function builds every level.
class MipBuilder {
 public:
  enum struct FilterTypes { Avg, Depth };
  void BuildMips(RenderGraph* rg, ShaderMemoryPool* pool, const MippedProxy& proxy,
                 FilterTypes filterType = FilterTypes::Avg) {
    (void)pool;
    auto viewId = proxy.imageViewProxy->Id();
    auto size = proxy.baseSize;
    int filter = filterType == FilterTypes::Avg ? GI_MIP_AVG : GI_MIP_DEPTH;
    rg->AddPass(RenderGraph::RenderPassDesc()
                    .SetColorAttachments({viewId})
                    .SetInputImages({viewId})
                    .SetRenderAreaExtent(Extent2D(size.x / 2, size.y / 2))
                    .SetProfilerInfo(Colors::nephritis, "MipBuilderPass")
                    .SetRecordFunc([viewId, size, filter](RenderGraph::RenderPassContext ctx) {
                      const auto& v = ctx.GetImageView(viewId);
                      Check(gi_build_mips(v.levels.data(), (int)size.x, (int)size.y, v.channels,
                                          (int)v.levels.size(), filter, ctx.GetCommandBuffer()),
                            "MipBuilderPass");
                    }));
  }
};

// BlurBuilder::ApplyBlur (BlurBuilder.h:14-46), plus the whole-pyramid form of
// the loops at SSVGIRenderer.h:209-221 (radius 0 at level 0, 2 above).
class BlurBuilder {
 public:
  void ApplyBlur(RenderGraph* rg, ShaderMemoryPool* pool, RenderGraph::ImageViewProxyId src,
                 RenderGraph::ImageViewProxyId dst, int radius) {
    (void)pool;
    uvec2 size = rg->GetMipSize(src, 0);
    if (!(size == rg->GetMipSize(dst, 0))) throw GiError(GI_ERR_INVALID_ARGUMENT, "ApplyBlur: size mismatch");
    rg->AddPass(RenderGraph::RenderPassDesc()
                    .SetColorAttachments({dst})
                    .SetInputImages({src})
                    .SetRenderAreaExtent(Extent2D(size.x, size.y))
                    .SetProfilerInfo(Colors::wisteria, "BlurPass")
                    .SetRecordFunc([src, dst, size, radius](RenderGraph::RenderPassContext ctx) {
                      const auto& s = ctx.GetImageView(src);
                      const auto& d = ctx.GetImageView(dst);
                      Check(gi_blur(s.level(0), d.level(0), (int)size.x, (int)size.y, s.channels, radius,
                                    ctx.GetCommandBuffer()),
                            "BlurPass");
                    }));
  }
  void ApplyBlurPyramid(RenderGraph* rg, ShaderMemoryPool* pool, RenderGraph::ImageViewProxyId src,
                        RenderGraph::ImageViewProxyId dst) {
    (void)pool;
    uvec2 size = rg->GetMipSize(src, 0);
    rg->AddPass(RenderGraph::RenderPassDesc()
                    .SetColorAttachments({dst})
                    .SetInputImages({src})
                    .SetRenderAreaExtent(Extent2D(size.x, size.y))
                    .SetProfilerInfo(Colors::wisteria, "BlurPyramidPass")
                    .SetRecordFunc([src, dst, size](RenderGraph::RenderPassContext ctx) {
                      const auto& s = ctx.GetImageView(src);
                      const auto& d = ctx.GetImageView(dst);
                      std::vector<const float*> sl(s.levels.begin(), s.levels.end());
                      Check(gi_blur_pyramid(sl.data(), d.levels.data(), (int)size.x, (int)size.y, s.channels,
                                            (int)s.levels.size(), ctx.GetCommandBuffer()),
                            "BlurPyramidPass");
                    }));
  }
};

// InterleaveBuilder (InterleaveBuilder.h:14-80).  Interleave runs the
// interleave map (the reference binds the deinterleave program there,
// InterleaveBuilder.h:60-62; the intended behaviour is implemented).
class InterleaveBuilder {
 public:
  void Deinterleave(RenderGraph* rg, ShaderMemoryPool* pool, RenderGraph::ImageViewProxyId interleaved,
                    RenderGraph::ImageViewProxyId deinterleaved, uvec2 gridSize) {
    Add(rg, pool, interleaved, deinterleaved, gridSize, false);
  }
  void Interleave(RenderGraph* rg, ShaderMemoryPool* pool, RenderGraph::ImageViewProxyId deinterleaved,
                  RenderGraph::ImageViewProxyId interleaved, uvec2 gridSize) {
    Add(rg, pool, deinterleaved, interleaved, gridSize, true);
  }

 private:
  void Add(RenderGraph* rg, ShaderMemoryPool*, RenderGraph::ImageViewProxyId src, RenderGraph::ImageViewProxyId dst,
           uvec2 grid, bool interleave) {
    uvec2 size = rg->GetMipSize(interleave ? dst : src, 0);
    rg->AddPass(RenderGraph::RenderPassDesc()
                    .SetColorAttachments({dst})
                    .SetInputImages({src})
                    .SetRenderAreaExtent(Extent2D(size.x, size.y))
                    .SetProfilerInfo(Colors::nephritis, interleave ? "Interleave" : "Deinterleave")
                    .SetRecordFunc([src, dst, size, grid, interleave](RenderGraph::RenderPassContext ctx) {
                      const auto& s = ctx.GetImageView(src);
                      const auto& d = ctx.GetImageView(dst);
                      int st = interleave ? gi_interleave(s.level(0), d.level(0), (int)size.x, (int)size.y,
                                                          s.channels, (int)grid.x, (int)grid.y, ctx.GetCommandBuffer())
                                          : gi_deinterleave(s.level(0), d.level(0), (int)size.x, (int)size.y,
                                                            s.channels, (int)grid.x, (int)grid.y,
                                                            ctx.GetCommandBuffer());
                      Check(st, interleave ? "Interleave" : "Deinterleave");
                    }));
  }
};

}  // namespace legit
