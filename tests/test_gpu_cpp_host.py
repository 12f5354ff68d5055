"""The drop-in boundary from C++: a host program written against the
reference's render-graph calls (MippedProxy / UnmippedProxy, MipBuilder::BuildMips,
BlurBuilder::ApplyBlur per level as SSVGIRenderer.h:207-221 does, and an
indirect-light pass added with AddPass(RenderPassDesc().SetRecordFunc(...)) that
calls gi_march), compiled with g++ against include/legit_gi.h and the shim,
linked to the library, run as a CUDA graph; its output equals the oracle's."""
import glob
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "legit_render_graph.h"

static std::vector<float> load(const std::string& path, size_t n) {
  std::vector<float> v(n);
  FILE* f = fopen(path.c_str(), "rb");
  if (!f || fread(v.data(), sizeof(float), n, f) != n) { fprintf(stderr, "read %s\n", path.c_str()); exit(2); }
  fclose(f);
  return v;
}

int main(int argc, char** argv) {
  const std::string dir = argv[1];
  const int W = atoi(argv[2]), H = atoi(argv[3]);
  gi_view view;
  FILE* f = fopen((dir + "/view.bin").c_str(), "rb");
  if (!f || fread(&view, sizeof(view), 1, f) != 1) return 2;
  fclose(f);
  try {
    using legit::Format;
    legit::RenderGraph rg;
    legit::ShaderMemoryPool pool;
    legit::uvec2 size((uint32_t)W, (uint32_t)H);
    legit::MippedProxy directLight(&rg, Format::R32G32B32A32Sfloat, size);
    legit::MippedProxy blurredDirectLight(&rg, Format::R32G32B32A32Sfloat, size);
    legit::MippedProxy depthMoments(&rg, Format::R32G32Sfloat, size);
    legit::MippedProxy blurredDepthMoments(&rg, Format::R32G32Sfloat, size);
    legit::UnmippedProxy normal(&rg, Format::R32G32B32A32Sfloat, size);
    legit::UnmippedProxy depthStencil(&rg, Format::R32Sfloat, size);
    legit::UnmippedProxy indirect(&rg, Format::R32G32B32A32Sfloat, size);
    auto upload = [&](legit::RenderGraph::ImageViewProxyId id, const char* name, int ch) {
      std::vector<float> h = load(dir + "/" + name, (size_t)W * H * ch);
      cudaMemcpy(rg.ResolveView(id).level(0), h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
    };
    upload(directLight.imageViewProxy->Id(), "direct.bin", 4);
    upload(depthMoments.imageViewProxy->Id(), "moments.bin", 2);
    upload(normal.imageViewProxy->Id(), "normal.bin", 4);
    upload(depthStencil.imageViewProxy->Id(), "ndc.bin", 1);

    legit::MipBuilder mipBuilder;
    legit::BlurBuilder blurBuilder;
    mipBuilder.BuildMips(&rg, &pool, directLight);
    mipBuilder.BuildMips(&rg, &pool, depthMoments);
    for (uint32_t mip = 0; mip < directLight.mipsCount; mip++) {
      blurBuilder.ApplyBlur(&rg, &pool, directLight.mipImageViewProxies[mip]->Id(),
                            blurredDirectLight.mipImageViewProxies[mip]->Id(), mip == 0 ? 0 : 2);
      blurBuilder.ApplyBlur(&rg, &pool, depthMoments.mipImageViewProxies[mip]->Id(),
                            blurredDepthMoments.mipImageViewProxies[mip]->Id(), mip == 0 ? 0 : 2);
    }
    const auto lightId = blurredDirectLight.imageViewProxy->Id(), depthId = blurredDepthMoments.imageViewProxy->Id();
    const auto normalId = normal.imageViewProxy->Id(), ndcId = depthStencil.imageViewProxy->Id();
    const auto outId = indirect.imageViewProxy->Id();
    rg.AddPass(legit::RenderGraph::RenderPassDesc()
                   .SetColorAttachments({outId})
                   .SetInputImages({lightId, depthId, normalId, ndcId})
                   .SetRenderAreaExtent(legit::Extent2D(W, H))
                   .SetProfilerInfo(legit::Colors::sunFlower, "IndirectLightPass")
                   .SetRecordFunc([&](legit::RenderGraph::RenderPassContext ctx) {
                     const auto& L = ctx.GetImageView(lightId);
                     const auto& D = ctx.GetImageView(depthId);
                     std::vector<const float*> l(L.levels.begin(), L.levels.end()), d(D.levels.begin(), D.levels.end());
                     gi_march_params p{8, 32, 4, 0, GI_MARCH_EXACT, GI_OCCLUSION_HARD};
                     legit::Check(gi_march(&view, &p, l.data(), d.data(), (int)l.size(),
                                           ctx.GetImageView(normalId).level(0), ctx.GetImageView(ndcId).level(0),
                                           ctx.GetImageView(outId).level(0), ctx.GetCommandBuffer()),
                                  "IndirectLightPass");
                   }));
    cudaStream_t stream;
    cudaStreamCreate(&stream);
    rg.Execute(stream, /*use_graph=*/true);
    cudaStreamSynchronize(stream);
    std::vector<float> out((size_t)W * H * 4);
    cudaMemcpy(out.data(), rg.ResolveView(outId).level(0), out.size() * sizeof(float), cudaMemcpyDeviceToHost);
    f = fopen((dir + "/out.bin").c_str(), "wb");
    fwrite(out.data(), sizeof(float), out.size(), f);
    fclose(f);
  } catch (const std::exception& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
'''


def _cudart_dir():
    for pat in ("/usr/local/cuda/lib64/libcudart.so", "/usr/local/cuda/targets/*/lib/libcudart.so"):
        hits = glob.glob(pat)
        if hits:
            return str(Path(hits[0]).parent)
    return None


def test_cpp_host_program_through_the_shim(gi, oracle, scene_small, tmp_path):
    lib = gi.lib()
    libdir = str(Path(lib._name).parent)
    cudart = _cudart_dir()
    if cudart is None:
        pytest.skip("no libcudart.so in the CUDA toolkit")
    s = scene_small
    gb, direct, view = s["gb"], s["direct"], s["view"]
    W, H = view.width, view.height
    for name, arr in (("direct.bin", direct), ("moments.bin", gb["moments"]), ("normal.bin", gb["normal"]),
                      ("ndc.bin", gb["ndc"])):
        np.ascontiguousarray(arr, np.float32).tofile(tmp_path / name)
    (tmp_path / "view.bin").write_bytes(bytes(view))
    src = tmp_path / "host.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "host"
    cmd = ["g++", "-std=c++17", "-O2", str(src), "-o", str(exe), f"-I{ROOT / 'legitengine_gb300' / 'csrc'}",
           f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include", f"-L{libdir}", "-lgi_gb300", f"-L{cudart}",
           "-lcudart", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cudart}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path), str(W), str(H)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "out.bin", np.float32).reshape(H, W, 4)
    L = gi.mip_level_count(W, H, 10)
    ref, _ = oracle.march(view, 8, 32, oracle.blur_pyramid(oracle.mip_chain(direct, L)),
                          oracle.blur_pyramid(oracle.mip_chain(gb["moments"], L)), gb["normal"], gb["ndc"])
    print(f"C++ host program: bit-identical {np.mean(got == ref) * 100:.3f}%")
    assert np.mean(got == ref) >= 0.999
    assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max()
