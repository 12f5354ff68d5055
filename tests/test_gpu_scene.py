"""Triangle-mesh scenes on the GPU: the mesh G-buffer and shadow map against the
oracle's restatement bit for bit, analytic primitives and meshes together, and
the headless scene renderer end to end against the oracle's frame."""
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

ROOM = str(Path(__file__).parent / "golden" / "scenes" / "room.json")


def host(t):
    return t.detach().cpu().numpy()


def _gpu_inputs(gi, torch, view, light_view, mesh, cull, prims=None):
    f = dict(dtype=torch.float32, device="cuda")
    H, W = view.height, view.width
    t = {k: torch.full((H, W, c), -9.0, **f) for k, c in (("albedo", 4), ("emissive", 4), ("normal", 4),
                                                          ("moments", 2), ("ndc", 1))}
    sm = torch.full((light_view.height, light_view.width, 1), -9.0, **f)
    pd, npr = (gi.prims_to_device(prims) if prims is not None else (None, 0))
    gi.gbuffer_mesh(view, mesh, t["albedo"], t["emissive"], t["normal"], t["moments"], t["ndc"], prims_dev=pd,
                    num_prims=npr, cull=cull)
    gi.shadow_map_mesh(light_view, mesh, sm, prims_dev=pd, num_prims=npr, cull=cull)
    return t, sm


@pytest.mark.parametrize("cull", [0, 1])
def test_mesh_gbuffer_and_shadow_bit_identical(gi, oracle, cuda, cull):
    torch = cuda
    from legitengine_gb300 import scene as S
    sc = S.load_scene(ROOM)
    cam, light = S.reference_cameras(gi)
    view = gi.view_from_camera(cam, 200, 120)
    lv = gi.view_from_camera(light, 160, 160)
    t, sm = _gpu_inputs(gi, torch, view, lv, gi.MeshDevice(sc), cull)
    torch.cuda.synchronize()
    gb = oracle.gbuffer_mesh(view, sc.objects, sc.triangles, cull=cull)
    osm = oracle.shadow_map_mesh(lv, sc.objects, sc.triangles, cull=cull)
    for k in ("albedo", "emissive", "normal", "moments", "ndc"):
        np.testing.assert_array_equal(host(t[k]), gb[k], err_msg=k)
    np.testing.assert_array_equal(host(sm), osm)
    # every pixel sees the room or an object; the floor under the light is lit
    assert (gb["moments"][..., 0] > 0).all()
    if cull:
        assert (osm < 1.0).mean() > 0.5  # the light sees through the room's ceiling onto the floor and objects


def test_meshes_and_analytic_primitives_together(gi, oracle, cuda):
    """Spheres and a box next to the meshes: the nearest of both kinds wins, as in the oracle."""
    torch = cuda
    from legitengine_gb300 import scene as S
    sc = S.load_scene(ROOM)
    prims = (gi.GiPrim * 3)()
    for i, (kind, a, b) in enumerate([(gi.GI_PRIM_SPHERE, (0.6, 0.4, 0.0), (0.35, 0, 0)),
                                      (gi.GI_PRIM_SPHERE, (-0.9, 0.3, 0.8), (0.25, 0, 0)),  # overlaps a block
                                      (gi.GI_PRIM_BOX, (-0.2, 0.0, 1.6), (0.3, 0.8, 2.0))]):
        prims[i].kind = kind
        prims[i].a[:] = a
        prims[i].b[:] = b
        prims[i].albedo[:] = (0.3 + 0.2 * i, 0.5, 0.7, 1.0)
    cam, light = S.reference_cameras(gi)
    view = gi.view_from_camera(cam, 160, 96)
    lv = gi.view_from_camera(light, 128, 128)
    t, sm = _gpu_inputs(gi, torch, view, lv, gi.MeshDevice(sc), 1, prims)
    torch.cuda.synchronize()
    gb = oracle.gbuffer_mesh(view, sc.objects, sc.triangles, prims=prims)
    osm = oracle.shadow_map_mesh(lv, sc.objects, sc.triangles, prims=prims)
    for k in ("albedo", "normal", "moments", "ndc"):
        np.testing.assert_array_equal(host(t[k]), gb[k], err_msg=k)
    np.testing.assert_array_equal(host(sm), osm)
    # the spheres are in the picture
    alb = gb["albedo"][..., 0]
    assert (np.isclose(alb, 0.3 ** 2.2, rtol=1e-6)).sum() > 50


def test_render_scene_matches_oracle(gi, oracle, cuda, tmp_path):
    """render_scene.py on the test scene (exact precision, 1 bounce, 8 directions):
    the GPU inputs equal the oracle's, the lit frame equals the oracle's frame on
    them, and the CLI writes the same image to a PFM file."""
    torch = cuda
    from legitengine_gb300 import render_scene as RS
    from legitengine_gb300 import scene as S
    W, H = 192, 112
    lit, info = RS.render(ROOM, W, H, dirs=8, cap=32, bounces=1, precision="exact")
    assert info["triangles"] == 44 and info["objects"] == 5
    sc = S.load_scene(ROOM)
    cam, light = S.reference_cameras(gi)
    view = gi.view_from_camera(cam, W, H)
    lv = gi.view_from_camera(light, sc.shadow_size, sc.shadow_size)
    gb = oracle.gbuffer_mesh(view, sc.objects, sc.triangles)
    osm = oracle.shadow_map_mesh(lv, sc.objects, sc.triangles)
    od = oracle.direct_light(view, lv, gb, osm)
    ref = oracle.render_frame(view, gb, od, 8, 32, bounces=1)
    e = rel_err(lit, ref["lit"])
    exact = float(np.mean(lit == ref["lit"]))
    print(f"scene frame: max rel {e.max():.3g}, bit-identical {exact * 100:.3f}%, {info}")
    assert e.max() <= 1e-3 and exact >= 0.999
    assert np.isfinite(lit).all() and lit[..., :3].mean() > 0.01
    out = tmp_path / "lit.pfm"
    assert RS.main([ROOM, "--out", str(out), "--width", str(W), "--height", str(H), "--dirs", "8", "--cap", "32",
                    "--bounces", "1", "--precision", "exact"]) == 0
    np.testing.assert_array_equal(RS.read_pfm(str(out)), lit[..., :3])


@pytest.mark.parametrize("learned,precision", [(False, "fast"), (True, "fast"), (False, "texture")])
def test_cpp_scene_renderer_matches_python(gi, cuda, tmp_path, learned, precision):
    """The C++ headless renderer (lib/gi_render_scene, C ABI only: gi_scene_load,
    mesh G-buffer and shadow map, direct light, GI renderer) writes the same image
    as the Python front end for the same scene and settings."""
    import json
    import subprocess

    from legitengine_gb300 import build as B
    from legitengine_gb300 import render_scene as RS
    from legitengine_gb300 import train_reconstructor as tr
    W, H = 224, 128
    out = tmp_path / "cpp.pfm"
    cmd = [str(B.CLI), ROOM, str(out), "--width", str(W), "--height", str(H), "--dirs", "8", "--cap", "32",
           "--bounces", "2"]
    if learned:
        cmd += ["--learned", str(tr.DEFAULT_WEIGHTS)]
    if precision == "texture":
        cmd += ["--texture"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    info = json.loads(r.stdout.strip().splitlines()[-1])
    assert info["triangles"] == 44 and info["objects"] == 5
    lit, _ = RS.render(ROOM, W, H, dirs=8, cap=32, bounces=2, precision=precision, learned=learned)
    np.testing.assert_array_equal(RS.read_pfm(str(out)), lit[..., :3])
