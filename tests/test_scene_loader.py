"""Scene files (the reference's bin/data/Scenes/*.json format) -> world-space
triangles: JSON with comments, OBJ parsing and triangulation, object placement,
the ReadJsonVec3f defaults (CPU only)."""
import json
import math
import os
from pathlib import Path

import numpy as np
import pytest

from legitengine_gb300 import scene as S

HERE = Path(__file__).parent
ROOM = HERE / "golden" / "scenes" / "room.json"


def _write(tmp_path, scene: str, meshes: dict):
    (tmp_path / "m").mkdir(exist_ok=True)
    for name, text in meshes.items():
        (tmp_path / "m" / name).write_text(text)
    p = tmp_path / "s.json"
    p.write_text(scene)
    return str(p)


QUAD = "v 0 0 0\nv 1 0 0\nv 1 0 1\nv 0 0 1\nvn 0 1 0\nf 1//1 4//1 3//1 2//1\n"


def test_comments_and_vector_defaults(tmp_path):
    """jsoncpp-style comments (also inside none of the strings), ReadJsonVec3f
    defaults: a missing vector or component reads as 0, so a missing "scale"
    collapses the mesh and a 2-component "pos" has z = 0."""
    scene = """// line comment
    { /* block
         comment */ "scene" : { "meshes" : [ { "name" : "q", "filename" : "m/q.obj", "scale" : [2, 1, 3] },
                                           { "name" : "flat", "filename" : "m/q.obj" } ],
        "objects" : [ { "mesh" : "q", "pos" : [1, 2], "albedoColor" : [0.5] },
                      { "mesh" : "flat" } ] },
      "renderer" : { "note" : "a // and a /* inside a string" } }"""
    sc = S.load_scene(_write(tmp_path, scene, {"q.obj": QUAD}))
    assert sc.names == ["q", "flat"] and sc.shadow_size == 1024
    p = sc.triangles["p"][:2].reshape(-1, 3)
    assert np.allclose(p.min(0), [1, 2, 0]) and np.allclose(p.max(0), [3, 2, 3])
    assert sc.objects[0]["albedo"].tolist() == [0.5, 0, 0, 1]
    assert np.all(sc.triangles["p"][2:] == 0)  # scale (0, 0, 0)


def test_triangulation_convex_fan_and_concave_ears(tmp_path):
    scene = '{"scene": {"meshes": [{"name": "q", "filename": "m/q.obj", "scale": [1, 1, 1]}], ' \
            '"objects": [{"mesh": "q"}]}}'
    sc = S.load_scene(_write(tmp_path, scene, {"q.obj": QUAD}))
    # the quad (1, 4, 3, 2) becomes the fan (1, 4, 3), (1, 3, 2) of tinyobjloader's ear clipping
    V = np.array([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]], np.float32)
    assert np.array_equal(sc.triangles["p"][0], V[[0, 3, 2]]) and np.array_equal(sc.triangles["p"][1], V[[0, 2, 1]])
    # L-shaped hexagon (notch.obj): 4 triangles, none across the notch, total area 3
    scene = '{"scene": {"meshes": [{"name": "n", "filename": "meshes/notch.obj", "scale": [1, 1, 1]}], ' \
            '"objects": [{"mesh": "n"}]}}'
    p = tmp_path / "n.json"
    p.write_text(scene)
    (tmp_path / "meshes").mkdir()
    (tmp_path / "meshes" / "notch.obj").write_text((HERE / "golden" / "scenes" / "meshes" / "notch.obj").read_text())
    t = S.load_scene(str(p)).triangles["p"].astype(np.float64)
    assert len(t) == 4
    assert math.isclose(sum(_area(x) for x in t), 3.0, rel_tol=1e-12)
    for x in t:
        c = x.mean(0)
        assert not (c[0] > 1 and c[2] > 1), "a triangle covers the notch"


def test_bad_files_fail_cleanly(tmp_path):
    from legitengine_gb300 import gi
    with pytest.raises(gi.GiError):
        S.load_scene(str(tmp_path / "missing.json"))
    with pytest.raises(gi.GiError):
        S.load_scene(_write(tmp_path, '{"scene": {"meshes": [ {"name": "q", "filename": "m/none.obj"} ]}}', {}))
    with pytest.raises(gi.GiError):
        S.load_scene(_write(tmp_path, '{"scene": /* unterminated', {}))


def _area(p):
    return 0.5 * np.linalg.norm(np.cross(p[1] - p[0], p[2] - p[0]))


def test_room_scene():
    sc = S.load_scene(str(ROOM))
    # the object with an undeclared mesh is skipped (Scene.h:95-99)
    assert sc.names == ["hall", "block", "block", "spike", "notch"]
    assert sc.objects["count"].tolist() == [12, 12, 12, 4, 4]
    assert sc.objects["first"].tolist() == [0, 12, 24, 36, 40]
    assert len(sc.triangles) == 44
    assert sc.shadow_size == 512
    # colours: missing albedoColor -> 0 (ReadJsonVec3f), alpha 1 (SSVGIRenderer.h:142-143)
    assert sc.objects[2]["albedo"].tolist() == [0, 0, 0, 1]
    assert np.allclose(sc.objects[2]["emissive"], [4, 2, 0.5, 1])
    # bounds hold every vertex of the object
    for o in sc.objects:
        p = sc.triangles["p"][o["first"]:o["first"] + o["count"]].reshape(-1, 3)
        assert (p >= o["lo"]).all() and (p <= o["hi"]).all()
    # the hall: scale (3, 1.5, 3) then translate (0, 1.5, 0) -> [-3, 3] x [0, 3] x [-3, 3]
    hall = sc.triangles["p"][0:12].reshape(-1, 3)
    assert np.allclose(hall.min(0), [-3, 0, -3]) and np.allclose(hall.max(0), [3, 3, 3])
    # block 1: rotated by pi/4 about y -> its corners reach 0.3 * sqrt(2) from the centre in x and z
    b = sc.triangles["p"][12:24].reshape(-1, 3) - np.array([-0.8, 0.3, 0.8], np.float32)
    assert np.isclose(np.abs(b[:, 0]).max(), 0.3 * math.sqrt(2), rtol=1e-5)
    assert np.isclose(np.abs(b[:, 1]).max(), 0.3, rtol=1e-6)
    # its normals turned with it: unit length, none axis-aligned in x-z
    n = sc.triangles["n"][12:24].reshape(-1, 3)
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-6)
    side = np.abs(n[:, 1]) < 0.5
    assert np.allclose(np.abs(n[side, 0]), math.sqrt(0.5), atol=1e-6)
    # spike: |angle| below 1e-3 is not applied; the corner without a normal gets (1, 0, 0)
    sp = sc.triangles[36:40]
    assert np.allclose(sp["p"][0, 0], np.array([0.0, 0.6, 0.0]) + [0.2, 0.2, 0.4])
    assert any(np.allclose(c, [1, 0, 0]) for c in sp["n"].reshape(-1, 3))
    # every fixture mesh is wound counter-clockwise about its stated normals
    gn = np.cross(sc.triangles["p"][:, 1] - sc.triangles["p"][:, 0], sc.triangles["p"][:, 2] - sc.triangles["p"][:, 0])
    assert (np.einsum("ij,ij->i", gn, sc.triangles["n"].mean(1)) > 0).all()


def test_reference_cube_scene_summary():
    """The reference's CubeScene.json as the loader reads it (summary written by
    tests/golden/make_scene_summary.py from the reference's own scene and mesh
    files): 6 objects (the hornbug mesh, the inward room, four cubes), 1944
    triangles.  When the reference files are at hand the loader is re-run on them
    and must reproduce the summary."""
    summ = json.loads((HERE / "golden" / "cube_scene_summary.json").read_text())
    assert summ["objects"] == 6 and summ["triangles"] == 1884 + 5 * 12
    assert [o["count"] for o in summ["per_object"]] == [1884, 12, 12, 12, 12, 12]
    assert sum(o["count"] for o in summ["per_object"]) == summ["triangles"]
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_scene_summary", HERE / "golden" / "make_scene_summary.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    scene = mod.reference_root() / mod.SCENE
    if not scene.is_file():
        pytest.skip("the reference's scene files are not present")
    assert mod.summarise(str(scene)) == summ
