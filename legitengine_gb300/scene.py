"""Scene files of the reference (bin/data/Scenes/*.json) as triangle meshes for
gi_gbuffer_mesh / gi_shadow_map_mesh: a binding of the library's loader
(gi_scene_load, csrc/gi_scene.cpp, which follows Scene.h:55-117 and Mesh.h:14-57),
returning numpy structured arrays with the layouts of gi_mesh_object and
gi_triangle, plus the reference application's camera and light.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

MESH_OBJECT_DTYPE = np.dtype([("lo", "<f4", 3), ("hi", "<f4", 3), ("first", "<i4"), ("count", "<i4"),
                              ("albedo", "<f4", 4), ("emissive", "<f4", 4), ("pad", "<i4", 4)])
TRIANGLE_DTYPE = np.dtype([("p", "<f4", (3, 3)), ("n", "<f4", (3, 3)), ("pad", "<f4", 2)])
assert MESH_OBJECT_DTYPE.itemsize == 80 and TRIANGLE_DTYPE.itemsize == 80


@dataclass
class Scene:
    objects: np.ndarray              # MESH_OBJECT_DTYPE
    triangles: np.ndarray            # TRIANGLE_DTYPE
    names: list = field(default_factory=list)  # mesh name of each object
    shadow_size: int = 1024          # the file's renderer.shadowmapSize[0]


def load_scene(path: str) -> Scene:
    """Loads a scene file with the library's loader (host memory only)."""
    from . import gi
    lib = gi.lib()
    h = C.c_void_p()
    gi._check(lib.gi_scene_load(str(path).encode(), C.byref(h)), "gi_scene_load")
    try:
        no, nt, ss = C.c_int(), C.c_int(), C.c_int()
        gi._check(lib.gi_scene_info(h, C.byref(no), C.byref(nt), C.byref(ss)), "gi_scene_info")
        objects = np.zeros(no.value, MESH_OBJECT_DTYPE)
        tris = np.zeros(nt.value, TRIANGLE_DTYPE)
        gi._check(lib.gi_scene_copy(h, objects.ctypes.data_as(C.c_void_p), tris.ctypes.data_as(C.c_void_p)),
                  "gi_scene_copy")
        names = [lib.gi_scene_object_mesh(h, i).decode() for i in range(no.value)]
    finally:
        lib.gi_scene_destroy(h)
    return Scene(objects, tris, names, ss.value)


def reference_cameras(gi):
    """main.cpp:164-172 and SSVGIRenderer.h:57-59: the camera at (0, 0.5, -2)
    (fovy 1, near 0.01, far 1000) and the light at (0, 5, 0) looking down
    (vertAngle 3.1415 / 2; fovy 0.8, aspect 1, near 0.1, far 100)."""
    cam = gi.GiCamera()
    cam.pos[:] = [0.0, 0.5, -2.0]
    cam.hor_angle, cam.vert_angle = 0.0, 0.0
    cam.fovy, cam.znear, cam.zfar = 1.0, 0.01, 1000.0
    light = gi.GiCamera()
    light.pos[:] = [0.0, 5.0, 0.0]
    light.hor_angle, light.vert_angle = 0.0, 3.1415 / 2.0
    light.fovy, light.znear, light.zfar = 0.8, 0.1, 100.0
    return cam, light
