"""Scene files of the reference (bin/data/Scenes/*.json) as triangle meshes for
gi_gbuffer_mesh / gi_shadow_map_mesh.

The reference loads a scene in Scene.h:55-117: each entry of "meshes" is an OBJ
file read by tinyobjloader with triangulation (Mesh.h:14-57: positions times the
entry's "scale", the vertex normal or (1, 0, 0) when a corner has none); each
entry of "objects" places a mesh by translate(pos) * rotate(|angle|, angle /
|angle|) (the rotation only when |angle| > 1e-3) with "albedoColor" and
"emissiveColor", which the G-buffer pass extends with alpha 1
(SSVGIRenderer.h:142-143).  Vectors are read as ReadJsonVec3f does
(main.cpp:24-27): a missing member reads as (0, 0, 0).  The JSON may hold C and
C++ comments (jsoncpp accepts them).  The camera and light are those main.cpp
sets up (main.cpp:164-172) with the projections of SSVGIRenderer.h:57-59.

Everything here runs on the host: it builds the world-space triangle and object
arrays (numpy structured arrays with the layouts of gi_triangle and
gi_mesh_object) that the G-buffer and shadow-map kernels ray cast.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

MESH_OBJECT_DTYPE = np.dtype([("lo", "<f4", 3), ("hi", "<f4", 3), ("first", "<i4"), ("count", "<i4"),
                              ("albedo", "<f4", 4), ("emissive", "<f4", 4), ("pad", "<i4", 4)])
TRIANGLE_DTYPE = np.dtype([("p", "<f4", (3, 3)), ("n", "<f4", (3, 3)), ("pad", "<f4", 2)])
assert MESH_OBJECT_DTYPE.itemsize == 80 and TRIANGLE_DTYPE.itemsize == 80


def strip_json_comments(text: str) -> str:
    """Removes // and /* */ comments outside string literals."""
    out, i, n = [], 0, len(text)
    in_str = False
    while i < n:
        c = text[i]
        if in_str:
            out.append(c)
            if c == "\\" and i + 1 < n:
                out.append(text[i + 1])
                i += 2
                continue
            if c == '"':
                in_str = False
            i += 1
        elif c == '"':
            in_str = True
            out.append(c)
            i += 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            if j < 0:
                raise ValueError("unterminated /* comment")
            out.append(" ")
            i = j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def vec3(node) -> np.ndarray:
    """ReadJsonVec3f (main.cpp:24-27): components 0-2, a missing one reads as 0."""
    v = [0.0, 0.0, 0.0]
    if isinstance(node, list):
        for k in range(min(3, len(node))):
            v[k] = float(node[k])
    return np.array(v, np.float64)


@dataclass
class ObjMesh:
    """Triangulated OBJ: per triangle three corners of (position, normal)."""
    positions: np.ndarray  # (T, 3, 3) float64, already scaled
    normals: np.ndarray    # (T, 3, 3) float64


def _parse_index(tok: str, nv: int, nn: int):
    parts = tok.split("/")

    def idx(s, count):
        if s == "":
            return -1
        k = int(s)
        return k - 1 if k > 0 else count + k

    v = idx(parts[0], nv)
    n = idx(parts[2], nn) if len(parts) >= 3 else -1
    return v, n


def _pnpoly(xs, ys, tx, ty) -> bool:
    """Crossing-number point-in-polygon test (W. R. Franklin's published method)."""
    inside = False
    j = len(xs) - 1
    for i in range(len(xs)):
        if ((ys[i] > ty) != (ys[j] > ty)) and (tx < (xs[j] - xs[i]) * (ty - ys[i]) / (ys[j] - ys[i]) + xs[i]):
            inside = not inside
        j = i
    return inside


def triangulate(face, verts) -> list:
    """Splits a polygon (list of (v, n) corners) into triangles the way the
    reference's tinyobjloader 1.4 does when asked to triangulate (ear clipping in
    the plane of the polygon's dominant axes, starting at corner 0): a triangle
    stays as it is, a convex polygon becomes the fan from its first corner."""
    if len(face) < 3:
        return []
    if len(face) == 3:
        return [tuple(face)]
    eps = np.finfo(np.float32).eps
    axes = [1, 2]
    npoly = len(face)
    for k in range(npoly):
        a, b, c = (verts[face[(k + j) % npoly][0]] for j in range(3))
        e0, e1 = b - a, c - b
        cx = abs(e0[1] * e1[2] - e0[2] * e1[1])
        cy = abs(e0[2] * e1[0] - e0[0] * e1[2])
        cz = abs(e0[0] * e1[1] - e0[1] * e1[0])
        if cx > eps or cy > eps or cz > eps:
            if not (cx > cy and cx > cz):
                axes[0] = 0
                if cz > cx and cz > cy:
                    axes[1] = 1
            break
    area = 0.0
    for k in range(npoly):
        p, q = verts[face[k][0]], verts[face[(k + 1) % npoly][0]]
        area += (p[axes[0]] * q[axes[1]] - p[axes[1]] * q[axes[0]]) * 0.5
    rem = list(face)
    tris = []
    guess = 0
    iters = len(rem)
    prev = len(rem)
    while len(rem) > 3 and iters > 0:
        npoly = len(rem)
        if guess >= npoly:
            guess -= npoly
        if prev != npoly:
            prev = npoly
            iters = npoly
        else:
            iters -= 1
        ind = [rem[(guess + k) % npoly] for k in range(3)]
        vx = [verts[c[0]][axes[0]] for c in ind]
        vy = [verts[c[0]][axes[1]] for c in ind]
        cross = (vx[1] - vx[0]) * (vy[2] - vy[1]) - (vy[1] - vy[0]) * (vx[2] - vx[1])
        if cross * area < 0.0:
            guess += 1
            continue
        overlap = False
        for other in range(3, npoly):
            o = verts[rem[(guess + other) % npoly][0]]
            if _pnpoly(vx, vy, o[axes[0]], o[axes[1]]):
                overlap = True
                break
        if overlap:
            guess += 1
            continue
        tris.append(tuple(ind))
        del rem[(guess + 1) % npoly]
    if len(rem) == 3:
        tris.append(tuple(rem))
    return tris


def load_obj(path: str, scale) -> ObjMesh:
    """OBJ positions, normals and faces (v, v/vt, v//vn, v/vt/vn; negative
    indices), triangulated; positions times `scale` (Mesh.h:44), normals as
    stored or (1, 0, 0) for a corner without one (Mesh.h:45-48)."""
    verts, norms, faces = [], [], []
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v" and len(t) >= 4:
                verts.append([float(t[1]), float(t[2]), float(t[3])])
            elif t[0] == "vn" and len(t) >= 4:
                norms.append([float(t[1]), float(t[2]), float(t[3])])
            elif t[0] == "f" and len(t) >= 4:
                faces.append([_parse_index(tok, len(verts), len(norms)) for tok in t[1:]])
    V = np.array(verts, np.float64).reshape(-1, 3)
    N = np.array(norms, np.float64).reshape(-1, 3)
    tri_p, tri_n = [], []
    for face in faces:
        if any(v < 0 or v >= len(V) for v, _ in face):
            continue
        for tri in triangulate(face, V):
            tri_p.append([V[v] * np.asarray(scale, np.float64) for v, _ in tri])
            tri_n.append([N[n] if 0 <= n < len(N) else np.array([1.0, 0.0, 0.0]) for _, n in tri])
    return ObjMesh(np.array(tri_p, np.float64).reshape(-1, 3, 3), np.array(tri_n, np.float64).reshape(-1, 3, 3))


def rotation(angle_vec) -> np.ndarray:
    """glm::rotate(|a|, a / |a|) as a 3x3 matrix (Rodrigues' formula)."""
    a = np.asarray(angle_vec, np.float64)
    th = float(np.linalg.norm(a))
    if th <= 1e-3:
        return np.eye(3)
    x, y, z = a / th
    c, s = math.cos(th), math.sin(th)
    K = np.array([[0.0, -z, y], [z, 0.0, -x], [-y, x, 0.0]])
    return c * np.eye(3) + s * K + (1.0 - c) * np.outer([x, y, z], [x, y, z])


@dataclass
class Scene:
    objects: np.ndarray              # MESH_OBJECT_DTYPE
    triangles: np.ndarray            # TRIANGLE_DTYPE
    names: list = field(default_factory=list)
    renderer: dict = field(default_factory=dict)

    @property
    def shadow_size(self) -> int:
        v = self.renderer.get("shadowmapSize")
        return int(v[0]) if isinstance(v, list) and v else 1024


def resolve_mesh_path(filename: str, scene_dir: str) -> str:
    """The reference opens mesh paths relative to its working directory, a
    sibling of bin/data (bin/<build>); tried: as given, next to the scene file,
    and from such a sibling directory of the scene's data folder."""
    cands = [filename, os.path.join(scene_dir, filename), os.path.join(scene_dir, "..", filename),
             os.path.join(scene_dir, "..", "..", "_", filename)]
    for c in cands:
        c = os.path.normpath(c)
        if os.path.isfile(c):
            return c
    raise FileNotFoundError(f"mesh {filename!r} (scene folder {scene_dir})")


def load_scene(path: str) -> Scene:
    """Scene.h:55-117 on the file at `path`: world-space triangles grouped by object."""
    with open(path, "r", encoding="utf-8") as f:
        root = json.loads(strip_json_comments(f.read()))
    sc = root.get("scene", {}) or {}
    scene_dir = os.path.dirname(os.path.abspath(path))
    meshes = {}
    for node in sc.get("meshes", []) or []:
        fn = node.get("filename", "<unspecified>")
        meshes[node.get("name", "<unspecified>")] = load_obj(resolve_mesh_path(fn, scene_dir), vec3(node.get("scale")))
    objs, tris_p, tris_n, names = [], [], [], []
    first = 0
    for node in sc.get("objects", []) or []:
        name = node.get("mesh", "<unspecified>")
        if name not in meshes:  # Scene.h:95-99: an unknown mesh skips the object
            continue
        m = meshes[name]
        R = rotation(vec3(node.get("angle")))
        t = vec3(node.get("pos"))
        p = (m.positions @ R.T + t).astype(np.float32)
        n = (m.normals @ R.T).astype(np.float32)
        o = np.zeros((), MESH_OBJECT_DTYPE)
        if len(p):
            lo, hi = p.reshape(-1, 3).min(0).astype(np.float64), p.reshape(-1, 3).max(0).astype(np.float64)
            pad = 1e-4 * max(1.0, float(np.abs(np.concatenate([lo, hi])).max()))
            o["lo"], o["hi"] = lo - pad, hi + pad
        o["first"], o["count"] = first, len(p)
        o["albedo"] = np.append(vec3(node.get("albedoColor")), 1.0)
        o["emissive"] = np.append(vec3(node.get("emissiveColor")), 1.0)
        objs.append(o)
        tris_p.append(p)
        tris_n.append(n)
        names.append(name)
        first += len(p)
    tri = np.zeros(first, TRIANGLE_DTYPE)
    if first:
        tri["p"] = np.concatenate(tris_p)
        tri["n"] = np.concatenate(tris_n)
    return Scene(np.array(objs, MESH_OBJECT_DTYPE).reshape(-1), tri, names, root.get("renderer", {}) or {})


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
