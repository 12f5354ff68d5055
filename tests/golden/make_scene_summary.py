"""Writes tests/golden/cube_scene_summary.json: the reference's
bin/data/Scenes/CubeScene.json (and the OBJ meshes it names) as
legitengine_gb300/scene.py loads them -- object and triangle counts, bounds and
per-object sums of the world-space vertices and normals.  Reads the reference's
files where they lie; writes only the summary.

Run: python tests/golden/make_scene_summary.py [REFERENCE_ROOT]
(the reference checkout's root: the argument, else the LEGIT_REFERENCE_ROOT
environment variable, else the default of oracle/build_ref.py).
"""
import json
import os
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[2]))

from legitengine_gb300 import scene as S  # noqa: E402
from oracle import build_ref  # noqa: E402

SCENE = "bin/data/Scenes/CubeScene.json"


def reference_root(arg: str | None = None) -> Path:
    if arg:
        return Path(arg)
    return Path(os.environ.get("LEGIT_REFERENCE_ROOT", build_ref.DEFAULT_REFERENCE_ROOT))


def summarise(path):
    sc = S.load_scene(path)
    per = []
    for name, o in zip(sc.names, sc.objects):
        t = sc.triangles[o["first"]:o["first"] + o["count"]]
        per.append({"mesh": name, "count": int(o["count"]),
                    "lo": [round(float(v), 6) for v in o["lo"]], "hi": [round(float(v), 6) for v in o["hi"]],
                    "albedo": [round(float(v), 6) for v in o["albedo"]],
                    "emissive": [round(float(v), 6) for v in o["emissive"]],
                    "sum_p": [round(float(v), 3) for v in t["p"].astype("f8").sum((0, 1))],
                    "sum_n": [round(float(v), 3) for v in t["n"].astype("f8").sum((0, 1))]})
    return {"scene": "bin/data/Scenes/CubeScene.json", "objects": int(len(sc.objects)),
            "triangles": int(len(sc.triangles)), "shadow_size": sc.shadow_size, "per_object": per}


if __name__ == "__main__":
    out = Path(__file__).parent / "cube_scene_summary.json"
    root = reference_root(sys.argv[1] if len(sys.argv) > 1 else None)
    if not (root / SCENE).exists():
        sys.exit(f"{root / SCENE} not found: pass the reference checkout's root")
    out.write_text(json.dumps(summarise(str(root / SCENE)), indent=1) + "\n")
    print("wrote", out)
