"""Helpers that rebuild scenes and cameras from the golden fixtures."""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from diffrender_tutorials_gb300.scene import CamInfo, Scene, Texture, TransformR, TriangleMesh  # noqa: E402


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def scene_from(d):
    s = Scene()
    for i in range(int(d["n_meshes"][0])):
        p = f"m{i}."
        get = lambda k: d.get(p + k)  # noqa: E731
        tex = []
        if p + "tex" in d:
            w, h, c = (int(x) for x in d[p + "tex_shape"])
            tex = [Texture(w, h, c, d[p + "tex"])]
        m = TriangleMesh(get("vertices"), get("indices"), colors=get("colors"), tc=get("tc"), normals=get("normals"),
                         tangents=get("tangents"), textures=tex)
        if p + "restricted" in d:
            s.add_mesh(m, [TransformR.from_params(q) for q in d[p + "restricted"].reshape(-1, 7)])
            continue
        tr = d[p + "transforms"].reshape(-1, 4, 4)
        s.add_mesh(m, [t.T.copy() for t in tr])  # stored column-major
    return s


def cams_from(d):
    la = d["cams_lookat"].reshape(-1, 11)
    fov = d["cams_fov"] if "cams_fov" in d else np.full(len(la), math.pi / 4, np.float32)
    return [CamInfo(origin=tuple(r[0:3]), target=tuple(r[3:6]), up=tuple(r[6:9]), width=int(r[9]), height=int(r[10]),
                    fov_rad=float(f)) for r, f in zip(la, fov)]


def dscene_from(d):
    """Concatenated DScene vector and per-dmesh layout rows."""
    n = int(d["out.n_dmeshes"][0])
    return (np.concatenate([d[f"out.dmesh{k}"] for k in range(n)]),
            np.stack([d[f"out.dmesh{k}.layout"] for k in range(n)]))


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = max(np.linalg.norm(b), 1e-30)
    return float(np.linalg.norm(a - b) / den)
