"""Inputs for the reference driver (oracle/ref/ref_driver.cpp) and a runner.

Test infrastructure only.  Scenes and cameras are written in ref_driver's
DRKV format (oracle/ref/kvio.py); `run` executes a ref_driver binary built by
oracle/ref/build_ref.py and returns its outputs.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import kvio  # noqa: E402


def scene_items(scene):
    it = {"n_meshes": np.array([len(scene.meshes)], np.int32)}
    for i, m in enumerate(scene.meshes):
        p = f"m{i}."
        it[p + "vertices"] = m.vertices.reshape(-1)
        it[p + "indices"] = m.indices
        for name in ("colors", "tc", "normals", "tangents"):
            a = getattr(m, name)
            if a is not None:
                it[p + name] = a.reshape(-1)
        if m.textures:
            t = m.textures[0]
            it[p + "tex"] = t.data
            it[p + "tex_shape"] = np.array([t.w, t.h, t.channels], np.int32)
        it[p + "transforms"] = scene.transforms_colmajor(i)
        rp = scene.restricted_params(i) if hasattr(scene, "restricted_params") else None
        if rp is not None:
            it[p + "restricted"] = rp
    return it


def cam_items(cams):
    la = np.array([[*c.origin, *c.target, *c.up, c.width, c.height] for c in cams], np.float32).reshape(-1)
    fov = np.array([c.fov_rad for c in cams], np.float32)
    return {"cams_lookat": la, "cams_fov": fov}


def run(exe, items, env=None):
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.kv"), os.path.join(d, "out.kv")
        kvio.save(fin, items)
        subprocess.check_call([exe, fin, fout], env=env)
        return kvio.load(fout)
