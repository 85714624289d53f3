"""Mesh and image files (diffrender_tutorials_gb300/io.py): round trips, and
the reference's own assets read through the reference's VSGF loader where the
reference sources are available."""
import os
import sys

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import io as IO

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def test_vsgf_round_trip(tmp_path):
    m = D.make_uv_sphere(6, 12, seed=1)
    m.tangents = np.roll(m.normals, 1, axis=1)
    p = str(tmp_path / "m.vsgf")
    IO.save_vsgf(p, m)
    r = IO.load_vsgf(p)
    assert np.array_equal(r.vertices, m.vertices) and np.array_equal(r.indices, m.indices)
    assert np.array_equal(r.normals, m.normals) and np.array_equal(r.tangents, m.tangents)
    m2 = D.TriangleMesh(m.vertices, m.indices)
    IO.save_vsgf(p, m2)
    r2 = IO.load_vsgf(p)
    assert r2.normals is None and r2.tangents is None and np.array_equal(r2.vertices, m.vertices)


def test_obj_round_trip_and_polygons(tmp_path):
    m = D.make_icosphere(1, seed=2)
    p = str(tmp_path / "m.obj")
    IO.save_obj(p, m)
    r = IO.load_obj(p)
    # vertices are numbered in order of first use by the faces
    assert r.face_count == m.face_count
    assert np.allclose(r.vertices[r.indices], m.vertices[m.indices], atol=1e-6)
    assert np.allclose(r.normals[r.indices], m.normals[m.indices], atol=1e-6)
    q = tmp_path / "quad.obj"
    q.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
                 "f 1/1 2/2 3/3 4/4\nf -4/-4 -2/-2 -1/-1\n")
    r = IO.load_obj(str(q))
    assert r.face_count == 3 and r.tc is not None and r.normals is None
    assert np.array_equal(r.indices.reshape(-1, 3)[0], [0, 1, 2])


def test_images(tmp_path):
    rng = np.random.default_rng(3)
    img = rng.uniform(0, 1.2, size=(7, 5, 3)).astype(np.float32)
    for ext in (".bmp", ".ppm"):
        p = str(tmp_path / ("i" + ext))
        IO.save_image(p, img)
        back = IO.load_image(p)
        assert back.shape == img.shape
        assert np.array_equal(IO.tonemap(back), IO.tonemap(img))
    # int(x^(1/2.2)*255+0.5) clamped: 0 -> 0, 1 -> 255, 0.5 -> 186
    assert list(IO.tonemap(np.array([0.0, 1.0, 0.5, 2.0, -1.0], np.float32))) == [0, 255, 186, 255, 0]
    p = str(tmp_path / "i.image3f")
    IO.save_image(p, img)
    assert np.array_equal(IO.load_image(p), img)
    with open(str(tmp_path / "i.bmp"), "rb") as f:
        assert f.read(2) == b"BM"


def reference_meshes():
    import build_ref
    d = os.path.join(build_ref.REF_ROOT, "data", "meshes")
    return d if os.path.isdir(d) else None


@pytest.mark.parametrize("name", ["teapot.vsgf", "vase.vsgf"])
def test_reference_vsgf_assets_match_reference_loader(name):
    d = reference_meshes()
    if d is None:
        pytest.skip("reference assets absent")
    import build_ref
    import refrun
    exe = build_ref.build()
    path = os.path.join(d, name)
    ref = refrun.run(exe, {"task": np.array([8], np.int32),
                           "path": np.frombuffer(path.encode(), np.uint8).astype(np.int32)})
    m = IO.load_vsgf(path)
    assert np.array_equal(m.vertices, ref["pos4"].reshape(-1, 4)[:, :3])
    assert np.array_equal(m.normals, ref["norm4"].reshape(-1, 4)[:, :3])
    assert np.array_equal(m.tc, ref["tc2"].reshape(-1, 2))
    assert np.array_equal(m.indices, ref["indices"])
    # and it renders (oracle silhouette of the normalised mesh)
    import pyoracle as O
    v = m.vertices - m.vertices.mean(0)
    m.vertices = (v / np.abs(v).max()).astype(np.float32)
    s = D.Scene()
    s.add_mesh(m)
    img = O.render(s, [D.CamInfo(origin=(0, 0, 3), width=24, height=24)], 1, 1)
    assert img.max() == 1.0 and img.mean() > 0.05


def test_reference_obj_asset():
    d = reference_meshes()
    if d is None:
        pytest.skip("reference assets absent")
    m = IO.load_obj(os.path.join(d, "sphere.obj"))
    assert m.face_count > 0 and np.isfinite(m.vertices).all()
