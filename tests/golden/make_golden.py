"""Generate golden fixtures by running the reference renderer itself.

The reference (FROL256/diffrender_tutorials) has no golden vectors of its
own; its tests compare against finite differences only (src/tests.cpp).  This
script compiles the reference's CPU path (oracle/ref/build_ref.py), runs it
through oracle/ref/ref_driver.cpp on small seeded scenes and stores inputs and
outputs as tests/golden/*.npz.  It needs the reference source tree and runs
in the development container only; the fixtures it writes are committed and
are all that the tests read.

    python tests/golden/make_golden.py              # all but the long runs
    python tests/golden/make_golden.py convergence  # 300-iteration optimiser runs
    python tests/golden/make_golden.py path_test    # the PATH_TEST mean image
    python tests/golden/make_golden.py fd_scenes    # scenes of the reference's derivative tests
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))

import build_ref  # noqa: E402
import kvio  # noqa: E402,F401
import refrun  # noqa: E402
from refrun import cam_items, scene_items  # noqa: E402
from diffrender_tutorials_gb300.scene import (Scene, TriangleMesh, Texture, TransformR, make_cube,  # noqa: E402
                                              make_icosphere, perturb_vertices, identity4)

OUT = os.path.dirname(os.path.abspath(__file__))
SIL, VC, TEX, LAMBERT, PHONG, GGX = 1, 2, 3, 4, 5, 6


def run(items):
    return refrun.run(build_ref.build(), items)


class Cam:
    def __init__(self, origin, width, height, fov=math.pi / 4, target=(0, 0, 0), up=(0, 1, 0)):
        self.origin, self.target, self.up = origin, target, up
        self.width, self.height, self.fov_rad = width, height, fov


def textured_sphere(sub=2, tex_size=16, seed=3):
    m = make_icosphere(sub, seed=seed)
    P = m.vertices.astype(np.float64)
    u = 0.5 + np.arctan2(P[:, 0], P[:, 2]) / (2 * math.pi)
    v = np.arccos(np.clip(P[:, 1], -1, 1)) / math.pi
    rng = np.random.default_rng(seed)
    tex = rng.uniform(0.1, 0.9, size=(tex_size, tex_size, 3)).astype(np.float32)
    return TriangleMesh(m.vertices, m.indices, tc=np.stack([u, v], 1).astype(np.float32), normals=m.normals,
                        textures=[Texture(tex_size, tex_size, 3, tex.reshape(-1))])


def path_test_scene():
    """Scene for shade<PATH_TEST> (src/shade_path_test.cpp): a textured
    sphere of radius 0.4 above a textured floor (y = -0.3), normals and
    tangents given, both outward-wound; the model's point light (0,0.7,0.7)
    lies outside the sphere.  Used with the camera PATH_TEST_CAM."""
    sph = textured_sphere(2, tex_size=8, seed=7)
    n = sph.normals.astype(np.float64)
    t = np.cross(np.array([0.0, 1.0, 0.0]), n)
    flat = np.linalg.norm(t, axis=1) < 1e-3
    t[flat] = (1.0, 0.0, 0.0)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    sph.vertices = (sph.vertices * np.float32(0.4) + np.array([0.0, 0.1, 0.0], np.float32)).astype(np.float32)
    sph.tangents = t.astype(np.float32)
    y = -0.3
    fv = np.array([[-2, y, -2], [2, y, -2], [2, y, 2], [-2, y, 2]], np.float32)
    checker = np.array([[0.8, 0.75, 0.6] if (i + j) % 2 == 0 else [0.3, 0.35, 0.5] for j in range(4) for i in range(4)],
                       np.float32)
    floor = TriangleMesh(fv, np.array([0, 2, 1, 0, 3, 2], np.uint32),
                         tc=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32),
                         normals=np.tile(np.array([0, 1, 0], np.float32), (4, 1)),
                         textures=[Texture(4, 4, 3, checker.reshape(-1))])
    floor.tangents = np.tile(np.array([1, 0, 0], np.float32), (4, 1))
    sc = Scene()
    sc.add_mesh(sph)
    sc.add_mesh(floor)
    return sc


PATH_TEST_CAM = dict(origin=(0.0, 0.7, 2.2), width=32, height=32)


def path_test():
    """The reference's PATH_TEST model (its shared rand() stream): mean
    image of 16 renders at 64 spp and the per-value variance across them."""
    build_ref.build(verbose=True)
    sc = path_test_scene()
    cam = Cam(PATH_TEST_CAM["origin"], PATH_TEST_CAM["width"], PATH_TEST_CAM["height"])
    items = {"task": np.array([2], np.int32), "mode": np.array([7], np.int32), "spp": np.array([64], np.int32),
             "repeats": np.array([16], np.int32), **scene_items(sc), **cam_items([cam])}
    save("render_path_test", **items, **prefixed("out.", run(items)))


def reference_fd_scenes():
    """The scenes and camera of the reference's derivative tests 1.1-1.5
    (src/tests.cpp:31-107), built by the reference's own src/scenes.cpp."""
    build_ref.build(verbose=True)
    save("fd_tests1_scenes", **prefixed("out.", run({"task": np.array([9], np.int32)})))


def pyramid(seed=4):
    """Square pyramid, 5 vertices / 6 triangles, random vertex colours."""
    v = np.array([[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [0.5, -0.5, 0.5], [-0.5, -0.5, 0.5], [0.0, 0.5, 0.0]],
                 np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3, 0, 4, 1, 1, 4, 2, 2, 4, 3, 3, 4, 0], np.uint32)
    col = np.random.default_rng(seed).uniform(0.2, 0.9, size=(5, 3)).astype(np.float32)
    return TriangleMesh(v, idx, colors=col)


def save(name, **arrays):
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def prefixed(prefix, d):
    return {prefix + k: v for k, v in d.items()}


def main():
    build_ref.build(verbose=True)

    # -- cameras (CamInfo, common_src/camera.h) ---------------------------
    cams = [Cam((0, 0, 3), 256, 256), Cam((3 * math.sin(math.pi / 4), 0, 3 * math.cos(math.pi / 4)), 512, 512),
            Cam((0.3, 1.2, -2.5), 64, 48, fov=0.9), Cam((-3, 0, 0), 1024, 1024)]
    items = {"task": np.array([0], np.int32), **cam_items(cams)}
    out = run(items)
    save("camera", **items, **prefixed("out.", out))

    # -- random streams and Hammersley points -----------------------------
    seeds = np.array([7777 + k * k + 1 for k in range(14)] + [1, 7, 100], np.int32)
    items = {"task": np.array([6], np.int32), "prng_seeds": seeds, "prng_count": np.array([64], np.int32)}
    out = run(items)
    ham = {}
    for n in (1, 4, 8, 16, 25, 32):
        ham[f"ham{n}"] = run({"task": np.array([7], np.int32), "ham_n": np.array([n], np.int32)})["ham"]
    save("random", **items, **prefixed("out.", out), **ham)

    # -- per-sample nearest hits ------------------------------------------
    cube = make_cube(seed=1)
    scene = Scene()
    scene.add_mesh(cube)
    tetra = TriangleMesh(np.array([[0, 0, 0], [0.6, 0, 0], [0, 0.6, 0], [0, 0, 0.6]], np.float32) + np.float32(0.2),
                         np.array([0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3], np.uint32),
                         colors=np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0]], np.float32))
    t1 = identity4(); t1[0, 3] = 0.9; t1[1, 3] = -0.2
    t2 = identity4(); t2[0, 3] = -1.1; t2[2, 3] = 0.4
    scene.add_mesh(tetra, [t1, t2])
    cam = Cam((0.4, 0.7, 3.0), 64, 64)
    rng = np.random.default_rng(5)
    g = (np.arange(64) + 0.5)
    grid = np.stack(np.meshgrid(g, g), -1).reshape(-1, 2)
    xy = np.concatenate([grid, rng.uniform(0, 64, size=(4096, 2))]).astype(np.float32)
    items = {"task": np.array([1], np.int32), **scene_items(scene), **cam_items([cam]), "hit_xy": xy.reshape(-1)}
    out = run(items)
    save("hits_cube_instanced", **items, **prefixed("out.", out))

    ico = make_icosphere(3, seed=2)
    scene = Scene()
    scene.add_mesh(ico)
    cam = Cam((0.0, 0.5, 2.8), 96, 96)
    xy = rng.uniform(0, 96, size=(12000, 2)).astype(np.float32)
    items = {"task": np.array([1], np.int32), **scene_items(scene), **cam_items([cam]), "hit_xy": xy.reshape(-1)}
    out = run(items)
    save("hits_icosphere3", **items, **prefixed("out.", out))

    # -- forward render ---------------------------------------------------
    scene = Scene()
    scene.add_mesh(make_cube(seed=1))
    cams = [Cam((0, 0, 3), 64, 64), Cam((2.0, 1.0, 2.0), 48, 40)]
    for mode, spp in ((VC, 16), (SIL, 9), (VC, 8)):
        items = {"task": np.array([2], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([spp], np.int32),
                 **scene_items(scene), **cam_items(cams)}
        out = run(items)
        save(f"render_cube_m{mode}_spp{spp}", **items, **prefixed("out.", out))
    ts = Scene()
    ts.add_mesh(textured_sphere())
    for mode in (TEX, LAMBERT, PHONG, GGX):
        items = {"task": np.array([2], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([4], np.int32),
                 **scene_items(ts), **cam_items([Cam((0.5, 0.8, 2.6), 48, 48)])}
        out = run(items)
        save(f"render_sphere_m{mode}", **items, **prefixed("out.", out))

    # -- derivatives ------------------------------------------------------
    true_cube = make_cube(seed=1)
    init_cube = perturb_vertices(true_cube, 0.1, seed=11)
    init_cube.colors = np.clip(true_cube.colors + np.random.default_rng(12).normal(0, 0.1, (8, 3)), 0, 1).astype(np.float32)
    tscene, iscene = Scene(), Scene()
    tscene.add_mesh(true_cube)
    iscene.add_mesh(init_cube)
    cams = [Cam((0, 0, 3), 64, 64)]
    tgt = run({"task": np.array([2], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([16], np.int32),
               **scene_items(tscene), **cam_items(cams)})["images"]
    for mode in (VC, SIL):
        items = {"task": np.array([4], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([16], np.int32),
                 **scene_items(iscene), **cam_items(cams), "targets": tgt, "edge_samples": np.array([64 * 64], np.int32),
                 "dmesh_ids": np.array([0], np.int32)}
        out = run(items)
        save(f"drc_cube_m{mode}", **items, **prefixed("out.", out))

    # instancing: two instances of the cube (Scene::add_mesh with two
    # matrices, BASE_TRANSFORM); gradients of positions and of both 4x3
    # transform blocks
    iscene2 = Scene()
    t0, t1 = identity4(), identity4()
    t0[0, 3], t0[1, 3] = -0.7, 0.1
    c, s_ = np.cos(0.4), np.sin(0.4)
    t1[:3, :3] = np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]]) * 0.8
    t1[0, 3], t1[2, 3] = 0.8, -0.3
    iscene2.add_mesh(init_cube, [t0, t1])
    tscene2 = Scene()
    tscene2.add_mesh(true_cube, [t0, t1])
    cams_i = [Cam((0, 0.5, 3.2), 64, 64)]
    tgt_i = run({"task": np.array([2], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([4], np.int32),
                 **scene_items(tscene2), **cam_items(cams_i)})["images"]
    items = {"task": np.array([4], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([4], np.int32),
             **scene_items(iscene2), **cam_items(cams_i), "targets": tgt_i, "edge_samples": np.array([64 * 64], np.int32),
             "dmesh_ids": np.array([0], np.int32)}
    out = run(items)
    save("drc_cube_instanced", **items, **prefixed("out.", out))

    # restricted transforms (TransformR: translation, rotation, scale per
    # instance; TEST 2.11 of src/tests.cpp:350-361): forward render through
    # to_mat, gradients of the 7 parameters per instance, and a trajectory
    pyr = pyramid()
    r_true = [TransformR((-0.6, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0), TransformR((0.6, 0.1, -0.2), (0.3, 0.0, 0.0), 0.8)]
    r_init = [TransformR((-0.55, 0.05, 0.0), (0.0, 0.2, 0.2), 1.05),
              TransformR((0.65, 0.05, -0.2), (0.25, -0.1, 0.15), 0.85)]
    tsr, isr = Scene(), Scene()
    tsr.add_mesh(pyr, r_true)
    isr.add_mesh(pyr, r_init)
    cams_r = [Cam((0.3, 0.9, 2.8), 64, 64)]
    items = {"task": np.array([2], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([16], np.int32),
             **scene_items(isr), **cam_items(cams_r)}
    save("render_pyramid_restricted", **items, **prefixed("out.", run(items)))
    # (the brute-force caster applies instance matrices twice, raytrace3d_bf.cpp:116-125,
    # so a silhouette model sees no edge of a rotated instance; VC and the point light do)
    for mode in (VC, 16):
        tg = run({"task": np.array([2], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([16], np.int32),
                  **scene_items(tsr), **cam_items(cams_r)})["images"]
        items = {"task": np.array([4], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([16], np.int32),
                 **scene_items(isr), **cam_items(cams_r), "targets": tg, "edge_samples": np.array([64 * 64], np.int32),
                 "dmesh_ids": np.array([0], np.int32)}
        save(f"drc_pyramid_restricted_m{mode}", **items, **prefixed("out.", run(items)))
    cams_o = [Cam((0.3, 0.9, 2.8), 48, 48)]
    tg = run({"task": np.array([2], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([16], np.int32),
              **scene_items(tsr), **cam_items(cams_o)})["images"]
    items = {"task": np.array([5], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([16], np.int32),
             **scene_items(isr), **cam_items(cams_o), "targets": tg, "iters": np.array([5], np.int32),
             "opt_alg": np.array([4], np.int32), "opt_pos_lr": np.array([0.0], np.float32),
             "opt_tfm_lr": np.array([0.05], np.float32), "opt_flags": np.array([2], np.int32),
             "dmesh_ids": np.array([0], np.int32)}
    save("optimize_pyramid_restricted", **items, **prefixed("out.", run(items)))

    # two meshes, a cube and a tetrahedron (one instance each), both
    # differentiable (DScene with two DMesh blocks; the optimiser's "Adam"
    # indexes its second-moment accumulator mesh-locally,
    # optimizer_simple.cpp:224), and the cube alone differentiable with the
    # tetrahedron as a static occluder
    tet = TriangleMesh(np.array([[0, 0, 0], [0.6, 0, 0], [0, 0.6, 0], [0, 0, 0.6]], np.float32) +
                       np.array([0.9, -0.1, 0.6], np.float32),
                       np.array([0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3], np.uint32),
                       colors=np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0]], np.float32))
    tet_init = perturb_vertices(tet, 0.05, seed=31)
    tet_init.colors = np.clip(tet.colors + np.random.default_rng(32).normal(0, 0.1, (4, 3)), 0, 1).astype(np.float32)
    tsm, ism = Scene(), Scene()
    tsm.add_mesh(true_cube)
    tsm.add_mesh(tet)
    ism.add_mesh(init_cube)
    ism.add_mesh(tet_init)
    cams_m = [Cam((0.4, 0.7, 3.0), 64, 64)]
    tgt_m = run({"task": np.array([2], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([4], np.int32),
                 **scene_items(tsm), **cam_items(cams_m)})["images"]
    for name, ids in (("drc_two_meshes", [0, 1]), ("drc_static_occluders", [0])):
        items = {"task": np.array([4], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([4], np.int32),
                 **scene_items(ism), **cam_items(cams_m), "targets": tgt_m,
                 "edge_samples": np.array([64 * 64], np.int32), "dmesh_ids": np.array(ids, np.int32)}
        save(name, **items, **prefixed("out.", run(items)))
    items = {"task": np.array([5], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([4], np.int32),
             **scene_items(ism), **cam_items(cams_m), "targets": tgt_m, "iters": np.array([5], np.int32),
             "opt_alg": np.array([4], np.int32), "opt_pos_lr": np.array([0.01], np.float32),
             "opt_base_lr": np.array([0.01], np.float32), "opt_flags": np.array([1 | 4], np.int32),
             "dmesh_ids": np.array([0, 1], np.int32)}
    save("optimize_two_meshes", **items, **prefixed("out.", run(items)))

    # two views, d_render with a given adjoint (accumulation over views)
    cams2 = [Cam((0, 0, 3), 48, 48), Cam((2.2, 1.0, 1.8), 48, 48)]
    adj = np.random.default_rng(13).normal(0, 0.5, size=2 * 48 * 48 * 3).astype(np.float32)
    items = {"task": np.array([3], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([4], np.int32),
             **scene_items(iscene), **cam_items(cams2), "adjoints": adj, "edge_samples": np.array([3000], np.int32),
             "dmesh_ids": np.array([0], np.int32)}
    out = run(items)
    save("drender_cube_2views", **items, **prefixed("out.", out))

    # textured sphere: texture derivatives (TEXTURE_COLOR, Lambert, Phong, GGX)
    tsph = textured_sphere()
    isph = tsph.copy()
    isph.textures[0].data[:] = 0.5
    isph.vertices = perturb_vertices(tsph, 0.02, seed=21).vertices
    tsc, isc = Scene(), Scene()
    tsc.add_mesh(tsph)
    isc.add_mesh(isph)
    cams = [Cam((0.5, 0.8, 2.6), 40, 40)]
    for mode in (TEX, LAMBERT, PHONG, GGX):
        tg = run({"task": np.array([2], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([4], np.int32),
                  **scene_items(tsc), **cam_items(cams)})["images"]
        items = {"task": np.array([4], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([4], np.int32),
                 **scene_items(isc), **cam_items(cams), "targets": tg, "edge_samples": np.array([1600], np.int32),
                 "dmesh_ids": np.array([0], np.int32)}
        out = run(items)
        save(f"drc_sphere_m{mode}", **items, **prefixed("out.", out))

    # -- optimiser trajectory ("Adam" variant, optimizer_simple.cpp) -------
    cams = [Cam((0, 0, 3), 32, 32)]
    tgt = run({"task": np.array([2], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([16], np.int32),
               **scene_items(tscene), **cam_items(cams)})["images"]
    items = {"task": np.array([5], np.int32), "mode": np.array([VC], np.int32), "spp": np.array([16], np.int32),
             **scene_items(iscene), **cam_items(cams), "targets": tgt, "iters": np.array([6], np.int32),
             "opt_alg": np.array([4], np.int32), "opt_pos_lr": np.array([0.01], np.float32),
             "opt_base_lr": np.array([0.01], np.float32), "opt_flags": np.array([1 | 4], np.int32),
             "dmesh_ids": np.array([0], np.int32)}
    out = run(items)
    save("optimize_cube_vc", **items, **prefixed("out.", out))
    path_test()
    reference_fd_scenes()


def _moved(mesh, m):
    v = np.c_[mesh.vertices.astype(np.float64), np.ones(len(mesh.vertices))] @ m.T
    return TriangleMesh(v[:, :3].astype(np.float32), mesh.indices.copy(), colors=mesh.colors.copy())


def _rot(axis, deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4)
    i, j = (0, 2) if axis == "y" else (0, 1)
    m[i, i], m[j, j] = c, c
    m[i, j], m[j, i] = (s, -s) if axis == "y" else (-s, s)
    return m


def _translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def convergence():
    """300-iteration runs in the shape of the reference's TESTS 2.1, 2.2 and
    2.4 (src/tests.cpp:144-260): the triangle and pyramid of
    src/scenes.cpp:69-117,190-238 restated (turned and moved apart between
    start and target), three cameras around at distance 5
    (create_cameras_around), 256x256, 16 spp, "Adam" with the tests'
    learning rates and otherwise default parameters.  Kept: the inputs, the
    final error and the last iteration's mesh."""
    build_ref.build(verbose=True)
    tri = TriangleMesh(np.array([[0, 1, 0], [1, -1, 1], [-1, -1, 1]], np.float32), np.array([0, 1, 2], np.uint32),
                       colors=np.ones((3, 3), np.float32))
    pyr = TriangleMesh(np.array([[0, 1, 0], [-1, -1, 1], [1, -1, 1], [1, -1, -1], [-1, -1, -1]], np.float32),
                       np.array([0, 1, 2, 0, 2, 3, 0, 3, 4, 0, 4, 1], np.uint32),
                       colors=np.array([[1, 0, 0], [1, 1, 0], [0, 0, 1], [0, 1, 0], [0, 1, 1]], np.float32))
    lift = _translate(0, 0.5, 0)
    half = np.diag([0.5, 0.5, 0.5, 1.0])
    tri_pair = (_moved(tri, lift @ _rot("y", -40)), _moved(tri, lift @ _rot("y", 30)))
    pyr_init = _moved(pyr, half @ lift @ _rot("y", -40) @ _rot("z", -30))
    pyr_init.colors[:] = 0.25
    pyr_pair = (pyr_init, _moved(pyr, half @ lift @ _rot("y", 50)))
    ry = 2 * math.pi / 3
    cams = [Cam((-5 * math.sin(ry * (i - 1)), 0.0, -5 * math.cos(ry * (i - 1))), 256, 256) for i in range(3)]
    iters = 300
    for name, (init, target), mode, tex_lr in (("converge_triangle_sil", tri_pair, 1, 0.1),
                                               ("converge_pyramid_sil", pyr_pair, 1, 0.1),
                                               ("converge_pyramid_vc", pyr_pair, 2, 0.0)):
        tscene, iscene = Scene(), Scene()
        tscene.add_mesh(target)
        iscene.add_mesh(init)
        tgt = run({"task": np.array([2], np.int32), "mode": np.array([mode], np.int32),
                   "spp": np.array([16], np.int32), **scene_items(tscene), **cam_items(cams)})["images"]
        items = {"task": np.array([5], np.int32), "mode": np.array([mode], np.int32), "spp": np.array([16], np.int32),
                 **scene_items(iscene), **cam_items(cams), "targets": tgt, "iters": np.array([iters], np.int32),
                 "opt_alg": np.array([4], np.int32), "opt_pos_lr": np.array([0.05], np.float32),
                 "opt_tex_lr": np.array([tex_lr], np.float32), "dmesh_ids": np.array([0], np.int32)}
        out = run(items)
        last = f"it{iters - 1}."
        keep = {k: v for k, v in out.items() if k in ("final_error", "n_iters") or k.startswith(last)}
        save(name, **items, **prefixed("out.", keep))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "convergence":
        convergence()
    elif len(sys.argv) > 1 and sys.argv[1] == "path_test":
        path_test()
    elif len(sys.argv) > 1 and sys.argv[1] == "fd_scenes":
        reference_fd_scenes()
    else:
        main()
