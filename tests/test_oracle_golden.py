"""The CPU oracle against fixtures produced by the reference itself.

These pin the oracle (oracle/oracle.c) before it is trusted as the checker
of the CUDA path: camera matrices, random streams, per-sample hit ids,
images, gradients and an optimiser trajectory must equal the reference's
output (bit-exact where the arithmetic is the same, tolerances noted where
the reference's own reduction order is nondeterministic).
"""
import math

import numpy as np
import pytest

import pyoracle as O
from fixtures import cams_from, dscene_from, load, scene_from


def test_camera_matrices_bit_exact():
    d = load("camera")
    for i, cam in enumerate(cams_from(d)):
        blk = O.camera(cam)
        assert np.array_equal(blk[0:16], d[f"out.cam{i}.worldview"])
        assert np.array_equal(blk[16:32], d[f"out.cam{i}.proj"])
        assert np.array_equal(blk[32:48], d[f"out.cam{i}.wvp"])
        assert np.array_equal(blk[48:64], d[f"out.cam{i}.proj_inv"])
        assert np.array_equal(blk[64:80], d[f"out.cam{i}.wv_inv"])


def test_prng_and_hammersley_bit_exact():
    d = load("random")
    cnt = int(d["prng_count"][0])
    got = np.concatenate([O.prng(int(s), cnt) for s in d["prng_seeds"]])
    assert np.array_equal(got, d["out.prng"])
    for n in (1, 4, 8, 16, 25, 32):
        assert np.array_equal(O.hammersley(n), d[f"ham{n}"])


def test_edge_random_table_matches_thread_streams():
    # sample i of thread k's static block uses stream 7777+k^2+1 in order
    n = 1000
    tab = O.edge_random_table(n, 14)
    d = load("random")
    cnt = int(d["prng_count"][0])
    q, r = divmod(n, 14)
    for k in range(14):
        b = k * q + min(k, r)
        stream = d["out.prng"][k * cnt:(k + 1) * cnt]
        m = min(cnt, 2 * (q + (1 if k < r else 0)))
        assert np.array_equal(tab[2 * b:2 * b + m], stream[:m])


@pytest.mark.parametrize("name", ["hits_cube_instanced", "hits_icosphere3"])
def test_hits_bit_exact(name):
    d = load(name)
    sc = scene_from(d)
    cam = cams_from(d)[0]
    got = O.cast_rays(sc, cam, d["hit_xy"])
    for k in ("prim", "inst", "geom"):
        assert np.array_equal(got[k], d["out." + k]), k
    for k in ("t", "u", "v"):
        assert np.array_equal(got[k], d["out." + k]), k
    assert np.array_equal(got["ray_pos"].reshape(-1), d["out.ray_pos"])
    assert np.array_equal(got["ray_dir"].reshape(-1), d["out.ray_dir"])
    assert (got["prim"] != 0xFFFFFFFF).sum() > 100


@pytest.mark.parametrize("name,mode,spp", [("render_cube_m2_spp16", 2, 16), ("render_cube_m1_spp9", 1, 9),
                                           ("render_cube_m2_spp8", 2, 8), ("render_sphere_m3", 3, 4),
                                           ("render_sphere_m4", 4, 4), ("render_sphere_m5", 5, 4),
                                           ("render_sphere_m6", 6, 4), ("render_pyramid_restricted", 2, 16)])
def test_render_bit_exact(name, mode, spp):
    d = load(name)
    img = O.render(scene_from(d), cams_from(d), mode, spp)
    assert np.array_equal(img, d["out.images"])
    assert img.max() > 0


@pytest.mark.parametrize("name,mode", [("drc_cube_m2", 2), ("drc_cube_m1", 1), ("drc_sphere_m3", 3),
                                       ("drc_sphere_m4", 4), ("drc_sphere_m5", 5), ("drc_sphere_m6", 6),
                                       ("drc_cube_instanced", 2), ("drc_pyramid_restricted_m2", 2),
                                       ("drc_pyramid_restricted_m16", 16), ("drc_two_meshes", 2),
                                       ("drc_static_occluders", 2)])
def test_d_render_and_compare(name, mode):
    d = load(name)
    loss, ds, imgs = O.d_render_and_compare(scene_from(d), cams_from(d), mode, int(d["spp"][0]), d["targets"],
                                            int(d["edge_samples"][0]), ids=d["dmesh_ids"])
    ref, lay = dscene_from(d)
    assert np.array_equal(imgs, d["out.images"])
    assert loss == pytest.approx(float(d["out.loss"][0]), rel=1e-6)
    olay, tot = O.dscene_layout(scene_from(d), mode, d["dmesh_ids"])
    assert np.array_equal(olay[:, :8], lay[:, :8]) and tot == ref.size
    # single view: the reference's reduction order is deterministic, so the
    # replayed 14-block accumulation reproduces it exactly
    assert np.array_equal(ds, ref)
    assert np.abs(ref).max() > 0


def test_d_render_two_views_bit_exact():
    d = load("drender_cube_2views")
    ds = O.d_render(scene_from(d), cams_from(d), 2, int(d["spp"][0]), d["adjoints"], int(d["edge_samples"][0]),
                    ids=d["dmesh_ids"])
    ref, _ = dscene_from(d)
    assert np.array_equal(ds, ref)


def test_optimizer_trajectory():
    d = load("optimize_cube_vc")
    p = O.opt_params(4, position_lr=float(d["opt_pos_lr"][0]), base_lr=float(d["opt_base_lr"][0]),
                     flags=int(d["opt_flags"][0]), dmesh_ids=[0])
    iters = int(d["iters"][0])
    r = O.optimize(scene_from(d), cams_from(d), 2, int(d["spp"][0]), d["targets"], p, iters)
    for k in range(iters):
        assert np.array_equal(r["vertices"][k], d[f"out.it{k}.m0.vertices"]), k
        assert np.array_equal(r["colors"][k], d[f"out.it{k}.m0.colors"]), k
    assert r["final_error"] == pytest.approx(float(d["out.final_error"][0]), rel=1e-6)


def test_optimizer_trajectory_two_meshes():
    """Two differentiable meshes: the reference's "Adam" divides every mesh's
    moment by the second-moment accumulator indexed mesh-locally
    (optimizer_simple.cpp:224), so the second mesh steps with the first
    mesh's accumulator."""
    d = load("optimize_two_meshes")
    p = O.opt_params(4, position_lr=float(d["opt_pos_lr"][0]), base_lr=float(d["opt_base_lr"][0]),
                     flags=int(d["opt_flags"][0]), dmesh_ids=[0, 1])
    iters = int(d["iters"][0])
    sc = scene_from(d)
    r = O.optimize(sc, cams_from(d), 2, int(d["spp"][0]), d["targets"], p, iters)
    n0v, n0c = 3 * sc.meshes[0].vertex_count, 3 * sc.meshes[0].vertex_count
    for k in range(iters):
        assert np.array_equal(r["vertices"][k][:n0v], d[f"out.it{k}.m0.vertices"]), k
        assert np.array_equal(r["vertices"][k][n0v:], d[f"out.it{k}.m1.vertices"]), k
        assert np.array_equal(r["colors"][k][:n0c], d[f"out.it{k}.m0.colors"]), k
        assert np.array_equal(r["colors"][k][n0c:], d[f"out.it{k}.m1.colors"]), k
    assert r["final_error"] == pytest.approx(float(d["out.final_error"][0]), rel=1e-6)


def test_optimizer_trajectory_restricted_transforms():
    """TEST 2.11 shape: only the TransformR parameters move (flags = transforms)."""
    d = load("optimize_pyramid_restricted")
    p = O.opt_params(4, position_lr=float(d["opt_pos_lr"][0]), transforms_lr=float(d["opt_tfm_lr"][0]),
                     flags=int(d["opt_flags"][0]), dmesh_ids=[0])
    iters = int(d["iters"][0])
    sc = scene_from(d)
    r = O.optimize(sc, cams_from(d), 2, int(d["spp"][0]), d["targets"], p, iters)
    for k in range(iters):
        assert np.array_equal(r["restricted"][k], d[f"out.it{k}.m0.restricted"]), k
        assert np.array_equal(r["vertices"][k], sc.meshes[0].vertices.reshape(-1)), k
    assert not np.array_equal(r["restricted"][-1], sc.restricted_params(0))
    assert r["final_error"] == pytest.approx(float(d["out.final_error"][0]), rel=1e-6)


def _to_mat64(p):
    """TransformR::to_mat in float64 (translate * rotZ * rotY * rotX * scale)."""
    tx, ty, tz, rx, ry, rz, s = (float(x) for x in p)
    c, n = math.cos, math.sin
    Rx = np.array([[1, 0, 0], [0, c(rx), -n(rx)], [0, n(rx), c(rx)]])
    Ry = np.array([[c(ry), 0, n(ry)], [0, 1, 0], [-n(ry), 0, c(ry)]])
    Rz = np.array([[c(rz), -n(rz), 0], [n(rz), c(rz), 0], [0, 0, 1]])
    M = np.zeros((3, 4))
    M[:, :3] = Rz @ Ry @ Rx * s
    M[:, 3] = (tx, ty, tz)
    return M.reshape(-1)  # row-major 3x4, the layout of the 12 transform gradients


def test_restricted_transform_jacobian_vs_central_differences():
    rng = np.random.default_rng(4)
    for _ in range(20):
        p = np.concatenate([rng.uniform(-1, 1, 3), rng.uniform(-math.pi, math.pi, 3), rng.uniform(0.3, 2, 1)])
        jac = O.restricted_jacobian(p.astype(np.float32)).astype(np.float64)
        p32 = p.astype(np.float32).astype(np.float64)
        h = 1e-6
        fd = np.stack([(_to_mat64(p32 + h * e) - _to_mat64(p32 - h * e)) / (2 * h) for e in np.eye(7)])
        assert np.abs(jac - fd).max() < 2e-6, np.abs(jac - fd).max()
        m = O.restricted_to_mat(p32.astype(np.float32)).reshape(4, 4).T  # column-major storage
        assert np.abs(m[:3].reshape(-1) - _to_mat64(p32)).max() < 1e-6
        assert np.array_equal(m[3], [0, 0, 0, 1])
