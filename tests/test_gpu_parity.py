"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs (golden fixtures) and against the CPU oracle.

Tolerances:
  * per-sample hit ids, t, u, v: bit-exact (ties resolve to the lowest
    flattened triangle, which is the triangle the brute-force loop keeps);
  * images: bit-exact (max abs 0 <= 1e-4);
  * gradients: relative L2 <= 1e-3 for the interior (colour/texture) block
    and <= 1e-2 for the edge (position/transform) block.  Float atomics make
    the summation order differ from the reference's, so exact equality is
    not expected; the observed errors are near 1e-7.
"""
import math

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
import pyoracle as O
from fixtures import cams_from, dscene_from, load, rel_l2, scene_from

pytestmark = pytest.mark.gpu

INTERIOR_TOL = 1e-3
EDGE_TOL = 1e-2


def make(mode, spp, bruteforce=False):
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), spp))
    if bruteforce:
        r.set_option(1, 1)
    return r


def split_grad(vec, layout):
    """(positions+transforms, colours+textures) parts of a DScene vector."""
    pos, col = [], []
    off = 0
    for row in layout:
        nv, ninst, p, c, t, tr, rt, full = (int(x) for x in row[:8])
        blk = vec[off:off + full]
        pos.append(blk[p:p + 3 * nv])
        if tr >= 0:
            pos.append(blk[tr:tr + 12 * ninst])
        if rt >= 0:  # restricted transform parameters, also from the edge term
            pos.append(blk[rt:rt + 7 * ninst])
        if c >= 0:
            col.append(blk[c:c + 3 * nv])
        if t >= 0:
            col.append(blk[t:tr if tr >= 0 else rt])
        off += full
    cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0, np.float32)  # noqa: E731
    return cat(pos), cat(col)


def assert_grad_close(got, ref, layout, edge_tol=EDGE_TOL, interior_tol=INTERIOR_TOL):
    gp, gc = split_grad(got, layout)
    rp, rc = split_grad(ref, layout)
    if np.abs(rp).max(initial=0) > 0:
        assert rel_l2(gp, rp) <= edge_tol, ("edge block", rel_l2(gp, rp))
    else:
        assert np.abs(gp).max(initial=0) == 0
    if rc.size and np.abs(rc).max() > 0:
        assert rel_l2(gc, rc) <= interior_tol, ("interior block", rel_l2(gc, rc))


# ---------------------------------------------------------------------------
# against the reference's own outputs
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("bruteforce", [False, True])
@pytest.mark.parametrize("name", ["hits_cube_instanced", "hits_icosphere3"])
def test_hits_bit_exact_vs_reference(name, bruteforce):
    d = load(name)
    sc = scene_from(d)
    r = make(2, 1, bruteforce)
    r.commit(sc)
    got = r.cast_rays(cams_from(d)[0], d["hit_xy"])
    for k in ("prim", "inst", "geom", "t", "u", "v"):
        assert np.array_equal(got[k], d["out." + k]), (k, int(np.sum(got[k] != d["out." + k])))


@pytest.mark.parametrize("name,mode,spp", [("render_cube_m2_spp16", 2, 16), ("render_cube_m1_spp9", 1, 9),
                                           ("render_cube_m2_spp8", 2, 8), ("render_sphere_m3", 3, 4),
                                           ("render_sphere_m4", 4, 4), ("render_sphere_m5", 5, 4),
                                           ("render_sphere_m6", 6, 4)])
def test_render_bit_exact_vs_reference(name, mode, spp):
    d = load(name)
    sc = scene_from(d)
    r = make(mode, spp)
    r.commit(sc)
    img = r.render(sc, cams_from(d)).reshape(-1)
    assert np.array_equal(img, d["out.images"]), float(np.abs(img - d["out.images"]).max())


@pytest.mark.parametrize("name,mode", [("drc_cube_m2", 2), ("drc_cube_m1", 1), ("drc_sphere_m3", 3),
                                       ("drc_sphere_m4", 4), ("drc_sphere_m5", 5), ("drc_sphere_m6", 6),
                                       ("drc_cube_instanced", 2), ("drc_two_meshes", 2),
                                       ("drc_static_occluders", 2)])
def test_d_render_and_compare_vs_reference(name, mode):
    d = load(name)
    sc = scene_from(d)
    r = make(mode, int(d["spp"][0]))
    r.commit(sc)
    ds = D.DScene(r, d["dmesh_ids"])
    cams = cams_from(d)
    imgs = np.zeros(d["targets"].size, np.float32)
    loss = r.d_render_and_compare(sc, cams, d["targets"], int(d["edge_samples"][0]), ds, out_images=imgs)
    ref, lay = dscene_from(d)
    assert np.array_equal(imgs, d["out.images"])
    assert loss == pytest.approx(float(d["out.loss"][0]), rel=1e-6)
    assert np.array_equal(ds.layout[:, :8], lay[:, :8])
    assert_grad_close(ds.data, ref, lay)


def test_d_render_two_views_accumulates_vs_reference():
    d = load("drender_cube_2views")
    sc = scene_from(d)
    r = make(2, int(d["spp"][0]))
    r.commit(sc)
    ds = D.DScene(r, d["dmesh_ids"])
    r.d_render(sc, cams_from(d), d["adjoints"], int(d["edge_samples"][0]), ds)
    ref, lay = dscene_from(d)
    assert_grad_close(ds.data, ref, lay)
    # d_render accumulates (+=) into the DScene
    before = ds.data.copy()
    r.d_render(sc, cams_from(d), d["adjoints"], int(d["edge_samples"][0]), ds)
    assert rel_l2(ds.data, 2 * before) < 1e-5


@pytest.mark.parametrize("deterministic", [0, 1])
def test_optimizer_trajectory_vs_reference(deterministic):
    # The gradient sums run in another order than the reference's 14
    # per-thread copies (atomics, or the deterministic sorted reduction), and
    # the reference's update m/sqrt(G) is normalised per component, so
    # last-bit differences of small components grow to ~1e-5 over the steps.
    d = load("optimize_cube_vc")
    sc = scene_from(d)
    r = make(2, int(d["spp"][0]))
    r.set_option(N.OPT_DETERMINISTIC, deterministic)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=float(d["opt_pos_lr"][0]))
    p.base_lr = float(d["opt_base_lr"][0])
    p.flags = int(d["opt_flags"][0])
    opt = D.CreateSimpleOptimizer()
    opt.Init(sc, r, cams_from(d), d["targets"], p)
    iters = int(d["iters"][0])
    for k in range(iters):
        opt.Run(1)
        cur = opt.current_scene().meshes[0]
        assert np.abs(cur.vertices.reshape(-1) - d[f"out.it{k}.m0.vertices"]).max() < 5e-5, k
        assert np.abs(cur.colors.reshape(-1) - d[f"out.it{k}.m0.colors"]).max() < 5e-5, k
    assert opt.losses[-1] == pytest.approx(float(d["out.final_error"][0]), rel=1e-4)


def test_optimizer_trajectory_two_meshes_vs_reference():
    """Two differentiable meshes, the second stepped with the first mesh's
    second-moment accumulator (the reference's mesh-local index).  The first
    step must match.  After it, the per-component normalised steps turn
    summation-order noise in near-zero gradient components into full
    learning-rate steps of either sign, so the second step of the first mesh
    is compared component-wise for most components; the second mesh divides
    by the first mesh's (unrelated, often near-zero) accumulator entries and
    is compared at the first step only."""
    d = load("optimize_two_meshes")
    sc = scene_from(d)
    r = make(2, int(d["spp"][0]))
    r.set_option(N.OPT_DETERMINISTIC, 1)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=float(d["opt_pos_lr"][0]), diff_mesh_ids=(0, 1))
    p.base_lr = float(d["opt_base_lr"][0])
    p.flags = int(d["opt_flags"][0])
    opt = D.CreateSimpleOptimizer()
    opt.Init(sc, r, cams_from(d), d["targets"], p)
    for k in range(2):
        opt.Run(1)
        cur = opt.current_scene()
        for m in range(2 if k == 0 else 1):
            for what, got in (("vertices", cur.meshes[m].vertices), ("colors", cur.meshes[m].colors)):
                ref = d[f"out.it{k}.m{m}.{what}"]
                close = np.abs(got.reshape(-1) - ref) <= 1e-4 * max(1.0, float(np.abs(ref).max()))
                if k == 0:
                    assert close.all(), (k, m, what)
                else:
                    assert close.mean() >= 0.75, (k, m, what, close.mean())


# ---------------------------------------------------------------------------
# against the oracle on the benchmark workloads (reduced where the oracle
# would be slow) and size-independent properties at full size
# ---------------------------------------------------------------------------
def cube_problem(res=256, spp=16):
    true = D.make_cube(seed=1)
    init = D.perturb_vertices(true, 0.1, seed=2)
    init.colors = np.clip(true.colors + np.random.default_rng(3).normal(0, 0.1, (8, 3)), 0, 1).astype(np.float32)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = [D.CamInfo(origin=(0, 0, 3), width=res, height=res)]
    return ts, isc, cams


def test_cube_config_full_size_vs_oracle():
    ts, isc, cams = cube_problem(256, 16)
    r = make(2, 16)
    r.commit(ts)
    tgt = r.render(ts, cams).reshape(-1)
    assert np.array_equal(tgt, O.render(ts, cams, 2, 16))
    r.commit(isc)
    ds = D.DScene(r, [0])
    imgs = np.zeros(tgt.size, np.float32)
    loss = r.d_render_and_compare(isc, cams, tgt, 256 * 256, ds, out_images=imgs)
    oloss, ods, oimgs = O.d_render_and_compare(isc, cams, 2, 16, tgt, 256 * 256)
    assert np.array_equal(imgs, oimgs)
    assert loss == pytest.approx(oloss, rel=1e-6)
    assert_grad_close(ds.data, ods, ds.layout)


def ico_problem(res, n_views, sub=4):
    true = D.make_icosphere(sub, seed=1)
    init = D.perturb_vertices(true, 0.02, seed=2, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = D.ring_cameras(n_views, 3.0, res, res)
    return ts, isc, cams


def test_icosphere_point_light_vs_oracle():
    ts, isc, cams = ico_problem(48, 2)
    mode, spp = 16, 4
    r = make(mode, spp)
    r.commit(ts)
    tgt = r.render(ts, cams).reshape(-1)
    otgt = O.render(ts, cams, mode, spp)
    assert np.array_equal(tgt, otgt), float(np.abs(tgt - otgt).max())
    r.commit(isc)
    ds = D.DScene(r, [0])
    imgs = np.zeros(tgt.size, np.float32)
    loss = r.d_render_and_compare(isc, cams, tgt, 48 * 48, ds, out_images=imgs)
    oloss, ods, oimgs = O.d_render_and_compare(isc, cams, mode, spp, tgt, 48 * 48)
    assert np.array_equal(imgs, oimgs)
    assert loss == pytest.approx(oloss, rel=1e-5)
    assert_grad_close(ds.data, ods, ds.layout)


@pytest.mark.parametrize("builder", [0, 1])  # LBVH, binned SAH
def test_bvh_equals_bruteforce_on_large_mesh(builder):
    true = D.displace_radially(D.make_uv_sphere(120, 240, seed=4), seed=5)
    sc = D.Scene()
    sc.add_mesh(true)
    cam = D.CamInfo(origin=(0.3, 0.4, 2.7), width=512, height=512)
    rng = np.random.default_rng(9)
    xy = rng.uniform(0, 512, size=(400000, 2)).astype(np.float32)
    a, b = make(2, 1), make(2, 1, bruteforce=True)
    a.set_option(N.OPT_BVH_BUILDER, builder)
    a.commit(sc)
    b.commit(sc)
    ha, hb = a.cast_rays(cam, xy), b.cast_rays(cam, xy)
    assert (ha["prim"] != 0xFFFFFFFF).mean() > 0.3
    same = ha["prim"] == hb["prim"]
    for k in ("t", "u", "v"):
        assert np.array_equal(ha[k][same], hb[k][same])
    # Every disagreement must be a clamped-determinant hit of the brute-force
    # test (invDet = sign/max(sign*det, 1e-6), raytrace3d_bf.cpp:131): the
    # caster then reports t = |(o-A).N|/1e-6, a point that is not on the
    # triangle, nearer than the true surface.  A BVH cannot find such hits by
    # culling on geometry; they are rare and listed here.
    mism = np.flatnonzero(~same)
    assert mism.size <= 1e-3 * xy.shape[0], mism.size
    V = true.vertices.astype(np.float64)
    F = true.indices.reshape(-1, 3)
    for i in mism:
        p = hb["prim"][i]
        assert p != 0xFFFFFFFF
        A, B, C = V[F[p]]
        nrm = np.cross(B - A, C - A)
        # the brute-force hit is nearer than the LBVH's, its determinant was
        # clamped (|d.(e1 x e2)| < 1e-6), and it sits at the clamped distance
        # |(o-A).N|/1e-6 (o = the camera position; float32 cancellation in
        # (o-A).N allows a few per cent)
        assert hb["t"][i] < ha["t"][i] or ha["prim"][i] == 0xFFFFFFFF
        o = np.array(cam.origin, np.float64)
        tc = abs(np.dot(A - o, nrm)) / 1e-6
        assert abs(tc - hb["t"][i]) <= 5e-2 * max(tc, 1e-3), (i, tc, hb["t"][i])


def test_full_size_point_light_iteration_properties():
    """512x512, 8 views, 16 spp, 5120 triangles: the benchmark workload."""
    ts, isc, cams = ico_problem(512, 8)
    r = make(16, 16)
    r.commit(ts)
    tgt = r.render(ts, cams).reshape(-1)
    assert np.isfinite(tgt).all() and tgt.max() > 0.1
    r.commit(isc)
    ds = D.DScene(r, [0])
    l1 = r.d_render_and_compare(isc, cams, tgt, 512 * 512, ds)
    g1 = ds.data.copy()
    l2 = r.d_render_and_compare(isc, cams, tgt, 512 * 512, ds)
    assert l1 == l2 and np.isfinite(g1).all()
    assert rel_l2(ds.data, g1) < 1e-5          # same result up to atomic order
    pos, col = split_grad(g1, ds.layout)
    assert np.abs(pos).max() > 0 and np.abs(col).max() > 0
    # the target itself has zero loss and zero gradient
    r.commit(ts)
    dz = D.DScene(r, [0])
    assert r.d_render_and_compare(ts, cams, tgt, 512 * 512, dz) == 0.0
    assert np.abs(dz.data).max() == 0.0


def test_path_diffuse_close_to_oracle():
    ts, _, cams = ico_problem(32, 1, sub=2)
    r = make(17, 4)
    r.commit(ts)
    img = r.render(ts, cams).reshape(-1)
    oimg = O.render(ts, cams, 17, 4)
    # same random sequence; only trigonometric rounding differs
    assert np.abs(img - oimg).mean() < 1e-4


def test_edge_cases():
    # empty scene renders background
    r = make(2, 4)
    s = D.Scene()
    r.commit(s)
    img = r.render(s, [D.CamInfo(width=16, height=16)])
    assert np.abs(img).max() == 0
    # a single triangle (the LBVH root is a leaf)
    tri = D.TriangleMesh(np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32), np.array([0, 1, 2], np.uint32),
                         colors=np.eye(3, dtype=np.float32))
    s = D.Scene()
    s.add_mesh(tri)
    r.commit(s)
    cams = [D.CamInfo(origin=(0, 0, 3), width=32, height=32)]
    assert np.array_equal(r.render(s, cams).reshape(-1), O.render(s, cams, 2, 4))
    # render before commit is an error; bad dmesh ids are an error
    r2 = make(2, 4)
    with pytest.raises(D.api.N.DrgbError):
        r2.render(None, cams)
    with pytest.raises(D.api.N.DrgbError):
        D.DScene(r, [3])


def test_kernels_were_launched():
    assert D.kernel_launches() > 0
