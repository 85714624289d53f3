"""Two-level hierarchy build for instanced scenes (DRGB_OPT_BVH_BUILDER 1,
the default, or 2):
one hierarchy per mesh, shared by its instances, under a hierarchy over the
instances; the reference's Embree caster likewise builds one BVH per mesh
and instances it (raytrace_src/raytrace3d_embree.cpp:35-50,
raytrace_src/EmbreeRT.cpp:146-255).  The composed hierarchy keeps
world-space boxes and triangles, so the traversal and its hit arithmetic
are those of the flat build: hits equal the brute-force caster's
(raytrace_src/raytrace3d_bf.cpp:102-156) except where its determinant
clamp reports a point off the triangle, which no hierarchy finds."""
import math

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
from fixtures import rel_l2

pytestmark = pytest.mark.gpu


def rot(ax, ay, az):
    cx, sx, cy, sy, cz, sz = math.cos(ax), math.sin(ax), math.cos(ay), math.sin(ay), math.cos(az), math.sin(az)
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return rz @ ry @ rx


def instanced_scene(seed=0, jitter=0.0):
    """27 rotated instances of an icosphere (1,280 triangles), 5 of a cube and
    one large sphere behind them (three meshes)."""
    rng = np.random.default_rng(seed)
    sc = D.Scene()
    ico = D.make_icosphere(3, seed=1)
    trs = []
    for i in range(27):
        c = (np.array([i % 3, (i // 3) % 3, i // 9], np.float64) - 1.0) * 0.6
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] = 0.4 * rot(*rng.uniform(0, 2 * math.pi, 3))
        m[:3, 3] = c / 1.4 + rng.normal(0.0, jitter, 3)
        trs.append(m)
    sc.add_mesh(ico, trs)
    cube = D.make_cube(seed=2)
    ctr = []
    for k in range(5):
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] = 0.3 * rot(*rng.uniform(0, 2 * math.pi, 3))
        m[:3, 3] = rng.uniform(-0.7, 0.7, 3)
        ctr.append(m)
    sc.add_mesh(cube, ctr)
    back = D.make_icosphere(2, radius=3.0, seed=3)
    mb = np.eye(4, dtype=np.float32)
    mb[:3, 3] = (0.0, 0.0, -4.0)
    sc.add_mesh(back, [mb])
    return sc


def renderer(mode, spp, builder=None, bruteforce=False):
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), spp))
    if builder is not None:
        r.set_option(N.OPT_BVH_BUILDER, builder)
    if bruteforce:
        r.set_option(N.OPT_TRACE_BRUTEFORCE, 1)
    return r


@pytest.mark.parametrize("builder", [0, 1, 2, 3])  # LBVH, default (two-level here), two-level, flat SAH
def test_instanced_hits_equal_bruteforce(builder):
    sc = instanced_scene()
    cam = D.CamInfo(origin=(0.4, 0.5, 3.0), width=512, height=512)
    xy = np.random.default_rng(5).uniform(0, 512, size=(300000, 2)).astype(np.float32)
    a, b = renderer(2, 1, builder), renderer(2, 1, bruteforce=True)
    a.commit(sc)
    b.commit(sc)
    ha, hb = a.cast_rays(cam, xy), b.cast_rays(cam, xy)
    assert_hits_match(ha, hb)


def assert_hits_match(ha, hb):
    hit = hb["prim"] != 0xFFFFFFFF
    assert hit.mean() > 0.3
    assert len(np.unique(hb["inst"][hit & (hb["geom"] == 0)])) > 20   # many instances are seen
    n = hit.size
    same = np.ones(n, bool)
    for k in ("prim", "inst", "geom"):
        same &= ha[k] == hb[k]
    for k in ("t", "u", "v"):
        assert np.array_equal(ha[k][same], hb[k][same])
    # the rest: brute-force hits nearer than any hierarchy's (clamped determinant)
    mism = np.flatnonzero(~same)
    assert mism.size <= 1e-3 * n, mism.size
    assert np.all((hb["t"][mism] < ha["t"][mism]) | (ha["prim"][mism] == 0xFFFFFFFF))


def test_two_level_render_and_gradient_equal_flat():
    sc = instanced_scene()
    cams = D.ring_cameras(2, 3.0, 128, 128)
    adj = np.random.default_rng(2).normal(0, 0.5, 2 * 128 * 128 * 3).astype(np.float32)
    imgs, grads = {}, {}
    for builder in (3, 2):  # flat, two-level
        r = renderer(2, 4, builder)
        r.commit(sc)
        imgs[builder] = r.render(sc, cams).reshape(-1)
        ds = D.DScene(r, [0, 1])
        r.d_render(sc, cams, adj, 128 * 128, ds)
        grads[builder] = ds.data.copy()
    differ = np.flatnonzero(imgs[3] != imgs[2])
    assert differ.size <= 1e-3 * imgs[3].size, differ.size
    assert np.abs(grads[3]).max() > 0
    assert rel_l2(grads[2], grads[3]) < 2e-2


def test_two_level_rebuilds_of_moving_instances():
    """Instance transforms optimised with a new topology every 2 iterations:
    the hierarchy the optimiser holds afterwards (built from the moved
    instances, refitted) gives the brute-force hits of its current scene."""
    ts, isc = instanced_scene(), instanced_scene(jitter=0.02)
    cams = D.ring_cameras(2, 3.0, 96, 96)
    r0 = renderer(2, 4)
    r0.commit(ts)
    tgt = r0.render(ts, cams)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.0, transforms_lr=0.004)
    p.flags = D.OptimizerParameters._OPT_TFM
    r = renderer(2, 4, 2)
    r.set_option(N.OPT_BVH_REBUILD, 2)
    opt = D.CreateSimpleOptimizer()
    opt.Init(isc, r, cams, tgt, p)
    opt.Run(7)
    cur = opt.current_scene()
    moved = np.concatenate([np.ravel(m) for m in cur.transforms[0]])
    start = np.concatenate([np.ravel(m) for m in isc.transforms[0]])
    assert np.abs(moved - start).max() > 0.01
    bf = renderer(2, 1, bruteforce=True)
    bf.commit(cur)
    cam = D.CamInfo(origin=(0.4, 0.5, 3.0), width=512, height=512)
    xy = np.random.default_rng(6).uniform(0, 512, size=(300000, 2)).astype(np.float32)
    assert_hits_match(r.cast_rays(cam, xy), bf.cast_rays(cam, xy))


@pytest.mark.parametrize("builder", [0, 1, 2, 3])
def test_degenerate_instancing_equals_bruteforce(builder):
    """A one-triangle mesh with 7 instances (the top hierarchy's leaves are
    single triangles), a mesh with vertices but no triangles, 3 instances,
    and a two-triangle quad; hits against the brute-force caster, and a
    gradient through the edge pass."""
    rng = np.random.default_rng(11)
    sc = D.Scene()
    tri = D.TriangleMesh(np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32), np.array([0, 1, 2], np.uint32),
                         colors=np.eye(3, dtype=np.float32))
    trs = []
    for k in range(7):
        m = np.eye(4, dtype=np.float32)
        m[:3, :3] = 0.3 * rot(*rng.uniform(0, 2 * math.pi, 3))
        m[:3, 3] = rng.uniform(-0.5, 0.5, 3)
        trs.append(m)
    sc.add_mesh(tri, trs)
    empty = D.TriangleMesh(np.zeros((3, 3), np.float32), np.zeros(0, np.uint32), colors=np.ones((3, 3), np.float32))
    sc.add_mesh(empty, [np.eye(4, dtype=np.float32)] * 3)
    quad = D.TriangleMesh(np.array([[-2, -2, -1], [2, -2, -1], [2, 2, -1], [-2, 2, -1]], np.float32),
                          np.array([0, 1, 2, 0, 2, 3], np.uint32), colors=rng.uniform(0, 1, (4, 3)).astype(np.float32))
    sc.add_mesh(quad)
    cam = D.CamInfo(origin=(0.2, 0.1, 3.0), width=256, height=256)
    xy = np.random.default_rng(12).uniform(0, 256, size=(100000, 2)).astype(np.float32)
    a, b = renderer(2, 1, builder), renderer(2, 1, bruteforce=True)
    a.commit(sc)
    b.commit(sc)
    ha, hb = a.cast_rays(cam, xy), b.cast_rays(cam, xy)
    assert (hb["geom"][hb["prim"] != 0xFFFFFFFF] == 0).mean() > 0.005   # the small triangles are hit
    same = np.ones(xy.shape[0], bool)
    for k in ("prim", "inst", "geom", "t", "u", "v"):
        same &= ha[k] == hb[k]
    assert (~same).sum() <= 1e-3 * xy.shape[0]
    cams = [cam]
    adj = np.random.default_rng(13).normal(0, 0.5, 256 * 256 * 3).astype(np.float32)
    ds = D.DScene(a, [0, 2])
    a.d_render(sc, cams, adj, 256 * 256, ds)
    assert np.isfinite(ds.data).all() and np.abs(ds.data).max() > 0
