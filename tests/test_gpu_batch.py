"""Batched optimisation (drgb_batch_*) against the plain one-job path.

A batch advances several jobs of different models, sizes and sample counts
with one fused launch sequence per iteration.  Each job must compute the
same thing alone and in the mix: the first iteration's loss is bit-identical
(the forward pass is deterministic) and later iterations agree to float
atomic-ordering noise.
"""
import math

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300.scene import Texture, TriangleMesh

pytestmark = pytest.mark.gpu


def textured_sphere(seed=3):
    m = D.make_icosphere(2, seed=seed)
    P = m.vertices.astype(np.float64)
    u = 0.5 + np.arctan2(P[:, 0], P[:, 2]) / (2 * math.pi)
    v = np.arccos(np.clip(P[:, 1], -1, 1)) / math.pi
    tex = np.random.default_rng(seed).uniform(0.1, 0.9, size=(16, 16, 3)).astype(np.float32)
    return TriangleMesh(m.vertices, m.indices, tc=np.stack([u, v], 1).astype(np.float32), normals=m.normals,
                        textures=[Texture(16, 16, 3, tex.reshape(-1))])


def jobs():
    out = []
    # vertex colours, one view
    true = D.make_cube(seed=1)
    init = D.perturb_vertices(true, 0.1, seed=2)
    out.append((true, init, [D.CamInfo(origin=(0, 0, 3), width=64, height=64)], D.SHADING_MODEL.VERTEX_COLOR, 16,
                0.01))
    # point light + vertex albedo, two views
    true = D.make_icosphere(3, seed=4)
    init = D.perturb_vertices(true, 0.02, seed=5, radial=True)
    out.append((true, init, D.ring_cameras(2, 3.0, 48, 48), D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 4, 0.005))
    # texture
    true = textured_sphere()
    init = true.copy()
    init.textures[0].data[:] = 0.5
    out.append((true, init, [D.CamInfo(origin=(0.5, 0.8, 2.6), width=40, height=40)], D.SHADING_MODEL.TEXTURE_COLOR,
                4, 0.01))
    return out


def params(lr, mode):
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=lr, tex_lr=0.05)
    p.base_lr = lr
    return p


def test_batch_matches_plain_path():
    # After the first step the parameters of the two paths differ only by the
    # order of the gradient's atomic additions (the update is continuous in
    # the gradient).  From the second forward pass on, that noise can move a
    # sample across a silhouette, a discrete change, so later iterations are
    # compared through their losses.
    plain, setups = [], []
    for true, init, cams, mode, spp, lr in jobs():
        ts, isc = D.Scene(), D.Scene()
        ts.add_mesh(true)
        isc.add_mesh(init)
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
        r.commit(ts)
        tgt = r.render(ts, cams)
        opt = D.CreateSimpleOptimizer()
        opt.Init(isc, r, cams, tgt, params(lr, mode))
        opt.Run(1)
        first = opt.current_scene()
        opt.Run(2)
        plain.append((np.array(opt.losses), first))
        setups.append((isc, cams, tgt, mode, spp, lr))
    b = D.BatchOptimizer()
    ids = [b.add_job(isc, cams, tgt, D.DiffRenderSettings(mode, spp), params(lr, mode))
           for isc, cams, tgt, mode, spp, lr in setups]
    assert b.size() == 3
    b.run(1)
    scenes = [b.job_scene(j) for j in ids]
    b.run(2)
    for (losses, scene), bs, jid in zip(plain, scenes, ids):
        bl = b.losses(jid)
        assert bl.size == 3
        assert bl[0] == losses[0]                       # same forward pass
        np.testing.assert_allclose(bl, losses, rtol=1e-3)
        assert np.abs(bs.meshes[0].vertices - scene.meshes[0].vertices).max() < 1e-5
        if scene.meshes[0].colors is not None:
            assert np.abs(bs.meshes[0].colors - scene.meshes[0].colors).max() < 1e-5
        if scene.meshes[0].textures:
            assert np.abs(bs.meshes[0].textures[0].data - scene.meshes[0].textures[0].data).max() < 1e-5


def test_batch_job_same_alone_and_in_mix():
    setups = []
    for true, init, cams, mode, spp, lr in jobs():
        ts, isc = D.Scene(), D.Scene()
        ts.add_mesh(true)
        isc.add_mesh(init)
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
        r.commit(ts)
        setups.append((isc, cams, r.render(ts, cams), mode, spp, lr))
    alone = D.BatchOptimizer()
    a = alone.add_job(*setups[1][:3], D.DiffRenderSettings(setups[1][3], setups[1][4]), params(setups[1][5], 16))
    alone.run(4)
    mix = D.BatchOptimizer()
    ids = [mix.add_job(isc, cams, tgt, D.DiffRenderSettings(mode, spp), params(lr, mode))
           for isc, cams, tgt, mode, spp, lr in setups]
    mix.run(2)
    # a job removed from and another added to a running batch do not disturb it
    mix.remove_job(ids[0])
    extra = mix.add_job(*setups[0][:3], D.DiffRenderSettings(setups[0][3], setups[0][4]), params(setups[0][5], 2))
    mix.run(2)
    la, lm = alone.losses(a), mix.losses(ids[1])
    assert la[0] == lm[0]
    np.testing.assert_allclose(lm, la, rtol=1e-3)
    assert mix.losses(extra).size == 2
    assert mix.device_bytes(ids[1]) > 0
