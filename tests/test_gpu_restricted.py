"""Restricted transforms (TransformR instances, common_src/scene.h:91-116) on
the GPU: the instance matrices come from to_mat of 7 parameters each and the
gradient holds d loss / d params, the 12 matrix gradients of the edge term
taken through the Jacobian of to_mat (src/drender.h:398-421).

The reference computes that Jacobian with the Enzyme plugin, absent here; the
fixtures come from the reference's own code with the oracle's analytic
Jacobian in its place (oracle/ref/ref_driver.cpp), and the oracle's tests pin
that Jacobian against central differences of to_mat.  Tolerances as in
test_gpu_parity: images bit-exact, edge-term gradients within 1e-2 relative
L2 (float atomics), trajectories within a few 1e-5.
"""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
from fixtures import cams_from, dscene_from, load, rel_l2, scene_from
from test_gpu_parity import assert_grad_close

pytestmark = pytest.mark.gpu


def make(mode, spp):
    return D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), spp))


def restricted_block(vec, layout):
    row = layout[0]
    return vec[int(row[6]):int(row[6]) + 7 * int(row[1])]


def test_render_bit_exact_vs_reference():
    d = load("render_pyramid_restricted")
    sc = scene_from(d)
    assert sc.restricted[0] is not None and len(sc.restricted[0]) == 2
    r = make(2, 16)
    r.commit(sc)
    img = r.render(sc, cams_from(d)).reshape(-1)
    assert np.array_equal(img, d["out.images"]), float(np.abs(img - d["out.images"]).max())


@pytest.mark.parametrize("name,mode", [("drc_pyramid_restricted_m2", 2), ("drc_pyramid_restricted_m16", 16)])
def test_d_render_and_compare_vs_reference(name, mode):
    d = load(name)
    sc = scene_from(d)
    r = make(mode, int(d["spp"][0]))
    r.commit(sc)
    ds = D.DScene(r, d["dmesh_ids"])
    imgs = np.zeros(d["targets"].size, np.float32)
    loss = r.d_render_and_compare(sc, cams_from(d), d["targets"], int(d["edge_samples"][0]), ds, out_images=imgs)
    ref, lay = dscene_from(d)
    assert np.array_equal(imgs, d["out.images"])
    assert loss == pytest.approx(float(d["out.loss"][0]), rel=1e-6)
    assert np.array_equal(ds.layout[:, :8], lay[:, :8])
    assert ds.get_dmeshes()[0].transform_mat() is None
    rt, rt_ref = ds.get_dmeshes()[0].restricted_transform().reshape(-1), restricted_block(ref, lay)
    assert np.abs(rt_ref).max() > 0
    assert rel_l2(rt, rt_ref) <= 1e-2, rel_l2(rt, rt_ref)
    assert_grad_close(ds.data, ref, lay)


def test_d_render_accumulates_and_deterministic_mode():
    d = load("drc_pyramid_restricted_m2")
    sc, cams = scene_from(d), cams_from(d)
    adj = np.random.default_rng(3).normal(0, 0.5, d["targets"].size).astype(np.float32)
    out = {}
    for det in (0, 1):
        r = make(2, 16)
        r.set_option(N.OPT_DETERMINISTIC, det)
        r.commit(sc)
        ds = D.DScene(r, [0])
        r.d_render(sc, cams, adj, 4096, ds)
        once = ds.data.copy()
        r.d_render(sc, cams, adj, 4096, ds)   # += ; the matrix scratch is cleared per call
        assert rel_l2(ds.data, 2 * once) < 1e-5
        out[det] = once
    assert np.abs(restricted_block(out[1], ds.layout)).max() > 0
    assert rel_l2(out[1], out[0]) < 1e-5


def test_optimizer_trajectory_vs_reference():
    d = load("optimize_pyramid_restricted")
    sc = scene_from(d)
    r = make(2, int(d["spp"][0]))
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=float(d["opt_pos_lr"][0]),
                              transforms_lr=float(d["opt_tfm_lr"][0]))
    p.flags = int(d["opt_flags"][0])
    opt = D.CreateSimpleOptimizer()
    opt.Init(sc, r, cams_from(d), d["targets"], p)
    for k in range(int(d["iters"][0])):
        opt.Run(1)
        cur = opt.current_scene()
        got = np.concatenate([t.params() for t in cur.restricted[0]])
        # float atomics in the edge term: the bound grows by 5e-5 per iteration
        assert np.abs(got - d[f"out.it{k}.m0.restricted"]).max() < 5e-5 * (k + 1), (k, got)
        assert np.array_equal(cur.meshes[0].vertices, sc.meshes[0].vertices)
        # the instance matrices follow the parameters
        for t, m in zip(cur.restricted[0], cur.transforms[0]):
            assert np.abs(t.to_mat() - m).max() < 1e-6
    assert opt.losses[-1] == pytest.approx(float(d["out.final_error"][0]), rel=1e-4)


def _setup():
    d = load("optimize_pyramid_restricted")
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.0, transforms_lr=float(d["opt_tfm_lr"][0]))
    p.flags = int(d["opt_flags"][0])
    return scene_from(d), cams_from(d), d["targets"], p


def test_batch_and_server_run_restricted_jobs():
    sc, cams, tgt, p = _setup()
    opt = D.CreateSimpleOptimizer()
    opt.Init(sc, make(2, 16), cams, tgt, p)
    opt.Run(3)
    plain = np.concatenate([t.params() for t in opt.current_scene().restricted[0]])
    # in a batch next to an unrestricted job
    b = D.BatchOptimizer()
    jid = b.add_job(sc, cams, tgt, D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 16), p)
    cube_t, cube_i = D.Scene(), D.Scene()
    cube_t.add_mesh(D.make_cube(seed=1))
    cube_i.add_mesh(D.perturb_vertices(D.make_cube(seed=1), 0.1, seed=2))
    ccams = [D.CamInfo(origin=(0, 0, 3), width=32, height=32)]
    rr = make(2, 4)
    rr.commit(cube_t)
    b.add_job(cube_i, ccams, rr.render(cube_t, ccams), D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 4),
              D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.01))
    b.run(3)
    batched = np.concatenate([t.params() for t in b.job_scene(jid).restricted[0]])
    assert b.losses(jid)[0] == opt.losses[0]
    assert np.abs(batched - plain).max() < 5e-5
    # served
    srv = D.OptimizationServer(worker=False)
    t = srv.submit(sc, cams, tgt, D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 16), p, 3)
    for _ in range(10):
        srv.step()
        if srv.info(t)["state"] == "done":
            break
    served = np.concatenate([x.params() for x in srv.result_scene(t).restricted[0]])
    assert np.abs(served - plain).max() < 5e-5
    srv.close()

