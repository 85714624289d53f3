"""Autotuning of the work-item shape and persistent grids
(drgb_optimizer_autotune, drgb_batch_autotune): it must leave the
optimisation state untouched and the results unchanged up to summation
order."""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D

pytestmark = pytest.mark.gpu


def problem():
    true = D.make_icosphere(3, seed=4)
    init = D.perturb_vertices(true, 0.02, seed=5, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    return ts, isc, D.ring_cameras(2, 3.0, 96, 96)


def optimiser(ts, isc, cams):
    st = D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 16)
    r = D.MakeDifferentialRenderer(st)
    r.commit(ts)
    tgt = r.render(ts, cams)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.005)
    p.base_lr = 0.005
    o = D.CreateSimpleOptimizer()
    o.Init(isc, r, cams, tgt, p)
    return o, tgt, st, p


def test_optimizer_autotune_keeps_state_and_results():
    ts, isc, cams = problem()
    ref, _, _, _ = optimiser(ts, isc, cams)
    ref.Run(2)
    o, _, _, _ = optimiser(ts, isc, cams)
    before = o.current_scene().meshes[0].vertices.copy()
    cfg = o.autotune(2)
    assert cfg["tile"][0] * cfg["tile"][1] * 16 in (32, 64)
    assert cfg["pixel_blocks_per_sm"] in (2, 4, 8, 16) and cfg["edge_blocks_per_sm"] in (2, 4, 8, 16)
    assert cfg["ms"] > 0
    assert np.array_equal(o.current_scene().meshes[0].vertices, before)
    o.Run(2)
    # the first loss only regroups the per-pixel partials; the second follows
    # a step whose gradient was summed in another atomic order
    lo, lr = np.array(o.losses), np.array(ref.losses)
    np.testing.assert_allclose(lo[0], lr[0], rtol=1e-6)
    np.testing.assert_allclose(lo[1], lr[1], rtol=1e-3)


def test_batch_autotune_keeps_state():
    ts, isc, cams = problem()
    o, tgt, st, p = optimiser(ts, isc, cams)
    b = D.BatchOptimizer()
    j = b.add_job(isc, cams, tgt, st, p)
    j2 = b.add_job(*problem()[1:], tgt, st, p)
    cfg = b.autotune(2)
    assert cfg["pixel_blocks_per_sm"] in (2, 4, 8, 16) and cfg["ms"] > 0
    assert b.losses(j).size == 0
    assert np.array_equal(b.job_scene(j).meshes[0].vertices, isc.meshes[0].vertices)
    b.run(2)
    o.Run(2)
    np.testing.assert_allclose(b.losses(j), np.array(o.losses), rtol=1e-4)
    assert b.losses(j2).size == 2
