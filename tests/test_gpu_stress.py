"""Differentiation checks of the stress configuration, at test sizes.

* stored adjoint hits (DRGB_OPT_ADJOINT_HITS) give the gradient of re-traced
  visibility: bit-identical under the deterministic reduction;
* the 2-bounce path model's gradient against the oracle;
* central finite differences (h = 1e-3) of the loss on 64 seeded vertex
  coordinates against the edge-sampled position gradient of the silhouette
  model, where that term is the whole derivative, and of the path model on
  silhouette vertices.
"""
import os
import sys

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
from diffrender_tutorials_gb300 import workloads as WL
from fixtures import rel_l2
from test_gpu_parity import O, assert_grad_close

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

pytestmark = pytest.mark.gpu


def sphere_problem(n_tris, res, seed=0, views=1):
    true = WL.sphere_with_triangles(n_tris, seed=seed)
    init = D.perturb_vertices(true, 0.01, seed=seed + 2, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = [D.CamInfo(origin=(0.0, 0.4, 2.6), width=res, height=res)] if views == 1 else \
        D.ring_cameras(views, 3.0, res, res)
    return ts, isc, cams


@pytest.mark.parametrize("mode,spp", [(17, 4), (16, 16), (2, 16)])
def test_stored_hits_give_the_recomputed_gradient(mode, spp):
    ts, isc, cams = sphere_problem(8000, 96, views=2)
    W = cams[0].width
    out = {}
    for hits in (0, 1):
        for det in (0, 1):
            r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), spp))
            r.set_option(N.OPT_ADJOINT_HITS, hits)
            r.set_option(N.OPT_DETERMINISTIC, det)
            r.commit(ts)
            tgt = r.render(ts, cams).reshape(-1)
            r.commit(isc)
            ds = D.DScene(r, [0])
            loss = r.d_render_and_compare(isc, cams, tgt, W * W, ds)
            out[(hits, det)] = (loss, ds.data.copy())
    assert np.abs(out[(0, 1)][1]).max() > 0
    assert out[(1, 1)][0] == out[(0, 1)][0]
    assert np.array_equal(out[(1, 1)][1], out[(0, 1)][1])
    assert rel_l2(out[(1, 0)][1], out[(0, 0)][1]) < 1e-5


def test_stored_hits_in_the_optimiser_loop():
    ts, isc, cams = sphere_problem(4000, 64)
    runs = []
    for hits in (0, 1):
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.PATH_DIFFUSE, 4))
        r.commit(ts)
        tgt = r.render(ts, cams)
        r.set_option(N.OPT_ADJOINT_HITS, hits)
        r.set_option(N.OPT_DETERMINISTIC, 1)
        p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.001)
        p.base_lr = 0.01
        opt = D.CreateSimpleOptimizer()
        opt.Init(isc, r, cams, tgt, p)
        opt.Run(4)
        runs.append((np.array(opt.losses), opt.current_scene().meshes[0].vertices))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


def test_path_model_gradient_vs_oracle():
    ts, isc, cams = sphere_problem(1200, 40)
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.PATH_DIFFUSE, 4))
    r.commit(ts)
    tgt = O.render(ts, cams, 17, 4)
    r.commit(isc)
    ds = D.DScene(r, [0])
    imgs = np.zeros(tgt.size, np.float32)
    loss = r.d_render_and_compare(isc, cams, tgt, 40 * 40, ds, out_images=imgs)
    oloss, ods, oimgs = O.d_render_and_compare(isc, cams, 17, 4, tgt, 40 * 40)
    # the bounce directions come from the same counter-based random numbers
    # and the same sin/cos polynomial on both sides, so the images agree
    # per pixel
    diff = np.abs(imgs - oimgs)
    print(f"path model vs oracle: image max abs {diff.max():.3g} ({int((diff > 0).sum())} values differ)")
    assert diff.max() <= 1e-4, (float(diff.max()), int((diff > 0).sum()))
    assert loss == pytest.approx(oloss, rel=1e-5)
    assert_grad_close(ds.data, ods, ds.layout)


def silhouette_coords(isc, cams, n, rng):
    V = isc.meshes[0].vertices.astype(np.float64)
    nrm = isc.meshes[0].normals.astype(np.float64)
    view = V - np.asarray(cams[0].origin, np.float64)
    cosang = np.abs(np.sum(view * nrm, 1)) / (np.linalg.norm(view, axis=1) * np.linalg.norm(nrm, axis=1))
    sil = np.argsort(cosang)[:max(4 * n, 200)]
    sv = rng.choice(sil, size=n, replace=False)
    return 3 * sv + rng.integers(0, 3, size=n)


def test_silhouette_gradient_vs_central_differences():
    """Silhouette model: coverage changes only at edges, so the edge term is
    the whole position derivative and must follow the finite differences.
    The reference's edge Jacobian drops the cross terms of the projection
    (src/drender.cpp:31-87) and h = 1e-3 moves an edge by a fraction of a
    pixel over a fixed sample grid, so the agreement is statistical."""
    ts, isc, cams = sphere_problem(3000, 256)
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.SILHOUETTE, 16))
    r.commit(ts)
    tgt = r.render(ts, cams)
    r.commit(isc)
    ds = D.DScene(r, [0])
    r.d_render_and_compare(isc, cams, tgt, 16 * 256 * 256, ds)
    gpos = ds.get_dmeshes()[0].pos().reshape(-1).copy()
    coords = silhouette_coords(isc, cams, 64, np.random.default_rng(7))
    res = bench.fd_check(r, isc, cams, tgt, gpos, coords)
    assert res["fd_norm"] > 0
    assert res["rel_l2"] < 0.5, res
    assert res["correlation"] > 0.9, res
    assert res["sign_agreement"] > 0.9, res


def test_path_model_silhouette_vertices_follow_central_differences():
    """Path model: at silhouette vertices the visibility term dominates the
    derivative; the smooth shading term the method does not differentiate
    makes the match looser than for the silhouette model."""
    ts, isc, cams = sphere_problem(3000, 256)
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.PATH_DIFFUSE, 4))
    r.commit(ts)
    tgt = r.render(ts, cams)
    r.commit(isc)
    ds = D.DScene(r, [0])
    r.d_render_and_compare(isc, cams, tgt, 16 * 256 * 256, ds)
    gpos = ds.get_dmeshes()[0].pos().reshape(-1).copy()
    coords = silhouette_coords(isc, cams, 64, np.random.default_rng(8))
    res = bench.fd_check(r, isc, cams, tgt, gpos, coords)
    assert res["correlation"] > 0.5, res
    assert res["sign_agreement"] > 0.7, res
