"""Silhouette-edge sampling (DRGB_OPT_EDGE_SET = 1) against all-edge sampling.

The reference samples every edge of the differentiable meshes in proportion
to its projected length (src/drender.h:274-285,306-345).  With continuous
shading across edges (interpolated normals and vertex albedo) only the
silhouette edges, where one adjacent triangle faces the camera and the other
faces away, and boundary edges carry a discontinuity; the others contribute
just the difference of two shading points 2e-3 px apart.  The silhouette
mode samples only those edges.

  * against the oracle's restatement of the same mode: images bit-exact,
    gradients within 1e-3 (interior) / 1e-2 (edge) relative L2;
  * on the smooth-shaded point-light icosphere, its gradient against the
    all-edge gradient, both with many samples per pixel.
"""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
import pyoracle as O
from fixtures import rel_l2

pytestmark = pytest.mark.gpu

INTERIOR_TOL, EDGE_TOL = 1e-3, 1e-2


def problem(sub, res, views):
    true = D.make_icosphere(sub, seed=1)
    init = D.perturb_vertices(true, 0.02, seed=2, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    return ts, isc, D.ring_cameras(views, 3.0, res, res)


def gradient(isc, ts, cams, mode, spp, edge_set, samples):
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), spp))
    r.set_option(N.OPT_EDGE_SET, edge_set)
    r.commit(ts)
    tgt = r.render(ts, cams).reshape(-1)
    r.commit(isc)
    ds = D.DScene(r, [0])
    loss = r.d_render_and_compare(isc, cams, tgt, samples, ds)
    return loss, ds, tgt


def test_silhouette_edges_vs_oracle():
    ts, isc, cams = problem(3, 96, 2)
    loss, ds, tgt = gradient(isc, ts, cams, 16, 4, 1, 96 * 96)
    oloss, ods, _ = O.d_render_and_compare(isc, cams, 16, 4, tgt, 96 * 96, mp=O.model_params(edge_set=1))
    assert loss == pytest.approx(oloss, rel=1e-6)
    nv, _, p, c = (int(x) for x in ds.layout[0][:4])
    assert np.abs(ods[p:p + 3 * nv]).max() > 0
    assert rel_l2(ds.data[p:p + 3 * nv], ods[p:p + 3 * nv]) <= EDGE_TOL
    assert rel_l2(ds.data[c:c + 3 * nv], ods[c:c + 3 * nv]) <= INTERIOR_TOL
    # every edge mode is a different estimator of the same boundary integral:
    # the oracle's all-edge gradient differs
    _, ods_all, _ = O.d_render_and_compare(isc, cams, 16, 4, tgt, 96 * 96)
    assert not np.array_equal(ods_all[p:p + 3 * nv], ods[p:p + 3 * nv])


def test_silhouette_edges_give_the_all_edge_gradient_on_smooth_shading():
    ts, isc, cams = problem(4, 256, 2)
    samples = 64 * 256 * 256
    _, ds_all, _ = gradient(isc, ts, cams, 16, 16, 0, samples)
    _, ds_sil, _ = gradient(isc, ts, cams, 16, 16, 1, samples)
    nv, _, p, c = (int(x) for x in ds_all.layout[0][:4])
    g_all, g_sil = ds_all.data[p:p + 3 * nv], ds_sil.data[p:p + 3 * nv]
    err = rel_l2(g_sil, g_all)
    print(f"silhouette vs all-edge position gradient: relative L2 {err:.4f}")
    assert err < 5e-2, err
    # the interior (albedo) term does not depend on the edge set
    assert np.array_equal(ds_all.data[c:c + 3 * nv], ds_sil.data[c:c + 3 * nv]) or \
        rel_l2(ds_sil.data[c:c + 3 * nv], ds_all.data[c:c + 3 * nv]) < 1e-5
