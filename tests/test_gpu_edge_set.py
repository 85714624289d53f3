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
  * on the silhouette model, both modes against central differences of the
    loss (there the two estimate the same derivative);
  * on the smooth-shaded point-light icosphere, its gradient against the
    all-edge gradient, both with many samples per pixel.
"""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
import pyoracle as O
from fixtures import rel_l2
from test_gpu_edge_jacobian import directional_fd, tilted_ring

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


def test_silhouette_edges_follow_central_differences():
    """Silhouette model, tilted ring cameras, full edge Jacobian: coverage
    changes only at silhouette and boundary edges, where the all-edge mode's
    other edges contribute exactly zero (both sides shade 1), so both modes
    estimate the same derivative; the silhouette mode puts every sample on
    the edges that matter.  Both are compared with central differences of
    the loss along random directions of all vertex coordinates."""
    res, spp = 256, 64
    true = D.make_icosphere(3, seed=5)
    init = D.perturb_vertices(true, 0.03, seed=6, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = tilted_ring(3, 3.0, 1.4, res)
    mode = D.SHADING_MODEL.SILHOUETTE
    ref = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
    ref.commit(ts)
    tgt = ref.render(ts, cams)
    grads = {}
    for edge_set in (0, 1):
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
        r.set_option(N.OPT_EDGE_JACOBIAN, 1)
        r.set_option(N.OPT_EDGE_SET, edge_set)
        r.commit(isc)
        ds = D.DScene(r, [0])
        r.d_render_and_compare(isc, cams, tgt, 16 * res * res, ds)
        grads[edge_set] = ds.get_dmeshes()[0].pos().reshape(-1).astype(np.float64)
    rng = np.random.default_rng(11)
    fd_r = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
    nv = isc.meshes[0].vertex_count
    err = {0: [], 1: []}
    fds = []
    for _ in range(12):
        d = rng.normal(size=3 * nv)
        d /= np.linalg.norm(d)
        fd = directional_fd(fd_r, isc, cams, tgt, d, 5e-2)
        fds.append(fd)
        for k in (0, 1):
            err[k].append(float(np.dot(grads[k], d)) - fd)
    e_all = float(np.linalg.norm(err[0]) / np.linalg.norm(fds))
    e_sil = float(np.linalg.norm(err[1]) / np.linalg.norm(fds))
    print(f"directional derivatives vs central differences: all edges {e_all:.4f}, silhouette edges {e_sil:.4f}")
    # measured 0.065 (all edges) and 0.039 (silhouette edges)
    assert e_sil < 0.08, (e_all, e_sil)
    assert e_sil <= e_all + 0.02, (e_all, e_sil)


def test_silhouette_edges_on_smooth_shading():
    """Point-light icosphere, 64 edge samples per pixel: the two modes'
    position gradients against each other.  They differ by the all-edge
    estimator's sampling noise (its gradients at N and 2N samples differ by
    about 3 % relative L2 here) and by the interior edges' contributions of
    the all-edge mode -- the shading difference of two points 2e-3 px apart
    across an edge where shading is continuous, about 3 % of its norm --
    which the silhouette mode leaves out."""
    ts, isc, cams = problem(4, 256, 2)
    samples = 64 * 256 * 256
    _, ds_all, _ = gradient(isc, ts, cams, 16, 16, 0, samples)
    _, ds_sil, _ = gradient(isc, ts, cams, 16, 16, 1, samples)
    nv, _, p, c = (int(x) for x in ds_all.layout[0][:4])
    g_all, g_sil = ds_all.data[p:p + 3 * nv], ds_sil.data[p:p + 3 * nv]
    err = rel_l2(g_sil, g_all)
    print(f"silhouette vs all-edge position gradient: relative L2 {err:.4f}")
    assert err < 0.1, err  # measured 0.074
    # the interior (albedo) term does not depend on the edge set
    assert rel_l2(ds_sil.data[c:c + 3 * nv], ds_all.data[c:c + 3 * nv]) < 1e-5
