"""Edge-term chain rule: the reference's edge_grad against the full Jacobian.

The reference's edge_grad (src/drender.cpp:31-87) keeps only dx/dX and
dy/dY for the x and y components of each endpoint's world-space gradient
(both terms for z) and maps it to mesh-local positions with mesh 0's inverse
transform.  That is exact for a camera on the z axis and biased otherwise.
DRGB_OPT_EDGE_JACOBIAN = 1 uses the full 2x3 Jacobian of the endpoint's
pixel position and the transpose of the edge's own instance transform.

  * against the oracle's restatement of the same mode (instanced, rotated
    and scaled meshes, tilted cameras): images bit-exact, gradients within
    1e-3 (interior) / 1e-2 (edge) relative L2;
  * against central differences of the loss (silhouette model, so the edge
    term is the whole position derivative) on ring cameras: the full
    Jacobian agrees with the differences, the reference's form does not.
"""
import math

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
import pyoracle as O
from fixtures import rel_l2

pytestmark = pytest.mark.gpu

INTERIOR_TOL, EDGE_TOL = 1e-3, 1e-2


def tilted_ring(n, radius, height, res):
    cams = []
    for k in range(n):
        a = 2 * math.pi * (k + 0.5) / n
        cams.append(D.CamInfo(origin=(radius * math.sin(a), height, radius * math.cos(a)), width=res, height=res))
    return cams


def rot_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], np.float32)


def instanced_problem():
    true = D.make_icosphere(2, seed=3)
    init = D.perturb_vertices(true, 0.02, seed=4, radial=True)
    tr = []
    for k, (ang, sc, dx) in enumerate(((0.3, 0.55, -0.6), (-0.7, 0.4, 0.6))):
        m = rot_y(ang) @ np.diag([sc, sc * 1.3, sc, 1.0]).astype(np.float32)
        m[0, 3] = dx
        m[1, 3] = 0.1 * k
        tr.append(m.astype(np.float32))
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true, tr)
    isc.add_mesh(init, tr)
    return ts, isc


def split(vec, layout):
    nv, ninst, p, c, t, tr = (int(x) for x in layout[0][:6])
    return np.concatenate([vec[p:p + 3 * nv], vec[tr:tr + 12 * ninst]]), vec[c:c + 3 * nv]


@pytest.mark.parametrize("exact", [0, 1])
def test_edge_jacobian_vs_oracle_instanced(exact):
    ts, isc = instanced_problem()
    cams = tilted_ring(2, 3.0, 1.2, 64)
    mode, spp = 16, 4
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), spp))
    r.set_option(N.OPT_EDGE_JACOBIAN, exact)
    r.commit(ts)
    tgt = r.render(ts, cams).reshape(-1)
    assert np.array_equal(tgt, O.render(ts, cams, mode, spp))
    r.commit(isc)
    ds = D.DScene(r, [0])
    loss = r.d_render_and_compare(isc, cams, tgt, 64 * 64, ds)
    oloss, ods, _ = O.d_render_and_compare(isc, cams, mode, spp, tgt, 64 * 64,
                                           mp=O.model_params(edge_jacobian=exact))
    assert loss == pytest.approx(oloss, rel=1e-6)
    gp, gc = split(ds.data, ds.layout)
    rp, rc = split(ods, ds.layout)
    assert np.abs(rp).max() > 0
    assert rel_l2(gp, rp) <= EDGE_TOL, rel_l2(gp, rp)
    assert rel_l2(gc, rc) <= INTERIOR_TOL, rel_l2(gc, rc)


def test_edge_jacobian_modes_differ_only_off_axis():
    """For a camera on the z axis looking down it, with identity transforms,
    dx/dY and dy/dX are zero (the view is a translation), so both forms give
    the same gradient; a tilted camera off the axis makes them differ."""
    true = D.make_icosphere(2, seed=3)
    init = D.perturb_vertices(true, 0.02, seed=4, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    grads = []
    for cams in ([D.CamInfo(origin=(0, 0, 3), width=64, height=64)], tilted_ring(1, 3.0, 1.5, 64)):
        g = []
        for exact in (0, 1):
            r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.SILHOUETTE, 4))
            r.set_option(N.OPT_EDGE_JACOBIAN, exact)
            r.set_option(N.OPT_DETERMINISTIC, 1)
            r.commit(ts)
            tgt = r.render(ts, cams)
            r.commit(isc)
            ds = D.DScene(r, [0])
            r.d_render_and_compare(isc, cams, tgt, 64 * 64, ds)
            g.append(ds.get_dmeshes()[0].pos().reshape(-1).copy())
        grads.append(rel_l2(g[1], g[0]))
    on_axis, off_axis = grads
    assert on_axis <= 1e-6, grads
    assert off_axis > 0.05, grads


def directional_fd(r, sc, cams, tgt, direction, h):
    vals = []
    for sgn in (1.0, -1.0):
        s = sc.copy()
        s.meshes[0].vertices = (s.meshes[0].vertices.reshape(-1) + sgn * h * direction).astype(
            np.float32).reshape(s.meshes[0].vertices.shape)
        r.commit(s)
        ds = D.DScene(r, [0])
        vals.append(r.d_render_and_compare(s, cams, tgt, 0, ds))
    n_pix = sum(c.width * c.height for c in cams)
    # the returned loss is the MSE / (views*W*H); the gradient belongs to the
    # sum of squared errors (src/drender.h:184-190)
    return (vals[0] - vals[1]) / (2 * h) * n_pix


def test_full_jacobian_matches_central_differences_on_ring_cameras():
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
    for exact in (0, 1):
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
        r.set_option(N.OPT_EDGE_JACOBIAN, exact)
        r.commit(isc)
        ds = D.DScene(r, [0])
        # 16 edge samples per pixel: sampling noise well below the gap between the forms
        r.d_render_and_compare(isc, cams, tgt, 16 * res * res, ds)
        grads[exact] = ds.get_dmeshes()[0].pos().reshape(-1).astype(np.float64)
    rng = np.random.default_rng(11)
    fd_r = D.MakeDifferentialRenderer(D.DiffRenderSettings(mode, spp))
    nv = isc.meshes[0].vertex_count
    err = {0: [], 1: []}
    fds = []
    for _ in range(12):
        # per vertex, a random displacement (all three axes move)
        d = rng.normal(size=3 * nv)
        d /= np.linalg.norm(d)
        fd = directional_fd(fd_r, isc, cams, tgt, d, 5e-2)
        fds.append(fd)
        for exact in (0, 1):
            err[exact].append(float(np.dot(grads[exact], d)) - fd)
    fds = np.array(fds)
    e0 = float(np.linalg.norm(err[0]) / np.linalg.norm(fds))
    e1 = float(np.linalg.norm(err[1]) / np.linalg.norm(fds))
    print(f"directional derivatives vs central differences: reference form {e0:.4f}, full Jacobian {e1:.4f}")
    # deterministic inputs (seeded mesh, directions and replayed edge
    # samples): measured 0.127 (reference form) and 0.065 (full Jacobian)
    assert e1 < 0.08, (e0, e1)
    assert e1 < 0.6 * e0, (e0, e1)
