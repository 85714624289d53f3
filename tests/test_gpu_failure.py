"""Device-side failure path: a traversal that runs out of its step budget.

Every traversal loop is bounded (a stack depth and a number of node visits
per ray).  A ray that reaches the bound stops with the nearest hit found so
far and sets an error flag; the call returns DRGB_ERR_KERNEL with a message
naming the limit, and the renderer stays usable.  The reference has no
status codes: it prints and returns (src/drender.h:103-107).  The limit is
lowered through DRGB_OPT_TRACE_STEP_LIMIT so that ordinary rays reach it;
nothing here faults, traps or hangs the GPU.
"""
import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
import pyoracle as O

pytestmark = pytest.mark.gpu


def scene_and_cams():
    s = D.Scene()
    s.add_mesh(D.make_icosphere(3, seed=1))
    return s, [D.CamInfo(origin=(0.4, 0.3, 3.0), width=48, height=48)]


def test_traversal_step_limit_returns_kernel_error_and_recovers():
    s, cams = scene_and_cams()
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 4))
    # camera samples and point-light shadow rays through the hierarchy (the
    # raster pass and the light-space cells resolve them without traversal)
    r.set_option(N.OPT_PRIMARY_RASTER, 0)
    r.commit(s)
    good = r.render(s, cams).reshape(-1)
    assert np.array_equal(good, O.render(s, cams, 16, 4))
    r.set_option(N.OPT_TRACE_STEP_LIMIT, 2)
    with pytest.raises(N.DrgbError) as e:
        r.render(s, cams)
    assert e.value.code == N.ERR_KERNEL
    assert "traversal step limit" in str(e.value)
    # the gradient path reports it the same way
    ds = D.DScene(r, [0])
    with pytest.raises(N.DrgbError) as e:
        r.d_render_and_compare(s, cams, good, 48 * 48, ds)
    assert e.value.code == N.ERR_KERNEL
    # back to the default bound: the next calls are correct again
    r.set_option(N.OPT_TRACE_STEP_LIMIT, 0)
    assert np.array_equal(r.render(s, cams).reshape(-1), good)
    assert r.d_render_and_compare(s, cams, good, 48 * 48, ds) == 0.0


def test_traversal_step_limit_in_the_optimiser_loop():
    """The optimiser replays its iteration as a CUDA graph; a raised flag
    surfaces from Run, and a later Run with the default bound succeeds."""
    s, cams = scene_and_cams()
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.LAMBERT_POINT_VCOLOR, 4))
    r.set_option(N.OPT_PRIMARY_RASTER, 0)  # every ray through the hierarchy
    r.commit(s)
    tgt = r.render(s, cams)
    init = D.Scene()
    init.add_mesh(D.perturb_vertices(s.meshes[0], 0.02, seed=2, radial=True))
    opt = D.CreateSimpleOptimizer()
    opt.Init(init, r, cams, tgt, D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.01))
    opt.Run(2)
    r.set_option(N.OPT_TRACE_STEP_LIMIT, 3)
    with pytest.raises(N.DrgbError) as e:
        opt.Run(1)
    assert e.value.code == N.ERR_KERNEL
    r.set_option(N.OPT_TRACE_STEP_LIMIT, 0)
    opt.Run(2)
    assert np.isfinite(opt.losses).all()


def test_trace_step_limit_option_is_validated():
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 1))
    with pytest.raises(N.DrgbError):
        r.set_option(N.OPT_TRACE_STEP_LIMIT, -1)
    with pytest.raises(N.DrgbError):
        r.set_option(N.OPT_TRACE_STEP_LIMIT, (1 << 24) + 1)
