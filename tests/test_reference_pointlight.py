"""The point-light vertex-albedo model inside the reference's own DiffRender<>
(oracle/ref/ref_pointlight.h, built by oracle/ref/build_ref.py) against the
oracle's restatement of the same model: the reference pipeline (camera rays,
brute-force caster, 14-thread interior and edge passes, loss) then runs the
benchmark workload, and its output pins the oracle for that model.

Runs where the reference sources are available (the reference tree or the
patched copy under oracle/_ref/src)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402
import pyoracle as O  # noqa: E402
import refrun  # noqa: E402

import diffrender_tutorials_gb300 as D  # noqa: E402


def driver():
    exe = build_ref.build()
    if exe is None:
        pytest.skip("reference sources absent")
    return exe


def test_reference_pipeline_with_point_light_matches_oracle():
    exe = driver()
    true = D.make_icosphere(3, seed=4)
    init = D.perturb_vertices(true, 0.02, seed=5, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = D.ring_cameras(2, 3.0, 40, 40)
    base = {"mode": np.array([16], np.int32), "spp": np.array([4], np.int32), **refrun.cam_items(cams)}
    ref_t = refrun.run(exe, {**base, **refrun.scene_items(ts), "task": np.array([2], np.int32)})["images"]
    tgt = O.render(ts, cams, 16, 4)
    assert np.array_equal(ref_t, tgt)
    out = refrun.run(exe, {**base, **refrun.scene_items(isc), "task": np.array([4], np.int32), "targets": tgt,
                           "dmesh_ids": np.array([0], np.int32), "edge_samples": np.array([40 * 40], np.int32)})
    oloss, ods, oimgs = O.d_render_and_compare(isc, cams, 16, 4, tgt, 40 * 40)
    assert np.array_equal(out["images"], oimgs)
    assert float(out["loss"][0]) == pytest.approx(oloss, rel=1e-6)
    g = out["dmesh0"]
    assert g.size == ods.size and np.abs(g).max() > 0
    assert np.array_equal(g, ods)
