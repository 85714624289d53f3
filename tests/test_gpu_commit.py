"""drgb_commit on the GPU: the reference commits the scene it is given on
every d_render_and_compare (src/drender.h:176), so a commit of a scene of
the same sizes reuses the device buffers of the last one, and a commit whose
arrays are pageable returns without waiting for the device.  These tests
check that the committed scene is the one given: images equal those of a
fresh renderer (bit-exact), whatever the caller does with its arrays after
the call, and a rejected commit leaves the previous scene in place.
"""
import numpy as np
import pytest
import torch

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N

pytestmark = pytest.mark.gpu

MODE = D.SHADING_MODEL.LAMBERT_POINT_VCOLOR


def renderer(bruteforce=False):
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(MODE, 4))
    r.set_option(N.OPT_TRACE_BRUTEFORCE, int(bruteforce))
    return r


def scene_of(mesh):
    s = D.Scene()
    s.add_mesh(mesh)
    return s


def fresh_image(scene, cams, bruteforce=False):
    r = renderer(bruteforce)
    r.commit(scene)
    return r.render(scene, cams)


def pinned_copy(a):
    """a numpy view of page-locked memory holding a copy of a"""
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
    out = t.numpy()
    out[...] = a
    return out, t


def test_commits_of_same_sized_scenes_render_each_scene():
    # the reference's triangle loop: the images do not depend on a hierarchy
    # built for an earlier scene of the same triangles
    cams = D.ring_cameras(2, 3.0, 96, 96)
    a = D.make_icosphere(3, seed=1)
    b = D.perturb_vertices(a, 0.05, seed=7, radial=True)
    b.colors = np.ascontiguousarray(b.colors[::-1])
    sa, sb = scene_of(a), scene_of(b)
    want_a, want_b = fresh_image(sa, cams, True), fresh_image(sb, cams, True)
    assert np.abs(want_a - want_b).max() > 0
    r = renderer(True)
    for s, want in ((sa, want_a), (sb, want_b), (sa, want_a), (sb, want_b)):
        r.commit(s)
        np.testing.assert_array_equal(r.render(s, cams), want)


@pytest.mark.parametrize("pinned", [False, True])
def test_arrays_changed_after_commit_do_not_reach_the_scene(pinned):
    cams = D.ring_cameras(2, 3.0, 96, 96)
    mesh = D.make_icosphere(3, seed=2)
    keep = []
    if pinned:  # page-locked arrays: the commit waits for its copies
        mesh.vertices, t1 = pinned_copy(mesh.vertices)
        mesh.colors, t2 = pinned_copy(mesh.colors)
        keep += [t1, t2]
    s = scene_of(mesh)
    want = fresh_image(scene_of(mesh.copy()), cams)
    r = renderer()
    for _ in range(3):
        r.commit(s)
        saved_v, saved_c = mesh.vertices.copy(), mesh.colors.copy()
        mesh.vertices[...] += 0.25  # changed at once: the committed scene keeps the old values
        mesh.colors[...] = 0.0
        got = r.render(s, cams)
        mesh.vertices[...] = saved_v
        mesh.colors[...] = saved_c
        np.testing.assert_array_equal(got, want)


def test_rejected_commit_keeps_the_committed_scene():
    cams = D.ring_cameras(1, 3.0, 96, 96)
    good = scene_of(D.make_icosphere(3, seed=3))
    other = D.make_icosphere(3, seed=4)
    other.indices = other.indices.copy()
    other.indices[-1] = other.vertex_count + 5  # out of range: rejected before anything changes
    bad = D.Scene()
    bad.add_mesh(D.make_icosphere(3, seed=5))  # a valid first mesh, then the bad one
    bad.add_mesh(other)
    r = renderer()
    r.commit(good)
    want = r.render(good, cams)
    with pytest.raises(N.DrgbError) as e:
        r.commit(bad)
    assert "index out of range" in str(e.value)
    np.testing.assert_array_equal(r.render(good, cams), want)
