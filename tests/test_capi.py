"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/drgb.h, reports errors through return codes, and its
host-side camera math equals the reference's bit for bit."""
import ctypes as C

import numpy as np
import pytest

from diffrender_tutorials_gb300 import native as N
from diffrender_tutorials_gb300.api import make_camera
from fixtures import cams_from, load


@pytest.fixture(scope="module")
def lib():
    return N.load()


def test_exports_every_declared_symbol(lib):
    declared = N.header_functions()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.drgb_abi_version() == 1


def test_camera_look_at_matches_reference(lib):
    d = load("camera")
    for i, cam in enumerate(cams_from(d)):
        c = make_camera(cam)
        assert np.array_equal(np.array(c.world_view[:], np.float32), d[f"out.cam{i}.worldview"])
        assert np.array_equal(np.array(c.proj[:], np.float32), d[f"out.cam{i}.proj"])


def test_null_arguments_are_errors(lib):
    assert lib.drgb_renderer_create(2, 16, 0, None) == -1
    assert "null" in N.last_error()
    assert lib.drgb_commit(None, None) == -1
    assert lib.drgb_render(None, None, 1, None) == -1
    assert lib.drgb_renderer_destroy(None) == -1


def test_bad_model_and_spp_rejected(lib):
    h = C.c_void_p()
    assert lib.drgb_renderer_create(99, 16, 0, C.byref(h)) == -6
    assert lib.drgb_renderer_create(2, 0, 0, C.byref(h)) == -1
    assert lib.drgb_renderer_create(2, 65, 0, C.byref(h)) == -1


def test_opt_params_default(lib):
    p = N.OptParams()
    assert lib.drgb_opt_params_default(4, C.byref(p)) == 0
    assert p.decay_period == 100 and abs(p.decay_mult - 0.75) < 1e-7
    assert abs(p.position_lr - 0.1) < 1e-7 and p.flags == 15
    assert lib.drgb_opt_params_default(1, C.byref(p)) == 0
    assert p.decay_period == 25


def test_camera_cache_is_keyed_by_value(lib):
    """make_camera keeps the library's matrices per camera: a camera built
    from equal parameters (tuples, lists or arrays) gets the same matrices
    as a fresh computation, and a changed camera gets its own."""
    from diffrender_tutorials_gb300 import api
    from diffrender_tutorials_gb300.scene import CamInfo

    def fresh(cam):
        c = api._make_camera(cam)
        return np.array(c.world_view[:] + c.proj[:] + [c.width, c.height], np.float32)

    def cached(cam):
        c = make_camera(cam)
        return np.array(c.world_view[:] + c.proj[:] + [c.width, c.height], np.float32)

    a = CamInfo(origin=(0.5, 1.0, 3.0), width=64, height=48)
    assert np.array_equal(cached(a), fresh(a))
    assert np.array_equal(cached(a), fresh(a))  # second call: from the cache
    for same in (CamInfo(origin=[0.5, 1.0, 3.0], width=64, height=48),
                 CamInfo(origin=np.array([0.5, 1.0, 3.0], np.float32), width=64, height=48)):
        assert np.array_equal(cached(same), fresh(a))
    a.origin = (0.5, 1.25, 3.0)  # a changed camera is not served the old matrices
    assert np.array_equal(cached(a), fresh(a))
    b = CamInfo(origin=(0.5, 1.0, 3.0), width=64, height=48, fov_rad=0.5)
    assert not np.array_equal(cached(b), cached(CamInfo(origin=(0.5, 1.0, 3.0), width=64, height=48)))
    arr = api.make_cameras([a, b, a])
    assert np.array_equal(np.array(arr[0].world_view[:]), np.array(arr[2].world_view[:]))
    assert np.array_equal(np.array(arr[1].proj[:], np.float32), fresh(b)[16:32])
