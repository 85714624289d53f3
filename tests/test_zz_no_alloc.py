"""drgb_d_render_and_compare_noalloc against drgb_d_render_and_compare_device.

The no-allocation entry point serves callers that cannot allocate GPU memory
while they run (programs that take all device memory from their own pool or
budget, loops that must not pay for an allocation mid-run).  It must produce
the same loss and gradient as the allocating device-pointer entry point,
call after call, and allocate nothing.  Both entry points shade the same
edge list with the same replayed random numbers and the same samples; only
the order of the float atomics differs, so the results agree to float
rounding.  The first call on a device may load the library's fixed array
onto it (the runtime does that when its address is looked up), so the
no-allocation check is made on the second call.  This file is collected last
on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import diffrender_tutorials_gb300 as D
from diffrender_tutorials_gb300 import native as N
from diffrender_tutorials_gb300.api import make_cameras

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2 of each gradient block: the same sums in another atomic order


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_noalloc_matches_device_entry_point():
    torch = pytest.importorskip("torch")
    lib = N.load()
    true = D.make_cube(seed=1)
    init = D.perturb_vertices(true, 0.1, seed=2)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = [D.CamInfo(origin=(0, 0, 3), width=96, height=96), D.CamInfo(origin=(2.0, 1.0, 2.0), width=96, height=96)]
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 16))
    r.commit(ts)
    targets = r.render(ts, cams).reshape(-1)
    r.commit(isc)
    ds = D.DScene(r, [0])
    ids = np.array([0], np.int32)
    ca = make_cameras(cams)
    n_edge = 96 * 96
    dev = torch.device("cuda:0")
    d_t = torch.from_numpy(targets).to(dev)
    ref_g = torch.zeros(ds.data.size, dtype=torch.float32, device=dev)
    ref_l = torch.zeros(1, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    N.check(lib.drgb_d_render_and_compare_device(r._h, ca, C.c_void_p(d_t.data_ptr()), len(cams), n_edge,
                                                 C.c_void_p(ids.ctypes.data), 1, C.c_void_p(ref_g.data_ptr()),
                                                 None, C.c_void_p(ref_l.data_ptr())))
    ref = ref_g.cpu().numpy()
    ref_loss = float(ref_l.item())
    lay = ds.layout[0]
    nv, pos, col, tr = int(lay[0]), int(lay[2]), int(lay[3]), int(lay[5])

    g = torch.full((ds.data.size,), 7.0, dtype=torch.float32, device=dev)  # stale contents must be cleared
    l = torch.zeros(1, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    for call in range(2):
        free_before = torch.cuda.mem_get_info(0)[0]
        N.check(lib.drgb_d_render_and_compare_noalloc(r._h, ca, C.c_void_p(d_t.data_ptr()), len(cams), n_edge,
                                                      C.c_void_p(ids.ctypes.data), 1, C.c_void_p(g.data_ptr()),
                                                      C.c_void_p(l.data_ptr())))
        free_after = torch.cuda.mem_get_info(0)[0]
        if call == 1:
            assert free_after == free_before, "the call allocated device memory"
        got = g.cpu().numpy()
        assert float(l.item()) == pytest.approx(ref_loss, rel=1e-6), call
        edge_got = np.concatenate([got[pos:pos + 3 * nv], got[tr:tr + 12]])
        edge_ref = np.concatenate([ref[pos:pos + 3 * nv], ref[tr:tr + 12]])
        assert np.abs(edge_ref).max() > 0
        assert _rel(edge_got, edge_ref) <= TOL, (call, _rel(edge_got, edge_ref))
        assert _rel(got[col:col + 3 * nv], ref[col:col + 3 * nv]) <= TOL, call


def test_noalloc_rejects_oversized_calls():
    torch = pytest.importorskip("torch")
    lib = N.load()
    s = D.Scene()
    s.add_mesh(D.make_cube(seed=1))
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 4))
    r.commit(s)
    ds = D.DScene(r, [0])
    big = [D.CamInfo(origin=(0, 0, 3), width=2048, height=2048)]
    dev = torch.device("cuda:0")
    d_t = torch.zeros(2048 * 2048 * 3, dtype=torch.float32, device=dev)
    g = torch.zeros(ds.data.size, dtype=torch.float32, device=dev)
    l = torch.zeros(1, dtype=torch.float32, device=dev)
    ids = np.array([0], np.int32)
    torch.cuda.synchronize()
    rc = lib.drgb_d_render_and_compare_noalloc(r._h, make_cameras(big), C.c_void_p(d_t.data_ptr()), 1, 2048 * 2048,
                                               C.c_void_p(ids.ctypes.data), 1, C.c_void_p(g.data_ptr()),
                                               C.c_void_p(l.data_ptr()))
    assert rc == -1
    assert "scratch" in N.last_error()


def test_noalloc_refuses_restricted_transform_meshes():
    """Their Jacobian step needs a scratch block beyond the caller's gradient vector."""
    torch = pytest.importorskip("torch")
    lib = N.load()
    s = D.Scene()
    s.add_mesh(D.make_cube(seed=1), [D.TransformR((0.1, 0.0, 0.0), (0.0, 0.3, 0.0), 1.0)])
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL.VERTEX_COLOR, 4))
    r.commit(s)
    ds = D.DScene(r, [0])
    cams = [D.CamInfo(origin=(0, 0, 3), width=32, height=32)]
    dev = torch.device("cuda:0")
    d_t = torch.zeros(32 * 32 * 3, dtype=torch.float32, device=dev)
    g = torch.zeros(ds.data.size, dtype=torch.float32, device=dev)
    l = torch.zeros(1, dtype=torch.float32, device=dev)
    ids = np.array([0], np.int32)
    torch.cuda.synchronize()
    rc = lib.drgb_d_render_and_compare_noalloc(r._h, make_cameras(cams), C.c_void_p(d_t.data_ptr()), 1, 32 * 32,
                                               C.c_void_p(ids.ctypes.data), 1, C.c_void_p(g.data_ptr()),
                                               C.c_void_p(l.data_ptr()))
    assert rc == -1
    assert "restricted" in N.last_error()
