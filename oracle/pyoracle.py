"""ctypes binding of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs as the checker.  The product path never uses it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

ORC_CAM_FLOATS = 82
SILHOUETTE, VERTEX_COLOR, TEXTURE_COLOR, LAMBERT = 1, 2, 3, 4
PATH_TEST = 7
LAMBERT_POINT_VCOLOR, PATH_DIFFUSE = 16, 17


def build(force=False):
    """Compile oracle.c with gcc (-ffp-contract=off keeps the reference's
    rounding on hosts whose compilers fuse multiply-adds by default;
    -fno-trapping-math only lets gcc turn the caster's compares into vector
    selects, it changes no value)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-std=c11", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                           "-fno-trapping-math", "-fPIC",
                           "-shared", "-Wall", "-Wno-unused-function", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class OrcMesh(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("n_indices", C.c_int32), ("vertices", C.c_void_p),
                ("colors", C.c_void_p), ("tc", C.c_void_p), ("normals", C.c_void_p), ("tangents", C.c_void_p),
                ("indices", C.c_void_p), ("n_instances", C.c_int32), ("transforms", C.c_void_p),
                ("tex_w", C.c_int32), ("tex_h", C.c_int32), ("tex_channels", C.c_int32), ("texture", C.c_void_p),
                ("restricted", C.c_void_p)]


class OrcModelParams(C.Structure):
    _fields_ = [("light_pos", C.c_float * 3), ("light_intensity", C.c_float), ("ambient", C.c_float),
                ("path_depth", C.c_int32), ("seed", C.c_uint32), ("edge_jacobian", C.c_int32),
                ("edge_set", C.c_int32)]


class OrcOptParams(C.Structure):
    _fields_ = [("alg", C.c_int32), ("decay_period", C.c_int32), ("decay_mult", C.c_float),
                ("base_lr", C.c_float), ("position_lr", C.c_float), ("textures_lr", C.c_float),
                ("transforms_lr", C.c_float), ("flags", C.c_int32), ("n_dmesh_ids", C.c_int32),
                ("dmesh_ids", C.c_int32 * 16)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
    return _lib


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _addr(a):
    return None if a is None else a.ctypes.data


class _Scene:
    """Keeps the numpy arrays alive while the C structs point at them."""

    def __init__(self, scene):
        self.keep = []
        self.arr = (OrcMesh * max(1, len(scene.meshes)))()
        for i, m in enumerate(scene.meshes):
            tr = scene.transforms_colmajor(i)
            rp = scene.restricted_params(i)
            self.keep += [tr, rp]
            tex = m.textures[0] if m.textures else None
            self.arr[i] = OrcMesh(m.vertex_count, m.indices.size, _addr(m.vertices), _addr(m.colors), _addr(m.tc),
                                  _addr(m.normals), _addr(m.tangents), _addr(m.indices), len(scene.transforms[i]),
                                  _addr(tr), tex.w if tex else 0, tex.h if tex else 0, tex.channels if tex else 0,
                                  _addr(tex.data) if tex else None, _addr(rp))
        self.n = len(scene.meshes)


def model_params(light_pos=(3.0, 3.0, 3.0), intensity=10.0, ambient=0.1, path_depth=2, seed=1, edge_jacobian=0,
                 edge_set=0):
    p = OrcModelParams()
    p.edge_jacobian = edge_jacobian
    p.edge_set = edge_set
    p.light_pos[:] = light_pos
    p.light_intensity = intensity
    p.ambient = ambient
    p.path_depth = path_depth
    p.seed = seed
    return p


def camera(cam):
    """82-float camera block (matrices computed like CamInfo)."""
    out = np.zeros(ORC_CAM_FLOATS, dtype=np.float32)
    L = lib()
    if cam.world_view is not None:
        wv = np.ascontiguousarray(np.asarray(cam.world_view, dtype=np.float32).reshape(16))
        pr = np.ascontiguousarray(np.asarray(cam.proj, dtype=np.float32).reshape(16))
        L.orc_camera_from_matrices(_ptr(wv), _ptr(pr), C.c_float(cam.width), C.c_float(cam.height), _ptr(out))
    else:
        o = np.asarray(cam.origin, dtype=np.float32)
        t = np.asarray(cam.target, dtype=np.float32)
        u = np.asarray(cam.up, dtype=np.float32)
        L.orc_camera_look_at(_ptr(o), _ptr(t), _ptr(u), C.c_float(cam.width), C.c_float(cam.height),
                             C.c_float(cam.fov_rad), C.c_float(cam.znear), C.c_float(cam.zfar), _ptr(out))
    return out


def cameras(cams):
    return np.ascontiguousarray(np.concatenate([camera(c) for c in cams]).astype(np.float32))


def cast_rays(scene, cam, xy):
    xy = np.ascontiguousarray(np.asarray(xy, dtype=np.float32).reshape(-1, 2))
    n = xy.shape[0]
    sc = _Scene(scene)
    cb = camera(cam)
    out = {k: np.zeros(n, dtype=np.uint32) for k in ("prim", "inst", "geom")}
    out.update({k: np.zeros(n, dtype=np.float32) for k in ("t", "u", "v")})
    out["ray_pos"] = np.zeros((n, 3), dtype=np.float32)
    out["ray_dir"] = np.zeros((n, 3), dtype=np.float32)
    lib().orc_cast_rays(sc.arr, sc.n, _ptr(cb), _ptr(xy), C.c_int64(n), _ptr(out["prim"]), _ptr(out["inst"]),
                        _ptr(out["geom"]), _ptr(out["t"]), _ptr(out["u"]), _ptr(out["v"]), _ptr(out["ray_pos"]),
                        _ptr(out["ray_dir"]))
    return out


def _img_total(cams):
    return sum(3 * int(c.width) * int(c.height) for c in cams)


def render(scene, cams, mode, spp, mp=None):
    sc = _Scene(scene)
    cb = cameras(cams)
    imgs = np.zeros(_img_total(cams), dtype=np.float32)
    mp = mp or model_params()
    lib().orc_render(sc.arr, sc.n, mode, spp, C.byref(mp), _ptr(cb), len(cams), _ptr(imgs))
    return imgs


def dscene_layout(scene, mode, ids):
    sc = _Scene(scene)
    ids = np.asarray(ids, dtype=np.int32)
    lay = np.zeros(9 * len(ids), dtype=np.int32)
    tot = C.c_int64(0)
    r = lib().orc_dscene_layout(sc.arr, sc.n, mode, _ptr(ids), len(ids), _ptr(lay), C.byref(tot))
    if r != 0:
        raise ValueError("bad dmesh ids")
    return lay.reshape(-1, 9), int(tot.value)


def d_render(scene, cams, mode, spp, adjoints, edge_samples, ids=(0,), mp=None):
    sc = _Scene(scene)
    cb = cameras(cams)
    ids = np.asarray(ids, dtype=np.int32)
    _, tot = dscene_layout(scene, mode, ids)
    ds = np.zeros(tot, dtype=np.float32)
    adj = np.ascontiguousarray(np.asarray(adjoints, dtype=np.float32).reshape(-1))
    mp = mp or model_params()
    r = lib().orc_d_render(sc.arr, sc.n, mode, spp, C.byref(mp), _ptr(cb), len(cams), _ptr(adj), edge_samples,
                           _ptr(ids), len(ids), _ptr(ds))
    if r != 0:
        raise RuntimeError("orc_d_render failed")
    return ds


def d_render_and_compare(scene, cams, mode, spp, targets, edge_samples, ids=(0,), mp=None):
    sc = _Scene(scene)
    cb = cameras(cams)
    ids = np.asarray(ids, dtype=np.int32)
    _, tot = dscene_layout(scene, mode, ids)
    ds = np.zeros(tot, dtype=np.float32)
    imgs = np.zeros(_img_total(cams), dtype=np.float32)
    tg = np.ascontiguousarray(np.asarray(targets, dtype=np.float32).reshape(-1))
    loss = C.c_float(0)
    mp = mp or model_params()
    r = lib().orc_d_render_and_compare(sc.arr, sc.n, mode, spp, C.byref(mp), _ptr(cb), len(cams), _ptr(tg),
                                       edge_samples, _ptr(ids), len(ids), _ptr(ds), _ptr(imgs), C.byref(loss))
    if r != 0:
        raise RuntimeError("orc_d_render_and_compare failed")
    return float(loss.value), ds, imgs


def opt_params(alg=4, **kw):
    p = OrcOptParams()
    lib().orc_opt_params_default(alg, C.byref(p))
    ids = kw.pop("dmesh_ids", None)
    for k, v in kw.items():
        setattr(p, k, v)
    if ids is not None:
        p.n_dmesh_ids = len(ids)
        for i, x in enumerate(ids):
            p.dmesh_ids[i] = x
    return p


def optimize(scene, cams, mode, spp, targets, params, iters, mp=None):
    sc = _Scene(scene)
    cb = cameras(cams)
    tg = np.ascontiguousarray(np.asarray(targets, dtype=np.float32).reshape(-1))
    nv = sum(3 * m.vertex_count for m in scene.meshes)
    nc = sum(3 * m.vertex_count for m in scene.meshes if m.colors is not None)
    nt = sum(m.textures[0].data.size for m in scene.meshes if m.textures)
    ntr = sum(16 * len(t) for t in scene.transforms)
    nrt = sum(7 * len(r) for r in scene.restricted if r is not None)
    trt = np.zeros(iters * max(nrt, 1), dtype=np.float32)
    tv = np.zeros(iters * nv, dtype=np.float32)
    tcol = np.zeros(iters * max(nc, 1), dtype=np.float32)
    ttex = np.zeros(iters * max(nt, 1), dtype=np.float32)
    ttr = np.zeros(iters * ntr, dtype=np.float32)
    losses = np.zeros(iters, dtype=np.float32)
    fe = C.c_float(0)
    mp = mp or model_params()
    r = lib().orc_optimize(sc.arr, sc.n, mode, spp, C.byref(mp), _ptr(cb), len(cams), _ptr(tg), C.byref(params),
                           iters, C.byref(fe), _ptr(losses), _ptr(tv), _ptr(tcol) if nc else None,
                           _ptr(ttex) if nt else None, _ptr(ttr), _ptr(trt) if nrt else None)
    if r != 0:
        raise RuntimeError("orc_optimize failed")
    return {"final_error": float(fe.value), "losses": losses, "vertices": tv.reshape(iters, -1),
            "colors": tcol[:iters * nc].reshape(iters, -1) if nc else None,
            "textures": ttex[:iters * nt].reshape(iters, -1) if nt else None,
            "transforms": ttr.reshape(iters, -1),
            "restricted": trt[:iters * nrt].reshape(iters, -1) if nrt else None}


def restricted_to_mat(params):
    """Column-major 4x4 of TransformR parameters (translate xyz, rotate xyz, scale)."""
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(7))
    out = np.zeros(16, dtype=np.float32)
    lib().orc_restricted_to_mat(_ptr(p), _ptr(out))
    return out


def restricted_jacobian(params):
    """jac[7][12]: derivative of the row-major 3x4 of to_mat by each parameter."""
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(7))
    out = np.zeros(84, dtype=np.float32)
    lib().orc_restricted_jacobian(_ptr(p), _ptr(out))
    return out.reshape(7, 12)


def prng(seed, count):
    out = np.zeros(count, dtype=np.float32)
    lib().orc_prng(seed, count, _ptr(out))
    return out


def edge_random_table(n, threads=14):
    out = np.zeros(2 * n, dtype=np.float32)
    lib().orc_edge_random_table(n, threads, _ptr(out))
    return out


def hammersley(n):
    out = np.zeros(2 * n, dtype=np.float32)
    lib().orc_hammersley(n, _ptr(out))
    return out


def set_threads(n):
    lib().orc_set_threads(n)
