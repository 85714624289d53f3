"""Python mirror of the reference's renderer and optimiser interfaces.

Names, argument meaning and accumulation semantics follow the reference:

* ``SHADING_MODEL`` and ``DiffRenderSettings`` -- src/dmesh.h:16-23,
  src/virtual_drender.h:8-12;
* ``MakeDifferentialRenderer`` / ``IDiffRender`` (``init``, ``commit``,
  ``render``, ``d_render``, ``d_render_and_compare``) --
  src/drender.cpp:89-147, src/virtual_drender.h:14-26;
* ``DScene`` / ``DMesh`` gradient containers -- src/dmesh.h:29-243;
* ``OptimizerParameters``, ``CreateSimpleOptimizer`` / ``IOptimizer``
  (``Init``, ``Run``) -- src/optimizer.h:9-61.

Every call runs on the GPU through libdrgb.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import native as N
from .scene import CamInfo, Scene, TransformR


class SHADING_MODEL(enum.IntEnum):
    UNDEFINED = 0
    SILHOUETTE = 1
    VERTEX_COLOR = 2
    TEXTURE_COLOR = 3
    LAMBERT = 4
    PHONG = 5
    GGX = 6
    PATH_TEST = 7              # path tracer of shade_path_test.cpp, counter-based random numbers
    LAMBERT_POINT_VCOLOR = 16  # point light + per-vertex albedo (no reference counterpart)
    PATH_DIFFUSE = 17          # fixed-depth diffuse path tracer (no reference counterpart)


@dataclass
class DiffRenderSettings:
    mode: SHADING_MODEL = SHADING_MODEL.SILHOUETTE
    spp: int = 1


@dataclass
class ModelParams:
    """Constants of the models without a reference counterpart."""
    light_pos: tuple = (3.0, 3.0, 3.0)
    light_intensity: float = 10.0
    ambient: float = 0.1
    path_depth: int = 2
    seed: int = 1


def _ptr(a):
    return None if a is None else a.ctypes.data


class _SceneHandle:
    """SceneDesc pointing at the numpy arrays of a Scene (kept alive here)."""

    def __init__(self, scene: Scene):
        self.keep = []
        n = len(scene.meshes)
        self.meshes = (N.MeshDesc * max(1, n))()
        for i, m in enumerate(scene.meshes):
            tr = scene.transforms_colmajor(i)
            rp = scene.restricted_params(i)
            self.keep += [tr, rp]
            tex = m.textures[0] if m.textures else None
            self.meshes[i] = N.MeshDesc(m.vertex_count, m.indices.size, _ptr(m.vertices), _ptr(m.colors), _ptr(m.tc),
                                        _ptr(m.normals), _ptr(m.tangents), _ptr(m.indices), len(scene.transforms[i]),
                                        _ptr(tr), tex.w if tex else 0, tex.h if tex else 0,
                                        tex.channels if tex else 0, _ptr(tex.data) if tex else None, _ptr(rp))
        self.desc = N.SceneDesc(n, C.cast(self.meshes, C.POINTER(N.MeshDesc)))


def _read_scene(template: Scene, get_mesh, get_restricted) -> Scene:
    """A copy of template with the optimised parameters read back through
    get_mesh(i, vertices, colors, texture, transforms) and, for restricted
    meshes, get_restricted(i, params)."""
    s = template.copy()
    for i, m in enumerate(s.meshes):
        v = np.zeros_like(m.vertices)
        col = np.zeros_like(m.colors) if m.colors is not None else None
        tex = np.zeros_like(m.textures[0].data) if m.textures else None
        tr = np.zeros(16 * len(s.transforms[i]), np.float32)
        N.check(get_mesh(i, _ptr(v), _ptr(col), _ptr(tex), _ptr(tr)))
        m.vertices = v
        if col is not None:
            m.colors = col
        if tex is not None:
            m.textures[0].data = tex
        s.transforms[i] = [t.T.copy() for t in tr.reshape(-1, 4, 4)]
        if s.restricted[i] is not None:
            p = np.zeros(7 * len(s.restricted[i]), np.float32)
            N.check(get_restricted(i, _ptr(p)))
            s.restricted[i] = [TransformR.from_params(q) for q in p.reshape(-1, 7)]
    return s


_CAMERA_CACHE = {}  # camera parameters -> drgb_camera (the library's matrices)


def _camera_key(cam: CamInfo, exact: bool = False):
    """The parameters of a camera as a dictionary key: as given when they are
    hashable (tuples of numbers), else converted to floats and bytes.  Equal
    keys give equal cameras; one camera may have two keys."""
    if cam.world_view is not None:
        return (np.asarray(cam.world_view, np.float32).tobytes(), np.asarray(cam.proj, np.float32).tobytes(),
                float(cam.width), float(cam.height))
    if not exact:
        return (cam.origin, cam.target, cam.up, cam.width, cam.height, cam.fov_rad, cam.znear, cam.zfar)
    return (tuple(float(x) for x in cam.origin), tuple(float(x) for x in cam.target), tuple(float(x) for x in cam.up),
            float(cam.width), float(cam.height), float(cam.fov_rad), float(cam.znear), float(cam.zfar))


def _cached_camera(cam: CamInfo):
    key = _camera_key(cam)
    try:
        return key, _CAMERA_CACHE.get(key)
    except TypeError:  # arrays or lists among the parameters
        key = _camera_key(cam, exact=True)
        return key, _CAMERA_CACHE.get(key)


def make_camera(cam: CamInfo) -> N.Camera:
    """drgb_camera of a CamInfo (matrices computed by the library; a camera
    seen before is taken from a cache keyed by its parameters)."""
    key, hit = _cached_camera(cam)
    if hit is not None:
        return N.Camera.from_buffer_copy(hit)
    c = _make_camera(cam)
    if len(_CAMERA_CACHE) >= 4096:
        _CAMERA_CACHE.clear()
    _CAMERA_CACHE[key] = N.Camera.from_buffer_copy(c)
    return c


def _make_camera(cam: CamInfo) -> N.Camera:
    c = N.Camera()
    if cam.world_view is not None:
        c.world_view[:] = [float(x) for x in np.asarray(cam.world_view, np.float32).reshape(16)]
        c.proj[:] = [float(x) for x in np.asarray(cam.proj, np.float32).reshape(16)]
        c.width, c.height = float(cam.width), float(cam.height)
        return c
    o = np.asarray(cam.origin, np.float32)
    t = np.asarray(cam.target, np.float32)
    u = np.asarray(cam.up, np.float32)
    N.check(N.load().drgb_camera_look_at(_ptr(o), _ptr(t), _ptr(u), float(cam.width), float(cam.height),
                                         float(cam.fov_rad), float(cam.znear), float(cam.zfar), C.byref(c)))
    return c


def make_cameras(cams: Sequence[CamInfo]):
    arr = (N.Camera * len(cams))()
    for i, c in enumerate(cams):
        hit = _cached_camera(c)[1]
        arr[i] = hit if hit is not None else make_camera(c)
    return arr


class DMesh:
    """View of one differentiable mesh's block of the gradient (dmesh.h:29-154)."""
    TRANSFORM_SIZE = 12

    def __init__(self, data: np.ndarray, layout: np.ndarray):
        self.data = data
        self.vertices, self.instances = int(layout[0]), int(layout[1])
        self._pos, self._col, self._tex, self._tr = (int(layout[2]), int(layout[3]), int(layout[4]), int(layout[5]))
        self._rt = int(layout[6])
        self.mesh_id = int(layout[8])

    def pos(self):
        return self.data[self._pos:self._pos + 3 * self.vertices].reshape(-1, 3)

    def color(self):
        return None if self._col < 0 else self.data[self._col:self._col + 3 * self.vertices].reshape(-1, 3)

    def tex(self):
        if self._tex < 0:
            return None
        return self.data[self._tex:self._tr if self._tr >= 0 else self._rt]

    def transform_mat(self):
        if self._tr < 0:
            return None
        return self.data[self._tr:self._tr + 12 * self.instances].reshape(-1, 12)

    def restricted_transform(self):
        """7 values per instance of a restricted mesh (dmesh.h:132), else None."""
        if self._rt < 0:
            return None
        return self.data[self._rt:self._rt + 7 * self.instances].reshape(-1, 7)

    def full_data(self):
        return self.data


class DScene:
    """Gradient of a scene w.r.t. its differentiable meshes (dmesh.h:155-243).

    ``data`` is the concatenation of the DMesh blocks in ``dmesh_ids`` order.
    """

    def __init__(self, renderer: "IDiffRender", dmesh_ids: Sequence[int]):
        self.dmesh_ids = [int(i) for i in dmesh_ids]
        ids = np.asarray(self.dmesh_ids, np.int32)
        lay = np.zeros(9 * len(ids), np.int32)
        tot = C.c_int64(0)
        N.check(N.load().drgb_dscene_layout(renderer._h, _ptr(ids), len(ids), _ptr(lay), C.byref(tot)))
        self.layout = lay.reshape(-1, 9)
        self.data = np.zeros(int(tot.value), np.float32)

    def clear(self):
        self.data[:] = 0.0

    def get_dmeshes(self) -> List[DMesh]:
        out, off = [], 0
        for row in self.layout:
            full = int(row[7])
            out.append(DMesh(self.data[off:off + full], row))
            off += full
        return out

    def get_dmesh(self, mesh_id: int) -> Optional[DMesh]:
        for d in self.get_dmeshes():
            if d.mesh_id == mesh_id:
                return d
        return None

    def full_size(self) -> int:
        return int(self.data.size)


class IDiffRender:
    """GPU implementation of IDiffRender (src/virtual_drender.h:14-26)."""

    def __init__(self):
        self._h = C.c_void_p()
        self.mode = SHADING_MODEL.UNDEFINED
        self.spp = 1
        self._scene_keep = None
        self._committed = None

    def init(self, settings: DiffRenderSettings, device: int = 0):
        lib = N.load()
        N.check(lib.drgb_renderer_create(int(settings.mode), int(settings.spp), int(device), C.byref(self._h)))
        self.mode = SHADING_MODEL(settings.mode)
        self.spp = int(settings.spp)

    def __del__(self):
        try:
            if self._h:
                N.load().drgb_renderer_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    # -- configuration -----------------------------------------------------
    def set_option(self, option: int, value: int):
        N.check(N.load().drgb_renderer_set_option(self._h, option, int(value)))

    def set_model_params(self, p: ModelParams):
        mp = N.ModelParams()
        mp.light_pos[:] = [float(x) for x in p.light_pos]
        mp.light_intensity, mp.ambient, mp.path_depth, mp.seed = p.light_intensity, p.ambient, p.path_depth, p.seed
        N.check(N.load().drgb_renderer_set_model_params(self._h, C.byref(mp)))

    def stream(self) -> int:
        return N.load().drgb_renderer_stream(self._h) or 0

    # -- IDiffRender -------------------------------------------------------
    def commit(self, scene: Scene):
        h = _SceneHandle(scene)
        N.check(N.load().drgb_commit(self._h, C.byref(h.desc)))
        self._committed = scene

    def _check_scene(self, scene):
        if scene is not None and scene is not self._committed:
            raise N.DrgbError(-4, "renderer was not prepared for this scene (commit it first)")

    def render(self, scene: Scene, cams: Sequence[CamInfo], images: Optional[np.ndarray] = None) -> np.ndarray:
        self._check_scene(scene)
        cams = list(cams)
        same = all(c.width == cams[0].width and c.height == cams[0].height for c in cams)
        total = sum(3 * int(c.width) * int(c.height) for c in cams)
        out = np.zeros(total, np.float32)
        ca = make_cameras(cams)
        N.check(N.load().drgb_render(self._h, ca, len(cams), _ptr(out)))
        if same:
            out = out.reshape(len(cams), int(cams[0].height), int(cams[0].width), 3)
        if images is not None:
            images[...] = out.reshape(images.shape)
            return images
        return out

    def d_render(self, scene: Scene, cams: Sequence[CamInfo], adjoints: np.ndarray, edge_samples_in_total: int,
                 d_scene: DScene):
        self._check_scene(scene)
        cams = list(cams)
        adj = np.ascontiguousarray(np.asarray(adjoints, np.float32).reshape(-1))
        ids = np.asarray(d_scene.dmesh_ids, np.int32)
        N.check(N.load().drgb_d_render(self._h, make_cameras(cams), _ptr(adj), len(cams), int(edge_samples_in_total),
                                       _ptr(ids), len(ids), _ptr(d_scene.data)))

    def d_render_and_compare(self, scene: Scene, cams: Sequence[CamInfo], target_images: np.ndarray,
                             edge_samples_in_total: int, d_scene: DScene, out_images: Optional[np.ndarray] = None):
        self._check_scene(scene)
        cams = list(cams)
        tg = np.ascontiguousarray(np.asarray(target_images, np.float32).reshape(-1))
        ids = np.asarray(d_scene.dmesh_ids, np.int32)
        loss = C.c_float(0)
        oi = None
        if out_images is not None:
            oi = np.zeros(tg.size, np.float32)
        N.check(N.load().drgb_d_render_and_compare(self._h, make_cameras(cams), _ptr(tg), len(cams),
                                                   int(edge_samples_in_total), _ptr(ids), len(ids),
                                                   _ptr(d_scene.data), _ptr(oi), C.byref(loss)))
        if out_images is not None:
            out_images[...] = oi.reshape(out_images.shape)
        return float(loss.value)

    def cast_rays(self, cam: CamInfo, xy: np.ndarray):
        """Per-sample SurfaceInfo of CastSingleRay at pixel positions xy."""
        xy = np.ascontiguousarray(np.asarray(xy, np.float32).reshape(-1, 2))
        n = xy.shape[0]
        out = {k: np.zeros(n, np.uint32) for k in ("prim", "inst", "geom")}
        out.update({k: np.zeros(n, np.float32) for k in ("t", "u", "v")})
        c = make_camera(cam)
        N.check(N.load().drgb_cast_rays(self._h, C.byref(c), _ptr(xy), n, _ptr(out["prim"]), _ptr(out["inst"]),
                                        _ptr(out["geom"]), _ptr(out["t"]), _ptr(out["u"]), _ptr(out["v"])))
        return out


def MakeDifferentialRenderer(settings: DiffRenderSettings, device: int = 0) -> IDiffRender:
    """MakeDifferentialRenderer (src/drender.cpp:89-147)."""
    r = IDiffRender()
    r.init(settings, device)
    return r


class OptimizerParameters:
    """OptimizerParameters (src/optimizer.h:9-50)."""
    GD_Naive, GD_AdaGrad, GD_RMSProp, GD_Adam = 1, 2, 3, 4
    _OPT_POS, _OPT_TFM, _OPT_COL, _OPT_TEX = 1, 2, 4, 8
    OPT_POS = _OPT_POS | _OPT_TFM
    OPT_TEX = _OPT_COL | _OPT_TEX
    OPT_ALL = OPT_POS | OPT_TEX

    def __init__(self, alg=GD_Naive, pos_lr=None, tex_lr=None, transforms_lr=0.1, diff_mesh_ids=(0,), verbose=False):
        self.alg = alg
        self.decayPeriod = 25
        self.decay_mult = 0.75
        self.base_lr = 0.1
        self.position_lr = 0.1
        self.textures_lr = 0.1
        self.transforms_lr = 0.1
        self.flags = self.OPT_ALL
        self.differentiable_mesh_ids = list(diff_mesh_ids)
        self.verbose = verbose
        if alg == self.GD_Adam:  # set_default (optimizer_simple.cpp:13-23)
            self.decayPeriod = 100
        if pos_lr is not None:
            self.position_lr = pos_lr
        if tex_lr is not None:
            self.textures_lr = tex_lr
        self.transforms_lr = transforms_lr

    def native(self) -> N.OptParams:
        p = N.OptParams()
        p.alg, p.decay_period, p.decay_mult = self.alg, self.decayPeriod, self.decay_mult
        p.base_lr, p.position_lr, p.textures_lr, p.transforms_lr = (self.base_lr, self.position_lr, self.textures_lr,
                                                                    self.transforms_lr)
        p.flags = self.flags
        p.n_dmesh_ids = len(self.differentiable_mesh_ids)
        for i, x in enumerate(self.differentiable_mesh_ids):
            p.dmesh_ids[i] = x
        return p


class IOptimizer:
    """OptSimple (src/optimizer_simple.cpp:25-309), run entirely on the GPU."""

    def __init__(self):
        self._r: Optional[IDiffRender] = None
        self._scene: Optional[Scene] = None
        self.losses: List[float] = []

    def Init(self, scene: Scene, renderer: IDiffRender, cams: Sequence[CamInfo], targets: np.ndarray,
             params: OptimizerParameters):
        self._r = renderer
        self._scene = scene.copy()
        self._cams = list(cams)
        h = _SceneHandle(self._scene)
        tg = np.ascontiguousarray(np.asarray(targets, np.float32).reshape(-1))
        p = params.native()
        N.check(N.load().drgb_optimizer_init(renderer._h, C.byref(h.desc), make_cameras(self._cams), _ptr(tg),
                                             len(self._cams), C.byref(p)))
        renderer._committed = self._scene

    def Run(self, num_iters: int):
        """Returns (scene, final_error); the per-iteration losses are kept in .losses."""
        losses = np.zeros(max(1, num_iters), np.float32)
        fe = C.c_float(0)
        N.check(N.load().drgb_optimizer_run(self._r._h, int(num_iters), C.byref(fe), _ptr(losses)))
        self.losses.extend(float(x) for x in losses[:num_iters])
        return self.current_scene(), float(fe.value)

    def run_async(self, num_iters: int):
        N.check(N.load().drgb_optimizer_run_async(self._r._h, int(num_iters)))

    def profile(self, num_iters: int = 3):
        """Mean CUDA-event ms per phase: pixels, edges, optimiser, refit, total."""
        out = np.zeros(5, np.float32)
        N.check(N.load().drgb_optimizer_profile(self._r._h, int(num_iters), _ptr(out)))
        return {k: float(v) for k, v in zip(("pixels", "edges", "optimizer", "refit", "total"), out)}

    def autotune(self, trial_iters: int = 3) -> dict:
        """Picks the work-item shape and the persistent grid sizes by timing
        the gradient passes of the optimiser's views (the state is unchanged)."""
        out = np.zeros(5, np.int32)
        ms = C.c_float(0.0)
        N.check(N.load().drgb_optimizer_autotune(self._r._h, int(trial_iters), _ptr(out), C.byref(ms)))
        return {"tile": (int(out[0]), int(out[1])), "pixel_blocks_per_sm": int(out[2]),
                "edge_blocks_per_sm": int(out[3]), "raster": bool(out[4]), "ms": float(ms.value)}

    def count_work(self):
        """Rays, box tests, triangle tests, shaded edge samples and footprint
        tests of the tile and cell lists of one iteration."""
        out = np.zeros(5, np.uint64)
        N.check(N.load().drgb_count_work(self._r._h, _ptr(out)))
        return {k: int(v) for k, v in zip(("rays", "box_tests", "tri_tests", "edge_samples", "footprint_tests"), out)}

    def current_scene(self) -> Scene:
        L, h = N.load(), self._r._h
        return _read_scene(self._scene, lambda i, *a: L.drgb_optimizer_get_mesh(h, i, *a),
                           lambda i, p: L.drgb_optimizer_get_restricted(h, i, p))


def CreateSimpleOptimizer() -> IOptimizer:
    return IOptimizer()


def _model_params_native(p: Optional[ModelParams]):
    if p is None:
        return None
    mp = N.ModelParams()
    mp.light_pos[:] = [float(x) for x in p.light_pos]
    mp.light_intensity, mp.ambient, mp.path_depth, mp.seed = p.light_intensity, p.ambient, p.path_depth, p.seed
    return mp


class BatchOptimizer:
    """Many independent optimisation jobs advanced by one fused launch
    sequence per iteration (drgb_batch_*).  Each job is the equivalent of
    IOptimizer.Init + Run on its own renderer."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        N.check(N.load().drgb_batch_create(int(device), C.byref(self._h)))
        self._scenes = {}

    def __del__(self):
        try:
            if self._h:
                N.load().drgb_batch_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    def add_job(self, scene: Scene, cams: Sequence[CamInfo], targets: np.ndarray, settings: DiffRenderSettings,
                params: OptimizerParameters, model_params: Optional[ModelParams] = None) -> int:
        h = _SceneHandle(scene)
        tg = np.ascontiguousarray(np.asarray(targets, np.float32).reshape(-1))
        p = params.native()
        mp = _model_params_native(model_params)
        jid = C.c_int32(0)
        N.check(N.load().drgb_batch_add_job(self._h, int(settings.mode), int(settings.spp),
                                            C.byref(mp) if mp is not None else None, C.byref(h.desc),
                                            make_cameras(list(cams)), _ptr(tg), len(cams), C.byref(p),
                                            C.byref(jid)))
        self._scenes[int(jid.value)] = scene.copy()
        return int(jid.value)

    def remove_job(self, job_id: int):
        N.check(N.load().drgb_batch_remove_job(self._h, int(job_id)))
        self._scenes.pop(job_id, None)

    def size(self) -> int:
        return int(N.load().drgb_batch_size(self._h))

    def set_option(self, option: int, value: int):
        N.check(N.load().drgb_batch_set_option(self._h, option, int(value)))

    def run(self, num_iters: int):
        N.check(N.load().drgb_batch_run(self._h, int(num_iters)))

    def run_async(self, num_iters: int):
        N.check(N.load().drgb_batch_run_async(self._h, int(num_iters)))

    def sync(self):
        N.check(N.load().drgb_batch_sync(self._h))

    def stream(self) -> int:
        return N.load().drgb_batch_stream(self._h) or 0

    def losses(self, job_id: int) -> np.ndarray:
        done = C.c_int64(0)
        N.check(N.load().drgb_batch_job_losses(self._h, int(job_id), 0, 0, None, C.byref(done)))
        out = np.zeros(max(1, done.value), np.float32)
        N.check(N.load().drgb_batch_job_losses(self._h, int(job_id), 0, done.value, _ptr(out), C.byref(done)))
        return out[:done.value]

    def autotune(self, trial_iters: int = 3) -> dict:
        """Picks the grid sizes of the batch's shared launches by timing its
        gradient passes (the jobs' state is unchanged)."""
        out = np.zeros(2, np.int32)
        ms = C.c_float(0.0)
        N.check(N.load().drgb_batch_autotune(self._h, int(trial_iters), _ptr(out), C.byref(ms)))
        return {"pixel_blocks_per_sm": int(out[0]), "edge_blocks_per_sm": int(out[1]), "ms": float(ms.value)}

    def device_bytes(self, job_id: int) -> int:
        return int(N.load().drgb_batch_job_device_bytes(self._h, int(job_id)))

    def job_scene(self, job_id: int) -> Scene:
        L, h, j = N.load(), self._h, int(job_id)
        return _read_scene(self._scenes[job_id], lambda i, *a: L.drgb_batch_get_mesh(h, j, i, *a),
                           lambda i, p: L.drgb_batch_get_restricted(h, j, i, p))


JOB_STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}


class OptimizationServer:
    """Serving loop over the batched engine (drgb_server_*): jobs are
    submitted at any time, admitted in arrival order by a device-memory budget
    and a slot count, and advanced together one iteration per batched step
    (continuous batching).  With worker=True a native worker thread steps the
    batch; otherwise call step()."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 150 * 10**9, max_jobs: int = 0,
                 worker: bool = True, deterministic: bool = False):
        cfg = N.ServerConfig(int(device), int(max_jobs), int(hbm_budget_bytes), 1 if worker else 0,
                             1 if deterministic else 0)
        self._h = C.c_void_p()
        N.check(N.load().drgb_server_create(C.byref(cfg), C.byref(self._h)))
        self._scenes = {}

    def close(self):
        if self._h:
            N.load().drgb_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scene: Scene, cams: Sequence[CamInfo], targets: np.ndarray, settings: DiffRenderSettings,
               params: OptimizerParameters, steps: int, model_params: Optional[ModelParams] = None) -> int:
        h = _SceneHandle(scene)
        tg = np.ascontiguousarray(np.asarray(targets, np.float32).reshape(-1))
        p = params.native()
        mp = _model_params_native(model_params)
        t = C.c_int32(0)
        N.check(N.load().drgb_server_submit(self._h, int(settings.mode), int(settings.spp),
                                            C.byref(mp) if mp is not None else None, C.byref(h.desc),
                                            make_cameras(list(cams)), _ptr(tg), len(cams), C.byref(p), int(steps),
                                            C.byref(t)))
        self._scenes[int(t.value)] = scene.copy()
        return int(t.value)

    def step(self) -> int:
        n = C.c_int32(0)
        N.check(N.load().drgb_server_step(self._h, C.byref(n)))
        return int(n.value)

    def wait(self, ticket: int = 0, timeout: float = -1.0):
        """Until the job (or, with ticket 0, every submitted job) is finished."""
        N.check(N.load().drgb_server_wait(self._h, int(ticket), float(timeout)))

    def info(self, ticket: int) -> dict:
        i = N.JobInfo()
        N.check(N.load().drgb_server_job_info(self._h, int(ticket), C.byref(i)))
        return {"state": JOB_STATES.get(i.state, str(i.state)), "error": i.error, "steps": i.steps,
                "steps_done": i.steps_done, "t_submit": i.t_submit, "t_admit": i.t_admit, "t_done": i.t_done,
                "device_bytes": i.device_bytes, "final_loss": i.final_loss}

    def losses(self, ticket: int) -> np.ndarray:
        n = self.info(ticket)["steps_done"]
        out = np.zeros(max(1, n), np.float32)
        N.check(N.load().drgb_server_job_losses(self._h, int(ticket), 0, n, _ptr(out)))
        return out[:n]

    def result_scene(self, ticket: int) -> Scene:
        L, h, t = N.load(), self._h, int(ticket)
        return _read_scene(self._scenes[ticket], lambda i, *a: L.drgb_server_get_mesh(h, t, i, *a),
                           lambda i, p: L.drgb_server_get_restricted(h, t, i, p))

    def release(self, ticket: int):
        N.check(N.load().drgb_server_release(self._h, int(ticket)))
        self._scenes.pop(ticket, None)

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.load().drgb_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in N.ServerStats._fields_}

    def step_times(self):
        """(device ms, resident jobs) of every batched step so far."""
        n = self.stats()["batch_steps"]
        ms = np.zeros(max(1, n), np.float32)
        jobs = np.zeros(max(1, n), np.int32)
        N.check(N.load().drgb_server_step_times(self._h, 0, n, _ptr(ms), _ptr(jobs)))
        return ms[:n], jobs[:n]


def estimate_job_bytes(scene: Scene, cams: Sequence[CamInfo], mode: int = 0, spp: int = 16) -> int:
    h = _SceneHandle(scene)
    return int(N.load().drgb_estimate_job_bytes(int(mode), int(spp), C.byref(h.desc), make_cameras(list(cams)),
                                                len(cams)))


def kernel_launches() -> int:
    return int(N.load().drgb_kernel_launches())
