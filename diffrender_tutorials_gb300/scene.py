"""Host-side scene description mirroring the reference's data types.

``TriangleMesh`` and ``Scene`` follow common_src/scene.h:40-70 and 121-247
(meshes with per-vertex attributes, an index buffer, optional texture, and a
list of instance transforms); ``CamInfo`` follows common_src/camera.h:6-44.
Arrays are numpy float32/uint32 so they can be handed to the C ABI without
copies.  Camera matrices are computed by the native library
(``drgb_camera_look_at``), not here, so that their rounding matches the
reference's float arithmetic exactly.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


def _f32(a, cols=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if cols is not None:
        a = a.reshape(-1, cols)
    return a


@dataclass
class Texture:
    """CPUTexture (common_src/scene.h:11-35): w*h*channels float32, row major."""
    w: int
    h: int
    channels: int
    data: np.ndarray

    def __post_init__(self):
        self.data = np.ascontiguousarray(np.asarray(self.data, dtype=np.float32).reshape(-1))
        if self.data.size != self.w * self.h * self.channels:
            raise ValueError("texture size does not match w*h*channels")


@dataclass
class TriangleMesh:
    """TriangleMesh (common_src/scene.h:40-70)."""
    vertices: np.ndarray
    indices: np.ndarray
    colors: Optional[np.ndarray] = None
    tc: Optional[np.ndarray] = None
    normals: Optional[np.ndarray] = None
    tangents: Optional[np.ndarray] = None
    textures: List[Texture] = field(default_factory=list)

    def __post_init__(self):
        self.vertices = _f32(self.vertices, 3)
        self.indices = np.ascontiguousarray(np.asarray(self.indices, dtype=np.uint32).reshape(-1))
        self.colors = _f32(self.colors, 3)
        self.tc = _f32(self.tc, 2)
        self.normals = _f32(self.normals, 3)
        self.tangents = _f32(self.tangents, 3)
        n = self.vertices.shape[0]
        for name in ("colors", "tc", "normals", "tangents"):
            a = getattr(self, name)
            if a is not None and a.shape[0] != n:
                raise ValueError(f"{name} has {a.shape[0]} rows, expected {n}")
        if self.indices.size % 3 != 0:
            raise ValueError("index count is not a multiple of 3")
        if self.indices.size and int(self.indices.max()) >= n:
            raise ValueError("index out of range")

    @property
    def vertex_count(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def face_count(self) -> int:
        return int(self.indices.size // 3)

    def copy(self) -> "TriangleMesh":
        return TriangleMesh(self.vertices.copy(), self.indices.copy(),
                            None if self.colors is None else self.colors.copy(),
                            None if self.tc is None else self.tc.copy(),
                            None if self.normals is None else self.normals.copy(),
                            None if self.tangents is None else self.tangents.copy(),
                            [Texture(t.w, t.h, t.channels, t.data.copy()) for t in self.textures])


def identity4() -> np.ndarray:
    return np.eye(4, dtype=np.float32)


def _mul44(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """float32 a @ b summed left to right over k (LiteMath.h:1536-1549)."""
    out = np.zeros((4, 4), np.float32)
    for r in range(4):
        for c in range(4):
            acc = np.float32(b[0, c] * a[r, 0])
            for k in range(1, 4):
                acc = np.float32(acc + np.float32(b[k, c] * a[r, k]))
            out[r, c] = acc
    return out


@dataclass
class TransformR:
    """TransformR (common_src/scene.h:91-116): translation, rotation angles
    about x, y and z (radians) and a uniform scale.  A mesh added with a list
    of these is a RESTRICTED_TRANSFORM mesh: its instance matrices are
    ``to_mat()`` and its gradient holds these 7 parameters per instance."""
    translate: tuple = (0.0, 0.0, 0.0)
    rotate: tuple = (0.0, 0.0, 0.0)
    scale: float = 1.0

    def params(self) -> np.ndarray:
        return np.asarray([*self.translate, *self.rotate, self.scale], np.float32)

    @staticmethod
    def from_params(p) -> "TransformR":
        p = [float(x) for x in np.asarray(p, np.float32).reshape(7)]
        return TransformR(tuple(p[0:3]), tuple(p[3:6]), p[6])

    def to_mat(self) -> np.ndarray:
        """translate * rotZ * rotY * rotX * scale (scene.h:99-104), M[row, col]."""
        p = self.params()
        f = np.float32
        T = identity4()
        T[:3, 3] = p[:3]
        c, s = f(math.cos(p[5])), f(math.sin(p[5]))
        Rz = identity4()
        Rz[0, 0], Rz[0, 1], Rz[1, 0], Rz[1, 1] = c, -s, s, c
        c, s = f(math.cos(p[4])), f(math.sin(p[4]))
        Ry = identity4()
        Ry[0, 0], Ry[0, 2], Ry[2, 0], Ry[2, 2] = c, s, -s, c
        c, s = f(math.cos(p[3])), f(math.sin(p[3]))
        Rx = identity4()
        Rx[1, 1], Rx[1, 2], Rx[2, 1], Rx[2, 2] = c, -s, s, c
        S = np.diag([p[6], p[6], p[6], f(1)]).astype(np.float32)
        return _mul44(_mul44(_mul44(_mul44(T, Rz), Ry), Rx), S)


class Scene:
    """Scene (common_src/scene.h:121-247): meshes, each with instance transforms.

    Transforms are 4x4 matrices given in the usual row/column sense
    (``M[row, col]``); they are passed to the native side in the reference's
    column-major memory order.  A mesh added with ``TransformR`` instances is
    a RESTRICTED_TRANSFORM mesh (scene.h:140-148): ``restricted[i]`` holds
    them and ``transforms[i]`` their matrices.
    """

    def __init__(self):
        self.meshes: List[TriangleMesh] = []
        self.transforms: List[List[np.ndarray]] = []
        self.restricted: List[Optional[List[TransformR]]] = []
        self.names: List[str] = []

    def add_mesh(self, mesh: TriangleMesh, transforms=None, name: str = "") -> int:
        if transforms is None:
            transforms = [identity4()]
        transforms = list(transforms)
        self.meshes.append(mesh)
        if transforms and all(isinstance(t, TransformR) for t in transforms):
            self.restricted.append(list(transforms))
            self.transforms.append([t.to_mat() for t in transforms])
        else:
            self.restricted.append(None)
            self.transforms.append([np.asarray(t, dtype=np.float32).reshape(4, 4) for t in transforms])
        self.names.append(name)
        return len(self.meshes) - 1

    def get_restricted_transform(self, i: int) -> Optional[List[TransformR]]:
        return self.restricted[i]

    def restricted_params(self, i: int) -> Optional[np.ndarray]:
        """7 floats per instance of a restricted mesh, else None."""
        r = self.restricted[i]
        return None if r is None else np.ascontiguousarray(np.concatenate([t.params() for t in r]))

    def get_mesh(self, i: int) -> TriangleMesh:
        return self.meshes[i]

    def transforms_colmajor(self, i: int) -> np.ndarray:
        """Instance transforms of mesh i in LiteMath memory order (column major)."""
        return np.ascontiguousarray(np.stack([t.T for t in self.transforms[i]]).astype(np.float32).reshape(-1))

    def copy(self) -> "Scene":
        s = Scene()
        for m, t, r, n in zip(self.meshes, self.transforms, self.restricted, self.names):
            s.add_mesh(m.copy(), list(r) if r is not None else [x.copy() for x in t], n)
        return s


@dataclass
class CamInfo:
    """Pinhole camera (common_src/camera.h:9-22): look-at parameters.

    ``world_view``/``proj`` may instead be given directly (column-major, as
    LiteMath stores them), which is how the reference's derivative tests set
    their camera (src/tests.cpp:39-44).
    """
    origin: tuple = (0.0, 0.0, 3.0)
    target: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    width: int = 256
    height: int = 256
    fov_rad: float = math.pi / 4
    znear: float = 0.01
    zfar: float = 100.0
    world_view: Optional[np.ndarray] = None
    proj: Optional[np.ndarray] = None


# ---------------------------------------------------------------------------
# Synthetic scene generators (seeded) for the workloads the renderer is
# measured on.
# ---------------------------------------------------------------------------

def make_cube(seed: int = 1, edge: float = 1.0) -> TriangleMesh:
    """Unit cube with 8 shared vertices / 12 triangles, outward winding,
    per-vertex RGB colours drawn U[0,1] from ``seed``."""
    h = edge / 2.0
    v = np.array([[x, y, z] for x in (-h, h) for y in (-h, h) for z in (-h, h)], dtype=np.float32)

    def vid(x, y, z):
        return (x > 0) * 4 + (y > 0) * 2 + (z > 0) * 1

    faces = []
    for axis in range(3):
        for sgn in (-1, 1):
            quad = []
            for a, b in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                p = [0, 0, 0]
                p[axis] = sgn
                p[(axis + 1) % 3] = a
                p[(axis + 2) % 3] = b
                quad.append(vid(*p))
            # orient outward: (p1-p0)x(p2-p0) must point along sgn*axis
            p0, p1, p2 = v[quad[0]], v[quad[1]], v[quad[2]]
            n = np.cross(p1 - p0, p2 - p0)
            if n[axis] * sgn < 0:
                quad = quad[::-1]
            faces.append((quad[0], quad[1], quad[2]))
            faces.append((quad[0], quad[2], quad[3]))
    rng = np.random.default_rng(seed)
    colors = rng.uniform(0.0, 1.0, size=(8, 3)).astype(np.float32)
    return TriangleMesh(v, np.array(faces, dtype=np.uint32).reshape(-1), colors=colors)


def make_icosphere(subdivisions: int = 4, radius: float = 1.0, seed: int = 1,
                   albedo_range=(0.2, 0.9)) -> TriangleMesh:
    """Icosphere: 10*4^s+2 vertices, 20*4^s triangles (s=4: 2562/5120),
    unit-length vertex normals, per-vertex albedo U[albedo_range]."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    P = np.array(verts, dtype=np.float64)
    rng = np.random.default_rng(seed)
    colors = rng.uniform(albedo_range[0], albedo_range[1], size=(len(P), 3)).astype(np.float32)
    return TriangleMesh((P * radius).astype(np.float32), np.array(faces, dtype=np.uint32).reshape(-1),
                        colors=colors, normals=P.astype(np.float32))


def make_uv_sphere(n_lat: int, n_lon: int, radius: float = 1.0, seed: int = 1,
                   albedo_range=(0.2, 0.9)) -> TriangleMesh:
    """Closed UV sphere with poles: (n_lat-1)*n_lon+2 vertices and
    2*n_lon*(n_lat-1) triangles."""
    verts = [(0.0, radius, 0.0)]
    for i in range(1, n_lat):
        th = math.pi * i / n_lat
        for j in range(n_lon):
            ph = 2 * math.pi * j / n_lon
            verts.append((radius * math.sin(th) * math.sin(ph), radius * math.cos(th), radius * math.sin(th) * math.cos(ph)))
    verts.append((0.0, -radius, 0.0))
    faces = []
    S = len(verts) - 1
    for j in range(n_lon):
        faces.append((0, 1 + j, 1 + (j + 1) % n_lon))
    for i in range(n_lat - 2):
        r0, r1 = 1 + i * n_lon, 1 + (i + 1) * n_lon
        for j in range(n_lon):
            a, b = r0 + j, r0 + (j + 1) % n_lon
            c, d = r1 + j, r1 + (j + 1) % n_lon
            faces.append((a, c, d))
            faces.append((a, d, b))
    base = 1 + (n_lat - 2) * n_lon
    for j in range(n_lon):
        faces.append((S, base + (j + 1) % n_lon, base + j))
    P = np.array(verts, dtype=np.float64)
    N = P / np.linalg.norm(P, axis=1, keepdims=True)
    rng = np.random.default_rng(seed)
    colors = rng.uniform(albedo_range[0], albedo_range[1], size=(len(P), 3)).astype(np.float32)
    return TriangleMesh(P.astype(np.float32), np.array(faces, dtype=np.uint32).reshape(-1), colors=colors,
                        normals=N.astype(np.float32))


def displace_radially(mesh: TriangleMesh, seed: int, n_waves: int = 8, amplitude: float = 0.05) -> TriangleMesh:
    """Radial displacement by a seeded sum of sinusoids of the unit direction;
    the total amplitude is bounded by ``amplitude``."""
    rng = np.random.default_rng(seed)
    P = mesh.vertices.astype(np.float64)
    r = np.linalg.norm(P, axis=1, keepdims=True)
    d = P / r
    disp = np.zeros(len(P))
    for _ in range(n_waves):
        k = rng.normal(size=3)
        k = k / np.linalg.norm(k) * rng.uniform(2.0, 8.0)
        ph = rng.uniform(0, 2 * math.pi)
        disp += np.sin(d @ k + ph)
    disp *= amplitude / n_waves
    out = mesh.copy()
    out.vertices = (d * (r + disp[:, None])).astype(np.float32)
    # normals from the displaced surface (area-weighted face normals)
    F = out.indices.reshape(-1, 3)
    V = out.vertices.astype(np.float64)
    fn = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    vn = np.zeros_like(V)
    for k in range(3):
        np.add.at(vn, F[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-12)
    out.normals = vn.astype(np.float32)
    return out


def perturb_vertices(mesh: TriangleMesh, sigma: float, seed: int, radial: bool = False) -> TriangleMesh:
    """Start state: vertices + N(0, sigma) noise (radial when ``radial``)."""
    rng = np.random.default_rng(seed)
    out = mesh.copy()
    if radial:
        P = out.vertices.astype(np.float64)
        d = P / np.linalg.norm(P, axis=1, keepdims=True)
        out.vertices = (P + d * rng.normal(0.0, sigma, size=(len(P), 1))).astype(np.float32)
    else:
        out.vertices = (out.vertices + rng.normal(0.0, sigma, size=out.vertices.shape)).astype(np.float32)
    return out


def ring_cameras(n: int, radius: float, width: int, height: int, fov_rad: float = math.pi / 4):
    """n cameras on a ring of the given radius in the y=0 plane, yaw k*360/n,
    all looking at the origin."""
    cams = []
    for k in range(n):
        a = 2 * math.pi * k / n
        cams.append(CamInfo(origin=(radius * math.sin(a), 0.0, radius * math.cos(a)), target=(0.0, 0.0, 0.0),
                            up=(0.0, 1.0, 0.0), width=width, height=height, fov_rad=fov_rad))
    return cams
