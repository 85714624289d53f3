"""Mesh and image files used with the reference renderer.

* VSGF meshes (common_src/cmesh.cpp:82-94 header and flags, 139-170 layout):
  a 24-byte header {u64 file size, u32 vertices, u32 indices, u32
  materials, u32 flags}, then float4 positions, float4 normals (unless
  flag 8, no normals), float4 tangents (flag 1), float2 texture
  coordinates, u32 indices and one u32 material index per triangle.
* Wavefront OBJ meshes (v / vt / vn / f, polygons fanned into triangles;
  every distinct v/vt/vn triple becomes one vertex).
* Images as LiteImage::SaveImage<float3> writes them
  (common_src/Image2d.cpp:580-588, 670-738): 8-bit channels
  int(pow(x, 1/gamma) * 255 + 0.5) clamped to [0, 255], gamma 2.2 by default,
  as BMP (24-bit, rows stored bottom-up so that image row 0 is the top) or
  PPM (P3); ``.image3f`` is the raw form {u32 width, u32 height, floats}.
"""
from __future__ import annotations

import os
import struct
from typing import Optional

import numpy as np

from .scene import TriangleMesh

HAS_TANGENT, HAS_NO_NORMALS = 1, 8


# ---- VSGF ------------------------------------------------------------------
def load_vsgf(path: str) -> TriangleMesh:
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 24:
        raise ValueError(f"{path}: not a VSGF file (short header)")
    _size, nv, ni, _nmat, flags = struct.unpack_from("<QIIII", data, 0)
    off = 24

    def take(count, dtype, width):
        nonlocal off
        n_bytes = count * width * np.dtype(dtype).itemsize
        if off + n_bytes > len(data):
            raise ValueError(f"{path}: truncated VSGF data")
        a = np.frombuffer(data, dtype, count * width, off).reshape(count, width) if width > 1 else \
            np.frombuffer(data, dtype, count, off)
        off += n_bytes
        return a

    pos = take(nv, np.float32, 4)
    nrm = None if flags & HAS_NO_NORMALS else take(nv, np.float32, 4)
    tan = take(nv, np.float32, 4) if flags & HAS_TANGENT else None
    tc = take(nv, np.float32, 2)
    idx = take(ni, np.uint32, 1)
    return TriangleMesh(pos[:, :3].copy(), idx.copy(), tc=tc.copy(),
                        normals=None if nrm is None else nrm[:, :3].copy(),
                        tangents=None if tan is None else tan[:, :3].copy())


def save_vsgf(path: str, mesh: TriangleMesh, material: int = 0) -> None:
    nv, ni = mesh.vertex_count, int(mesh.indices.size)
    flags = (0 if mesh.normals is not None else HAS_NO_NORMALS) | (HAS_TANGENT if mesh.tangents is not None else 0)

    def four(a):
        out = np.zeros((nv, 4), np.float32)
        out[:, :3] = np.asarray(a, np.float32).reshape(nv, 3)
        return out

    parts = [four(mesh.vertices).tobytes()]
    if mesh.normals is not None:
        parts.append(four(mesh.normals).tobytes())
    if mesh.tangents is not None:
        parts.append(four(mesh.tangents).tobytes())
    tc = mesh.tc if mesh.tc is not None else np.zeros((nv, 2), np.float32)
    parts.append(np.asarray(tc, np.float32).reshape(nv, 2).tobytes())
    parts.append(np.asarray(mesh.indices, np.uint32).reshape(-1).tobytes())
    parts.append(np.full(ni // 3, material, np.uint32).tobytes())
    body = b"".join(parts)
    header = struct.pack("<QIIII", 24 + len(body), nv, ni, 1, flags)
    with open(path, "wb") as f:
        f.write(header + body)


# ---- OBJ -------------------------------------------------------------------
def load_obj(path: str) -> TriangleMesh:
    P, T, N = [], [], []
    verts, remap, idx = [], {}, []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts or parts[0].startswith("#"):
                continue
            if parts[0] == "v":
                P.append([float(x) for x in parts[1:4]])
            elif parts[0] == "vt":
                T.append([float(x) for x in parts[1:3]])
            elif parts[0] == "vn":
                N.append([float(x) for x in parts[1:4]])
            elif parts[0] == "f":
                corner = []
                for tok in parts[1:]:
                    ids = (tok.split("/") + ["", ""])[:3]

                    def ref(s, n):
                        if not s:
                            return -1
                        k = int(s)
                        return k - 1 if k > 0 else n + k

                    key = (ref(ids[0], len(P)), ref(ids[1], len(T)), ref(ids[2], len(N)))
                    if key not in remap:
                        remap[key] = len(verts)
                        verts.append(key)
                    corner.append(remap[key])
                for k in range(1, len(corner) - 1):
                    idx += [corner[0], corner[k], corner[k + 1]]
    if not verts:
        raise ValueError(f"{path}: no faces")
    V = np.asarray([P[p] for p, _, _ in verts], np.float32)
    tc = np.asarray([T[t] for _, t, _ in verts], np.float32) if all(t >= 0 for _, t, _ in verts) else None
    nr = np.asarray([N[n] for _, _, n in verts], np.float32) if all(n >= 0 for _, _, n in verts) else None
    return TriangleMesh(V, np.asarray(idx, np.uint32), tc=tc, normals=nr)


def save_obj(path: str, mesh: TriangleMesh) -> None:
    with open(path, "w") as f:
        for p in mesh.vertices.reshape(-1, 3):
            f.write(f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
        if mesh.tc is not None:
            for t in mesh.tc.reshape(-1, 2):
                f.write(f"vt {t[0]:.9g} {t[1]:.9g}\n")
        if mesh.normals is not None:
            for n in mesh.normals.reshape(-1, 3):
                f.write(f"vn {n[0]:.9g} {n[1]:.9g} {n[2]:.9g}\n")
        has_t, has_n = mesh.tc is not None, mesh.normals is not None
        for tri in mesh.indices.reshape(-1, 3):
            c = []
            for v in tri + 1:
                c.append(f"{v}/{v if has_t else ''}/{v}" if has_n else (f"{v}/{v}" if has_t else f"{v}"))
            f.write("f " + " ".join(c) + "\n")


# ---- images ----------------------------------------------------------------
def tonemap(img: np.ndarray, gamma: float = 2.2) -> np.ndarray:
    """float image -> uint8 as LiteImage's tonemap: int(x^(1/gamma)*255+0.5), clamped."""
    x = np.asarray(img, np.float32)
    with np.errstate(invalid="ignore"):
        v = np.power(x.astype(np.float64), 1.0 / gamma) * 255.0 + 0.5
    v = np.where(np.isnan(v), 0.0, v)
    return np.clip(np.trunc(v), 0, 255).astype(np.uint8)


def save_image(path: str, img: np.ndarray, gamma: float = 2.2) -> None:
    """img: (H, W, 3) floats (the renderer's images reshaped)."""
    img = np.asarray(img, np.float32)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("image must be (height, width, 3)")
    h, w, _ = img.shape
    ext = os.path.splitext(path)[1].lower()
    if ext == ".image3f":
        with open(path, "wb") as f:
            f.write(struct.pack("<II", w, h) + img.tobytes())
        return
    q = tonemap(img, gamma)
    if ext == ".ppm":
        with open(path, "w") as f:
            f.write(f"P3\n{w} {h} 255\n")
            f.write(" ".join(str(int(c)) for c in q.reshape(-1)) + " ")
        return
    if ext != ".bmp":
        raise ValueError(f"unsupported image extension {ext!r} (.bmp, .ppm, .image3f)")
    row = (w * 3 + 3) & ~3
    pix = np.zeros((h, row), np.uint8)
    pix[:, :3 * w] = q[::-1, :, ::-1].reshape(h, 3 * w)  # bottom-up rows, BGR
    size = 54 + pix.size
    header = struct.pack("<2sIHHI", b"BM", size, 0, 0, 54) + \
        struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, pix.size, 2835, 2835, 0, 0)
    with open(path, "wb") as f:
        f.write(header + pix.tobytes())


def load_image(path: str, gamma: float = 2.2) -> np.ndarray:
    """(H, W, 3) floats; 8-bit files are mapped back through x^gamma."""
    ext = os.path.splitext(path)[1].lower()
    with open(path, "rb") as f:
        data = f.read()
    if ext == ".image3f":
        w, h = struct.unpack_from("<II", data, 0)
        return np.frombuffer(data, np.float32, w * h * 3, 8).reshape(h, w, 3).copy()
    if ext == ".bmp":
        off = struct.unpack_from("<I", data, 10)[0]
        w, h = struct.unpack_from("<ii", data, 18)
        bpp = struct.unpack_from("<H", data, 28)[0]
        if bpp != 24:
            raise ValueError(f"{path}: only 24-bit BMP files are read")
        row = (w * 3 + 3) & ~3
        pix = np.frombuffer(data, np.uint8, row * abs(h), off).reshape(abs(h), row)[:, :3 * w].reshape(abs(h), w, 3)
        q = pix[:, :, ::-1]
        if h > 0:
            q = q[::-1]
    elif ext == ".ppm":
        tok = data.decode().split()
        if tok[0] != "P3":
            raise ValueError(f"{path}: only P3 files are read")
        w, h = int(tok[1]), int(tok[2])
        q = np.asarray(tok[4:4 + 3 * w * h], np.float64).reshape(h, w, 3)
    else:
        raise ValueError(f"unsupported image extension {ext!r}")
    return np.power(np.asarray(q, np.float64) / 255.0, gamma).astype(np.float32)


def mesh_from_file(path: str, colors: Optional[np.ndarray] = None) -> TriangleMesh:
    ext = os.path.splitext(path)[1].lower()
    m = load_vsgf(path) if ext == ".vsgf" else load_obj(path) if ext == ".obj" else None
    if m is None:
        raise ValueError(f"unsupported mesh extension {ext!r} (.vsgf, .obj)")
    if colors is not None:
        m.colors = np.asarray(colors, np.float32).reshape(-1, 3)
    return m
