"""Build libdrgb.so (the CUDA kernels and the C ABI) in-tree with nvcc.

Every translation unit is compiled for sm_103a only.  Device code is built
with -fmad=false so that the renderer's float arithmetic rounds exactly like
the reference's CPU code, and host code with -ffp-contract=off for the same
reason (camera matrices, Hammersley points).
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdrgb.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["bvh.cu", "render.cu", "edge.cu", "optim.cu", "engine.cu", "capi.cu", "noalloc.cu", "batch.cu", "serve.cu", "detsum.cu",
           "raster.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def flags():
    return ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I", INCLUDE, "-I", CSRC]


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=(), out=None):
    """Compile the library; `out` names another output path (and object
    directory) for builds with different `extra_flags`."""
    lib = out or LIB
    objdir = os.path.dirname(os.path.abspath(lib))
    os.makedirs(objdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "drgb.h"))
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    if not force and not _stale(lib, srcs + headers + [__file__]):
        return lib
    cc = nvcc()
    objs = []

    def comp(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [cc, *flags(), *extra_flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(comp, srcs))
    tmp = lib + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
