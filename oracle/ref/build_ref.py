"""Build the reference renderer's CPU path (brute-force caster + OpenMP) into
oracle/_ref/ so that golden fixtures can be generated from the reference itself.

Test infrastructure only.  Recipe:
  1. copy the reference sources this path needs into oracle/_ref/src/ (a
     git-ignored scratch tree; nothing is copied into the repository);
  2. apply one compile-compatibility edit: ``TransformR`` in
     common_src/scene.h:105-115 wraps float3 members in an anonymous union,
     a clang extension that g++ rejects ("member with constructor not allowed
     in anonymous aggregate").  The union becomes plain members; the aliased
     ``M[7]`` view (read only by the restricted-transform Jacobian) becomes a
     mutable array that ``to_mat()`` -- called by every prepare_for_render
     before a gradient pass -- fills with the same 7 values;
  3. compile with g++ -O3 -fopenmp -DUSE_OMP (the flags of the reference's
     own CMakeLists.txt:79-85,91) together with oracle/ref/ref_driver.cpp and
     the oracle's C file, whose analytic TransformR Jacobian stands in for the
     absent Enzyme plugin (src/drender_autodiff.cpp:97-107).

The reference's CMake build, Embree (missing binary) and Mitsuba (not
installed) are not used.  Where the reference tree is absent, the patched copy under oracle/_ref/src
(made earlier and shipped with the working tree) is compiled instead, so that
ref_driver can be rebuilt on a machine of another architecture.
"""
import os
import platform
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $DRGB_REFERENCE_ROOT, else a directory named
# "reference" beside this repository's root
REF_ROOT = os.environ.get("DRGB_REFERENCE_ROOT",
                          os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference"))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
# objects and binaries per machine architecture (the source copy is shared)
BIN = os.path.join(OUT, platform.machine())

COMPILE = [
    "src/drender.cpp", "src/functions.cpp", "src/shade_simple.cpp", "src/shade_lambert.cpp",
    "src/shade_path_test.cpp", "src/shade_common.cpp", "src/utils.cpp", "src/optimizer_simple.cpp",
    "common_src/scene_utils.cpp", "common_src/qmc.cpp", "common_src/Image2d.cpp", "common_src/cmesh.cpp",
    "raytrace_src/raytrace3d_bf.cpp", "src/scenes.cpp",
]
HEADER_DIRS = ["src", "common_src", "raytrace_src"]


def _copy_tree():
    src_root = os.path.join(OUT, "src")
    if os.path.isdir(src_root):
        shutil.rmtree(src_root)
    for d in HEADER_DIRS:
        os.makedirs(os.path.join(src_root, d), exist_ok=True)
        for name in os.listdir(os.path.join(REF_ROOT, d)):
            if name.endswith((".h", ".cpp")):
                shutil.copy(os.path.join(REF_ROOT, d, name), os.path.join(src_root, d, name))
    # The only header of the Mitsuba stub directory that src/ might include.
    stub = os.path.join(REF_ROOT, "mitsuba_src", "stub")
    if os.path.isdir(stub):
        os.makedirs(os.path.join(src_root, "stub"), exist_ok=True)
        for name in os.listdir(stub):
            shutil.copy(os.path.join(stub, name), os.path.join(src_root, "stub", name))
    scene_h = os.path.join(src_root, "common_src", "scene.h")
    text = open(scene_h).read()
    pat = re.compile(r"union\s*\{\s*struct\s*\{\s*float3 translate;\s*float3 rotate;\s*float scale;\s*\};\s*float M\[7\];\s*\};")
    new, n = pat.subn("float3 translate; float3 rotate; float scale; mutable float M[7];", text)
    if n != 1:
        raise RuntimeError("TransformR union not found in scene.h; the reference layout changed")
    fill = ("M[0] = translate.x; M[1] = translate.y; M[2] = translate.z; "
            "M[3] = rotate.x; M[4] = rotate.y; M[5] = rotate.z; M[6] = scale;")
    new, n = re.subn(r"(float4x4 to_mat\(\) const\s*\{)", lambda m: m.group(1) + " " + fill, new)
    if n != 1:
        raise RuntimeError("TransformR::to_mat not found in scene.h; the reference layout changed")
    open(scene_h, "w").write(new)
    return src_root


def _source_tree(verbose=False):
    """The patched copy of the reference sources: made from the reference
    tree where it exists, else the copy made earlier (a machine without the
    reference tree receives oracle/_ref/src with the repository)."""
    src_root = os.path.join(OUT, "src")
    if os.path.isdir(REF_ROOT):
        stamp = os.path.join(src_root, ".copied")
        if not os.path.exists(stamp) or os.path.getmtime(stamp) < os.path.getmtime(__file__):
            _copy_tree()
            open(stamp, "w").close()
        return src_root
    if os.path.isdir(os.path.join(src_root, "src")):
        return src_root
    if verbose:
        print("reference sources absent; skipping oracle/_ref build")
    return None


def _includes(src_root):
    incs = []
    for d in HEADER_DIRS + ["stub"]:
        incs += ["-I", os.path.join(src_root, d)]
    return incs + ["-I", HERE, "-I", ORACLE]


FLAGS = ["g++", "-std=c++17", "-O3", "-fopenmp", "-DUSE_OMP", "-ffp-contract=off", "-w"]


def _objects(src_root):
    """The reference's translation units, compiled in parallel when stale."""
    incs = _includes(src_root)
    objs, procs = [], []
    for rel in COMPILE:
        src = os.path.join(src_root, rel)
        if rel == "src/drender.cpp":
            # compiled through drender_unit.cpp, which adds the point-light model
            src = os.path.join(HERE, "drender_unit.cpp")
        obj = os.path.join(BIN, rel.replace("/", "_") + ".o")
        objs.append(obj)
        deps = [src, os.path.join(HERE, "ref_pointlight.h"), os.path.join(src_root, "src", "drender.cpp"),
                os.path.join(src_root, "src", "drender.h")]
        if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
            continue
        cmd = FLAGS + incs + ["-c", src, "-o", obj]
        procs.append((subprocess.Popen(cmd), cmd))
    for p, cmd in procs:
        if p.wait() != 0:
            raise RuntimeError("reference compile failed: " + " ".join(cmd))
    return objs


def _stale(exe, deps):
    return not os.path.exists(exe) or any(os.path.getmtime(exe) < os.path.getmtime(d) for d in deps)


def _oracle_object():
    """oracle.c compiled for ref_driver (its TransformR Jacobian)."""
    src, hdr = os.path.join(ORACLE, "oracle.c"), os.path.join(ORACLE, "oracle.h")
    obj = os.path.join(BIN, "oracle.o")
    if _stale(obj, [src, hdr, __file__]):
        subprocess.check_call(["gcc", "-std=c11", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
                               "-fno-trapping-math", "-w", "-c",
                               src, "-o", obj])
    return obj


def build(verbose=False):
    """oracle/_ref/<arch>/ref_driver: the reference's CPU path behind ref_driver.cpp."""
    src_root = _source_tree(verbose)
    if src_root is None:
        return None
    os.makedirs(BIN, exist_ok=True)
    exe = os.path.join(BIN, "ref_driver")
    objs = _objects(src_root) + [_oracle_object()]
    deps = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "kvio.h"), __file__] + objs
    if _stale(exe, deps):
        subprocess.check_call(FLAGS + _includes(src_root) + [os.path.join(HERE, "ref_driver.cpp")] + objs +
                              ["-o", exe])
    return exe


def build_gpu_driver(verbose=False):
    """oracle/_ref/<arch>/ref_driver_gpu: the same driver with the GPU renderer and
    optimiser of diffrender_tutorials_gb300/cpp/gpu_drender.cpp behind the
    reference's interfaces (backend 1 and 2), linked to libdrgb.so."""
    src_root = _source_tree(verbose)
    if src_root is None:
        return None
    sys.path.insert(0, os.path.dirname(ORACLE))
    from diffrender_tutorials_gb300 import build as drgb_build
    lib = drgb_build.build()
    adapter = os.path.join(os.path.dirname(ORACLE), "diffrender_tutorials_gb300", "cpp")
    include = os.path.join(os.path.dirname(ORACLE), "include")
    os.makedirs(BIN, exist_ok=True)
    exe = os.path.join(BIN, "ref_driver_gpu")
    objs = _objects(src_root) + [_oracle_object()]
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(adapter, "gpu_drender.cpp")]
    deps = srcs + [os.path.join(adapter, "gpu_drender.h"), os.path.join(HERE, "kvio.h"), __file__, lib] + objs
    if _stale(exe, deps):
        libdir = os.path.dirname(lib)
        subprocess.check_call(FLAGS + ["-DDRGB_WITH_GPU", "-I", adapter, "-I", include] + _includes(src_root) + srcs +
                              objs + ["-L", libdir, "-ldrgb", "-Wl,-rpath," + libdir, "-o", exe])
    return exe


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
