"""Build the reference renderer's CPU path (brute-force caster + OpenMP) into
oracle/_ref/ so that golden fixtures can be generated from the reference itself.

Test infrastructure only.  Recipe:
  1. copy the reference sources this path needs into oracle/_ref/src/ (a
     git-ignored scratch tree; nothing is copied into the repository);
  2. apply one compile-compatibility edit: ``TransformR`` in
     common_src/scene.h:105-115 wraps float3 members in an anonymous union,
     a clang extension that g++ rejects ("member with constructor not allowed
     in anonymous aggregate").  The union becomes plain members; the aliased
     ``M[7]`` view is only read by the Enzyme restricted-transform Jacobian,
     which is stubbed to zero because the Enzyme plugin is absent;
  3. compile with g++ -O3 -fopenmp -DUSE_OMP (the flags of the reference's
     own CMakeLists.txt:79-85,91) together with oracle/ref/ref_driver.cpp.

The reference's CMake build, Embree (missing binary) and Mitsuba (not
installed) are not used.  Only runs where the reference tree exists; the
output is x86-specific and is not needed on other machines.
"""
import os
import re
import shutil
import subprocess
import sys

REF_ROOT = os.environ.get("DRGB_REFERENCE_ROOT", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")

COMPILE = [
    "src/drender.cpp", "src/functions.cpp", "src/shade_simple.cpp", "src/shade_lambert.cpp",
    "src/shade_path_test.cpp", "src/shade_common.cpp", "src/utils.cpp", "src/optimizer_simple.cpp",
    "common_src/scene_utils.cpp", "common_src/qmc.cpp", "common_src/Image2d.cpp",
    "raytrace_src/raytrace3d_bf.cpp",
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
    new, n = pat.subn("float3 translate; float3 rotate; float scale; float M[7];", text)
    if n != 1:
        raise RuntimeError("TransformR union not found in scene.h; the reference layout changed")
    open(scene_h, "w").write(new)
    return src_root


def build(verbose=False):
    if not os.path.isdir(REF_ROOT):
        if verbose:
            print("reference tree absent; skipping oracle/_ref build")
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_driver")
    stamp_src = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "kvio.h"), __file__]
    if os.path.exists(exe) and all(os.path.getmtime(exe) >= os.path.getmtime(s) for s in stamp_src):
        return exe
    src_root = _copy_tree()
    incs = []
    for d in HEADER_DIRS + ["stub"]:
        incs += ["-I", os.path.join(src_root, d)]
    incs += ["-I", HERE]
    objs = []
    procs = []
    for rel in COMPILE:
        obj = os.path.join(OUT, rel.replace("/", "_") + ".o")
        cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-DUSE_OMP", "-ffp-contract=off", "-w"] + incs + ["-c", os.path.join(src_root, rel), "-o", obj]
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(obj)
    for p, cmd in procs:
        if p.wait() != 0:
            raise RuntimeError("reference compile failed: " + " ".join(cmd))
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-DUSE_OMP", "-ffp-contract=off", "-w"] + incs + [
        os.path.join(HERE, "ref_driver.cpp")] + objs + ["-o", exe]
    subprocess.check_call(cmd)
    return exe


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
