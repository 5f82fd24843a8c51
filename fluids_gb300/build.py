"""Builds fluids_gb300/lib/libsph_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel (one -gencode, -O3 -lineinfo) and linked into
one shared library that exports the C ABI of include/sph_capi.h; the CUDA runtime is linked
statically so the library has no dependency on a particular libcudart on the target.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libsph_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["sph_sort.cu", "sph_grid.cu", "sph_wcsph.cu", "sph_pcisph.cu", "sph_boundary.cu", "sph_context.cu",
           "sph_scene.cpp", "sph_sort_noalloc.cu", "sph_adjoint.cu", "sph_render.cu", "sph_mesh.cu", "sph_state.cu"]
# The screen-space surface and voxelizer kernels round every multiply and add separately (no
# FMA contraction) so their images and voxels are reproducible operation for operation; the
# host scene builders likewise, so Arm and x86 hosts sample the same particles.
SOURCE_FLAGS = {"sph_render.cu": ["-fmad=false"], "sph_mesh.cu": ["-fmad=false"],
                "sph_scene.cpp": ["-Xcompiler", "-ffp-contract=off"]}
_lock = threading.Lock()


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src, extra):
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    newest = max([os.path.getmtime(path)] + [os.path.getmtime(h) for h in _headers()] +
                 [os.path.getmtime(os.path.abspath(__file__))])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj + ".tmp", "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-I", CSRC] + ARCH + SOURCE_FLAGS.get(src, []) + extra
    if src.endswith(".cpp"):
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(force=False, verbose=False, extra=None):
    """Compiles and links the library if any source is newer than it; returns its path."""
    with _lock:
        os.makedirs(OBJ_DIR, exist_ok=True)
        if force:
            for f in os.listdir(OBJ_DIR):
                os.remove(os.path.join(OBJ_DIR, f))
        extra = list(extra or [])
        with cf.ThreadPoolExecutor(max_workers=min(8, len(SOURCES))) as ex:
            objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
        newest = max(os.path.getmtime(o) for o in objs)
        if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
            tmp = LIB + ".tmp%d" % os.getpid()
            cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
            os.replace(tmp, LIB)
        if verbose:
            print("built", LIB)
        return LIB


DRIVER_SRC = os.path.join(PKG, "driver", "sph_driver.cpp")
DRIVER = os.path.join(OUT_DIR, "sph_driver")


def build_driver(force=False):
    """The headless C++ driver (driver/sph_driver.cpp) over include/sph_fluid.hpp, linked
    against the library with an rpath to its own directory."""
    lib = build()
    deps = [DRIVER_SRC, os.path.join(INCLUDE, "sph_fluid.hpp"), os.path.join(INCLUDE, "sph_capi.h"), lib]
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(d) for d in deps):
        return DRIVER
    tmp = DRIVER + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, DRIVER_SRC, "-o", tmp, "-L", OUT_DIR, "-lsph_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, DRIVER)
    return DRIVER


def ptxas_report(src="sph_wcsph.cu", extra=None):
    """Registers / spills / shared memory per kernel (nvcc -Xptxas -v) for one source, with
    the flags the build gives it."""
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", os.devnull, "-std=c++17", "-O3", "-Xptxas", "-v",
           "-I", INCLUDE, "-I", CSRC] + ARCH + SOURCE_FLAGS.get(src, []) + list(extra or [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr
