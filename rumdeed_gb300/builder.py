"""Builds librumdeed_gb300.so for sm_103a in-tree (rumdeed_gb300/_lib/).

Every translation unit is compiled in parallel with one -gencode
(arch=compute_103a,code=sm_103a) and linked with the static CUDA runtime, so
the library has no dependency beyond the driver.  No PyTorch is involved.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "librumdeed_gb300.so")
DRIVER_SRC = os.path.join(HERE, "driver", "rd_main.cpp")
DRIVER = os.path.join(OUT_DIR, "rd_main")
SOURCES = ["rd_force.cu", "rd_field.cu", "rd_step.cu", "rd_engine.cu", "rd_noalloc.cu"]
HEADERS = ["rd_internal.h", "rd_device.cuh", "rd_pair.cuh", "rd_tiles.cuh", "rd_split.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I", os.path.join(HERE, "..", "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    paths.append(os.path.join(HERE, "..", "include", "rumdeed_gpu.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def build_driver(force=False):
    """The native main-loop driver rd_main (g++), linked against the library."""
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(
            os.path.getmtime(DRIVER_SRC), os.path.getmtime(LIB)):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-o", DRIVER, DRIVER_SRC, "-L" + OUT_DIR, "-lrumdeed_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return DRIVER


def build(force=False, verbose=False, extra=()):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        build_driver()
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_driver(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
