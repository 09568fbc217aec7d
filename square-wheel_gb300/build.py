"""Build the GB300 rendering library (libswgpu.so) in-tree with nvcc for sm_103a.

Usage: python square-wheel_gb300/build.py [--force]

Translation units are compiled in parallel; the shared library lands in square-wheel_gb300/lib/.
Flags that matter for parity: --fmad=false (never contract a*b+c into an FMA), IEEE division and
square root, and -ffp-contract=off for the host-side C++ (exposure update, blur weights).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIB_DIR = os.path.join(PKG, "lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIB_DIR, "libswgpu.so")
SOURCES = ["swgpu.cu", "surfaces.cu", "raster.cu", "prep.cu", "post.cu", "post_noalloc.cu", "upscaler.cu", "lightmaps.cu", "effects.cu",
           "sims.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def common_flags():
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I", os.path.join(PKG, "..", "include"),
    ]


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(PKG, "..", "include", "swgpu.h"))
    # the per-polygon preparation code shared with the host side
    headers += [os.path.join(PKG, "host", f) for f in ("prep_math.h", "hmath.h")]
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([cc] + common_flags() + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err)
    if jobs or not os.path.exists(LIB):
        run([cc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs)
    build_host(force, verbose)
    return LIB


HOST_SOURCES = ["scene.cpp", "frame.cpp", "swhost.cpp", "sqwm.cpp", "sims.cpp"]
HOST_LIB = os.path.join(LIB_DIR, "libswhost.so")


def build_host(force=False, verbose=False):
    """Host side (visibility, per-polygon setup, scene generator) as libswhost.so, linked to libswgpu.so."""
    host_dir = os.path.join(PKG, "host")
    inc = os.path.join(PKG, "..", "include")
    deps = [os.path.join(host_dir, f) for f in os.listdir(host_dir) if f.endswith((".h", ".cpp"))]
    deps += [os.path.join(inc, "swgpu.h"), os.path.join(inc, "swhost.h"), LIB]
    if not force and _newer(HOST_LIB, deps):
        return HOST_LIB
    cxx = shutil.which("g++") or "g++"
    objs = []
    cmds = []
    for src in HOST_SOURCES:
        o = os.path.join(BUILD_DIR, "host_" + src.replace(".cpp", ".o"))
        objs.append(o)
        cmds.append([cxx, "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wextra",
                     "-Wno-unused-parameter", "-I", inc, "-c", os.path.join(host_dir, src), "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for err in ex.map(run, cmds):
            if verbose and err:
                print(err)
    run([cxx, "-shared", "-o", HOST_LIB] + objs + ["-L", LIB_DIR, "-lswgpu", "-Wl,-rpath,$ORIGIN", "-lpthread"])
    return HOST_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
