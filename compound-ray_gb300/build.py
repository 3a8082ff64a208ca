"""Builds libEyeRenderer3.so in place (sm_103a only).

The CUDA translation unit is compiled with --use_fast_math, matching the
reference's shader build flags (CMakeLists.txt:154-159); host C++ is built
with -ffp-contract=off so the loader's double-precision transform arithmetic
is the same on x86-64 and aarch64.  Objects go to ``_build/`` next to this
file, the shared library next to this file.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libEyeRenderer3.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["render.cu", "lbvh.cu", "mlp.cu", "mlp_tc.cu"]
CPP_SOURCES = ["gltf.cpp", "png.cpp", "bvh.cpp", "wbvh.cpp", "denoiser.cpp", "eye_renderer.cpp"]


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return proc.stdout


def _newer(src_paths, out):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(p) > t for p in src_paths)


def build(verbose=False, force=False, extra_nvcc=()):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "libEyeRenderer.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer([s] + headers, o):
            jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "--use_fast_math", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", *extra_nvcc, "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer([s] + headers, o):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I" + os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs])
        shutil.move(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
