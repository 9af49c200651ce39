"""Builds the in-tree shared library optix_pt_gb300/_lib/liboptpt.so.

CUDA translation units are compiled by nvcc for sm_103a only; host-only C++
by g++ without floating-point contraction (so scene generation and other
host arithmetic give identical results on x86 and Arm). Translation units
compile in parallel; an up-to-date library is not rebuilt.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(ROOT, "_build", "optpt")
LIB = os.path.join(OUT_DIR, "liboptpt.so")

CUDA_SOURCES = ["bvh_build.cu", "bvh8_build.cu", "wavefront.cu", "engine.cu", "metrics.cu", "guide.cu", "image_out.cu", "deform.cu"]
CXX_SOURCES = ["scenes.cpp", "autotune.cpp", "gltf.cpp", "image_io.cpp", "image_encode.cpp", "jpeg.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _inputs():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", "optpt.h")]
    inc = os.path.join(ROOT, "include", "optix_pt")
    files += [os.path.join(inc, f) for f in os.listdir(inc)]
    return files + [os.path.abspath(__file__)]


def _up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def build(force=False, verbose=False):
    if not force and _up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include")]
    jobs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD_DIR, src + ".o")
        jobs.append((obj, [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", *inc,
                           "-c", os.path.join(CSRC, src), "-o", obj]))
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD_DIR, src + ".o")
        jobs.append((obj, ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", *inc,
                           "-I", "/usr/local/cuda/include", "-c", os.path.join(CSRC, src), "-o", obj]))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[1]), jobs))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *[j[0] for j in jobs]])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
