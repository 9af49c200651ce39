"""Build recipe for the oracle (test infrastructure).

* oracle/liboracle.so: the project's CPU restatement (oracle_capi.cpp,
  oracle_render.cpp), compiled with g++ without floating-point contraction.
* oracle/_ref/libref.so: the reference's own BSDF, light-sampling, tone-map
  and barycentric headers plus src/light.cpp, compiled UNMODIFIED for the host
  from the reference tree, with the stand-in headers in oracle/ref_shim.
  Built only where the reference tree is present (it is not on GPU hosts).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE = os.environ.get("OPTIX_PT_REFERENCE", "/root/reference")
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")

ORACLE_SOURCES = ["oracle_capi.cpp", "oracle_render.cpp"]


def _newer(target, inputs):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(f) <= t for f in inputs)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))


def build_oracle(force=False):
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle_bsdf.hpp"), os.path.join(HERE, "query_abi.h"),
                   os.path.join(ROOT, "include", "optpt.h"), os.path.abspath(__file__)]
    if not force and _newer(LIB, deps):
        return LIB
    tmp = LIB + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I", HERE,
          "-I", os.path.join(ROOT, "include"), *srcs, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


def build_reference(force=False):
    """Returns the path of libref.so, or None when the reference tree is absent."""
    inc = os.path.join(REFERENCE, "include")
    if not os.path.isdir(inc):
        return None
    drv = os.path.join(HERE, "ref_driver.cpp")
    shim = os.path.join(HERE, "ref_shim")
    deps = [drv, os.path.join(HERE, "query_abi.h"), os.path.abspath(__file__)]
    deps += [os.path.join(dp, f) for dp, _, fs in os.walk(shim) for f in fs]
    if not force and _newer(REF_LIB, deps):
        return REF_LIB
    os.makedirs(os.path.dirname(REF_LIB), exist_ok=True)
    tmp = REF_LIB + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I", shim, "-I", HERE,
          "-I", inc, "-I", os.path.join(REFERENCE, "cu"), "-I", "/usr/local/cuda/include",
          drv, os.path.join(REFERENCE, "src", "light.cpp"), "-o", tmp])
    os.replace(tmp, REF_LIB)
    return REF_LIB


def build(force=False):
    return build_oracle(force), build_reference(force)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
