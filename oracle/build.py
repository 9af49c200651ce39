"""Build recipe for the oracle (test infrastructure).

* oracle/liboracle.so: the project's CPU restatement (oracle_capi.cpp,
  oracle_render.cpp), compiled with g++ without floating-point contraction.
* oracle/liboracle_fma.so: the same sources with contraction allowed (fused
  multiply-adds wherever the compiler forms them, on hosts that have them):
  a second FP32 evaluation of the same algorithm that rounds differently,
  used to tell rounding-sensitive pixels of a paired render apart.
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
# The reference tree: $OPTIX_PT_REFERENCE, else a `reference` directory beside
# the repository. Absent on GPU hosts, where only the oracle is built.
REFERENCE = os.environ.get("OPTIX_PT_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
LIB = os.path.join(HERE, "liboracle.so")
LIB_FMA = os.path.join(HERE, "liboracle_fma.so")
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


def build_oracle(force=False, variant=""):
    """variant "": no floating-point contraction; "fma": contraction allowed."""
    lib = LIB_FMA if variant == "fma" else LIB
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle_bsdf.hpp"), os.path.join(HERE, "query_abi.h"),
                   os.path.join(ROOT, "include", "optpt.h"), os.path.abspath(__file__)]
    if not force and _newer(lib, deps):
        return lib
    tmp = lib + ".tmp"
    contract = "-ffp-contract=fast" if variant == "fma" else "-ffp-contract=off"
    _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", contract, "-I", HERE,
          "-I", os.path.join(ROOT, "include"), *srcs, "-o", tmp])
    os.replace(tmp, lib)
    return lib


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
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(3) as ex:
        jobs = [ex.submit(build_oracle, force), ex.submit(build_oracle, force, "fma"), ex.submit(build_reference, force)]
        return tuple(j.result() for j in jobs)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
