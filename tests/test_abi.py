"""The C ABI boundary: the library loads, exports every declared entry point,
and the struct layouts seen by C, ctypes and numpy agree (no GPU needed)."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "optpt.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(optpt_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    from optix_pt_gb300 import _ffi
    names = _declared()
    assert len(names) >= 25
    lib = ctypes.CDLL(_ffi.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows them all
    assert set(names) <= set(_ffi.EXPORTS)


def test_version_and_error_message(built):
    from optix_pt_gb300 import _ffi
    assert _ffi.lib.optpt_version() >= 100
    rc = _ffi.lib.optpt_scene_procedural(b"no-such-scene", 1, ctypes.byref(_ffi.SceneStruct()))
    assert rc == -1
    assert b"no-such-scene" in _ffi.lib.optpt_last_error()


C_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "optpt.h"
#define S(T) printf(#T " %zu\n", sizeof(T))
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  S(Light); S(MaterialData); S(LaunchParams); S(optpt_scene); S(optpt_texture); S(optpt_options);
  S(optpt_stats); S(optpt_kernel_times); S(optpt_bsdf_query); S(optpt_bsdf_result); S(TextureTransform);
  S(optpt_guiding_options); S(optpt_view); S(optpt_autotune_request); S(optpt_autotune_trial);
  S(optpt_gltf_info_t); S(optpt_deformation); S(optpt_image);
  O(optpt_deformation, numVertices); O(optpt_guiding_options, trainSpp);
  O(MaterialData, baseColour); O(MaterialData, ior); O(MaterialData, category); O(MaterialData, hasSheenRoughnessTexture);
  O(LaunchParams, traversable); O(LaunchParams, gammaTerm); O(LaunchParams, bgColour);
  O(optpt_scene, camEye); O(optpt_scene, maxDepth); O(optpt_bsdf_query, xs); O(optpt_bsdf_result, pdf);
  return 0;
}
"""


def test_struct_layouts_match_c(built):
    from optix_pt_gb300 import _ffi
    cc = "gcc"
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(src, "w").write(C_PROBE)
        p = subprocess.run([cc, "-I", os.path.join(ROOT, "include"), src, "-o", exe], capture_output=True,
                           text=True)
        if p.returncode != 0:
            pytest.skip("no C compiler: " + p.stderr[:200])
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    c = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    c = {k: int(v) for k, v in c.items()}
    py = {"Light": _ffi.Light, "MaterialData": _ffi.MaterialData, "LaunchParams": _ffi.LaunchParams,
          "optpt_scene": _ffi.SceneStruct, "optpt_texture": _ffi.Texture, "optpt_options": _ffi.Options,
          "optpt_stats": _ffi.Stats, "optpt_kernel_times": _ffi.KernelTimes,
          "TextureTransform": _ffi.TextureTransform, "optpt_guiding_options": _ffi.GuidingOptions,
          "optpt_view": _ffi.View, "optpt_autotune_request": _ffi.AutotuneRequest,
          "optpt_autotune_trial": _ffi.AutotuneTrial, "optpt_gltf_info_t": _ffi.GltfInfo,
          "optpt_deformation": _ffi.Deformation, "optpt_image": _ffi.Image}
    for name, cls in py.items():
        assert ctypes.sizeof(cls) == c[name], name
    assert _ffi.BSDF_QUERY.itemsize == c["optpt_bsdf_query"]
    assert _ffi.BSDF_RESULT.itemsize == c["optpt_bsdf_result"]
    assert _ffi.MaterialData.ior.offset == c["MaterialData.ior"]
    assert _ffi.MaterialData.category.offset == c["MaterialData.category"]
    assert _ffi.LaunchParams.traversable.offset == c["LaunchParams.traversable"]
    assert _ffi.LaunchParams.bgColour.offset == c["LaunchParams.bgColour"]
    assert _ffi.SceneStruct.maxDepth.offset == c["optpt_scene.maxDepth"]
    assert _ffi.Deformation.numVertices.offset == c["optpt_deformation.numVertices"]
    assert _ffi.GuidingOptions.trainSpp.offset == c["optpt_guiding_options.trainSpp"]
    assert _ffi.BSDF_QUERY.fields["xs"][1] == c["optpt_bsdf_query.xs"]
    assert _ffi.BSDF_RESULT.fields["pdf"][1] == c["optpt_bsdf_result.pdf"]


CPP_DROPIN = r"""
#include "optix_pt/renderer.hpp"
#include <cstdio>
int main(int argc, char **argv) {
    optix_pt::SceneDesc sd(argv[1]);
    std::printf("%d %d %u\n", sd.resX, sd.resY, sd.scene.numTriangles);
    try { optix_pt::SceneDesc bad("/nonexistent/list.json"); return 2; }
    catch (const std::runtime_error &) { std::printf("caught\n"); }
    return 0;
}
"""


def test_cpp_dropin_header_compiles_and_parses_configs(built):
    """include/optix_pt/renderer.hpp: the reference-named C++ classes over the C ABI."""
    from optix_pt_gb300 import _ffi
    libdir = os.path.dirname(_ffi.LIB_PATH)
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "t.cpp"), os.path.join(d, "t")
        open(src, "w").write(CPP_DROPIN)
        p = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o",
                            exe, "-L", libdir, "-loptpt", "-Wl,-rpath," + libdir], capture_output=True, text=True)
        if p.returncode != 0:
            if "not found" in p.stderr and "g++" in p.stderr:
                pytest.skip("no C++ compiler")
            raise AssertionError(p.stderr)
        out = subprocess.run([exe, os.path.join(ROOT, "configs", "scene_selection.json")], capture_output=True,
                             text=True, check=True).stdout.split()
    assert out[:3] == ["512", "512", "36"] and out[3] == "caught"


def test_oracle_query_layout_matches_product(built):
    from optix_pt_gb300 import _ffi
    from oracle.abi import BSDF_QUERY
    assert BSDF_QUERY.itemsize == _ffi.BSDF_QUERY.itemsize
    assert list(BSDF_QUERY.names) == list(_ffi.BSDF_QUERY.names)
    assert np.dtype(BSDF_QUERY).descr == np.dtype(_ffi.BSDF_QUERY).descr


def test_calls_without_gpu_fail_cleanly(built):
    """Argument validation happens before any device work and reports errors."""
    from optix_pt_gb300 import _ffi
    h = ctypes.c_void_p()
    assert _ffi.lib.optpt_create(None, None, ctypes.byref(h)) == -1
    assert _ffi.lib.optpt_render(None, 1, None) == -1
    assert _ffi.lib.optpt_launch(None) == -1
    assert _ffi.lib.optpt_get_frame_buffer(None) is None or not _ffi.lib.optpt_get_frame_buffer(None)
    # pipelined frame loop: a NULL renderer or output pointer is refused
    frame = ctypes.POINTER(ctypes.c_float)()
    assert _ffi.lib.optpt_launch_pipelined(None, ctypes.byref(frame)) == -1
    assert _ffi.lib.optpt_launch_flush(None, ctypes.byref(frame)) == -1
    assert _ffi.lib.optpt_guide_mixture_eval(None, 4, None, None, None) == -1


def test_renderer_rejects_an_unknown_tree_builder(built):
    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("cornell")
    with pytest.raises(ValueError):
        opt.Renderer(sc, bvh_builder="sah")
