"""ctypes wrapper of the oracle library (test infrastructure only)."""
import ctypes
import os

import numpy as np

from .abi import BSDF_QUERY, BSDF_RESULT

HERE = os.path.dirname(os.path.abspath(__file__))
_libs = {}
_ref = None


def lib(variant=""):
    """The oracle library; variant "fma" is the build with floating-point
    contraction (a second FP32 rounding of the same algorithm)."""
    _lib = _libs.get(variant)
    if _lib is None:
        from .build import build_oracle
        _lib = ctypes.CDLL(build_oracle(variant=variant))
        _libs[variant] = _lib
        P = ctypes.c_void_p
        _lib.orc_scene_view.restype = P
        _lib.orc_scene_view.argtypes = [P, ctypes.c_int]
        _lib.orc_scene_view_free.argtypes = [P]
        _lib.orc_bvh.argtypes = [P, P, P, P, ctypes.c_uint32, P]
        _lib.orc_bvh8.argtypes = [P, P, ctypes.c_uint32, P, P]
        _lib.orc_trace.argtypes = [P, P, P, ctypes.c_uint32, ctypes.c_int, ctypes.c_int]
        _lib.orc_render.argtypes = [P, P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_int, ctypes.c_int, P, P, P, ctypes.c_int]
        for f in ("orc_bsdf_query_f32", "orc_bsdf_query_f64"):
            getattr(_lib, f).argtypes = [P, P, ctypes.c_int]
        _lib.orc_tonemap_f64.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double]
        _lib.orc_light_sample_f64.argtypes = [P, P, P, ctypes.c_int]
        _lib.orc_barycentric_f64.argtypes = [P, P, P, ctypes.c_int]
    return _lib


def ref():
    """The reference's own headers compiled for the host, or None if unavailable."""
    global _ref
    if _ref is None:
        from .build import REF_LIB, build_reference
        path = build_reference()
        if path is None:
            path = REF_LIB if os.path.exists(REF_LIB) else None
        if path is None:
            return None
        _ref = ctypes.CDLL(path)
    return _ref


def bsdf_query(q, precision=64):
    q = np.ascontiguousarray(q, dtype=BSDF_QUERY)
    r = np.zeros(len(q), BSDF_RESULT)
    fn = lib().orc_bsdf_query_f64 if precision == 64 else lib().orc_bsdf_query_f32
    fn(q.ctypes.data, r.ctypes.data, len(q))
    return r


def ref_bsdf_query(q):
    q = np.ascontiguousarray(q, dtype=BSDF_QUERY)
    r = np.zeros(len(q), BSDF_RESULT)
    ref().ref_bsdf_query(ctypes.c_void_p(q.ctypes.data), ctypes.c_void_p(r.ctypes.data), len(q))
    return r


def tonemap(rgba, tone=True, impl=1, gamma=True, gamma_term=2.2):
    x = np.ascontiguousarray(rgba, dtype=np.float64).reshape(-1, 4)
    y = np.empty_like(x)
    lib().orc_tonemap_f64(x.ctypes.data, y.ctypes.data, len(x), int(tone), impl, int(gamma), gamma_term)
    return y


class SceneView:
    """Host BVH + integrator over a product scene struct (same memory layout)."""

    def __init__(self, scene_struct, leaf_size=4, variant=""):
        self._keep = scene_struct
        self._lib = lib(variant)
        self._h = self._lib.orc_scene_view(ctypes.addressof(scene_struct), leaf_size)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_scene_view_free(self._h)
            self._h = None

    def bvh(self, n_tris):
        counts = np.zeros(3, np.uint32)
        self._lib.orc_bvh(self._h, None, None, None, 0, counts.ctypes.data)
        codes = np.zeros(n_tris, np.uint32)
        order = np.zeros(n_tris, np.int32)
        nodes = np.zeros((max(int(counts[0]), 1), 4), np.int32)
        rc = self._lib.orc_bvh(self._h, codes.ctypes.data, order.ctypes.data, nodes.ctypes.data, int(counts[0]),
                           counts.ctypes.data)
        assert rc == 0
        return codes, order, nodes[:counts[0]], int(counts[1]), int(counts[2])

    def bvh8(self, n_tris):
        """(nodes as a (N, 80) uint8 array, primitive per BVH8 triangle slot)."""
        counts = np.zeros(4, np.uint32)
        self._lib.orc_bvh8(self._h, None, 0, None, counts.ctypes.data)
        nodes = np.zeros((max(int(counts[0]), 1), 80), np.uint8)
        order = np.zeros(max(n_tris, 1), np.int32)
        rc = self._lib.orc_bvh8(self._h, nodes.ctypes.data, int(counts[0]), order.ctypes.data, counts.ctypes.data)
        assert rc == 0
        return nodes[:counts[0]], order[:n_tris]

    def trace(self, rays, any_hit=False, threads=None):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.zeros((len(rays), 4), np.float32)
        self._lib.orc_trace(self._h, rays.ctypes.data, hits.ctypes.data, len(rays), int(any_hit),
                        threads or os.cpu_count())
        return hits

    def render(self, camera15, w, h, seed, sample_base, spp, max_depth, y0=0, y1=None, precision=64,
               threads=None, sums=None, vis=0):
        y1 = h if y1 is None else y1
        if sums is None:
            sums = (np.zeros((h * w, 3)), np.zeros((h * w, 3)))
        cnt = np.zeros(4, np.uint64)
        cam = np.ascontiguousarray(camera15, dtype=np.float32)
        self._lib.orc_render(self._h, cam.ctypes.data, w, h, seed, sample_base, spp, max_depth, y0, y1, precision,
                         threads or os.cpu_count(), sums[0].ctypes.data, sums[1].ctypes.data, cnt.ctypes.data, vis)
        return sums[0], sums[1], cnt
