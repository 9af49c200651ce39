"""optix_pt_gb300: GB300-native progressive path tracer behind optix_pt's render surface.

Python mirror of the reference's host interface (class Renderer,
include/renderer.h:19-206, and SceneDesc, include/scene_desc.h:9-39) over the
C ABI in include/optpt.h. The reference's method names are kept
(setupOutputBuffer, setupCamera, updateLaunchParams, launch, getFrameBuffer,
getSampleCount, resetSampleCount, set/getVis, set/getToneMapping*,
set/getGammaCorrection*); OptiX set-up steps that have no counterpart are
accepted as no-ops so a caller's init sequence runs unchanged.
"""
import ctypes

import numpy as np

from . import _ffi
from ._ffi import BSDF_QUERY, BSDF_RESULT, OptptError, check, lib

__all__ = ["Scene", "SceneDesc", "GltfModel", "Animator", "decode_png", "decode_jpeg", "encode_png", "encode_hdr", "encode_exr", "Renderer", "OptptError", "bsdf_batch", "BSDF_QUERY", "BSDF_RESULT",
           "library_path", "render_batch_scenes", "autotune"]

library_path = _ffi.LIB_PATH


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)  # torch.cuda.Stream


class Scene:
    """A flattened triangle scene (the reference's SceneProperties + SceneDesc)."""

    def __init__(self, struct, owned):
        self._s = struct
        self._owned = owned

    @classmethod
    def procedural(cls, name, seed=1):
        s = _ffi.SceneStruct()
        check(lib.optpt_scene_procedural(name.encode(), seed, ctypes.byref(s)))
        return cls(s, True)

    @classmethod
    def from_config(cls, scene_list_path):
        s = _ffi.SceneStruct()
        check(lib.optpt_scene_from_config(str(scene_list_path).encode(), ctypes.byref(s)))
        return cls(s, True)

    @classmethod
    def from_gltf(cls, path, up=(0.0, 1.0, 0.0)):
        """Imports a glTF 2.0 file (.gltf or .glb): GltfLoader + Renderer::loadScene."""
        s = _ffi.SceneStruct()
        u = (ctypes.c_float * 3)(*up)
        check(lib.optpt_scene_from_gltf(str(path).encode(), ctypes.cast(u, ctypes.c_void_p), ctypes.byref(s)))
        return cls(s, True)

    def textures(self):
        """Copies of the texture images: list of dicts (rgba HxWx4 uint8, wrapS, wrapT, srgb, filter)."""
        out = []
        for t in range(self._s.numTextures):
            tx = self._s.textures[t]
            px = np.ctypeslib.as_array(ctypes.cast(tx.rgba, ctypes.POINTER(ctypes.c_uint8)),
                                       shape=(tx.height * tx.width * 4,)).copy().reshape(tx.height, tx.width, 4)
            out.append({"rgba": px, "wrapS": tx.wrapS, "wrapT": tx.wrapT, "srgb": tx.srgb, "filter": tx.filter})
        return out

    def materials(self):
        """The MaterialData records as a list of ctypes structures (copies)."""
        return [_ffi.MaterialData.from_buffer_copy(self._s.materials[i]) for i in range(self._s.numMaterials)]

    def lights(self):
        return [_ffi.Light.from_buffer_copy(self._s.lights[i]) for i in range(self._s.numLights)]

    def __del__(self):
        if getattr(self, "_owned", False):
            lib.optpt_scene_release(ctypes.byref(self._s))
            self._owned = False

    @property
    def struct(self):
        return self._s

    @property
    def num_triangles(self):
        return self._s.numTriangles

    def _arr(self, ptr, n, width, dtype):
        if not ptr or n == 0:
            return None
        return np.ctypeslib.as_array(ptr, shape=(n * width,)).astype(dtype).reshape(n, width) if width > 1 else \
            np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype)

    def arrays(self):
        """Copies of the scene arrays as numpy (for the oracle and tests)."""
        s = self._s
        out = {
            "positions": self._arr(s.positions, s.numVertices, 3, np.float32),
            "normals": self._arr(s.normals, s.numVertices, 3, np.float32),
            "texCoords": self._arr(s.texCoords, s.numVertices, 2, np.float32),
            "triIndices": self._arr(s.triIndices, s.numTriangles, 3, np.int32),
            "matIndices": self._arr(s.matIndices, s.numTriangles, 1, np.int32),
            "materials": bytes(ctypes.string_at(s.materials, ctypes.sizeof(_ffi.MaterialData) * s.numMaterials)),
            "numMaterials": s.numMaterials,
            "lights": bytes(ctypes.string_at(s.lights, ctypes.sizeof(_ffi.Light) * s.numLights))
            if s.numLights else b"",
            "numLights": s.numLights,
            "camEye": list(s.camEye), "camTarget": list(s.camTarget), "camUp": list(s.camUp),
            "camFovYDeg": s.camFovYDeg, "resX": s.resX, "resY": s.resY, "bgColour": list(s.bgColour),
            "spp": s.spp, "maxDepth": s.maxDepth,
        }
        return out


    def save(self, path):
        """Writes the scene arrays, material and light records and textures to
        an .npz file that the oracle can read without this library
        (oracle.scene_file.load)."""
        a = self.arrays()
        out = {k: v for k, v in a.items() if v is not None and k not in ("materials", "lights")}
        out["materials"] = np.frombuffer(a["materials"], np.uint8)
        out["lights"] = np.frombuffer(a["lights"], np.uint8)
        for i, t in enumerate(self.textures()):
            out["texture%d" % i] = t["rgba"]
            out["texture%d_modes" % i] = np.array([t["wrapS"], t["wrapT"], t["srgb"], t["filter"]], np.int32)
        out["numTextures"] = len(self.textures())
        np.savez(path, **out)


def _decode(fn, data):
    img = _ffi.Image()
    buf = ctypes.create_string_buffer(bytes(data), len(data))
    check(fn(buf, len(data), ctypes.byref(img)))
    try:
        return np.ctypeslib.as_array(img.rgba, shape=(img.height * img.width * 4,)).copy().reshape(
            img.height, img.width, 4)
    finally:
        lib.optpt_image_release(ctypes.byref(img))


def decode_png(data):
    """Decodes PNG bytes to an HxWx4 uint8 array with the library's decoder."""
    return _decode(lib.optpt_image_decode_png, data)


def decode_jpeg(data):
    """Decodes baseline JPEG bytes to an HxWx4 uint8 array with the library's decoder."""
    return _decode(lib.optpt_image_decode_jpeg, data)


class GltfModel:
    """A glTF scene kept for posing (node tree, skins, one animation): the
    reference's GltfLoader + the animation half of Renderer::updateScene."""

    def __init__(self, path, up=(0.0, 1.0, 0.0)):
        self._h = None
        h = ctypes.c_void_p()
        u = (ctypes.c_float * 3)(*up)
        check(lib.optpt_gltf_open(str(path).encode(), ctypes.cast(u, ctypes.c_void_p), ctypes.byref(h)))
        self._h = h.value
        inf = _ffi.GltfInfo()
        check(lib.optpt_gltf_info(self._h, ctypes.byref(inf)))
        self.info = {k: getattr(inf, k) for k, _ in _ffi.GltfInfo._fields_}

    def close(self):
        if self._h:
            lib.optpt_gltf_close(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def scene(self, time=0.0, animate=False):
        s = _ffi.SceneStruct()
        check(lib.optpt_gltf_scene(self._h, time, 1 if animate else 0, ctypes.byref(s)))
        return Scene(s, True)

    def deformation(self):
        d = _ffi.Deformation()
        check(lib.optpt_gltf_deformation(self._h, ctypes.byref(d)))
        return d

    def pose(self, time):
        """(shape matrices (S, 16), shape normal matrices (S, 9), joint matrices (J, 16)) at `time`."""
        S, J = self.info["numShapes"], self.info["numJointSlots"]
        m = np.zeros((S, 16), np.float32)
        n = np.zeros((S, 9), np.float32)
        j = np.zeros((max(J, 1), 16), np.float32)
        check(lib.optpt_gltf_pose(self._h, time, m.ctypes.data, n.ctypes.data, j.ctypes.data))
        return m, n, j[:J]

    def apply(self, time):
        """Positions (and normals) of every vertex at `time`, evaluated on the host."""
        nv = self.info["numVertices"]
        p = np.zeros((nv, 3), np.float32)
        n = np.zeros((nv, 3), np.float32)
        check(lib.optpt_gltf_apply(self._h, time, p.ctypes.data, n.ctypes.data))
        return p, n


class Animator:
    """Drives a renderer from a GltfModel as the reference's per-frame
    updateScene does: the clock advances 0.02 per frame, the pose is
    evaluated on the host (a few matrices) and the vertices are deformed and
    the BVH refit on the GPU."""

    def __init__(self, renderer, model, dt=0.02):
        self.r, self.model, self.dt, self.t = renderer, model, dt, 0.0
        check(lib.optpt_set_deformation(renderer._h, ctypes.byref(model.deformation())))

    def pose(self, time, stream=None):
        self.t = time
        m, n, j = self.model.pose(time)
        check(lib.optpt_deform(self.r._h, m.ctypes.data, n.ctypes.data, j.ctypes.data if len(j) else None,
                               _stream_handle(stream)))

    def step(self, stream=None):
        self.pose(self.t + self.dt, stream)


def _encoded(fn, *args):
    out, size = ctypes.c_void_p(), ctypes.c_size_t()
    check(fn(*args, ctypes.byref(out), ctypes.byref(size)))
    try:
        return ctypes.string_at(out.value, size.value)
    finally:
        lib.optpt_free(out)


def encode_png(rgba):
    """(h, w, 4) uint8 -> PNG bytes (the library's encoder)."""
    a = np.ascontiguousarray(rgba, np.uint8)
    return _encoded(lib.optpt_encode_png, a.ctypes.data, a.shape[1], a.shape[0], a.shape[1] * 4)


def encode_hdr(rgba):
    """(h, w, 4) float32 -> Radiance RGBE bytes."""
    a = np.ascontiguousarray(rgba, np.float32)
    return _encoded(lib.optpt_encode_hdr, a.ctypes.data, a.shape[1], a.shape[0])


def encode_exr(rgba, compression=3):
    """(h, w, 4) float32 -> OpenEXR bytes (HALF A, B, G, R; A = 1)."""
    a = np.ascontiguousarray(rgba, np.float32)
    return _encoded(lib.optpt_encode_exr, a.ctypes.data, a.shape[1], a.shape[0], compression)


SceneDesc = Scene.from_config  # the reference constructs SceneDesc from the scene list


class Renderer:
    """The reference's Renderer (include/renderer.h:19-206) on the GB300 engine."""

    def __init__(self, scene, spp_batch=0, block_size=0, leaf_size=0, use_graph=True, bvh_width=8, compaction=0,
                 node_budget=0, tail_bounce=0, bvh_builder="lbvh"):
        """tail_bounce: first bounce finished by the path-completion kernel
        (0 = the library's default, -1 = none: per-bounce kernels only).
        bvh_builder: "lbvh" (default) or "ploc", the binary tree the 8-wide
        BVH is collapsed from (the binary BVH is always the LBVH)."""
        self.scene = scene
        if bvh_builder not in ("ploc", "lbvh"):
            raise ValueError("bvh_builder must be 'ploc' or 'lbvh'")
        opt = _ffi.Options(spp_batch, block_size, leaf_size, 1 if use_graph else 0, bvh_width, compaction,
                           node_budget, tail_bounce & 0xFFFFFFFF, 1 if bvh_builder == "ploc" else 0)
        h = ctypes.c_void_p()
        check(lib.optpt_create(ctypes.byref(scene.struct), ctypes.byref(opt), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib.optpt_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # ---- init sequence of the reference (src/main_window.cpp:36-49) ----
    def initOptix(self):
        pass

    def createContext(self):
        pass

    def loadScene(self):
        pass

    def buildAccel(self, build=True):
        pass

    def setupCompilationOptions(self):
        pass

    def createModules(self):
        pass

    def createProgramGroups(self):
        pass

    def createPipeline(self):
        pass

    def setupSbt(self):
        pass

    def createDenoiser(self):
        pass

    def createRandomState(self):
        pass

    def setupLaunchParams(self, scene_desc=None):
        pass

    def setupOutputBuffer(self, width, height):
        check(lib.optpt_setup_output_buffer(self._h, width, height))

    def setupCamera(self, eye, target, up, fov_y_deg):
        check(lib.optpt_setup_camera(self._h, _ffi.f3(*eye), _ffi.f3(*target), _ffi.f3(*up), fov_y_deg))

    # ---- per frame ----
    def launch_params(self):
        lp = _ffi.LaunchParams()
        check(lib.optpt_get_launch_params(self._h, ctypes.byref(lp)))
        return lp

    def updateLaunchParams(self, lp=None):
        if lp is not None:
            check(lib.optpt_set_launch_params(self._h, ctypes.byref(lp)))

    def _set(self, **kw):
        lp = self.launch_params()
        for k, v in kw.items():
            setattr(lp, k, v)
        check(lib.optpt_set_launch_params(self._h, ctypes.byref(lp)))

    def launch(self):
        """1 sample per pixel, wait, copy the frame buffer to host (src/renderer.cpp:940-958)."""
        check(lib.optpt_launch(self._h))

    def _frame_view(self, p, copy):
        if not p:
            return None
        lp = self.launch_params()
        a = np.ctypeslib.as_array(p, shape=(lp.h, lp.w, 4))
        return a.copy() if copy else a

    def launch_pipelined(self, copy=True):
        """launch() as a pipelined frame loop: renders a frame and starts its
        copy to host memory; returns the previous call's frame (None after a
        flush or a resize). With copy=False the array is a view of the
        renderer's pinned buffer, valid until the second call after."""
        p = ctypes.POINTER(ctypes.c_float)()
        check(lib.optpt_launch_pipelined(self._h, ctypes.byref(p)))
        return self._frame_view(p, copy)

    def launch_flush(self, copy=True):
        """The last pipelined frame, once its copy has finished (None if none is pending)."""
        p = ctypes.POINTER(ctypes.c_float)()
        check(lib.optpt_launch_flush(self._h, ctypes.byref(p)))
        return self._frame_view(p, copy)

    def getFrameBuffer(self):
        p = lib.optpt_get_frame_buffer(self._h)
        if not p:
            return None
        lp = self.launch_params()
        return np.ctypeslib.as_array(p, shape=(lp.h, lp.w, 4)).copy()

    def getSampleCount(self):
        return lib.optpt_get_sample_count(self._h)

    def resetSampleCount(self):
        check(lib.optpt_reset_sample_count(self._h))

    def setVis(self, vis):
        self._set(vis=vis)

    def getVis(self):
        return self.launch_params().vis

    def setToneMappingState(self, enable):
        self._set(toneMapping=1 if enable else 0)

    def getToneMappingState(self):
        return bool(self.launch_params().toneMapping)

    def setToneMappingImpl(self, impl):
        self._set(toneMappingImpl=impl)

    def getToneMappingImpl(self):
        return self.launch_params().toneMappingImpl

    def setGammaCorrectionState(self, enable):
        self._set(gammaCorrection=1 if enable else 0)

    def getGammaCorrectionState(self):
        return self.launch_params().gammaCorrection

    def setGammaCorrectionTerm(self, value):
        self._set(gammaTerm=value)

    def getGammaCorrectionTerm(self):
        return self.launch_params().gammaTerm

    def dumpFramebuffer(self, path=None):
        """Renderer::dumpFramebuffer: PNG of processImage's RGBA8 (default output.png)."""
        check(lib.optpt_save_image(self._h, 0, None if path is None else str(path).encode()))

    def dumpAccumFramebufferRgbe(self, path=None):
        """Renderer::dumpAccumFramebufferRgbe: Radiance .hdr of the mean radiance (default output.hdr)."""
        check(lib.optpt_save_image(self._h, 1, None if path is None else str(path).encode()))

    def dumpAccumFramebufferExr(self, path=None):
        """The EXR dump: HALF RGBA of the mean radiance, ZIP (default output.exr)."""
        check(lib.optpt_save_image(self._h, 2, None if path is None else str(path).encode()))

    def getDenoiserState(self):
        return False

    def setDenoiserState(self, on):
        if on:
            raise OptptError(-1, "the OptiX denoiser is not part of this renderer")

    # ---- extensions ----
    def set_max_depth(self, depth):
        self._set(maxDepth=depth)

    def set_seed(self, seed):
        self._set(seed=seed)

    def render(self, spp, stream=None):
        check(lib.optpt_render(self._h, spp, _stream_handle(stream)))

    def frame_buffer(self, stream=None):
        lp = self.launch_params()
        out = np.empty((lp.h, lp.w, 4), np.float32)
        check(lib.optpt_read_frame_buffer(self._h, out.ctypes.data, _stream_handle(stream)))
        return out

    def accum(self, stream=None):
        """FP64 per-pixel (sum, sum of squares, samples): arrays (h, w, 3)."""
        lp = self.launch_params()
        s = np.empty((lp.h, lp.w, 4), np.float64)
        q = np.empty((lp.h, lp.w, 4), np.float64)
        check(lib.optpt_read_accum(self._h, s.ctypes.data, q.ctypes.data, _stream_handle(stream)))
        return s[..., :3], q[..., :3], self.getSampleCount()

    def rgba8(self, stream=None):
        """processImage's packed RGBA8 of the tone-mapped frame: (h, w, 4) uint8."""
        lp = self.launch_params()
        out = np.empty((lp.h, lp.w), np.uint32)
        check(lib.optpt_read_rgba8(self._h, out.ctypes.data, _stream_handle(stream)))
        return out.view(np.uint8).reshape(lp.h, lp.w, 4)

    def image_out(self, rgba8=None, rgbe=None, half_rows=None, stream=None):
        """The fused output kernel into caller device buffers (torch tensors or None)."""
        ptr = (lambda t: None if t is None else t.data_ptr())
        check(lib.optpt_image_out(self._h, ptr(rgba8), ptr(rgbe), ptr(half_rows), _stream_handle(stream)))

    def update_vertices(self, positions, normals=None, stream=None):
        p = np.ascontiguousarray(positions, np.float32)
        n = None if normals is None else np.ascontiguousarray(normals, np.float32)
        # pageable host memory: the copy has consumed the arrays when the call returns
        check(lib.optpt_update_vertices(self._h, p.ctypes.data, None if n is None else n.ctypes.data,
                                        _stream_handle(stream)))

    def read_vertices(self, stream=None):
        nv = self.scene.struct.numVertices
        p = np.empty((nv, 3), np.float32)
        n = np.empty((nv, 3), np.float32)
        check(lib.optpt_read_vertices(self._h, p.ctypes.data, n.ctypes.data, _stream_handle(stream)))
        return p, n

    def refit_profile(self, reps=20):
        """Milliseconds per BVH8 refit of the current vertices."""
        ms = ctypes.c_float()
        check(lib.optpt_refit_profiled(self._h, reps, ctypes.byref(ms)))
        return ms.value

    def image_out_profile(self, reps=20):
        """Milliseconds per output-kernel launch (all payloads, L2 evicted before each)."""
        ms = ctypes.c_float()
        check(lib.optpt_image_out_profiled(self._h, reps, ctypes.byref(ms)))
        return ms.value

    def device_buffers(self):
        fb, afb, s, q = (ctypes.c_void_p() for _ in range(4))
        check(lib.optpt_device_buffers(self._h, ctypes.byref(fb), ctypes.byref(afb), ctypes.byref(s),
                                       ctypes.byref(q)))
        return fb.value, afb.value, s.value, q.value

    def stats(self):
        st = _ffi.Stats()
        check(lib.optpt_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _ffi.Stats._fields_}

    def profile(self, spp, stream=None):
        kt = _ffi.KernelTimes()
        check(lib.optpt_render_profiled(self._h, spp, _stream_handle(stream), ctypes.byref(kt)))
        names = ["generate", "extend", "shade", "shadow", "accumulate", "guide_infer", "guide_train", "finish"]
        return {"ms": dict(zip(names, list(kt.ms))), "launches": dict(zip(names, list(kt.launches))),
                "extensionRays": kt.extensionRays, "shadowRays": kt.shadowRays}

    def queue_counts(self):
        """Per-bounce queue lengths of the last pass: (extension, point shadow, emissive shadow)."""
        d = self.launch_params().maxDepth
        a, b, c = (np.zeros(d, np.uint32) for _ in range(3))
        check(lib.optpt_queue_counts(self._h, a.ctypes.data, b.ctypes.data, c.ctypes.data, d))
        return a, b, c

    def traversal_counts(self, spp, stream=None):
        c = _ffi.TraversalCounts()
        check(lib.optpt_traversal_counts(self._h, spp, _stream_handle(stream), ctypes.byref(c)))
        return {k: getattr(c, k) for k, _ in _ffi.TraversalCounts._fields_}

    def trace(self, rays_ptr, hits_ptr, n, any_hit=False, stream=None):
        """Device pointers: rays (2 x float4 per ray), hits (float4 per ray)."""
        check(lib.optpt_trace(self._h, rays_ptr, hits_ptr, n, 1 if any_hit else 0, _stream_handle(stream)))

    def bvh_leaf_order(self):
        n = self.scene.num_triangles
        codes = np.zeros(n, np.uint32)
        order = np.zeros(n, np.int32)
        check(lib.optpt_bvh_leaf_order(self._h, codes.ctypes.data, order.ctypes.data))
        return codes, order

    def bvh8_nodes(self):
        """(nodes as (N, 80) uint8, primitive per BVH8 triangle slot)."""
        cnt = ctypes.c_uint32()
        check(lib.optpt_bvh8_nodes(self._h, None, 0, ctypes.byref(cnt), None))
        nodes = np.zeros((max(cnt.value, 1), 80), np.uint8)
        order = np.zeros(max(self.scene.num_triangles, 1), np.int32)
        check(lib.optpt_bvh8_nodes(self._h, nodes.ctypes.data, cnt.value, ctypes.byref(cnt), order.ctypes.data))
        return nodes[:cnt.value], order[:self.scene.num_triangles]

    def set_guiding(self, mode):
        """0: plain BSDF sampling; 1: learned guiding with online training;
        2: learned guiding, network frozen."""
        check(lib.optpt_set_guiding(self._h, int(mode)))

    def render_batch(self, views, stream=None):
        """Renders views [(eye, target, up, fovYDeg, width, height, spp), ...]
        of this scene in shared wavefront passes."""
        arr = (_ffi.View * len(views))()
        for i, (eye, target, up, fov, w, h, spp) in enumerate(views):
            arr[i] = _ffi.View(_ffi.f3(*eye), _ffi.f3(*target), _ffi.f3(*up), fov, w, h, spp, 0)
        check(lib.optpt_render_batch(self._h, arr, len(views), _stream_handle(stream)))
        self._batch_shapes = [(v[4], v[5]) for v in views]

    def batch_view(self, v, stream=None):
        """(sum (h*w, 3) float64, sum of squares, samples) of batch view v."""
        n = ctypes.c_uint32()
        check(lib.optpt_batch_view(self._h, v, None, None, None, ctypes.byref(n)))
        w, h = self._batch_shapes[v]
        s = np.zeros((h * w, 4), np.float64)
        q = np.zeros((h * w, 4), np.float64)
        check(lib.optpt_batch_read_view(self._h, v, s.ctypes.data, q.ctypes.data, _stream_handle(stream)))
        return s[:, :3], q[:, :3], n.value

    def guiding_options(self, **kw):
        """Reads, and with keyword arguments updates, the guiding controls
        (trainSteps, trainStride, maxDepth, alphaMin, alphaMax, alphaRamp,
        learningRate, lobeLoss)."""
        o = _ffi.GuidingOptions()
        if kw:
            for k, v in kw.items():
                setattr(o, k, v)
            check(lib.optpt_set_guiding_options(self._h, ctypes.byref(o)))
        check(lib.optpt_get_guiding_options(self._h, ctypes.byref(o)))
        return {k: getattr(o, k) for k, _ in o._fields_}

    def guiding_batch(self):
        """The last pass's training samples, (n, 16) float32."""
        n = ctypes.c_uint32()
        check(lib.optpt_guiding_batch(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), 16), np.float32)
        check(lib.optpt_guiding_batch(self._h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out[:n.value]

    def guide(self):
        """The renderer's guiding network (owned by the renderer), or None."""
        h = ctypes.c_void_p()
        check(lib.optpt_get_guide(self._h, ctypes.byref(h)))
        return None if not h.value else Guide._borrow(h, self)

    def bvh_nodes(self):
        cnt = ctypes.c_uint32()
        check(lib.optpt_bvh_nodes(self._h, None, 0, ctypes.byref(cnt)))
        nodes = np.zeros((max(cnt.value, 1), 4), np.int32)
        check(lib.optpt_bvh_nodes(self._h, nodes.ctypes.data, cnt.value, ctypes.byref(cnt)))
        return nodes[:cnt.value]


def relmse(sum_ptr, n_samples, ref_ptr, num_pixels, out_ptr, stream=None):
    """GPU FP64 relMSE of sum / n_samples against ref (double4 per pixel, device pointers)."""
    check(lib.optpt_relmse(sum_ptr, n_samples, ref_ptr, num_pixels, out_ptr, _stream_handle(stream)))


def bsdf_batch(queries_ptr, results_ptr, n, stream=None):
    """Device BSDF queries (optpt_bsdf_query -> optpt_bsdf_result), device pointers."""
    check(lib.optpt_bsdf_batch(queries_ptr, results_ptr, n, _stream_handle(stream)))


class Guide:
    """The learned path-guiding network (hash grid + MLP on the tensor cores,
    8 vMF lobes out) over the world-space box [lo, hi]."""

    MLP_PARAMS = 5 * 64 * 64
    HASH_PARAMS = 16 * (1 << 19) * 2

    def __init__(self, lo, hi, seed=1):
        h = ctypes.c_void_p()
        check(lib.optpt_guide_create(_ffi.f3(*lo), _ffi.f3(*hi), seed, ctypes.byref(h)))
        self._h = h

    @classmethod
    def _borrow(cls, handle, owner):
        g = cls.__new__(cls)
        g._h = handle
        g._owner = owner     # keeps the renderer (which frees the network) alive
        return g

    def close(self):
        if getattr(self, "_h", None) and getattr(self, "_owner", None) is None:
            lib.optpt_guide_destroy(self._h)
        self._h = None

    __del__ = close

    def params(self):
        mlp = np.zeros(self.MLP_PARAMS, np.float32)
        hsh = np.zeros(self.HASH_PARAMS, np.float32)
        check(lib.optpt_guide_params(self._h, mlp.ctypes.data, hsh.ctypes.data, 0))
        return mlp, hsh

    def set_params(self, mlp=None, hash_params=None):
        m = None if mlp is None else np.ascontiguousarray(mlp, np.float32)
        hp = None if hash_params is None else np.ascontiguousarray(hash_params, np.float32)
        check(lib.optpt_guide_params(self._h, None if m is None else m.ctypes.data,
                                     None if hp is None else hp.ctypes.data, 1))

    def geometry(self):
        """(level resolutions, dense flags, lo, invExt) as the oracle takes them."""
        res = np.zeros(16, np.float32)
        dense = np.zeros(16, np.uint32)
        lo = np.zeros(3, np.float32)
        inv = np.zeros(3, np.float32)
        check(lib.optpt_guide_levels(self._h, res.ctypes.data, dense.ctypes.data, lo.ctypes.data, inv.ctypes.data))
        return res, dense, lo, inv

    def infer(self, queries_ptr, n, mixtures_ptr, stream=None):
        check(lib.optpt_guide_infer(self._h, queries_ptr, n, mixtures_ptr, _stream_handle(stream)))

    @staticmethod
    def mixture_eval(mixtures_ptr, n, xi_ptr, dir_pdf_ptr, stream=None):
        """The renderer's mixture sampler and density (device pointers):
        with xi_ptr, rows of (direction, density) drawn as a guided vertex
        draws them; with xi_ptr None, densities at the given directions."""
        check(lib.optpt_guide_mixture_eval(mixtures_ptr, n, xi_ptr, dir_pdf_ptr, _stream_handle(stream)))

    def gradients(self, samples_ptr, count_ptr, capacity, stream=None):
        dm = np.zeros(self.MLP_PARAMS, np.float32)
        dh = np.zeros(self.HASH_PARAMS, np.float32)
        loss = ctypes.c_double()
        check(lib.optpt_guide_gradients(self._h, samples_ptr, count_ptr, capacity, dm.ctypes.data, dh.ctypes.data,
                                        ctypes.byref(loss), _stream_handle(stream)))
        return loss.value, dm, dh

    def train_step(self, samples_ptr, count_ptr, capacity, stream=None):
        check(lib.optpt_guide_train_step(self._h, samples_ptr, count_ptr, capacity, _stream_handle(stream)))

    def status(self):
        """(tensor-core wait expired?, loss of the last step, its samples)."""
        st = ctypes.c_int()
        loss = ctypes.c_double()
        n = ctypes.c_double()
        check(lib.optpt_guide_status(self._h, ctypes.byref(st), ctypes.byref(loss), ctypes.byref(n)))
        return st.value, loss.value, n.value


def render_batch_scenes(renderers, views, stream=None):
    """Views of several scenes in one batch (optpt_render_batch_scenes):
    views = [(scene index, (eye, target, up, fovYDeg, width, height, spp)),
    ...]; renderers[k] renders scene k. Every pass is one graph launch over
    all scenes. Afterwards renderers[k].batch_view(j) is the j-th view of
    scene k; returns, per view in the order given, (k, j)."""
    arr = (_ffi.View * len(views))()
    where, count = [], [0] * len(renderers)
    for i, (k, (eye, target, up, fov, w, h, spp)) in enumerate(views):
        arr[i] = _ffi.View(_ffi.f3(*eye), _ffi.f3(*target), _ffi.f3(*up), fov, w, h, spp, k)
        where.append((k, count[k]))
        count[k] += 1
    hs = (ctypes.c_void_p * len(renderers))(*[r._h.value for r in renderers])
    check(lib.optpt_render_batch_scenes(hs, len(renderers), arr, len(views), _stream_handle(stream)))
    for k, r in enumerate(renderers):
        r._batch_shapes = [(v[4], v[5]) for kk, v in views if kk == k]
    return where


def autotune(scene, width, height, spp, warmup_spp=2, guiding=0):
    """Times every (tree, block size, compaction) candidate on `scene`;
    returns (best options as a dict, [trial dicts])."""
    req = _ffi.AutotuneRequest(width, height, spp, warmup_spp, guiding)
    best = _ffi.Options()
    trials = (_ffi.AutotuneTrial * 64)()
    n = ctypes.c_uint32()
    check(lib.optpt_autotune(ctypes.byref(scene.struct), ctypes.byref(req), ctypes.byref(best), trials, 64,
                             ctypes.byref(n)))
    opts = lambda o: {k: getattr(o, k) for k, _ in o._fields_}
    return opts(best), [dict(opts(t.options), samples_per_s=t.samplesPerS, mrays_per_s=t.mraysPerS)
                        for t in trials[:n.value]]
