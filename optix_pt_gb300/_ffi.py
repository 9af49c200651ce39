"""ctypes binding of the optpt C ABI (include/optpt.h).

Loads the in-tree optix_pt_gb300/_lib/liboptpt.so. There is no fallback: if
the library is missing the import fails with an error naming the build step.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liboptpt.so")

OPTPT_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "I/O error", -4: "parse error",
          -5: "out of memory", -6: "device wait timed out", -7: "call out of order"}


class OptptError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("liboptpt.so is not built (%s): run "
                          "python -c 'import __graft_entry__ as g; g.build()'" % LIB_PATH)
    return ctypes.CDLL(LIB_PATH)


lib = _load()

f3 = ctypes.c_float * 3


class Light(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("radiance", f3), ("colour", f3), ("power", f3), ("p0", f3),
                ("p1", f3), ("p2", f3), ("normal", f3), ("v1", f3), ("v2", f3), ("area", ctypes.c_float),
                ("radius", ctypes.c_float), ("distance", ctypes.c_float), ("widthRad", ctypes.c_float),
                ("cosWidth", ctypes.c_float), ("cosFalloffStart", ctypes.c_float)]


class TextureTransform(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_float * 2), ("scale", ctypes.c_float * 2), ("rotation", ctypes.c_float)]


class MaterialData(ctypes.Structure):
    _fields_ = [("baseColourTexture", ctypes.c_int32), ("normalTexture", ctypes.c_int32),
                ("metallicRoughnessTexture", ctypes.c_int32), ("emissiveTexture", ctypes.c_int32),
                ("sheenColourTexture", ctypes.c_int32), ("sheenRoughnessTexture", ctypes.c_int32),
                ("baseColour", ctypes.c_float * 4), ("alphaMode", ctypes.c_int32), ("alphaCutoff", ctypes.c_float),
                ("sheenColour", f3), ("emission", f3),
                ("baseColourTexTf", TextureTransform), ("normalTexTf", TextureTransform),
                ("metallicRoughnessTexTf", TextureTransform), ("emissiveTexTf", TextureTransform),
                ("sheenColourTexTf", TextureTransform), ("sheenRoughnessTexTf", TextureTransform),
                ("ior", ctypes.c_float), ("roughness", ctypes.c_float), ("metallic", ctypes.c_float),
                ("specular", ctypes.c_float), ("transmissionWeight", ctypes.c_float),
                ("subsurfaceWeight", ctypes.c_float), ("coatWeight", ctypes.c_float),
                ("coatRoughness", ctypes.c_float), ("sheenRoughness", ctypes.c_float),
                ("type", ctypes.c_uint32), ("category", ctypes.c_uint32),
                ("hasBaseColourTexture", ctypes.c_uint8), ("hasNormalTexture", ctypes.c_uint8),
                ("hasMetallicRoughnessTexture", ctypes.c_uint8), ("hasEmissiveTexture", ctypes.c_uint8),
                ("hasSheenColourTexture", ctypes.c_uint8), ("hasSheenRoughnessTexture", ctypes.c_uint8),
                ("pad", ctypes.c_uint8 * 2)]


class LaunchParams(ctypes.Structure):
    _fields_ = [("frameBuffer", ctypes.c_void_p), ("accumFrameBuffer", ctypes.c_void_p),
                ("w", ctypes.c_uint32), ("h", ctypes.c_uint32), ("sample", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("eye", f3), ("U", f3), ("V", f3), ("W", f3),
                ("traversable", ctypes.c_uint64), ("lights", ctypes.c_void_p), ("numLights", ctypes.c_uint32),
                ("numEmissiveTriangles", ctypes.c_uint32), ("randState", ctypes.c_void_p), ("vis", ctypes.c_int32),
                ("toneMapping", ctypes.c_int32), ("toneMappingImpl", ctypes.c_int32),
                ("gammaCorrection", ctypes.c_int32), ("gammaTerm", ctypes.c_float),
                ("maxDepth", ctypes.c_uint32), ("bgColour", f3)]


class Texture(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("rgba", ctypes.c_void_p),
                ("wrapS", ctypes.c_int32), ("wrapT", ctypes.c_int32), ("srgb", ctypes.c_int32),
                ("filter", ctypes.c_int32)]


class Image(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("rgba", ctypes.POINTER(ctypes.c_uint8))]


class GltfInfo(ctypes.Structure):
    _fields_ = [("numVertices", ctypes.c_uint32), ("numShapes", ctypes.c_uint32), ("numJointSlots", ctypes.c_uint32),
                ("numChannels", ctypes.c_uint32), ("duration", ctypes.c_float), ("skinned", ctypes.c_int32)]


class Deformation(ctypes.Structure):
    _fields_ = [("restPositions", ctypes.c_void_p), ("restNormals", ctypes.c_void_p),
                ("vertexShape", ctypes.c_void_p), ("joints", ctypes.c_void_p), ("weights", ctypes.c_void_p),
                ("numVertices", ctypes.c_uint32), ("numShapes", ctypes.c_uint32), ("numJoints", ctypes.c_uint32)]


class SceneStruct(ctypes.Structure):
    _fields_ = [("positions", ctypes.POINTER(ctypes.c_float)), ("numVertices", ctypes.c_uint32),
                ("normals", ctypes.POINTER(ctypes.c_float)), ("texCoords", ctypes.POINTER(ctypes.c_float)),
                ("triIndices", ctypes.POINTER(ctypes.c_int32)), ("numTriangles", ctypes.c_uint32),
                ("matIndices", ctypes.POINTER(ctypes.c_int32)), ("materials", ctypes.POINTER(MaterialData)),
                ("numMaterials", ctypes.c_uint32), ("lights", ctypes.POINTER(Light)), ("numLights", ctypes.c_uint32),
                ("textures", ctypes.POINTER(Texture)), ("numTextures", ctypes.c_uint32),
                ("camEye", f3), ("camTarget", f3), ("camUp", f3), ("camFovYDeg", ctypes.c_float),
                ("resX", ctypes.c_uint32), ("resY", ctypes.c_uint32), ("bgColour", f3),
                ("spp", ctypes.c_uint32), ("maxDepth", ctypes.c_uint32)]


class Options(ctypes.Structure):
    _fields_ = [("sppBatch", ctypes.c_uint32), ("blockSize", ctypes.c_uint32), ("leafSize", ctypes.c_uint32),
                ("useGraph", ctypes.c_uint32), ("bvhWidth", ctypes.c_uint32), ("compaction", ctypes.c_uint32),
                ("nodeBudget", ctypes.c_uint32), ("tailBounce", ctypes.c_uint32), ("bvhBuilder", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("extensionRays", ctypes.c_uint64), ("shadowRays", ctypes.c_uint64),
                ("pathSamples", ctypes.c_uint64), ("nanSamples", ctypes.c_uint64), ("bvhNodes", ctypes.c_uint32),
                ("bvhLeaves", ctypes.c_uint32), ("bvh8Nodes", ctypes.c_uint32), ("bvhWidth", ctypes.c_uint32),
                ("sppBatch", ctypes.c_uint32), ("blockSize", ctypes.c_uint32),
                ("traversalStackOverflows", ctypes.c_uint64), ("traversalBudgetExhausted", ctypes.c_uint64),
                ("bvh8Levels", ctypes.c_uint32), ("tailBounce", ctypes.c_uint32)]


class KernelTimes(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * 8), ("launches", ctypes.c_uint64 * 8), ("extensionRays", ctypes.c_uint64),
                ("shadowRays", ctypes.c_uint64)]


class GuidingOptions(ctypes.Structure):
    _fields_ = [("trainSteps", ctypes.c_uint32), ("trainStride", ctypes.c_uint32), ("maxDepth", ctypes.c_uint32),
                ("alphaMin", ctypes.c_float), ("alphaMax", ctypes.c_float), ("alphaRamp", ctypes.c_float),
                ("learningRate", ctypes.c_float), ("lobeLoss", ctypes.c_int32), ("trainSpp", ctypes.c_uint32),
                ("primaryShare", ctypes.c_int32)]


class AutotuneRequest(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
                ("warmupSpp", ctypes.c_uint32), ("guiding", ctypes.c_uint32)]


class AutotuneTrial(ctypes.Structure):
    _fields_ = [("options", Options), ("samplesPerS", ctypes.c_double), ("mraysPerS", ctypes.c_double)]


class View(ctypes.Structure):
    _fields_ = [("eye", f3), ("target", f3), ("up", f3), ("fovYDeg", ctypes.c_float), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32), ("scene", ctypes.c_uint32)]


class TraversalCounts(ctypes.Structure):
    _fields_ = [("extensionRays", ctypes.c_uint64), ("extensionNodes", ctypes.c_uint64),
                ("extensionTris", ctypes.c_uint64), ("shadowRays", ctypes.c_uint64),
                ("shadowNodes", ctypes.c_uint64), ("shadowTris", ctypes.c_uint64)]


BSDF_QUERY = np.dtype([
    ("baseColour", "<f4", 3), ("emission", "<f4", 3), ("sheenColour", "<f4", 3),
    ("metallic", "<f4"), ("roughness", "<f4"), ("specular", "<f4"),
    ("transmissionWeight", "<f4"), ("subsurfaceWeight", "<f4"), ("coatWeight", "<f4"),
    ("coatRoughness", "<f4"), ("sheenRoughnessMat", "<f4"), ("sheenRoughness", "<f4"),
    ("ior", "<f4"), ("category", "<u4"),
    ("n", "<f4", 3), ("wo", "<f4", 3), ("wi", "<f4", 3), ("xs", "<f4", 12),
])
BSDF_RESULT = np.dtype([
    ("category", "<u4"), ("ret", "<i4"), ("used", "<i4"), ("categoryWeight", "<f4"),
    ("f", "<f4", 3), ("dir", "<f4", 3), ("bsdf", "<f4", 3), ("pdf", "<f4"),
])

_P = ctypes.c_void_p
_H = ctypes.c_void_p  # optpt_renderer*
_sigs = {
    "optpt_last_error": (ctypes.c_char_p, []),
    "optpt_version": (ctypes.c_int, []),
    "optpt_scene_procedural": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(SceneStruct)]),
    "optpt_scene_release": (None, [ctypes.POINTER(SceneStruct)]),
    "optpt_scene_from_config": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(SceneStruct)]),
    "optpt_scene_from_gltf": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.POINTER(SceneStruct)]),
    "optpt_image_decode_png": (ctypes.c_int, [_P, ctypes.c_size_t, ctypes.POINTER(Image)]),
    "optpt_image_decode_jpeg": (ctypes.c_int, [_P, ctypes.c_size_t, ctypes.POINTER(Image)]),
    "optpt_image_release": (None, [ctypes.POINTER(Image)]),
    "optpt_gltf_open": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.POINTER(_P)]),
    "optpt_gltf_close": (None, [_P]),
    "optpt_gltf_info": (ctypes.c_int, [_P, ctypes.POINTER(GltfInfo)]),
    "optpt_gltf_scene": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int, ctypes.POINTER(SceneStruct)]),
    "optpt_gltf_deformation": (ctypes.c_int, [_P, ctypes.POINTER(Deformation)]),
    "optpt_gltf_pose": (ctypes.c_int, [_P, ctypes.c_float, _P, _P, _P]),
    "optpt_gltf_apply": (ctypes.c_int, [_P, ctypes.c_float, _P, _P]),
    "optpt_update_vertices": (ctypes.c_int, [_H, _P, _P, _P]),
    "optpt_set_deformation": (ctypes.c_int, [_H, ctypes.POINTER(Deformation)]),
    "optpt_deform": (ctypes.c_int, [_H, _P, _P, _P, _P]),
    "optpt_read_vertices": (ctypes.c_int, [_H, _P, _P, _P]),
    "optpt_refit_profiled": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]),
    "optpt_image_out": (ctypes.c_int, [_H, _P, _P, _P, _P]),
    "optpt_read_rgba8": (ctypes.c_int, [_H, _P, _P]),
    "optpt_image_out_profiled": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float)]),
    "optpt_save_image": (ctypes.c_int, [_H, ctypes.c_int, ctypes.c_char_p]),
    "optpt_encode_png": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_size_t, ctypes.POINTER(_P),
                                        ctypes.POINTER(ctypes.c_size_t)]),
    "optpt_encode_hdr": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_P),
                                        ctypes.POINTER(ctypes.c_size_t)]),
    "optpt_encode_exr": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(_P),
                                        ctypes.POINTER(ctypes.c_size_t)]),
    "optpt_free": (None, [_P]),
    "optpt_create": (ctypes.c_int, [ctypes.POINTER(SceneStruct), ctypes.POINTER(Options), ctypes.POINTER(_H)]),
    "optpt_destroy": (ctypes.c_int, [_H]),
    "optpt_setup_output_buffer": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.c_uint32]),
    "optpt_setup_camera": (ctypes.c_int, [_H, f3, f3, f3, ctypes.c_float]),
    "optpt_get_launch_params": (ctypes.c_int, [_H, ctypes.POINTER(LaunchParams)]),
    "optpt_set_launch_params": (ctypes.c_int, [_H, ctypes.POINTER(LaunchParams)]),
    "optpt_render": (ctypes.c_int, [_H, ctypes.c_uint32, _P]),
    "optpt_launch": (ctypes.c_int, [_H]),
    "optpt_launch_pipelined": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.POINTER(ctypes.c_float))]),
    "optpt_launch_flush": (ctypes.c_int, [_H, ctypes.POINTER(ctypes.POINTER(ctypes.c_float))]),
    "optpt_get_frame_buffer": (ctypes.POINTER(ctypes.c_float), [_H]),
    "optpt_get_sample_count": (ctypes.c_uint32, [_H]),
    "optpt_reset_sample_count": (ctypes.c_int, [_H]),
    "optpt_device_buffers": (ctypes.c_int, [_H, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                                            ctypes.POINTER(_P)]),
    "optpt_read_frame_buffer": (ctypes.c_int, [_H, _P, _P]),
    "optpt_read_accum": (ctypes.c_int, [_H, _P, _P, _P]),
    "optpt_get_stats": (ctypes.c_int, [_H, ctypes.POINTER(Stats)]),
    "optpt_render_profiled": (ctypes.c_int, [_H, ctypes.c_uint32, _P, ctypes.POINTER(KernelTimes)]),
    "optpt_traversal_counts": (ctypes.c_int, [_H, ctypes.c_uint32, _P, ctypes.POINTER(TraversalCounts)]),
    "optpt_relmse": (ctypes.c_int, [_P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, _P]),
    "optpt_relmse_noalloc": (ctypes.c_int, [_P, ctypes.c_uint32, _P, ctypes.c_uint32, _P, _P]),
    "optpt_trace": (ctypes.c_int, [_H, _P, _P, ctypes.c_uint32, ctypes.c_int, _P]),
    "optpt_bvh_leaf_order": (ctypes.c_int, [_H, _P, _P]),
    "optpt_bvh_nodes": (ctypes.c_int, [_H, _P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]),
    "optpt_bvh8_nodes": (ctypes.c_int, [_H, _P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), _P]),
    "optpt_bsdf_batch": (ctypes.c_int, [_P, _P, ctypes.c_uint32, _P]),
    "optpt_tc_selftest": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "optpt_guide_create": (ctypes.c_int, [f3, f3, ctypes.c_uint32, ctypes.POINTER(_P)]),
    "optpt_guide_destroy": (ctypes.c_int, [_P]),
    "optpt_guide_params": (ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    "optpt_guide_levels": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "optpt_guide_infer": (ctypes.c_int, [_P, _P, ctypes.c_uint32, _P, _P]),
    "optpt_guide_mixture_eval": (ctypes.c_int, [_P, ctypes.c_uint32, _P, _P, _P]),
    "optpt_guide_gradients": (ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, _P, _P, ctypes.POINTER(ctypes.c_double),
                                             _P]),
    "optpt_guide_train_step": (ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, _P]),
    "optpt_guide_status": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "optpt_set_guiding": (ctypes.c_int, [_H, ctypes.c_int]),
    "optpt_get_guide": (ctypes.c_int, [_H, ctypes.POINTER(_P)]),
    "optpt_queue_counts": (ctypes.c_int, [_H, _P, _P, _P, ctypes.c_uint32]),
    "optpt_guiding_batch": (ctypes.c_int, [_H, _P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]),
    "optpt_render_batch": (ctypes.c_int, [_H, ctypes.POINTER(View), ctypes.c_uint32, _P]),
    "optpt_render_batch_scenes": (ctypes.c_int, [ctypes.POINTER(_H), ctypes.c_uint32, ctypes.POINTER(View),
                                                 ctypes.c_uint32, _P]),
    "optpt_autotune": (ctypes.c_int, [ctypes.POINTER(SceneStruct), ctypes.POINTER(AutotuneRequest),
                                      ctypes.POINTER(Options), ctypes.POINTER(AutotuneTrial), ctypes.c_uint32,
                                      ctypes.POINTER(ctypes.c_uint32)]),
    "optpt_batch_read_view": (ctypes.c_int, [_H, ctypes.c_uint32, _P, _P, _P]),
    "optpt_batch_view": (ctypes.c_int, [_H, ctypes.c_uint32, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P),
                                        ctypes.POINTER(ctypes.c_uint32)]),
    "optpt_set_guiding_options": (ctypes.c_int, [_H, ctypes.POINTER(GuidingOptions)]),
    "optpt_get_guiding_options": (ctypes.c_int, [_H, ctypes.POINTER(GuidingOptions)]),
}
EXPORTS = tuple(_sigs)
for _name, (_res, _args) in _sigs.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


def check(rc):
    if rc != OPTPT_OK:
        raise OptptError(rc, lib.optpt_last_error().decode())
    return rc
