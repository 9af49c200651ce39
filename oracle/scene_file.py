"""A scene read from the .npz file the library's Scene.save writes, laid out
as the C ABI's optpt_scene record (include/optpt.h) so that the oracle's
SceneView can walk it -- without loading the CUDA library (test
infrastructure: the CPU baseline times the oracle on scenes the library
generated in an earlier step)."""
import ctypes

import numpy as np

_f3 = ctypes.c_float * 3
_P = ctypes.c_void_p


class TextureRecord(ctypes.Structure):
    """optpt_texture."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("rgba", _P), ("wrapS", ctypes.c_int32),
                ("wrapT", ctypes.c_int32), ("srgb", ctypes.c_int32), ("filter", ctypes.c_int32)]


class SceneRecord(ctypes.Structure):
    """optpt_scene; materials and lights stay raw MaterialData / Light bytes."""
    _fields_ = [("positions", _P), ("numVertices", ctypes.c_uint32), ("normals", _P), ("texCoords", _P),
                ("triIndices", _P), ("numTriangles", ctypes.c_uint32), ("matIndices", _P), ("materials", _P),
                ("numMaterials", ctypes.c_uint32), ("lights", _P), ("numLights", ctypes.c_uint32),
                ("textures", _P), ("numTextures", ctypes.c_uint32),
                ("camEye", _f3), ("camTarget", _f3), ("camUp", _f3), ("camFovYDeg", ctypes.c_float),
                ("resX", ctypes.c_uint32), ("resY", ctypes.c_uint32), ("bgColour", _f3),
                ("spp", ctypes.c_uint32), ("maxDepth", ctypes.c_uint32)]


class FileScene:
    """Keeps the arrays alive; `.struct` is the optpt_scene record,
    `.arrays()` the camera and array fields as the library's Scene gives them."""

    def __init__(self, path):
        z = np.load(path)
        self._a = {k: z[k] for k in z.files}
        a = self._a
        s = SceneRecord()

        def ptr(name, dtype):
            if name not in a:
                return None
            a[name] = np.ascontiguousarray(a[name], dtype)
            return a[name].ctypes.data

        s.positions = ptr("positions", np.float32)
        s.numVertices = len(a["positions"])
        s.normals = ptr("normals", np.float32)
        s.texCoords = ptr("texCoords", np.float32)
        s.triIndices = ptr("triIndices", np.int32)
        s.numTriangles = len(a["triIndices"])
        s.matIndices = ptr("matIndices", np.int32)
        s.materials = ptr("materials", np.uint8)
        s.numMaterials = int(a["numMaterials"])
        s.lights = ptr("lights", np.uint8) if int(a["numLights"]) else None
        s.numLights = int(a["numLights"])
        nt = int(a["numTextures"])
        self._tex = (TextureRecord * max(1, nt))()
        for i in range(nt):
            px = np.ascontiguousarray(a["texture%d" % i], np.uint8)
            a["texture%d" % i] = px
            m = a["texture%d_modes" % i]
            self._tex[i] = TextureRecord(px.shape[1], px.shape[0], px.ctypes.data, int(m[0]), int(m[1]), int(m[2]),
                                         int(m[3]))
        s.textures = ctypes.addressof(self._tex) if nt else None
        s.numTextures = nt
        s.camEye[:], s.camTarget[:], s.camUp[:] = (list(map(float, a[k])) for k in ("camEye", "camTarget", "camUp"))
        s.camFovYDeg = float(a["camFovYDeg"])
        s.resX, s.resY = int(a["resX"]), int(a["resY"])
        s.bgColour[:] = list(map(float, a["bgColour"]))
        s.spp, s.maxDepth = int(a["spp"]), int(a["maxDepth"])
        self.struct = s
        self.num_triangles = s.numTriangles

    def arrays(self):
        a = self._a
        out = {k: a[k] for k in ("positions", "triIndices", "matIndices") if k in a}
        for k in ("camEye", "camTarget", "camUp", "bgColour"):
            out[k] = [float(x) for x in a[k]]
        out["camFovYDeg"] = float(a["camFovYDeg"])
        for k in ("resX", "resY", "spp", "maxDepth"):
            out[k] = int(a[k])
        return out


def load(path):
    return FileScene(path)
