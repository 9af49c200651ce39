"""numpy dtypes for the oracle's flat query records (oracle/query_abi.h)."""
import numpy as np

NXS = 12

BSDF_QUERY = np.dtype([
    ("baseColour", "<f4", 3), ("emission", "<f4", 3), ("sheenColour", "<f4", 3),
    ("metallic", "<f4"), ("roughness", "<f4"), ("specular", "<f4"),
    ("transmissionWeight", "<f4"), ("subsurfaceWeight", "<f4"), ("coatWeight", "<f4"),
    ("coatRoughness", "<f4"), ("sheenRoughnessMat", "<f4"), ("sheenRoughness", "<f4"),
    ("ior", "<f4"), ("category", "<u4"),
    ("n", "<f4", 3), ("wo", "<f4", 3), ("wi", "<f4", 3), ("xs", "<f4", NXS),
])

BSDF_RESULT = np.dtype([
    ("category", "<u4"), ("ret", "<i4"), ("used", "<i4"), ("pad", "<i4"),
    ("categoryWeight", "<f8"), ("f", "<f8", 3), ("dir", "<f8", 3), ("bsdf", "<f8", 3), ("pdf", "<f8"),
])

LIGHT = np.dtype([
    ("type", "<i4"), ("radiance", "<f4", 3), ("p0", "<f4", 3), ("normal", "<f4", 3),
    ("distance", "<f4"), ("cosWidth", "<f4"), ("cosFalloffStart", "<f4"),
])

LIGHT_SAMPLE = np.dtype([
    ("lightDir", "<f4", 3), ("radiance", "<f4", 3), ("pdf", "<f4"), ("lightDist", "<f4"),
])
