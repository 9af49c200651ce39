"""Generates the golden fixtures in tests/golden/ from the reference itself.

The reference's BSDF, light-sampling, tone-mapping and barycentric headers
(and src/light.cpp) are compiled unmodified for the host by oracle/build.py
(oracle/_ref/libref.so); this script feeds them seeded inputs and stores
inputs and outputs as small .npz files. Run from the repository root:

    python tests/golden/make_golden.py

It needs the reference tree, so it runs where that tree is mounted; the
fixtures it writes are committed and used everywhere else.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as orc  # noqa: E402
from oracle.abi import LIGHT, LIGHT_SAMPLE  # noqa: E402
from bsdf_cases import make_fixed_category_queries, make_queries  # noqa: E402


def main():
    ref = orc.ref()
    if ref is None:
        raise SystemExit("the reference tree is not available; fixtures cannot be regenerated here")
    P = ctypes.c_void_p

    # BSDF queries: runtime-categorised and host-categorised materials.
    q = np.concatenate([make_queries(6000, 7), make_fixed_category_queries(2000, 8)])
    r = orc.ref_bsdf_query(q)
    np.savez_compressed(os.path.join(HERE, "bsdf_golden.npz"), queries=q, results=r)

    # Tone mapping + gamma (cu/device_programs.cu:84-96).
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.exponential(1.0, (3000, 4)), rng.uniform(0.0, 50.0, (1000, 4)),
                        np.zeros((4, 4))]).astype(np.float32)
    x[:, 3] = 0.0
    outs = {}
    for tone in (0, 1):
        for impl in (0, 1):
            for gamma in (0, 1):
                y = np.zeros_like(x)
                ref.ref_tonemap(P(x.ctypes.data), P(y.ctypes.data), len(x), tone, impl, gamma, ctypes.c_float(2.2))
                outs["t%d_i%d_g%d" % (tone, impl, gamma)] = y.copy()
    np.savez_compressed(os.path.join(HERE, "tonemap_golden.npz"), inputs=x, **outs)

    # Punctual-light sampling (cu/light_sampling.cu:6-81).
    n = 3000
    lights = np.zeros(n, LIGHT)
    lights["type"] = np.arange(n) % 3
    lights["radiance"] = rng.uniform(1.0, 100.0, (n, 3))
    lights["p0"] = rng.uniform(-5.0, 5.0, (n, 3))
    nn = rng.normal(size=(n, 3))
    lights["normal"] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    lights["distance"] = rng.uniform(1.0, 100.0, n)
    cw = rng.uniform(0.0, 0.9, n)
    lights["cosWidth"] = cw
    lights["cosFalloffStart"] = cw + rng.uniform(0.01, 0.09, n)
    pts = rng.uniform(-5.0, 5.0, (n, 3)).astype(np.float32)
    ls = np.zeros(n, LIGHT_SAMPLE)
    ref.ref_light_sample(P(lights.ctypes.data), P(pts.ctypes.data), P(ls.ctypes.data), n)
    # Light construction (src/light.cpp:5-73): point and spot radiance.
    made = []
    for k in range(200):
        typ = 0 if k % 2 == 0 else 2
        a = rng.uniform(-5, 5, 3).astype(np.float32)
        b = rng.normal(size=3).astype(np.float32)
        w0, w1 = np.float32(rng.uniform(10, 80)), np.float32(rng.uniform(1, 9))
        watt = np.float32(rng.uniform(1, 500))
        col = rng.uniform(0.1, 1.0, 3).astype(np.float32)
        rad = np.zeros(3, np.float32)
        extra = np.zeros(5, np.float32)
        ref.ref_create_light(typ, P(a.ctypes.data), P(b.ctypes.data), ctypes.c_float(w0), ctypes.c_float(w1),
                             ctypes.c_float(watt), P(col.ctypes.data), P(rad.ctypes.data), P(extra.ctypes.data))
        made.append(np.concatenate([[typ], a, b, [w0, w1, watt], col, rad, extra]).astype(np.float32))
    np.savez_compressed(os.path.join(HERE, "light_golden.npz"), lights=lights, points=pts, samples=ls,
                        created=np.array(made))

    # Barycentrics of points on triangles (include/barycentrics.h:17-44).
    m = 3000
    tri = rng.uniform(-3.0, 3.0, (m, 9)).astype(np.float32)
    uv = rng.uniform(0.0, 1.0, (m, 2))
    fold = uv.sum(1) > 1.0
    uv[fold] = 1.0 - uv[fold]
    p = (tri[:, 0:3] + (tri[:, 3:6] - tri[:, 0:3]) * uv[:, :1] + (tri[:, 6:9] - tri[:, 0:3]) * uv[:, 1:2])
    p = p.astype(np.float32)
    uvw = np.zeros((m, 3), np.float32)
    ref.ref_barycentric(P(tri.ctypes.data), P(p.ctypes.data), P(uvw.ctypes.data), m)
    np.savez_compressed(os.path.join(HERE, "barycentric_golden.npz"), tri=tri, points=p, uvw=uvw)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
