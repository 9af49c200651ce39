"""Rendering imported glTF scenes on the GPU.

* A procedural scene exported to glTF and imported again renders bit for
  bit like the procedural original (same BVH, materials and random streams).
* A textured glTF scene (nearest-filtered clamped base colour, a normal map,
  an alpha-masked card, an emissive texture, point, spot and directional
  lights, the document's camera) follows the oracle's paths with paired
  random streams, and a high-spp render is unbiased against an independent
  FP64 oracle render.
"""
import math

import numpy as np
import pytest

from gltf_writer import Gltf, from_scene, png_bytes
from gpu_util import paired_agreement, pixel_stats, render_pair

pytestmark = pytest.mark.gpu


def test_exported_cornell_renders_bit_identically(cuda_dev, tmp_path):
    import torch

    import optix_pt_gb300 as opt
    proc = opt.Scene.procedural("cornell")
    imp = opt.Scene.from_gltf(from_scene(proc).save(tmp_path / "c.glb", glb=True))
    out = []
    for sc in (proc, imp):
        r = opt.Renderer(sc, spp_batch=4)
        r.setupOutputBuffer(96, 96)
        a = proc.arrays()
        r.setupCamera(a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"])
        r.render(16, torch.cuda.current_stream())
        torch.cuda.synchronize()
        out.append(r.accum())
        r.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def _textured_scene(tmp_path):
    g = Gltf()
    rng = np.random.default_rng(11)
    checker = ((np.indices((16, 16)).sum(0) % 2)[..., None] * np.array([200, 180, 40, 255]) +
               (1 - np.indices((16, 16)).sum(0) % 2)[..., None] * np.array([30, 60, 190, 255]))
    t_check = g.texture(g.image(png_bytes(checker, 6, 8)), {"wrapS": 33071, "wrapT": 33071, "magFilter": 9728})
    bumps = np.zeros((32, 32, 3), np.int64)
    yy, xx = np.mgrid[0:32, 0:32]
    bumps[..., 0] = 128 + (60 * np.sin(xx / 3.0)).astype(np.int64)
    bumps[..., 1] = 128 + (60 * np.cos(yy / 4.0)).astype(np.int64)
    bumps[..., 2] = 230
    t_norm = g.texture(g.image(png_bytes(bumps, 2, 8), embed="data"))
    alpha = np.zeros((16, 16, 2), np.int64)
    alpha[..., 0] = 150
    alpha[..., 1] = np.where((xx[:16, :16] - 8) ** 2 + (yy[:16, :16] - 8) ** 2 < 40, 255, 0)
    t_alpha = g.texture(g.image(png_bytes(alpha, 4, 8), embed="card.png"))
    glow = rng.integers(80, 256, (8, 8, 3))
    t_glow = g.texture(g.image(png_bytes(glow, 2, 8)))
    floor = g.material(pbrMetallicRoughness={"baseColorTexture": {
        "index": t_check, "extensions": {"KHR_texture_transform": {"scale": [3.0, 3.0], "offset": [-0.5, -0.5]}}},
        "metallicFactor": 0.0, "roughnessFactor": 0.7})
    wall = g.material(pbrMetallicRoughness={"baseColorFactor": [0.7, 0.7, 0.75, 1], "metallicFactor": 0.0,
                                            "roughnessFactor": 0.5}, normalTexture={"index": t_norm},
                      extensions={"KHR_materials_specular": {"specularFactor": 0.0}})
    card = g.material(pbrMetallicRoughness={"baseColorTexture": {"index": t_alpha}, "metallicFactor": 0.0},
                      alphaMode="MASK", alphaCutoff=0.5, doubleSided=True)
    lamp = g.material(emissiveFactor=[1.0, 0.9, 0.8], emissiveTexture={"index": t_glow},
                      extensions={"KHR_materials_emissive_strength": {"emissiveStrength": 6.0}})
    gold = g.material(pbrMetallicRoughness={"baseColorFactor": [1.0, 0.8, 0.4, 1], "metallicFactor": 1.0,
                                            "roughnessFactor": 0.3})

    def quad(c, u, v):
        c, u, v = (np.asarray(x, np.float32) for x in (c, u, v))
        p = np.stack([c - u - v, c + u - v, c + u + v, c - u + v])
        n = np.cross(u, v)
        n = np.tile(n / np.linalg.norm(n), (4, 1))
        return p, np.array([0, 1, 2, 0, 2, 3], np.uint32), n, np.array([[0, 1], [1, 1], [1, 0], [0, 0]], np.float32)

    prims = []
    for mat, q in ((floor, quad([0, 0, 0], [3, 0, 0], [0, 0, -3])), (wall, quad([0, 1.5, -3], [3, 0, 0], [0, 1.5, 0])),
                   (card, quad([0.6, 0.8, -0.5], [0.6, 0, 0.2], [0, 0.6, 0])),
                   (lamp, quad([-1.8, 2.2, -1.5], [0.4, 0, 0], [0, 0, 0.4]))):
        p, i, n, uv = q
        prims.append(g.primitive(p, i, n, uv, material=mat))
    # a small gold box-ish prism via a triangle fan
    fan = np.array([[-0.8, 0.0, -0.8], [-0.3, 0.0, -0.6], [-0.4, 0.9, -0.9], [-1.0, 0.7, -1.2]], np.float32)
    fn = np.tile(np.array([[0.3, 0.3, 0.9]], np.float32), (4, 1))
    prims.append(g.primitive(fan, None, fn, np.zeros((4, 2), np.float32), material=gold, mode=6))
    g.node(mesh=g.mesh(prims))
    lp = g.light(type="point", intensity=6000.0, color=[1.0, 0.85, 0.7])
    ls = g.light(type="spot", intensity=20000.0, spot={"innerConeAngle": 0.25, "outerConeAngle": 0.5})
    ld = g.light(type="directional", intensity=1.5, color=[0.6, 0.7, 1.0])
    g.node(translation=[1.5, 2.5, 0.5], extensions={"KHR_lights_punctual": {"light": lp}})
    down = [-math.sin(math.pi / 4), 0.0, 0.0, math.cos(math.pi / 4)]  # -z -> -y
    g.node(translation=[0.5, 3.0, -1.0], rotation=down, extensions={"KHR_lights_punctual": {"light": ls}})
    tilt = [-math.sin(0.5), 0.0, 0.0, math.cos(0.5)]
    g.node(rotation=tilt, extensions={"KHR_lights_punctual": {"light": ld}})
    cam = g.camera(0.9)
    look = [-math.sin(0.15), 0.0, 0.0, math.cos(0.15)]
    g.node(translation=[0.0, 1.6, 3.2], rotation=look, camera=cam)
    return g.save(tmp_path / "textured.gltf")


@pytest.fixture()
def textured(tmp_path):
    import optix_pt_gb300 as opt
    return opt.Scene.from_gltf(_textured_scene(tmp_path))


def test_textured_scene_follows_oracle_paths(cuda_dev, textured):
    assert textured.struct.numTextures == 4 and textured.struct.numLights == 3
    g, c, st, cnt, f = render_pair(textured, 96, 72, 2, 2, 0, 32, batch=2, classify=True)
    robust, sensitive, overall = paired_agreement(g, c, f)
    print("robust-pixel agreement %.4f, rounding-sensitive pixels %.4f, all pixels %.4f" % (
        robust, sensitive, overall))
    assert robust >= 0.995 and overall >= 0.995, (robust, overall)
    assert sensitive <= 0.05, sensitive
    assert abs(int(st["extensionRays"]) - int(cnt[0])) <= 0.02 * int(cnt[0])
    assert abs(int(st["shadowRays"]) - int(cnt[1])) <= 0.02 * max(1, int(cnt[1]))


def test_textured_scene_unbiased_against_fp64(cuda_dev, textured):
    g, c, st, cnt = render_pair(textured, 64, 48, 1024, 256, 1 << 20, 64)
    frac, dmean, se, gm, cm, live = pixel_stats(g, c)
    print("z>3 fraction %.4f, mean diff %.3g (SE %.3g)" % (frac, dmean, se))
    assert frac < 0.015, frac
    assert dmean < 4 * se, (dmean, se)
