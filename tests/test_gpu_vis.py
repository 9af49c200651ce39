"""Material visualisation modes (LaunchParams::vis 1-12) against the oracle.

The reference replaces the path's radiance with a material quantity at the
first hit and ends the path (cu/path_tracer.cu:252-315): metallic,
roughness, occlusion, emission, shading normal, geometric normal, albedo,
"glossy colour" (metallic x albedo x specular), 9 (unfinished: radiance
unchanged), sheen colour, sheen roughness and alpha. Each mode is rendered on
the GPU and by the FP32 oracle with the same random streams (same camera
jitter, so the same first hits) on a glTF scene that feeds every one of those
quantities from a texture: a metallic-roughness map (occlusion, roughness,
metalness), sheen colour and roughness maps, base colour with alpha, a
normal map and an emissive map.
"""
import numpy as np
import pytest

from gltf_writer import Gltf, png_bytes

pytestmark = pytest.mark.gpu


def _vis_scene(tmp_path):
    g = Gltf()
    yy, xx = np.mgrid[0:16, 0:16]
    rng = np.random.default_rng(4)
    base = np.zeros((16, 16, 4), np.int64)
    base[..., :3] = rng.integers(20, 250, (16, 16, 3))
    base[..., 3] = 64 + 12 * ((xx + yy) % 16)
    t_base = g.texture(g.image(png_bytes(base, 6, 8)))
    orm = np.zeros((16, 16, 3), np.int64)
    orm[..., 0] = 40 + 13 * xx                  # occlusion
    orm[..., 1] = 30 + 14 * yy                  # roughness
    orm[..., 2] = np.where(xx < 3, 5, 25 + 14 * xx)   # metalness, below the 0.04 threshold on the left
    t_orm = g.texture(g.image(png_bytes(orm, 2, 8)))
    bumps = np.zeros((32, 32, 3), np.int64)
    y2, x2 = np.mgrid[0:32, 0:32]
    bumps[..., 0] = 128 + (50 * np.sin(x2 / 3.0)).astype(np.int64)
    bumps[..., 1] = 128 + (50 * np.cos(y2 / 4.0)).astype(np.int64)
    bumps[..., 2] = 230
    t_norm = g.texture(g.image(png_bytes(bumps, 2, 8)))
    sheen_c = rng.integers(30, 255, (8, 8, 3))
    t_sheen_c = g.texture(g.image(png_bytes(sheen_c, 2, 8)))
    sheen_r = np.zeros((8, 8, 4), np.int64)
    sheen_r[..., :3] = 255
    sheen_r[..., 3] = rng.integers(10, 255, (8, 8))
    t_sheen_r = g.texture(g.image(png_bytes(sheen_r, 6, 8)))
    glow = rng.integers(80, 256, (8, 8, 3))
    t_glow = g.texture(g.image(png_bytes(glow, 2, 8)))

    floor = g.material(pbrMetallicRoughness={
        "baseColorTexture": {"index": t_base, "extensions": {"KHR_texture_transform": {"scale": [2.0, 2.0]}}},
        "metallicRoughnessTexture": {"index": t_orm}, "metallicFactor": 0.9, "roughnessFactor": 0.8},
        normalTexture={"index": t_norm}, extensions={"KHR_materials_specular": {"specularFactor": 0.7}})
    velvet = g.material(pbrMetallicRoughness={"baseColorFactor": [0.5, 0.2, 0.6, 1], "metallicFactor": 0.0,
                                              "roughnessFactor": 0.9},
                        extensions={"KHR_materials_sheen": {
                            "sheenColorFactor": [0.9, 0.8, 0.7], "sheenColorTexture": {"index": t_sheen_c},
                            "sheenRoughnessFactor": 0.8, "sheenRoughnessTexture": {"index": t_sheen_r}}})
    lamp = g.material(emissiveFactor=[1.0, 0.9, 0.8], emissiveTexture={"index": t_glow})

    def quad(c, u, v):
        c, u, v = (np.asarray(x, np.float32) for x in (c, u, v))
        p = np.stack([c - u - v, c + u - v, c + u + v, c - u + v])
        n = np.cross(u, v)
        n = np.tile(n / np.linalg.norm(n), (4, 1))
        return p, np.array([0, 1, 2, 0, 2, 3], np.uint32), n, np.array([[0, 1], [1, 1], [1, 0], [0, 0]], np.float32)

    prims = []
    for mat, q in ((floor, quad([0, 0, 0], [3, 0, 0], [0, 0, -3])),
                   (velvet, quad([0, 1.5, -3], [3, 0, 0], [0, 1.5, 0])),
                   (lamp, quad([-1.5, 1.2, -1.0], [0.5, 0, 0.2], [0, 0.5, 0]))):
        p, i, n, uv = q
        prims.append(g.primitive(p, i, n, uv, material=mat))
    g.node(mesh=g.mesh(prims))
    lp = g.light(type="point", intensity=3000.0)
    g.node(translation=[1.0, 2.5, 0.5], extensions={"KHR_lights_punctual": {"light": lp}})
    cam = g.camera(0.9)
    look = [-np.sin(0.2), 0.0, 0.0, np.cos(0.2)]
    g.node(translation=[0.0, 1.5, 3.0], rotation=[float(x) for x in look], camera=cam)
    return g.save(tmp_path / "vis.gltf")


@pytest.mark.parametrize("vis", list(range(1, 13)))
def test_vis_mode_matches_oracle(cuda_dev, tmp_path, vis):
    import torch

    import optix_pt_gb300 as opt
    from oracle import oracle as orc
    sc = opt.Scene.from_gltf(_vis_scene(tmp_path))
    assert sc.struct.numTextures == 6
    w, h, spp = 80, 60, 2
    r = opt.Renderer(sc, spp_batch=spp)
    r.setupOutputBuffer(w, h)
    r.setVis(vis)
    r.render(spp, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, _, n = r.accum()
    lp = r.launch_params()
    cam = list(lp.eye) + list(lp.U) + list(lp.V) + list(lp.W) + list(lp.bgColour)
    cs, _, _ = orc.SceneView(sc.struct, 4).render(cam, w, h, lp.seed, 0, spp, lp.maxDepth, precision=32, vis=vis)
    gm, cm = s.reshape(-1, 3) / n, cs / spp
    r.close()
    # Texture lookups, material arithmetic and hits are the same operations on
    # both sides, so those modes agree bit for bit; the normals (5, 6) come
    # from cross products, a tangent frame and normalisations, whose rounding
    # may differ by a few ULP where the device fuses multiply-adds.
    tol = 1e-5 if vis in (5, 6) else 0.0
    close = (np.abs(gm - cm) <= tol * np.maximum(1.0, np.abs(cm))).all(1)
    print("vis %d: %.5f of pixels agree; value range %.3g..%.3g" % (vis, close.mean(), cm.min(), cm.max()))
    assert close.mean() >= 0.999, close.mean()
    if vis != 9:
        assert np.ptp(cm) > 0.05   # the mode shows something that varies across the frame
