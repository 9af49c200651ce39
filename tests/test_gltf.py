"""glTF 2.0 import and PNG decoding (host side, no GPU).

* PNG: every colour type and bit depth, palettes and tRNS, Adam7, all five
  row filters and every DEFLATE block type decode exactly to the four-
  component RGBA8 stb_image gives; corrupt files are errors.
* JPEG (baseline): grey and YCbCr with 4:4:4, 4:2:2, 4:4:0, 4:2:0 and 4:1:1
  sampling, Adobe RGB, restart intervals, one scan per component, 16-bit
  quantisation tables, sizes that are not whole blocks, decode within one
  level of a float64 reconstruction of the encoder's coefficients
  (tests/jpeg_writer.py); progressive files are reported as unsupported.
* glTF: a procedural scene exported to glTF (.gltf with a data-URI buffer,
  external .bin, and .glb) imports to the identical flattened arrays; node
  transforms (matrix and T*R*S, nested), normals through the inverse
  transpose, skins in their rest pose, strips and fans, materials with the
  reference's extension handling and defaults, textures with their sampler,
  sRGB and filter settings, punctual lights and the camera follow
  src/gltf_loader.cpp; the scene-description route and the error codes.
"""
import json
import math
import os
import struct
import zlib

import numpy as np
import pytest

import optix_pt_gb300 as opt
from gltf_writer import Gltf, expected_rgba, from_scene, material_json, png_bytes


def _png_case(rng, ct, depth, h=13, w=29):
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ct]
    pal = trns = None
    if ct == 3:
        npal = min(1 << depth, 200)
        s = rng.integers(0, npal, (h, w, 1))
        pal = rng.integers(0, 256, (npal, 3))
        trns = bytes(rng.integers(0, 256, min(npal, 7)).astype(np.uint8))
    else:
        s = rng.integers(0, 1 << depth, (h, w, ch))
        if ct == 0:
            trns = int(s[0, 0, 0]).to_bytes(2, "big")
        elif ct == 2:
            trns = b"".join(int(v).to_bytes(2, "big") for v in s[1, 1])
    return s, pal, trns


FORMATS = [(0, d) for d in (1, 2, 4, 8, 16)] + [(3, d) for d in (1, 2, 4, 8)] + \
          [(2, 8), (2, 16), (4, 8), (4, 16), (6, 8), (6, 16)]
STRATEGIES = {"dynamic": (6, zlib.Z_DEFAULT_STRATEGY), "fixed": (6, zlib.Z_FIXED),
              "huffman_only": (6, zlib.Z_HUFFMAN_ONLY), "rle": (6, zlib.Z_RLE), "stored": (0, 0)}


@pytest.mark.parametrize("ct,depth", FORMATS)
@pytest.mark.parametrize("interlace", [False, True])
def test_png_decodes_every_format(ct, depth, interlace):
    rng = np.random.default_rng(ct * 100 + depth + (7 if interlace else 0))
    for name, (level, strategy) in STRATEGIES.items():
        s, pal, trns = _png_case(rng, ct, depth)
        b = png_bytes(s, ct, depth, palette=pal, trns=trns, interlace=interlace, level=level, strategy=strategy)
        got = opt.decode_png(b)
        assert np.array_equal(got, expected_rgba(s, ct, depth, palette=pal, trns=trns)), name


@pytest.mark.parametrize("h,w", [(1, 1), (1, 37), (9, 1), (8, 8), (64, 65)])
def test_png_sizes_and_single_filters(h, w):
    rng = np.random.default_rng(h * 1000 + w)
    s = rng.integers(0, 256, (h, w, 4))
    for f in range(5):
        got = opt.decode_png(png_bytes(s, 6, 8, filters=(f,), interlace=(f % 2 == 1)))
        assert np.array_equal(got, s.astype(np.uint8))


def test_png_large_smooth_image_long_matches():
    # A smooth image compresses into long back-references (length 258,
    # distances across rows) through zlib's dynamic blocks.
    y, x = np.mgrid[0:300, 0:400]
    s = np.stack([(x // 3) % 256, (y // 5) % 256, ((x + y) // 7) % 256, np.full_like(x, 255)], -1)
    b = png_bytes(s, 6, 8, filters=(1, 2, 4), level=9)
    assert len(b) < s.size // 10
    assert np.array_equal(opt.decode_png(b), s.astype(np.uint8))


def test_png_errors():
    rng = np.random.default_rng(5)
    s = rng.integers(0, 256, (16, 16, 4))
    good = png_bytes(s, 6, 8)
    opt.decode_png(good)
    bad_crc = bytearray(good)
    bad_crc[30] ^= 0xFF  # inside IHDR data or CRC
    bad_sig = b"\x89PNX" + good[4:]
    truncated = good[:len(good) // 2]
    for b in (bytes(bad_crc), bad_sig, truncated, b"", b"\x89PNG\r\n\x1a\n"):
        with pytest.raises(opt.OptptError):
            opt.decode_png(b if b else b"x")
    # Corrupt compressed data with valid chunk CRCs: Adler-32 / stream errors.
    co = zlib.compressobj(6)
    raw = b"".join(b"\0" + bytes(s[y].astype(np.uint8).reshape(-1)) for y in range(16))
    z = bytearray(co.compress(raw) + co.flush())
    z[-1] ^= 0x55
    ihdr = good[8:8 + 25]

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    with pytest.raises(opt.OptptError, match="Adler"):
        opt.decode_png(good[:8] + ihdr + chunk(b"IDAT", bytes(z)) + chunk(b"IEND", b""))


def _cornell_gltf(tmp_path, **save_kw):
    sc = opt.Scene.procedural("cornell")
    g = from_scene(sc)
    return sc, g.save(tmp_path / "cornell.gltf" if not save_kw.get("glb") else tmp_path / "cornell.glb", **save_kw)


@pytest.mark.parametrize("variant", ["data_uri", "external_bin", "glb"])
def test_exported_scene_imports_identically(tmp_path, variant):
    for name in ("cornell", "spheres"):
        sc = opt.Scene.procedural(name)
        g = from_scene(sc)
        if variant == "glb":
            path = g.save(tmp_path / (name + ".glb"), glb=True)
        elif variant == "external_bin":
            path = g.save(tmp_path / (name + ".gltf"), buffer_uri=name + " data.bin")
        else:
            path = g.save(tmp_path / (name + ".gltf"))
        imp = opt.Scene.from_gltf(path)
        a, b = sc.arrays(), imp.arrays()
        assert imp.num_triangles == sc.num_triangles
        # Vertices are re-emitted per primitive: compare per-triangle corners.
        pa = a["positions"][a["triIndices"]]
        pb = b["positions"][b["triIndices"]]
        assert np.array_equal(pa, pb)
        if a["normals"] is not None:
            assert np.array_equal(a["normals"][a["triIndices"]], b["normals"][b["triIndices"]])
        else:
            assert b["normals"] is None
        assert np.array_equal(a["matIndices"], b["matIndices"])
        assert a["materials"] == b["materials"], "MaterialData records differ"
        assert b["camUp"] == [0.0, 1.0, 0.0]


def _transform_scene():
    g = Gltf()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 2, 0], [0, 0, 3]], np.float32)
    nrm = np.array([[0, 0, 1], [0, 1, 0], [1, 0, 0], [0.6, 0.8, 0]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    m = g.mesh([g.primitive(tri, idx, nrm, material=g.material())])
    q = np.array([0.2, -0.4, 0.1, 0.0], np.float64)
    q[3] = math.sqrt(1 - (q[:3] ** 2).sum())
    child = g.node(root=False, mesh=m, translation=[1.5, -2.0, 0.25], rotation=q.tolist(), scale=[2.0, 0.5, 1.25])
    parent_m = np.array([[0, 1, 0, 0], [-1, 0, 0, 0], [0, 0, 1, 0], [3, 4, 5, 1]], np.float64)  # column-major rows
    g.node(matrix=parent_m.reshape(-1).tolist(), children=[child])
    g.node(mesh=m)  # the same mesh instanced at the root, untransformed
    return g, tri, nrm, idx, q, parent_m


def _quat_matrix(q):
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def test_node_transforms_and_instancing(tmp_path):
    g, tri, nrm, idx, q, parent_m = _transform_scene()
    sc = opt.Scene.from_gltf(g.save(tmp_path / "t.gltf"))
    a = sc.arrays()
    assert sc.num_triangles == 4
    local = np.eye(4)
    local[:3, :3] = _quat_matrix(q) @ np.diag([2.0, 0.5, 1.25])
    local[:3, 3] = [1.5, -2.0, 0.25]
    world = parent_m.T @ local
    P = a["positions"]
    want = (world @ np.c_[tri, np.ones(4)].T).T[:, :3]
    assert np.allclose(P[:4], want, rtol=1e-5, atol=1e-5)
    nm = np.linalg.inv(world[:3, :3]).T
    assert np.allclose(a["normals"][:4], (nm @ nrm.T).T, rtol=1e-5, atol=1e-5)
    # instanced copy at the root: raw vertices, raw normals
    assert np.array_equal(P[4:], tri) and np.array_equal(a["normals"][4:], nrm)
    assert np.array_equal(a["triIndices"], np.concatenate([idx, idx + 4]).reshape(-1, 3))


def test_strips_fans_missing_normals_and_texcoords(tmp_path):
    g = Gltf()
    mat = g.material()
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 2, 0]], np.float32)
    uv = np.array([[0, 0], [1, 0], [0, 1], [1, 1], [0, 2]], np.float32)
    n = np.tile(np.array([[0, 0, 1]], np.float32), (5, 1))
    prims = [g.primitive(v, None, n, uv, material=mat, mode=5),              # strip: 3 triangles
             g.primitive(v, np.arange(5, dtype=np.uint16), None, None, material=mat, mode=6, index_type=5123),
             g.primitive(v[:3], np.array([0, 1, 2], np.uint8), n[:3], None, index_type=5121),  # no material
             g.primitive(v, None, n, uv, material=mat, mode=1)]              # lines: skipped
    g.node(mesh=g.mesh(prims))
    sc = opt.Scene.from_gltf(g.save(tmp_path / "s.gltf"))
    a = sc.arrays()
    assert sc.num_triangles == 3 + 3 + 1
    P, I = a["positions"], a["triIndices"]
    strip = P[I[:3]]
    # glTF strip order: triangle k = (k, k + 1 + k % 2, k + 2 - k % 2)
    assert np.array_equal(strip[0], v[[0, 1, 2]]) and np.array_equal(strip[1], v[[1, 3, 2]])
    assert np.array_equal(strip[2], v[[2, 3, 4]])
    fan = P[I[3:6]]
    assert np.array_equal(fan[0], v[[0, 1, 2]]) and np.array_equal(fan[2], v[[0, 3, 4]])
    # the fan had no normals in a scene that has some: flat face normals
    for t in range(3, 6):
        c = P[I[t]]
        fn = np.cross(c[1] - c[0], c[2] - c[0])
        assert np.allclose(a["normals"][I[t]], fn / np.linalg.norm(fn))
    # the fan had no texture coordinates: zeros
    assert not a["texCoords"][I[3:6]].any()
    assert np.array_equal(a["texCoords"][I[:3]], uv[[[0, 1, 2], [1, 3, 2], [2, 3, 4]]])
    # no material: the glTF default material, appended after the document's
    mats = sc.materials()
    assert len(mats) == 2 and a["matIndices"][-1] == 1
    assert mats[1].metallic == 1.0 and mats[1].roughness == 1.0 and list(mats[1].baseColour) == [1, 1, 1, 1]


def test_material_extensions_and_quirks(tmp_path):
    g = Gltf()
    rng = np.random.default_rng(3)
    png = png_bytes(rng.integers(0, 256, (8, 8, 4)), 6, 8)
    img = g.image(png)
    t_clamp = g.texture(img, {"wrapS": 33071, "wrapT": 33648, "magFilter": 9728})
    t_plain = g.texture(img)
    tt = {"KHR_texture_transform": {"offset": [0.25, 0.5], "rotation": 0.3, "scale": [2.0, 4.0]}}
    m0 = g.material(pbrMetallicRoughness={"baseColorFactor": [0.5, 0.6, 0.7, 0.8], "metallicFactor": 0.3,
                                          "roughnessFactor": 0.4,
                                          "baseColorTexture": {"index": t_clamp, "extensions": tt},
                                          "metallicRoughnessTexture": {"index": t_clamp}},
                    normalTexture={"index": t_clamp}, alphaMode="MASK", alphaCutoff=0.25,
                    emissiveFactor=[0.0, 0.0, 0.0], emissiveTexture={"index": t_plain},
                    extensions={"KHR_materials_transmission": {"transmissionFactor": 0.7},
                                "KHR_materials_ior": {"ior": 1.33},
                                "KHR_materials_clearcoat": {"clearcoatFactor": 0.5,
                                                            "clearcoatRoughnessFactor": 0.2},
                                "KHR_materials_sheen": {"sheenRoughnessFactor": 0.9,
                                                        "sheenColorTexture": {"index": t_plain}}})
    m1 = g.material(emissiveFactor=[0.5, 0.25, 1.0], emissiveTexture={"index": t_plain},
                    extensions={"KHR_materials_emissive_strength": {"emissiveStrength": 4.0},
                                "KHR_materials_specular": {"specularFactor": 0.0},
                                "KHR_materials_sheen": {"sheenColorFactor": [0.1, 0.2, 0.3],
                                                        "sheenColorTexture": {"index": t_plain}}})
    m2 = g.material(alphaMode="BLEND")
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    g.node(mesh=g.mesh([g.primitive(tri, None, None, [[0, 0], [1, 0], [0, 1]], material=m)
                        for m in (m0, m1, m2)]))
    sc = opt.Scene.from_gltf(g.save(tmp_path / "m.gltf"))
    M = sc.materials()
    a, b, c = M
    assert list(a.baseColour) == pytest.approx([0.5, 0.6, 0.7, 0.8])
    assert (a.metallic, a.roughness, a.ior) == pytest.approx((0.3, 0.4, 1.33))
    assert a.specular == 1.0  # KHR_materials_specular absent: 1
    assert a.transmissionWeight == pytest.approx(0.7)
    assert (a.coatWeight, a.coatRoughness) == pytest.approx((0.5, 0.2))
    assert a.alphaMode == 2 and a.alphaCutoff == 0.25
    assert a.hasBaseColourTexture and a.hasNormalTexture and a.hasMetallicRoughnessTexture
    assert not a.hasEmissiveTexture  # emissiveFactor zero: texture ignored
    assert not a.hasSheenColourTexture and list(a.sheenColour) == [0, 0, 0]  # no sheenColorFactor
    assert a.sheenRoughness == pytest.approx(0.9)
    assert (a.baseColourTexTf.offset[0], a.baseColourTexTf.offset[1]) == (0.25, 0.5)
    assert (a.baseColourTexTf.scale[0], a.baseColourTexTf.scale[1]) == (2.0, 4.0)
    assert a.baseColourTexTf.rotation == pytest.approx(0.3)
    assert a.category == 0  # metallic in (0, 1): chosen per hit
    assert list(b.emission) == pytest.approx([2.0, 1.0, 4.0])
    assert b.hasEmissiveTexture and b.hasSheenColourTexture and b.specular == 0.0
    assert c.alphaMode == 1 and c.metallic == 1.0 and c.roughness == 1.0
    tex = sc.textures()
    # base colour: sampler (clamp, mirror, nearest), sRGB
    bc = tex[a.baseColourTexture]
    assert (bc["wrapS"], bc["wrapT"], bc["filter"], bc["srgb"]) == (1, 2, 1, 1)
    # normal / metallic-roughness: linear, sampler not applied
    for k in (a.normalTexture, a.metallicRoughnessTexture):
        assert (tex[k]["wrapS"], tex[k]["wrapT"], tex[k]["filter"], tex[k]["srgb"]) == (0, 0, 0, 0)
    assert a.normalTexture == a.metallicRoughnessTexture  # same image and settings: shared
    assert tex[b.emissiveTexture]["srgb"] == 1 and tex[b.sheenColourTexture]["srgb"] == 1
    assert np.array_equal(bc["rgba"], opt.decode_png(png))


def test_lights_and_camera(tmp_path):
    g = Gltf()
    lp = g.light(type="point", intensity=683.0, color=[1.0, 0.5, 0.25])
    ld = g.light(type="directional", intensity=10.0)
    ls = g.light(type="spot", intensity=100.0, spot={"innerConeAngle": 0.2, "outerConeAngle": 0.6})
    cam = g.camera(0.8)
    rot = [0.0, math.sin(math.pi / 4), 0.0, math.cos(math.pi / 4)]  # 90 degrees about +y: -z -> -x
    g.node(translation=[1, 2, 3], extensions={"KHR_lights_punctual": {"light": lp}})
    g.node(rotation=rot, extensions={"KHR_lights_punctual": {"light": ld}})
    g.node(translation=[0, 5, 0], rotation=rot, extensions={"KHR_lights_punctual": {"light": ls}})
    g.node(translation=[4, 5, 6], rotation=rot, camera=cam)
    g.node(translation=[9, 9, 9], camera=cam)  # only the first camera counts
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    g.node(mesh=g.mesh([g.primitive(tri, material=g.material())]))
    sc = opt.Scene.from_gltf(g.save(tmp_path / "l.gltf"), up=(0.0, 0.0, 1.0))
    L = sc.lights()
    assert [l.type for l in L] == [0, 1, 2]
    watt = 683.0 / 683.0 * 4 * math.pi
    assert list(L[0].p0) == pytest.approx([1, 2, 3])
    assert list(L[0].radiance) == pytest.approx([watt / (4 * math.pi) * c for c in (1.0, 0.5, 0.25)], rel=1e-6)
    assert list(L[1].normal) == pytest.approx([-1, 0, 0], abs=1e-6)
    assert list(L[1].p0) == pytest.approx([1000, 0, 0], abs=1e-3) and L[1].distance == 1000.0
    w2 = 100.0 / 683.0 * 4 * math.pi
    cos_t = 0.5 * (math.cos(0.6) + math.cos(0.2))
    assert L[2].radiance[0] == pytest.approx(w2 / (2 * math.pi * (1 - cos_t)), rel=1e-5)
    assert (L[2].cosWidth, L[2].cosFalloffStart) == pytest.approx((math.cos(0.6), math.cos(0.2)), rel=1e-6)
    assert list(L[2].p0) == pytest.approx([0, 5, 0]) and list(L[2].normal) == pytest.approx([-1, 0, 0], abs=1e-6)
    a = sc.arrays()
    assert a["camEye"] == pytest.approx([4, 5, 6])
    assert a["camTarget"] == pytest.approx([3, 5, 6], abs=1e-6)
    assert a["camFovYDeg"] == pytest.approx(math.degrees(0.8), rel=1e-6)
    assert a["camUp"] == [0.0, 0.0, 1.0]


def test_skin_rest_pose(tmp_path):
    g = Gltf()
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32)
    joints = np.array([[0, 1, 0, 0]] * 4, np.uint16)
    weights = np.array([[1, 0, 0, 0], [0.5, 0.5, 0, 0], [0.25, 0.75, 0, 0], [0, 1, 0, 0]], np.float32)
    prim = g.primitive(v, np.array([0, 1, 2, 1, 3, 2], np.uint32), material=g.material())
    prim["attributes"]["JOINTS_0"] = g.accessor(joints, 5123)
    prim["attributes"]["WEIGHTS_0"] = g.accessor(weights)
    j0 = g.node(root=False, translation=[0, 0, 1])
    j1 = g.node(root=False, translation=[2, 0, 0])
    ibm = np.stack([np.eye(4), np.eye(4)]).astype(np.float32)
    ibm[1][3, :3] = [-1, 0, 0]  # column-major: translation in the last column
    g.doc["skins"] = [{"joints": [j0, j1], "inverseBindMatrices": g.accessor(ibm.reshape(2, 16), typ="MAT4")}]
    g.node(mesh=g.mesh([prim]), skin=0, translation=[0, 10, 0])
    g.node(children=[j0, j1])
    sc = opt.Scene.from_gltf(g.save(tmp_path / "k.gltf"))
    P = sc.arrays()["positions"]
    J0 = np.eye(4)
    J0[:3, 3] = [0, 0, 1]
    J1 = np.eye(4)
    J1[:3, 3] = [2 - 1, 0, 0]
    want = []
    for p, w in zip(v, weights):
        M = w[0] * J0 + w[1] * J1
        want.append((M @ np.r_[p, 1])[:3])
    # node world * inverse(node world) * joint world * IBM: the node's own
    # translation cancels (src/renderer.cpp:1163-1182)
    assert np.allclose(P, want, atol=1e-5)


def test_scene_description_route(tmp_path):
    sc, path = _cornell_gltf(tmp_path)
    os.makedirs(tmp_path / "configs")
    with open(tmp_path / "configs" / "scene_selection.json", "w") as f:
        json.dump({"scene": "2", "1": "other", "2": "box"}, f)
    with open(tmp_path / "configs" / "box.json", "w") as f:
        json.dump({"scene": {"gltf scene file": "../cornell.gltf", "gltf up hint": [0, 0, 1],
                             "renderer": {"dimensions": [320, 200], "background colour": [0.1, 0.2, 0.3]}}}, f)
    s2 = opt.Scene.from_config(tmp_path / "configs" / "scene_selection.json")
    a = s2.arrays()
    assert (a["resX"], a["resY"]) == (320, 200)
    assert a["bgColour"] == pytest.approx([0.1, 0.2, 0.3])
    assert a["camUp"] == [0.0, 0.0, 1.0]
    assert s2.num_triangles == sc.num_triangles


def test_gltf_errors(tmp_path):
    with pytest.raises(opt.OptptError) as e:
        opt.Scene.from_gltf(tmp_path / "missing.gltf")
    assert e.value.code == -3
    (tmp_path / "bad.gltf").write_text("{ not json")
    with pytest.raises(opt.OptptError) as e:
        opt.Scene.from_gltf(tmp_path / "bad.gltf")
    assert e.value.code == -4
    g = Gltf()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    g.node(mesh=g.mesh([g.primitive(tri, np.array([0, 1, 7], np.uint32))]))
    with pytest.raises(opt.OptptError, match="index out of range"):
        opt.Scene.from_gltf(g.save(tmp_path / "idx.gltf"))
    g = Gltf()
    g.node(mesh=g.mesh([g.primitive(tri)]))
    del g.doc["scene"]
    with pytest.raises(opt.OptptError, match="no scene"):
        opt.Scene.from_gltf(g.save(tmp_path / "noscene.gltf"))
    g = Gltf()
    jpg = g.image(b"\xff\xd8\xff\xe0" + b"\0" * 64, mime="image/jpeg")
    m = g.material(pbrMetallicRoughness={"baseColorTexture": {"index": g.texture(jpg)}})
    g.node(mesh=g.mesh([g.primitive(tri, material=m)]))
    with pytest.raises(opt.OptptError, match="JPEG"):
        opt.Scene.from_gltf(g.save(tmp_path / "badjpg.gltf"))
    g = Gltf()
    gif = g.image(b"GIF89a" + b"\0" * 64, mime="image/gif")
    m = g.material(pbrMetallicRoughness={"baseColorTexture": {"index": g.texture(gif)}})
    g.node(mesh=g.mesh([g.primitive(tri, material=m)]))
    with pytest.raises(opt.OptptError, match="only PNG and JPEG"):
        opt.Scene.from_gltf(g.save(tmp_path / "gif.gltf"))
    g = Gltf()
    g.node(mesh=g.mesh([g.primitive(tri)]))
    g.doc["asset"]["version"] = "1.0"
    with pytest.raises(opt.OptptError, match="version"):
        opt.Scene.from_gltf(g.save(tmp_path / "v1.gltf"))


def _jpeg_image(h, w, grey, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    base = np.stack([(x * 3) % 256, (y * 2 + x) % 256, 128 + 60 * np.sin(x / 7.0) * np.cos(y / 5.0)], -1)
    a = np.clip(base + rng.normal(0, 6, base.shape), 0, 255).astype(np.uint8)
    return a[..., 0] if grey else a


JPEG_CASES = [dict(hs=1, vs=1), dict(hs=2, vs=2), dict(hs=2, vs=1), dict(hs=1, vs=2), dict(hs=4, vs=1),
              dict(hs=2, vs=2, restart=3), dict(hs=2, vs=2, separate_scans=True), dict(hs=1, vs=1, q16=True),
              dict(hs=1, vs=1, adobe_rgb=True)]


@pytest.mark.parametrize("case", range(len(JPEG_CASES)))
@pytest.mark.parametrize("h,w", [(37, 53), (16, 16), (1, 1), (70, 33)])
def test_jpeg_decodes_within_one_level(case, h, w):
    from jpeg_writer import encode_jpeg, reconstruct
    b, info = encode_jpeg(_jpeg_image(h, w, False, case), quality=80, seed=case, **JPEG_CASES[case])
    d = np.abs(opt.decode_jpeg(b).astype(int) - reconstruct(info).astype(int))
    assert d.max() <= 1 and (h * w < 256 or d.mean() < 0.05), (d.max(), d.mean())


def test_jpeg_grey_and_errors():
    from jpeg_writer import encode_jpeg, reconstruct
    b, info = encode_jpeg(_jpeg_image(29, 41, True, 1), quality=50, restart=2)
    d = np.abs(opt.decode_jpeg(b).astype(int) - reconstruct(info).astype(int))
    assert d.max() <= 1
    progressive = bytearray(b)
    i = progressive.index(b"\xff\xc0")
    progressive[i + 1] = 0xC2
    with pytest.raises(opt.OptptError, match="progressive"):
        opt.decode_jpeg(bytes(progressive))
    for bad in (b[: len(b) // 3], b"\xff\xd8\xff\xd9", b"\x00\x01"):
        with pytest.raises(opt.OptptError):
            opt.decode_jpeg(bad)


def test_gltf_with_jpeg_texture(tmp_path):
    from jpeg_writer import encode_jpeg, reconstruct
    b, info = encode_jpeg(_jpeg_image(24, 40, False, 3), quality=90, hs=2, vs=2)
    g = Gltf()
    m = g.material(pbrMetallicRoughness={"baseColorTexture": {"index": g.texture(g.image(b, mime="image/jpeg"))}})
    g.node(mesh=g.mesh([g.primitive(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32),
                                    texcoords=[[0, 0], [1, 0], [0, 1]], material=m)]))
    sc = opt.Scene.from_gltf(g.save(tmp_path / "j.glb", glb=True))
    tex = sc.textures()
    assert len(tex) == 1 and tex[0]["srgb"] == 1
    d = np.abs(tex[0]["rgba"].astype(int) - reconstruct(info).astype(int))
    assert d.max() <= 1
