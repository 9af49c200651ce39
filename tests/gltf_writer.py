"""Test-side writers for PNG images and glTF 2.0 files.

The library only decodes; these encoders make the fixtures its importer is
tested on. PNG rows can be written with any of the five filter types (chosen
per row), every colour type and bit depth, tRNS and Adam7 interlacing, and
the zlib stream with any of zlib's strategies (stored, fixed Huffman,
dynamic, Huffman-only, RLE), so the decoder sees every DEFLATE block type.
"""
import base64
import json
import struct
import zlib

import numpy as np

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _pack_row(samples, depth):
    """One row of samples (1-D, already interleaved) to bytes."""
    s = np.asarray(samples, dtype=np.uint32)
    if depth == 8:
        return s.astype(np.uint8).tobytes()
    if depth == 16:
        return s.astype(">u2").tobytes()
    per = 8 // depth
    n = len(s)
    padded = np.zeros(((n + per - 1) // per) * per, np.uint32)
    padded[:n] = s
    padded = padded.reshape(-1, per)
    out = np.zeros(len(padded), np.uint32)
    for k in range(per):
        out |= padded[:, k] << (8 - depth * (k + 1))
    return out.astype(np.uint8).tobytes()


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(rows, bpp, filters):
    out = bytearray()
    prev = np.zeros(len(rows[0]), np.int32) if rows else None
    for i, r in enumerate(rows):
        x = np.frombuffer(r, np.uint8).astype(np.int32)
        a = np.concatenate([np.zeros(bpp, np.int32), x[:-bpp]]) if len(x) > bpp else np.zeros_like(x)
        if len(x) > bpp:
            a[:bpp] = 0
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]]) if len(x) > bpp else np.zeros_like(x)
        b = prev
        ft = filters[i % len(filters)]
        if ft == 0:
            y = x
        elif ft == 1:
            y = x - a
        elif ft == 2:
            y = x - b
        elif ft == 3:
            y = x - (a + b) // 2
        else:
            y = x - _paeth(a, b, c)
        out.append(ft)
        out += (y & 0xFF).astype(np.uint8).tobytes()
        prev = x
    return bytes(out)


def _chunk(tag, data):
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def png_bytes(samples, colour_type=6, depth=8, palette=None, trns=None, interlace=False, filters=(0, 1, 2, 3, 4),
              level=6, strategy=zlib.Z_DEFAULT_STRATEGY, idat_split=3):
    """samples: H x W x channels array of raw sample values (palette
    indices for colour type 3)."""
    samples = np.asarray(samples)
    h, w = samples.shape[:2]
    ch = CHANNELS[colour_type]
    samples = samples.reshape(h, w, ch)
    bpp = max(1, ch * depth // 8)

    def encode(img):
        rows = [_pack_row(img[y].reshape(-1), depth) for y in range(img.shape[0])]
        return _filter_rows(rows, bpp, filters)

    if not interlace:
        raw = encode(samples)
    else:
        raw = b""
        for x0, y0, dx, dy in ADAM7:
            sub = samples[y0::dy, x0::dx]
            if sub.shape[0] and sub.shape[1]:
                raw += encode(sub)
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = co.compress(raw) + co.flush()
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, colour_type, 0, 0,
                                                             1 if interlace else 0))
    if palette is not None:
        out += _chunk(b"PLTE", np.asarray(palette, np.uint8).reshape(-1).tobytes())
    if trns is not None:
        out += _chunk(b"tRNS", trns)
    step = max(1, len(z) // idat_split + 1)
    for i in range(0, len(z), step):
        out += _chunk(b"IDAT", z[i:i + step])
    return out + _chunk(b"IEND", b"")


def expected_rgba(samples, colour_type, depth, palette=None, trns=None):
    """What a four-component stb-style decode gives."""
    s = np.asarray(samples).astype(np.int64)
    h, w = s.shape[:2]
    s = s.reshape(h, w, CHANNELS[colour_type])

    def to8(v):
        if depth == 16:
            return v >> 8
        if depth == 8:
            return v
        return v * (255 // ((1 << depth) - 1))

    out = np.zeros((h, w, 4), np.int64)
    if colour_type == 0:
        g = to8(s[..., 0])
        out[..., 0] = out[..., 1] = out[..., 2] = g
        out[..., 3] = 255
        if trns is not None:
            key = struct.unpack(">H", trns)[0]
            out[..., 3] = np.where(s[..., 0] == key, 0, 255)
    elif colour_type == 2:
        out[..., :3] = to8(s)
        out[..., 3] = 255
        if trns is not None:
            key = np.array(struct.unpack(">HHH", trns))
            out[..., 3] = np.where((s == key).all(-1), 0, 255)
    elif colour_type == 3:
        pal = np.concatenate([np.asarray(palette, np.int64).reshape(-1, 3),
                              np.full((len(palette), 1), 255, np.int64)], 1)
        if trns is not None:
            t = np.frombuffer(trns, np.uint8)
            pal[:len(t), 3] = t
        out = pal[s[..., 0]]
    elif colour_type == 4:
        out[..., 0] = out[..., 1] = out[..., 2] = to8(s[..., 0])
        out[..., 3] = to8(s[..., 1])
    else:
        out[...] = to8(s)
    return out.astype(np.uint8)


class Gltf:
    """A minimal glTF 2.0 document builder: one binary buffer, accessors,
    meshes, nodes, materials, textures, lights and cameras."""

    def __init__(self):
        self.doc = {"asset": {"version": "2.0", "generator": "optpt tests"}, "scene": 0,
                    "scenes": [{"nodes": []}], "nodes": [], "meshes": [], "accessors": [], "bufferViews": [],
                    "buffers": [], "materials": []}
        self.bin = bytearray()

    def _view(self, data, stride=None):
        while len(self.bin) % 4:
            self.bin.append(0)
        v = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)}
        if stride:
            v["byteStride"] = stride
        self.bin += data
        self.doc["bufferViews"].append(v)
        return len(self.doc["bufferViews"]) - 1

    def accessor(self, arr, ctype=5126, typ=None, normalized=False, stride=None):
        arr = np.asarray(arr)
        comps = 1 if arr.ndim == 1 else arr.shape[1]
        typ = typ or {1: "SCALAR", 2: "VEC2", 3: "VEC3", 4: "VEC4", 16: "MAT4"}[comps]
        dt = {5126: "<f4", 5125: "<u4", 5123: "<u2", 5121: "u1", 5122: "<i2", 5120: "i1"}[ctype]
        a = np.ascontiguousarray(arr.astype(dt))
        if stride:
            row = a.reshape(len(a), -1).view(np.uint8)
            buf = np.zeros((len(a), stride), np.uint8)
            buf[:, :row.shape[1]] = row
            view = self._view(buf.tobytes(), stride)
        else:
            view = self._view(a.tobytes())
        acc = {"bufferView": view, "componentType": ctype, "count": int(len(a)), "type": typ}
        if normalized:
            acc["normalized"] = True
        if typ == "VEC3" and ctype == 5126:
            acc["min"] = a.min(0).tolist() if len(a) else [0, 0, 0]
            acc["max"] = a.max(0).tolist() if len(a) else [0, 0, 0]
        self.doc["accessors"].append(acc)
        return len(self.doc["accessors"]) - 1

    def mesh(self, primitives):
        self.doc["meshes"].append({"primitives": primitives})
        return len(self.doc["meshes"]) - 1

    def primitive(self, positions, indices=None, normals=None, texcoords=None, material=None, mode=None,
                  index_type=5125):
        p = {"attributes": {"POSITION": self.accessor(np.asarray(positions, np.float32))}}
        if normals is not None:
            p["attributes"]["NORMAL"] = self.accessor(np.asarray(normals, np.float32))
        if texcoords is not None:
            p["attributes"]["TEXCOORD_0"] = self.accessor(np.asarray(texcoords, np.float32))
        if indices is not None:
            p["indices"] = self.accessor(np.asarray(indices).reshape(-1), index_type)
        if material is not None:
            p["material"] = material
        if mode is not None:
            p["mode"] = mode
        return p

    def node(self, root=True, **kw):
        self.doc["nodes"].append(dict(kw))
        i = len(self.doc["nodes"]) - 1
        if root:
            self.doc["scenes"][0]["nodes"].append(i)
        return i

    def material(self, **kw):
        self.doc["materials"].append(kw)
        return len(self.doc["materials"]) - 1

    def image(self, png, embed="view", mime="image/png"):
        imgs = self.doc.setdefault("images", [])
        if embed == "view":
            imgs.append({"bufferView": self._view(png), "mimeType": mime})
        elif embed == "data":
            imgs.append({"uri": "data:%s;base64,%s" % (mime, base64.b64encode(png).decode())})
        else:  # a file name written beside the .gltf by save()
            imgs.append({"uri": embed})
            self.files = getattr(self, "files", {})
            self.files[embed] = png
        return len(imgs) - 1

    def texture(self, image, sampler=None):
        t = {"source": image}
        if sampler is not None:
            ss = self.doc.setdefault("samplers", [])
            ss.append(sampler)
            t["sampler"] = len(ss) - 1
        self.doc.setdefault("textures", []).append(t)
        return len(self.doc["textures"]) - 1

    def light(self, **kw):
        ext = self.doc.setdefault("extensions", {}).setdefault("KHR_lights_punctual", {"lights": []})
        ext["lights"].append(kw)
        return len(ext["lights"]) - 1

    def camera(self, yfov, aspect=None):
        persp = {"yfov": yfov, "znear": 0.01}
        if aspect:
            persp["aspectRatio"] = aspect
        self.doc.setdefault("cameras", []).append({"type": "perspective", "perspective": persp})
        return len(self.doc["cameras"]) - 1

    def save(self, path, glb=False, buffer_uri="data"):
        path = str(path)
        doc = json.loads(json.dumps(self.doc))
        binary = bytes(self.bin)
        import os
        base = os.path.dirname(path)
        for name, data in getattr(self, "files", {}).items():
            with open(os.path.join(base, name), "wb") as f:
                f.write(data)
        if glb:
            doc["buffers"] = [{"byteLength": len(binary)}]
            js = json.dumps(doc).encode()
            js += b" " * ((4 - len(js) % 4) % 4)
            bn = binary + b"\0" * ((4 - len(binary) % 4) % 4)
            body = struct.pack("<I", len(js)) + b"JSON" + js + struct.pack("<I", len(bn)) + b"BIN\0" + bn
            with open(path, "wb") as f:
                f.write(b"glTF" + struct.pack("<II", 2, 12 + len(body)) + body)
            return path
        if buffer_uri == "data":
            doc["buffers"] = [{"byteLength": len(binary),
                               "uri": "data:application/octet-stream;base64," + base64.b64encode(binary).decode()}]
        else:
            with open(os.path.join(base, buffer_uri), "wb") as f:
                f.write(binary)
            doc["buffers"] = [{"byteLength": len(binary), "uri": buffer_uri.replace(" ", "%20")}]
        with open(path, "w") as f:
            json.dump(doc, f, indent=1)
        return path


def material_json(m):
    """glTF material for a MaterialData record (factors only)."""
    mj = {"pbrMetallicRoughness": {"baseColorFactor": [float(v) for v in m.baseColour],
                                   "metallicFactor": float(m.metallic), "roughnessFactor": float(m.roughness)},
          "extensions": {"KHR_materials_specular": {"specularFactor": float(m.specular)},
                         "KHR_materials_ior": {"ior": float(m.ior)}}}
    if max(m.emission) > 0:
        mj["emissiveFactor"] = [float(v) for v in m.emission]  # unclamped, as tinygltf accepts
    if m.transmissionWeight:
        mj["extensions"]["KHR_materials_transmission"] = {"transmissionFactor": float(m.transmissionWeight)}
    if m.coatWeight:
        mj["extensions"]["KHR_materials_clearcoat"] = {"clearcoatFactor": float(m.coatWeight),
                                                       "clearcoatRoughnessFactor": float(m.coatRoughness)}
    if max(m.sheenColour) > 0:
        mj["extensions"]["KHR_materials_sheen"] = {"sheenColorFactor": [float(v) for v in m.sheenColour],
                                                   "sheenRoughnessFactor": float(m.sheenRoughness)}
    if m.alphaMode:
        mj["alphaMode"] = {1: "BLEND", 2: "MASK"}[m.alphaMode]
        mj["alphaCutoff"] = float(m.alphaCutoff)
    return mj


def from_scene(scene):
    """A glTF document holding a flattened scene: one mesh node whose
    primitives are the runs of equal material, triangle order kept."""
    a = scene.arrays()
    g = Gltf()
    for m in scene.materials():
        g.material(**material_json(m))
    P, N, T, I, M = a["positions"], a["normals"], a["texCoords"], a["triIndices"], a["matIndices"]
    prims = []
    start = 0
    for k in range(1, len(M) + 1):
        if k == len(M) or M[k] != M[start]:
            tri = I[start:k]
            used, inv = np.unique(tri.reshape(-1), return_inverse=True)
            prims.append(g.primitive(P[used], inv.reshape(-1, 3).astype(np.uint32),
                                     None if N is None else N[used], None if T is None else T[used],
                                     material=int(M[start])))
            start = k
    g.node(mesh=g.mesh(prims))
    return g


def _box(c, h):
    """12-triangle box (24 vertices with face normals) centred at c, half size h."""
    c, h = np.asarray(c, np.float32), np.asarray(h, np.float32)
    P, N, I = [], [], []
    for ax in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3, np.float32)
            n[ax] = sgn
            u = np.zeros(3, np.float32)
            u[(ax + 1) % 3] = 1
            v = np.cross(n, u)
            base = len(P)
            for a, b in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                P.append(c + h * (n + a * u + b * v))
                N.append(n)
            I += [base, base + 1, base + 2, base, base + 2, base + 3]
    return np.array(P, np.float32), np.array(N, np.float32), np.array(I, np.uint32)


def animated_scene(num_animations=3):
    """A small animated document: a rotating arm carrying a box that steps
    along (node translation STEP), a skinned strip bent by two animated
    joints (rotation LINEAR, scale CUBICSPLINE), a static ground and an
    emissive panel on the arm. The animation that moves things is the one
    the reference selects (index 2 when there are three or more, else 0);
    the others move the ground, which must therefore stay still."""
    g = Gltf()
    grey = g.material(pbrMetallicRoughness={"baseColorFactor": [0.7, 0.7, 0.7, 1], "metallicFactor": 0.0},
                      extensions={"KHR_materials_specular": {"specularFactor": 0.0}})
    red = g.material(pbrMetallicRoughness={"baseColorFactor": [0.8, 0.2, 0.1, 1], "metallicFactor": 0.0,
                                           "roughnessFactor": 0.5})
    lamp = g.material(emissiveFactor=[1.0, 1.0, 0.9], extensions={"KHR_materials_emissive_strength":
                                                                  {"emissiveStrength": 8.0}})
    bp, bn, bi = _box([0, 0, 0], [0.3, 0.3, 0.3])
    box = g.mesh([g.primitive(bp, bi, bn, material=red)])
    panel = g.mesh([g.primitive(np.array([[-0.3, 0, -0.3], [0.3, 0, -0.3], [0.3, 0, 0.3], [-0.3, 0, 0.3]],
                                         np.float32), np.array([0, 2, 1, 0, 3, 2], np.uint32),
                                np.tile(np.array([[0, -1, 0]], np.float32), (4, 1)), material=lamp)])
    # skinned strip along x in [-1, 1], 9 columns x 2 rows
    xs = np.linspace(-1, 1, 9, dtype=np.float32)
    sp = np.array([[x, 0.0, z] for x in xs for z in (-0.2, 0.2)], np.float32)
    sn = np.tile(np.array([[0, 1, 0]], np.float32), (len(sp), 1))
    si = []
    for k in range(8):
        a, b, c, d = 2 * k, 2 * k + 1, 2 * k + 2, 2 * k + 3
        si += [a, b, d, a, d, c]
    w1 = np.clip((sp[:, 0] + 1) / 2, 0, 1)
    joints = np.tile(np.array([[0, 1, 0, 0]], np.uint16), (len(sp), 1))
    weights = np.stack([1 - w1, w1, np.zeros_like(w1), np.zeros_like(w1)], 1).astype(np.float32)
    strip = g.primitive(sp, np.array(si, np.uint32), sn, material=grey)
    strip["attributes"]["JOINTS_0"] = g.accessor(joints, 5123)
    strip["attributes"]["WEIGHTS_0"] = g.accessor(weights)
    strip_mesh = g.mesh([strip])
    gp = np.array([[-3, 0, -3], [3, 0, -3], [3, 0, 3], [-3, 0, 3]], np.float32)
    ground = g.mesh([g.primitive(gp, np.array([0, 2, 1, 0, 3, 2], np.uint32),
                                 np.tile(np.array([[0, 1, 0]], np.float32), (4, 1)), material=grey)])
    box_node = g.node(root=False, mesh=box, translation=[1.0, 0.5, 0.0])
    panel_node = g.node(root=False, mesh=panel, translation=[0.0, 2.0, 0.0])
    arm = g.node(children=[box_node, panel_node], translation=[0.0, 0.2, 0.0])
    bone0 = g.node(root=False, translation=[-1.0, 0.0, 0.0])
    bone1 = g.node(root=False, translation=[2.0, 0.0, 0.0])
    g.doc["nodes"][bone0]["children"] = [bone1]
    ibm = np.stack([np.eye(4), np.eye(4)]).astype(np.float32)
    ibm[0][3, :3] = [1.0, 0, 0]   # column-major: translations in the last column
    ibm[1][3, :3] = [-1.0, 0, 0]
    g.doc["skins"] = [{"joints": [bone0, bone1], "inverseBindMatrices": g.accessor(ibm.reshape(2, 16), typ="MAT4")}]
    strip_node = g.node(mesh=strip_mesh, skin=0, translation=[0.0, 1.0, -1.0])
    rig = g.node(children=[bone0], translation=[0.0, 1.0, -1.0])
    ground_node = g.node(mesh=ground)

    def sampler(times, values, interp):
        t = g.accessor(np.asarray(times, np.float32).reshape(-1))
        v = g.accessor(np.asarray(values, np.float32))
        return {"input": t, "output": v, "interpolation": interp}

    s2, c2 = 0.7071067811865476, 0.7071067811865476
    moving = {"samplers": [
        sampler([0.0, 1.0, 2.0], [[0, 0, 0, 1], [0, s2, 0, c2], [0, 1, 0, 0]], "LINEAR"),            # arm yaw
        sampler([0.5, 1.5], [[1.0, 0.5, 0.0], [1.5, 0.8, 0.3]], "STEP"),                              # box steps
        sampler([0.0, 1.0, 2.0], [[0, 0, 0, 1], [0, 0, 0.3826834, 0.9238795], [0, 0, 0, 1]], "LINEAR"),  # bone0 bend
        sampler([0.0, 1.0, 2.0],                                                                        # bone1 scale
                [[0, 0, 0], [1, 1, 1], [0.5, 0, 0], [-0.5, 0, 0], [1.5, 1, 1], [0, 0, 0],
                 [0, 0, 0], [1, 1, 1], [0, 0, 0]], "CUBICSPLINE")],
        "channels": [{"sampler": 0, "target": {"node": arm, "path": "rotation"}},
                     {"sampler": 1, "target": {"node": box_node, "path": "translation"}},
                     {"sampler": 2, "target": {"node": bone0, "path": "rotation"}},
                     {"sampler": 3, "target": {"node": bone1, "path": "scale"}}]}
    decoy = {"samplers": [sampler([0.0, 1.0], [[0, 0, 0], [0, 5, 0]], "LINEAR")],
             "channels": [{"sampler": 0, "target": {"node": ground_node, "path": "translation"}}]}
    anims = [decoy] * num_animations
    anims[2 if num_animations >= 3 else 0] = moving
    g.doc["animations"] = anims
    cam = g.camera(0.8)
    g.node(translation=[0.0, 2.0, 5.0], rotation=[-0.1305262, 0, 0, 0.9914449], camera=cam)
    g.light(type="point", intensity=3000.0)
    g.node(translation=[2.0, 3.0, 2.0], extensions={"KHR_lights_punctual": {"light": 0}})
    return g
