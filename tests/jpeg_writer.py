"""A test-side baseline JPEG encoder (ITU-T T.81 sequential, Huffman) and the
ideal reconstruction of what it encoded.

The library only decodes; this encoder makes its fixtures: grey or YCbCr
(or Adobe RGB) images, any luma sampling factors with 1x1 chroma,
interleaved or one-scan-per-component frames, 8- or 16-bit quantisation
tables, restart intervals, and Huffman tables built from the image's own
symbol statistics (length-limited to 16 bits, no all-ones code).
`reconstruct` decodes the quantised coefficients in float64 with the
reconstruction rules the library documents (inverse DCT, rounding, centred
bilinear chroma upsampling, JFIF YCbCr -> RGB), for comparison within a
level of rounding.
"""
import heapq
import struct

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27,
                   20, 13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58,
                   59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


def _dct_matrix():
    c = np.zeros((8, 8))
    for u in range(8):
        for x in range(8):
            c[u, x] = (np.sqrt(0.5) if u == 0 else 1.0) * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16)
    return c


C = _dct_matrix()


def quant_table(quality, chroma, rng):
    base = rng.integers(8, 60, 64) if chroma else rng.integers(4, 40, 64)
    base = np.sort(base)[np.argsort(np.argsort(ZIGZAG))]  # rising along the zigzag
    scale = 5000 / quality if quality < 50 else 200 - 2 * quality
    return np.clip((base * scale + 50) // 100, 1, 255).astype(np.int64)


def _huffman_lengths(freq):
    """Code lengths (<= 16) for symbols with freq > 0, plus a reserved
    all-ones code that no symbol gets."""
    f = {s: v for s, v in freq.items() if v > 0}
    while True:
        heap = [(v, i, [s]) for i, (s, v) in enumerate(sorted(f.items()))]
        heap.append((0.5, -1, [None]))  # the reserved code
        heapq.heapify(heap)
        depth = {s: 0 for s in list(f) + [None]}
        cnt = len(heap)
        while len(heap) > 1:
            a = heapq.heappop(heap)
            b = heapq.heappop(heap)
            for s in a[2] + b[2]:
                depth[s] += 1
            heapq.heappush(heap, (a[0] + b[0], cnt, a[2] + b[2]))
            cnt += 1
        if max(depth.values()) <= 16:
            return depth
        f = {s: max(1, v // 2) for s, v in f.items()}


def _canonical(depth):
    """BITS counts, HUFFVAL symbols and {symbol: (code, length)}; the reserved
    code is the last (all ones) of the longest length and is dropped."""
    order = sorted(depth, key=lambda s: (depth[s], s is None, -1 if s is None else s))
    codes, code, prev = {}, 0, 0
    for s in order:
        L = depth[s]
        code <<= (L - prev)
        prev = L
        codes[s] = (code, L)
        code += 1
    del codes[None]
    bits = [0] * 16
    vals = []
    for s in order:
        if s is None:
            continue
        bits[depth[s] - 1] += 1
        vals.append(s)
    return bits, vals, codes


def _category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _bits_of(v, s):
    return v if v >= 0 else v + (1 << s) - 1


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, v, k):
        for i in range(k - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        while self.n:
            self.put(1, 1)


def _seg(marker, payload):
    return struct.pack(">BBH", 0xFF, marker, len(payload) + 2) + payload


def encode_jpeg(img, quality=75, hs=2, vs=2, restart=0, separate_scans=False, q16=False, adobe_rgb=False, seed=0):
    """img: (H, W) grey or (H, W, 3) RGB uint8. Returns (bytes, info) where
    info holds what `reconstruct` needs."""
    rng = np.random.default_rng(seed)
    img = np.asarray(img, np.float64)
    H, W = img.shape[:2]
    grey = img.ndim == 2
    if grey:
        planes, factors = [img], [(1, 1)]
        hs = vs = 1
    else:
        R, G, B = img[..., 0], img[..., 1], img[..., 2]
        if adobe_rgb:
            ys = [R, G, B]
        else:
            ys = [0.299 * R + 0.587 * G + 0.114 * B, -0.168736 * R - 0.331264 * G + 0.5 * B + 128,
                  0.5 * R - 0.418688 * G - 0.081312 * B + 128]
        planes = [ys[0]]
        factors = [(hs, vs), (1, 1), (1, 1)]
        for ch in ys[1:]:
            ph, pw = -(-H // vs) * vs, -(-W // hs) * hs
            padded = np.pad(ch, ((0, ph - H), (0, pw - W)), mode="edge")
            planes.append(padded.reshape(ph // vs, vs, pw // hs, hs).mean((1, 3)))
    hmax, vmax = max(f[0] for f in factors), max(f[1] for f in factors)
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    qts = [quant_table(quality, False, rng), quant_table(quality, True, rng)]
    comps = []
    for ci, (pl, (h, v)) in enumerate(zip(planes, factors)):
        bw, bh = mcux * h, mcuy * v
        pad = np.pad(pl, ((0, bh * 8 - pl.shape[0]), (0, bw * 8 - pl.shape[1])), mode="edge")
        blocks = pad.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3) - 128.0
        coef = np.einsum("ux,abxy,vy->abuv", C, blocks, C)
        q = qts[0 if ci == 0 else 1].reshape(8, 8)
        quant = np.rint(coef / q).astype(np.int64)
        comps.append({"id": ci + 1, "h": h, "v": v, "tq": 0 if ci == 0 else 1, "q": quant, "bw": bw, "bh": bh,
                      "cw": -(-W * h // hmax), "ch": -(-H * v // vmax)})
    # symbol statistics for per-class Huffman tables
    def units(scan):
        if len(scan) == 1:
            c = scan[0]
            ux, uy = -(-c["cw"] // 8), -(-c["ch"] // 8)
            return [[(c, bx, by)] for by in range(uy) for bx in range(ux)]
        return [[(c, mx * c["h"] + bx, my * c["v"] + by) for c in scan for by in range(c["v"]) for bx in range(c["h"])]
                for my in range(mcuy) for mx in range(mcux)]

    scans = [[c] for c in comps] if separate_scans else [comps]
    freqs = {("dc", 0): {}, ("dc", 1): {}, ("ac", 0): {}, ("ac", 1): {}}

    def walk(scan, emit):
        preds = {c["id"]: 0 for c in scan}
        for u, unit in enumerate(units(scan)):
            if restart and u and u % restart == 0:
                emit("rst", (u // restart - 1) % 8)
                preds = {c["id"]: 0 for c in scan}
            for c, bx, by in unit:
                t = 0 if c["id"] == 1 else 1
                blk = c["q"][by, bx].reshape(-1)[ZIGZAG]
                d = int(blk[0]) - preds[c["id"]]
                preds[c["id"]] = int(blk[0])
                emit(("dc", t), (_category(d), d))
                run = 0
                last = max([k for k in range(1, 64) if blk[k] != 0], default=0)
                for k in range(1, last + 1):
                    if blk[k] == 0:
                        run += 1
                        continue
                    while run > 15:
                        emit(("ac", t), (0xF0, None))
                        run -= 16
                    s = _category(int(blk[k]))
                    emit(("ac", t), ((run << 4) | s, int(blk[k])))
                    run = 0
                if last < 63:
                    emit(("ac", t), (0x00, None))

    def count(kind, val):
        if kind == "rst":
            return
        sym = val[0]
        freqs[kind][sym] = freqs[kind].get(sym, 0) + 1

    for sc in scans:
        walk(sc, count)
    tables = {}
    for key, f in freqs.items():
        if not f:
            f = {0: 1}
        tables[key] = _canonical(_huffman_lengths(f))
    out = bytearray(b"\xff\xd8")
    out += _seg(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    if adobe_rgb:
        out += _seg(0xEE, b"Adobe\x00\x64\x00\x00\x00\x00\x00")
    for t, qt in enumerate(qts[:1 if grey else 2]):
        zz = qt[ZIGZAG]
        if q16:
            out += _seg(0xDB, bytes([0x10 | t]) + b"".join(struct.pack(">H", int(v)) for v in zz))
        else:
            out += _seg(0xDB, bytes([t]) + bytes(int(v) for v in zz))
    sof = struct.pack(">BHHB", 8, H, W, len(comps))
    for c in comps:
        sof += bytes([c["id"], (c["h"] << 4) | c["v"], c["tq"]])
    out += _seg(0xC0, sof)
    for (kind, t), (bits, vals, _) in tables.items():
        if grey and t == 1:
            continue
        out += _seg(0xC4, bytes([(0 if kind == "dc" else 1) << 4 | t]) + bytes(bits) + bytes(vals))
    if restart:
        out += _seg(0xDD, struct.pack(">H", restart))
    for sc in scans:
        sos = bytes([len(sc)])
        for c in sc:
            t = 0 if c["id"] == 1 else 1
            sos += bytes([c["id"], (t << 4) | t])
        out += _seg(0xDA, sos + b"\x00\x3f\x00")
        bw = _BitWriter()

        def write(kind, val):
            if kind == "rst":
                bw.flush()
                bw.out += bytes([0xFF, 0xD0 + val])
                return
            sym, extra = val
            code, L = tables[kind][2][sym]
            bw.put(code, L)
            size = sym if kind[0] == "dc" else sym & 15
            if size:
                bw.put(_bits_of(extra, size), size)

        walk(sc, write)
        bw.flush()
        out += bw.out
    out += b"\xff\xd9"
    return bytes(out), {"comps": comps, "qts": qts, "W": W, "H": H, "hmax": hmax, "vmax": vmax, "grey": grey,
                        "adobe_rgb": adobe_rgb}


def reconstruct(info):
    """The decoded image (H, W, 4) uint8 in float64 arithmetic."""
    W, H, hmax, vmax = info["W"], info["H"], info["hmax"], info["vmax"]
    planes = []
    for c in info["comps"]:
        q = info["qts"][c["tq"]].reshape(8, 8)
        coef = c["q"] * q
        blocks = np.einsum("ux,abuv,vy->abxy", C, coef, C) + 128.0
        pix = np.clip(np.floor(blocks + 0.5), 0, 255)
        bh, bw = c["bh"], c["bw"]
        plane = pix.transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)
        if c["h"] == hmax and c["v"] == vmax:
            planes.append(plane[:H, :W])
            continue
        cw, ch = c["cw"], c["ch"]
        xs = (np.arange(W) + 0.5) * c["h"] / hmax - 0.5
        ys = (np.arange(H) + 0.5) * c["v"] / vmax - 0.5
        x0, y0 = np.floor(xs).astype(int), np.floor(ys).astype(int)
        fx, fy = xs - x0, ys - y0
        cx = lambda a: np.clip(a, 0, cw - 1)
        cy = lambda a: np.clip(a, 0, ch - 1)
        p00 = plane[cy(y0)][:, cx(x0)]
        p10 = plane[cy(y0)][:, cx(x0 + 1)]
        p01 = plane[cy(y0 + 1)][:, cx(x0)]
        p11 = plane[cy(y0 + 1)][:, cx(x0 + 1)]
        top = p00 + (p10 - p00) * fx[None]
        bot = p01 + (p11 - p01) * fx[None]
        planes.append(top + (bot - top) * fy[:, None])
    out = np.full((H, W, 4), 255, np.uint8)
    if info["grey"]:
        out[..., :3] = planes[0][..., None].astype(np.uint8)
        return out
    Y, cb, cr = planes
    if info["adobe_rgb"]:
        rgb = [Y, cb, cr]
    else:
        rgb = [Y + 1.402 * (cr - 128), Y - 0.344136 * (cb - 128) - 0.714136 * (cr - 128), Y + 1.772 * (cb - 128)]
    for k in range(3):
        out[..., k] = np.clip(np.floor(rgb[k] + 0.5), 0, 255).astype(np.uint8)
    return out
