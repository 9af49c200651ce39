"""Image-output oracle (test infrastructure only; never on a product path).

A numpy restatement of the reference's frame-output arithmetic, and
independent readers for the files the library writes:

* ``process_image``: processImage (cu/kernels.cu:22-33 of the reference):
  r = int(clamp(255.99 * x, 0, 255)) in float32, packed
  0xff000000 | r | g << 8 | b << 16;
* ``rgbe``: the shared-exponent conversion stbi_write_hdr applies to the
  accumulation buffer (src/renderer.cpp:1009-1017; Ward's RGBE: mantissa of
  frexp(max(r, g, b)), channel = c * 256 * m / max truncated);
* ``half_rows``: the accumulation buffer as IEEE halves (OpenEXR's
  Imf::Rgba, cu/kernels.cu:57-76), A = 1, scanlines channel-planar
  A, B, G, R;
* ``read_png`` / ``read_hdr`` / ``read_exr``: format readers written from the
  PNG, Radiance and OpenEXR specifications with Python's zlib, used to check
  what the library's encoders wrote.

Parity is pinned by construction (the reference's formulas are restated in
float32 numpy) and by the readers agreeing with the library's own decoder.
"""
import struct
import zlib

import numpy as np


def process_image(fb):
    """fb: (..., 4) float32 tone-mapped frame buffer -> (..., 4) uint8."""
    f = np.asarray(fb, np.float32)[..., :3]
    q = np.maximum(np.float32(0), np.minimum(np.float32(255.99) * f, np.float32(255))).astype(np.int32)
    out = np.empty(f.shape[:-1] + (4,), np.uint8)
    out[..., :3] = q
    out[..., 3] = 255
    return out


def rgbe(rgba):
    """(..., >=3) float32 -> (..., 4) uint8 RGBE, as float32 operations."""
    c = np.asarray(rgba, np.float32)[..., :3]
    m = np.maximum(c[..., 0], np.maximum(c[..., 1], c[..., 2]))
    ok = m >= np.float32(1e-32)
    mm = np.where(ok, m, np.float32(1))
    f, e = np.frexp(mm)
    scale = (f.astype(np.float32) * np.float32(256)) / mm
    q = np.minimum(np.maximum(c * scale[..., None], np.float32(0)), np.float32(255)).astype(np.uint8)
    out = np.zeros(c.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.where(ok[..., None], q, 0)
    out[..., 3] = np.where(ok, np.minimum(e + 128, 255), 0).astype(np.uint8)
    return out


def half_rows(rgba):
    """(h, w, >=3) float32 -> (h, 4, w) float16 rows: A = 1, B, G, R."""
    c = np.asarray(rgba, np.float32)
    h, w = c.shape[:2]
    rows = np.empty((h, 4, w), np.float16)
    rows[:, 0] = np.float16(1.0)
    rows[:, 1] = c[..., 2].astype(np.float16)
    rows[:, 2] = c[..., 1].astype(np.float16)
    rows[:, 3] = c[..., 0].astype(np.float16)
    return rows


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def read_png(data):
    """8-bit RGBA, non-interlaced PNG -> (h, w, 4) uint8 (the subset the
    library writes), checking every chunk CRC."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(tag + body) & 0xFFFFFFFF == crc, tag
        if tag == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
        pos += 12 + n
    w, h, depth, ct, _, _, inter = hdr
    assert depth == 8 and ct == 6 and inter == 0
    raw = zlib.decompress(idat)
    rb = w * 4
    assert len(raw) == h * (rb + 1)
    out = np.zeros((h, rb), np.uint8)
    prev = np.zeros(rb, np.int64)
    for y in range(h):
        ft = raw[y * (rb + 1)]
        x = np.frombuffer(raw, np.uint8, rb, y * (rb + 1) + 1).astype(np.int64)
        cur = np.zeros(rb, np.int64)
        if ft == 0:
            cur = x
        elif ft == 2:
            cur = (x + prev) & 255
        else:
            for i in range(rb):
                a = cur[i - 4] if i >= 4 else 0
                b = prev[i]
                c = prev[i - 4] if i >= 4 else 0
                pred = a if ft == 1 else (a + b) // 2 if ft == 3 else _paeth(a, b, c)
                cur[i] = (x[i] + pred) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 4)


def read_hdr(data):
    """Radiance RGBE file -> (h, w, 4) uint8 RGBE pixels."""
    end = data.index(b"\n\n")
    header = data[:end].decode()
    assert header.startswith("#?RADIANCE") and "FORMAT=32-bit_rle_rgbe" in header
    nl = data.index(b"\n", end + 2)
    parts = data[end + 2:nl].decode().split()
    assert parts[0] == "-Y" and parts[2] == "+X"
    h, w = int(parts[1]), int(parts[3])
    pos = nl + 1
    out = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w < 32768 and data[pos] == 2 and data[pos + 1] == 2:
            assert (data[pos + 2] << 8) | data[pos + 3] == w
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        n -= 128
                        out[y, x:x + n, c] = data[pos]
                        pos += 1
                    else:
                        assert n > 0
                        out[y, x:x + n, c] = np.frombuffer(data, np.uint8, n, pos)
                        pos += n
                    x += n
                assert x == w
        else:
            out[y] = np.frombuffer(data, np.uint8, w * 4, pos).reshape(w, 4)
            pos += w * 4
    assert pos == len(data)
    return out


def read_exr(data):
    """Single-part scanline OpenEXR with HALF channels, compression NONE or
    ZIP -> (dict of channel -> (h, w) float16, header dict)."""
    magic, version = struct.unpack("<II", data[:8])
    assert magic == 20000630 and (version & 0xFF) == 2
    pos, hdr = 8, {}
    while data[pos] != 0:
        name_end = data.index(b"\0", pos)
        name = data[pos:name_end].decode()
        type_end = data.index(b"\0", name_end + 1)
        typ = data[name_end + 1:type_end].decode()
        size, = struct.unpack("<I", data[type_end + 1:type_end + 5])
        hdr[name] = (typ, data[type_end + 5:type_end + 5 + size])
        pos = type_end + 5 + size
    pos += 1
    chans, p = [], 0
    cl = hdr["channels"][1]
    while cl[p] != 0:
        e = cl.index(b"\0", p)
        ptype, = struct.unpack("<i", cl[e + 1:e + 5])
        assert ptype == 1  # HALF
        chans.append(cl[p:e].decode())
        p = e + 1 + 16
    comp = hdr["compression"][1][0]
    x0, y0, x1, y1 = struct.unpack("<iiii", hdr["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = {0: 1, 2: 1, 3: 16}[comp]
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack("<%dQ" % nchunks, data[pos:pos + 8 * nchunks])
    img = {c: np.zeros((h, w), np.float16) for c in chans}
    for off in offsets:
        y, size = struct.unpack("<iI", data[off:off + 8])
        block = data[off + 8:off + 8 + size]
        n = min(lines, y1 + 1 - y)
        raw_len = n * w * 2 * len(chans)
        if comp != 0 and size < raw_len:
            t = np.frombuffer(zlib.decompress(block), np.uint8).astype(np.int64)
            t = np.cumsum(np.concatenate([[t[0]], t[1:] - 128])) & 255
            half = (len(t) + 1) // 2
            raw = np.empty(len(t), np.uint8)
            raw[0::2] = t[:half]
            raw[1::2] = t[half:]
            block = raw.tobytes()
        assert len(block) == raw_len
        a = np.frombuffer(block, "<f2").reshape(n, len(chans), w)
        for k, c in enumerate(chans):
            img[c][y - y0:y - y0 + n] = a[:, k]
    return img, hdr
