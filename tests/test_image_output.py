"""Image writers on the host (no GPU): the PNG, Radiance .hdr and OpenEXR
encoders against independent readers (Python's zlib and the format
specifications, oracle/image_oracle.py) and the library's own PNG decoder.

* PNG: noise (stored blocks), smooth images (long matches), a multi-piece
  stream compressed on several threads; every chunk CRC checked.
* HDR: run-length scanlines (and flat ones for narrow images) carry exactly
  the RGBE pixels of Ward's conversion as the reference's writer applies it.
* EXR: NONE and ZIP scanline files carry exactly numpy's float16 of every
  channel (round to nearest even), A = 1; the float-to-half conversion is
  bit-exact on 200,000 random bit patterns and the rounding edges.
"""
import struct
import zlib

import numpy as np
import pytest

import optix_pt_gb300 as opt
from oracle import image_oracle as io


def _smooth(h, w, noise=0, seed=0):
    y, x = np.mgrid[0:h, 0:w]
    img = np.stack([(x // 3) % 256, (y // 5) % 256, ((x + y) // 7) % 256, np.full_like(x, 255)], -1)
    if noise:
        rng = np.random.default_rng(seed)
        img[..., :3] = np.clip(img[..., :3] + rng.integers(-noise, noise + 1, (h, w, 3)), 0, 255)
    return img.astype(np.uint8)


@pytest.mark.parametrize("kind,h,w", [("noise", 37, 53), ("smooth", 64, 64), ("noisy", 31, 17), ("one", 1, 1)])
def test_png_round_trip_small(kind, h, w):
    rng = np.random.default_rng(h * w)
    img = rng.integers(0, 256, (h, w, 4)).astype(np.uint8) if kind in ("noise", "one") else \
        _smooth(h, w, 3 if kind == "noisy" else 0)
    b = opt.encode_png(img)
    assert np.array_equal(io.read_png(b), img)
    assert np.array_equal(opt.decode_png(b), img)


def test_png_multi_piece_stream():
    img = _smooth(900, 1000, noise=4, seed=2)  # 3.6 MB of filtered rows: several pieces
    b = opt.encode_png(img)
    assert len(b) < img.size * 0.6
    pos, z = 8, b""
    while pos < len(b):
        n, = struct.unpack(">I", b[pos:pos + 4])
        if b[pos + 4:pos + 8] == b"IDAT":
            z += b[pos + 8:pos + 8 + n]
        pos += 12 + n
    raw = zlib.decompress(z)  # zlib validates the stream and its Adler-32
    assert len(raw) == 900 * (1000 * 4 + 1)
    assert np.array_equal(opt.decode_png(b), img)


def _radiance(h, w, seed):
    rng = np.random.default_rng(seed)
    img = (rng.lognormal(0, 3, (h, w, 4)) * rng.choice([0, 1], (h, w, 4), p=[0.1, 0.9])).astype(np.float32)
    img[0, :10] = 0
    img[1, :20] = img[1, 0]
    img[2, 3] = [-1.0, 2.0, 0.5, 1.0]  # negative channels clamp to 0
    img[3, 4] = [1e-35, 0, 0, 0]       # below 1e-32: black
    return img


@pytest.mark.parametrize("w", [5, 8, 41, 300])
def test_hdr_carries_reference_rgbe(w):
    img = _radiance(23, w, w)
    assert np.array_equal(io.read_hdr(opt.encode_hdr(img)), io.rgbe(img))


@pytest.mark.parametrize("compression", [0, 3])
def test_exr_carries_half_channels(compression):
    img = _radiance(37, 29, 7)
    with np.errstate(over="ignore"):
        rows = io.half_rows(img)
    ch, hdr = io.read_exr(opt.encode_exr(img, compression))
    assert list(ch) == ["A", "B", "G", "R"]
    assert hdr["compression"][1][0] == compression
    for k, c in enumerate("ABGR"):
        assert np.array_equal(ch[c].view(np.uint16), rows[:, k].view(np.uint16)), c


def test_half_conversion_bit_exact():
    rng = np.random.default_rng(3)
    edges = np.array([0, 0x80000000, 0x33000000, 0x33000001, 0x32FFFFFF, 0x33800000, 0x387FC000, 0x387FE000,
                      0x38800000, 0x477FE000, 0x477FF000, 0x477FEFFF, 0x47800000, 0x7F800000, 0x7FC00000,
                      0xFF800000, 0x00000001, 0x3F800000, 0x3F801000, 0x3F803000, 0x3F802000], np.uint32)
    bits = np.concatenate([rng.integers(0, 2 ** 32, 200000 - len(edges), dtype=np.uint64).astype(np.uint32), edges])
    f = bits.view(np.float32).reshape(200, 1000)
    img = np.zeros((200, 1000, 4), np.float32)
    img[..., 0] = f
    ch, _ = io.read_exr(opt.encode_exr(img, 0))
    with np.errstate(over="ignore", invalid="ignore"):
        want = f.astype(np.float16)
    nan = np.isnan(f)
    assert np.array_equal(ch["R"].view(np.uint16)[~nan], want.view(np.uint16)[~nan])
    assert np.isnan(ch["R"][nan]).all()


def test_encoder_errors():
    with pytest.raises(opt.OptptError):
        opt.encode_exr(np.zeros((4, 4, 4), np.float32), compression=1)
    with pytest.raises(opt.OptptError):
        opt.encode_png(np.zeros((0, 4, 4), np.uint8))
