"""Frame output on the GPU against the image oracle.

* processImage's RGBA8 of the tone-mapped frame buffer, bit-exact.
* The fused output kernel's RGBE and HALF payloads of the accumulated mean,
  bit-exact against Ward's RGBE and numpy float16 of the FP64 mean.
* dumpFramebuffer / dumpAccumFramebufferRgbe / the EXR dump write files
  whose pixels read back (independent readers) to exactly those payloads,
  under the reference's default names when no path is given.
"""
import numpy as np
import pytest

from oracle import image_oracle as io

pytestmark = pytest.mark.gpu


@pytest.fixture()
def rendered(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("cornell")
    r = opt.Renderer(sc, spp_batch=4)
    r.setupOutputBuffer(83, 61)  # odd sizes: rows straddle warps and blocks
    r.render(12, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = r.accum()
    mean = np.zeros(s.shape[:2] + (4,), np.float32)
    mean[..., :3] = (s * (1.0 / n)).astype(np.float32)
    yield r, mean
    r.close()


def test_rgba8_matches_process_image(rendered):
    r, _ = rendered
    fb = r.frame_buffer()
    assert np.array_equal(r.rgba8(), io.process_image(fb))


def test_fused_payloads_bit_exact(rendered):
    import torch
    r, mean = rendered
    h, w = mean.shape[:2]
    dev = torch.device("cuda")
    rgba8 = torch.empty(h * w, dtype=torch.int32, device=dev)
    rgbe = torch.empty(h * w, dtype=torch.int32, device=dev)
    rows = torch.empty(h * w * 4, dtype=torch.float16, device=dev)
    r.image_out(rgba8, rgbe, rows, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert np.array_equal(rgba8.cpu().numpy().view(np.uint8).reshape(h, w, 4), io.process_image(r.frame_buffer()))
    assert np.array_equal(rgbe.cpu().numpy().view(np.uint8).reshape(h, w, 4), io.rgbe(mean))
    want = io.half_rows(mean)
    assert np.array_equal(rows.cpu().numpy().view(np.uint16).reshape(h, 4, w), want.view(np.uint16))
    # payloads are partial when pointers are NULL: RGBE alone
    rgbe2 = torch.zeros(h * w, dtype=torch.int32, device=dev)
    r.image_out(None, rgbe2, None, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert torch.equal(rgbe, rgbe2)


def test_dumps_write_reference_files(rendered, tmp_path, monkeypatch):
    r, mean = rendered
    monkeypatch.chdir(tmp_path)
    r.dumpFramebuffer()
    r.dumpAccumFramebufferRgbe()
    r.dumpAccumFramebufferExr()
    png = (tmp_path / "output.png").read_bytes()
    assert np.array_equal(io.read_png(png), r.rgba8())
    assert np.array_equal(io.read_hdr((tmp_path / "output.hdr").read_bytes()), io.rgbe(mean))
    ch, _ = io.read_exr((tmp_path / "output.exr").read_bytes())
    want = io.half_rows(mean)
    for k, c in enumerate("ABGR"):
        assert np.array_equal(ch[c].view(np.uint16), want[:, k].view(np.uint16))
    r.dumpFramebuffer(tmp_path / "named.png")
    assert (tmp_path / "named.png").read_bytes() == png
