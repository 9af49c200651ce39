"""The allocation-free relMSE entry point, called through the C ABI.

optpt_relmse_noalloc serves callers that cannot allocate device memory when
they call it: a viewer's frame loop that makes no allocator call per frame
(cudaMalloc and cudaFree can synchronise the device), or a host whose own
memory pool owns the device memory. It must give the same result as
optpt_relmse, on consecutive calls that reuse its fixed scratch array, up to
and including the largest image that array covers, and refuse larger images.
This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _relmse_pair(lib, torch, dev, s, r, n_samples):
    sd = torch.from_numpy(s).to(dev)
    rd = torch.from_numpy(r).to(dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    npix = s.shape[0]
    rc = lib.optpt_relmse(ctypes.c_void_p(sd.data_ptr()), n_samples, ctypes.c_void_p(rd.data_ptr()), npix,
                          ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 0, lib.optpt_last_error()
    rc = lib.optpt_relmse_noalloc(ctypes.c_void_p(sd.data_ptr()), n_samples, ctypes.c_void_p(rd.data_ptr()), npix,
                                  ctypes.c_void_p(out.data_ptr() + 8), stream)
    assert rc == 0, lib.optpt_last_error()
    torch.cuda.synchronize()
    a, b = out.tolist()
    return a, b


def test_noalloc_matches_allocating_entry_point(cuda_dev):
    import torch

    from optix_pt_gb300 import _ffi
    lib = _ffi.lib
    rng = np.random.default_rng(77)
    # two calls in a row on different images: the second must not see the first's partials
    for npix, n_samples in ((1920 * 1080, 64), (300_001, 7)):
        s = rng.exponential(2.0, (npix, 4)) * n_samples
        r = rng.exponential(0.3, (npix, 4))
        a, b = _relmse_pair(lib, torch, cuda_dev, s, r, n_samples)
        assert b == pytest.approx(a, rel=1e-12)
        i = s[:, :3] / n_samples
        expect = np.mean(np.sum((i - r[:, :3]) ** 2 / (r[:, :3] ** 2 + 1e-2), axis=1))
        assert b == pytest.approx(expect, rel=1e-12)


def test_noalloc_rejects_images_beyond_its_scratch(cuda_dev):
    import torch

    from optix_pt_gb300 import _ffi
    lib = _ffi.lib
    buf = torch.zeros(8, dtype=torch.float64, device=cuda_dev)
    p = ctypes.c_void_p(buf.data_ptr())
    rc = lib.optpt_relmse_noalloc(p, 1, p, 8_388_609, p, None)   # rejected before any device work
    assert rc == -1
    assert b"8388608" in lib.optpt_last_error()
    for npix in (4_294_967_295, 4_294_965_249):                   # would wrap a 32-bit tile count
        assert lib.optpt_relmse_noalloc(p, 1, p, npix, p, None) == -1
    rc = lib.optpt_relmse_noalloc(p, 1, p, 1, p, None)          # a one-pixel image is fine
    torch.cuda.synchronize()
    assert rc == 0


def test_noalloc_at_its_exact_limit(cuda_dev):
    """8,388,608 pixels: every one of the 4,096 scratch entries is written and
    read; the result equals the allocating entry point's, twice in a row."""
    import torch

    from optix_pt_gb300 import _ffi
    lib = _ffi.lib
    npix = 8_388_608
    g = torch.Generator(device=cuda_dev).manual_seed(5)
    out = torch.zeros(4, dtype=torch.float64, device=cuda_dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for k, n_samples in enumerate((16, 3)):
        s = torch.rand((npix, 4), dtype=torch.float64, device=cuda_dev, generator=g) * (2.0 * n_samples)
        r = torch.rand((npix, 4), dtype=torch.float64, device=cuda_dev, generator=g)
        rc = lib.optpt_relmse(ctypes.c_void_p(s.data_ptr()), n_samples, ctypes.c_void_p(r.data_ptr()), npix,
                              ctypes.c_void_p(out.data_ptr() + 16 * k), stream)
        assert rc == 0, lib.optpt_last_error()
        rc = lib.optpt_relmse_noalloc(ctypes.c_void_p(s.data_ptr()), n_samples, ctypes.c_void_p(r.data_ptr()), npix,
                                      ctypes.c_void_p(out.data_ptr() + 16 * k + 8), stream)
        assert rc == 0, lib.optpt_last_error()
        torch.cuda.synchronize()
        i = s[:, :3] / n_samples
        expect = float((((i - r[:, :3]) ** 2) / (r[:, :3] ** 2 + 1e-2)).sum(1).mean())
        a, b = out[2 * k].item(), out[2 * k + 1].item()
        assert b == pytest.approx(a, rel=1e-12)
        assert b == pytest.approx(expect, rel=1e-12)
        del s, r
