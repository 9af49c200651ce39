"""The allocation-free relMSE entry point, called through the C ABI.

optpt_relmse_noalloc serves callers that cannot allocate device memory when
they call it (inside a stream capture, in allocation-free frame loops, or under
a host-owned memory pool). It must give the same result as optpt_relmse, on
consecutive calls that reuse its fixed scratch array, and refuse images larger
than that array covers. This file is collected last on purpose.
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
    rc = lib.optpt_relmse_noalloc(p, 1, p, 1, p, None)          # the largest-but-one case is fine
    torch.cuda.synchronize()
    assert rc == 0
