"""GPU FP64 relMSE reduction against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _relmse_np(s, n, r):
    i = s[:, :3] / n
    return float(np.mean(np.sum((i - r[:, :3]) ** 2 / (r[:, :3] ** 2 + 1e-2), axis=1)))


@pytest.mark.parametrize("npix", [1, 255, 2048, 2049, 1920 * 1080])
def test_relmse_matches_numpy(cuda_dev, npix):
    import torch

    import optix_pt_gb300 as opt
    rng = np.random.default_rng(npix)
    s = rng.exponential(3.0, (npix, 4)) * 16
    r = rng.exponential(0.2, (npix, 4))
    sd = torch.from_numpy(s).to(cuda_dev)
    rd = torch.from_numpy(r).to(cuda_dev)
    out = torch.zeros(1, dtype=torch.float64, device=cuda_dev)
    opt.relmse(sd.data_ptr(), 16, rd.data_ptr(), npix, out.data_ptr(), torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert out.item() == pytest.approx(_relmse_np(s, 16, r), rel=1e-12)


def test_relmse_of_renderer_accumulation(cuda_dev):
    """The renderer's FP64 sums against a reference mean, on the device."""
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("cornell")
    r = opt.Renderer(sc)
    r.setupOutputBuffer(64, 64)
    r.render(16, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = r.accum()
    ref = np.zeros((64 * 64, 4))
    ref[:, :3] = (s.reshape(-1, 3) / n) * 0.9 + 0.01
    _, _, sum_ptr, _ = r.device_buffers()
    rd = torch.from_numpy(ref).to(cuda_dev)
    out = torch.zeros(1, dtype=torch.float64, device=cuda_dev)
    opt.relmse(sum_ptr, n, rd.data_ptr(), 64 * 64, out.data_ptr(), torch.cuda.current_stream())
    torch.cuda.synchronize()
    full = np.zeros((64 * 64, 4))
    full[:, :3] = s.reshape(-1, 3)
    assert out.item() == pytest.approx(_relmse_np(full, n, ref), rel=1e-12)
    r.close()


def test_relmse_rejects_empty(built):
    import optix_pt_gb300 as opt
    with pytest.raises(opt.OptptError):
        opt.relmse(None, 1, None, 0, None)
