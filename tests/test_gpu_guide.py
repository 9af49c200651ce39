"""Learned path guiding on the tensor cores.

* tcgen05 operand layouts: a 128x64x64 K-major MMA and a 64x64x128 MN-major
  MMA (the weight-gradient shape) against FP32 products of the same BF16
  values.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(rng, shape):
    x = rng.standard_normal(shape).astype(np.float32)
    bits = (x.view(np.uint32) + 0x8000) >> 16          # round to nearest (ties away)
    return bits.astype(np.uint16), (bits.astype(np.uint32) << 16).view(np.float32)


def test_tcgen05_operand_layouts(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    rng = np.random.default_rng(3)
    (A, a), (B, b), (G, g), (X, x) = (_bf16(rng, s) for s in ((128, 64), (64, 64), (128, 64), (128, 64)))
    dev = [torch.from_numpy(v.view(np.int16)).to(cuda_dev) for v in (A, B, G, X)]
    c = torch.zeros((128, 64), dtype=torch.float32, device=cuda_dev)
    dw = torch.zeros((128, 64), dtype=torch.float32, device=cuda_dev)
    st = torch.zeros(1, dtype=torch.int32, device=cuda_dev)
    opt.check(opt.lib.optpt_tc_selftest(*[d.data_ptr() for d in dev], c.data_ptr(), dw.data_ptr(), st.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st.item() == 0
    c, dw = c.cpu().numpy(), dw.cpu().numpy()
    ref_c = a.astype(np.float64) @ b.astype(np.float64).T
    ref_dw = g.astype(np.float64).T @ x.astype(np.float64)
    print("C max err", np.abs(c - ref_c).max())
    # where do the 64 rows of the M = 64 result sit among the 128 TMEM lanes?
    lanes = {}
    for r in range(64):
        d = np.abs(dw - ref_dw[r][None, :]).max(1)
        lanes[r] = int(d.argmin()) if d.min() < 1e-3 * (1 + np.abs(ref_dw[r]).max()) else -1
    print("M=64 row -> lane:", lanes)
    assert np.allclose(c, ref_c, rtol=1e-5, atol=1e-4)
    # M = 64: rows 16q .. 16q + 15 in lanes 32q .. 32q + 15 of each lane quarter
    assert lanes == {r: (r // 16) * 32 + r % 16 for r in range(64)}, lanes
    for r in range(64):
        np.testing.assert_allclose(dw[(r // 16) * 32 + r % 16], ref_dw[r], rtol=1e-5, atol=1e-4)
