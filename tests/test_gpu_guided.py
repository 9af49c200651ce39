"""Learned path guiding inside the renderer (indirect-lit interior).

* Guiding off is the plain renderer, bit for bit.
* Guided renders (online training, and a frozen trained network) are
  unbiased against an independent FP64 oracle render of the plain estimator:
  per-pixel z test on the FP64 sums and sums of squares, frame mean within 4
  standard errors.
* The trained network pays: at equal samples per pixel the guided image's
  relMSE against a high-spp plain render is lower than the plain image's.
"""
import numpy as np
import pytest

from gpu_util import pixel_stats
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _render(scene, w, h, spp, mode, batch=0, seed=None, warm=0):
    import torch

    import optix_pt_gb300 as opt
    r = opt.Renderer(scene, spp_batch=batch)
    r.setupOutputBuffer(w, h)
    if seed is not None:
        r.set_seed(seed)
    if warm:
        r.set_guiding(1)
        r.render(warm, torch.cuda.current_stream())   # training passes, then start over
        r.resetSampleCount()
        r.set_seed((seed or 1) + 7919)                # random streams independent of training
    if mode:
        r.set_guiding(mode)
    r.render(spp, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = r.accum()
    st = r.guide().status() if mode else (0, 0.0)
    return r, (s.reshape(-1, 3), q.reshape(-1, 3), n), st


def test_guiding_off_is_bit_identical(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("interior_small")
    a, ga, _ = _render(sc, 64, 36, 8, 0, batch=4)
    b = opt.Renderer(sc, spp_batch=4)
    b.setupOutputBuffer(64, 36)
    b.set_guiding(1)
    b.set_guiding(0)
    b.render(8, torch.cuda.current_stream())
    torch.cuda.synchronize()
    sb, qb, nb = b.accum()
    assert np.array_equal(ga[0], sb.reshape(-1, 3)) and np.array_equal(ga[1], qb.reshape(-1, 3))
    a.close()
    b.close()


@pytest.mark.parametrize("mode", [1, 2])
def test_guided_render_is_unbiased(cuda_dev, mode):
    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("interior_small")
    w, h = 96, 54
    # mode 2 freezes a network trained on 256 spp first (then the accumulator restarts)
    r, g, st = _render(sc, w, h, 2048, mode, warm=256 if mode == 2 else 0)
    assert st[0] == 0
    lp = r.launch_params()
    cam = list(lp.eye) + list(lp.U) + list(lp.V) + list(lp.W) + list(lp.bgColour)
    v = orc.SceneView(sc.struct, 4)
    cs, cq, _ = v.render(cam, w, h, lp.seed, 1 << 20, 256, lp.maxDepth, precision=64)
    frac, dmean, se, gm, cm, live = pixel_stats(g, (cs, cq, 256))
    print("guided mode %d: z>3 fraction %.4f, mean diff %.3g (SE %.3g)" % (mode, frac, dmean, se))
    assert frac < 0.015, frac
    assert dmean < 4 * se, (dmean, se)
    r.close()


def test_guiding_lowers_relmse_at_equal_spp(cuda_dev):
    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("interior_small")
    w, h = 96, 54
    ref_r, ref, _ = _render(sc, w, h, 32768, 0, seed=99)
    R = ref[0] / ref[2]
    ref_r.close()
    errs = {}
    for mode in (0, 1):
        r, g, st = _render(sc, w, h, 512, mode, seed=7)
        I = g[0] / g[2]
        errs[mode] = float(np.mean(((I - R) ** 2 / (R ** 2 + 1e-2)).sum(1)))
        r.close()
    print("relMSE at 512 spp: plain %.4g, guided %.4g (ratio %.2f)" % (errs[0], errs[1], errs[0] / errs[1]))
    assert errs[1] < 0.8 * errs[0]
