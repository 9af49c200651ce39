"""The path-completion kernel (kFinish): from bounce tailBounce on, one launch
finishes every remaining path with the same functions, in the same order, as
the per-bounce kernels. Images, sums of squares, ray totals and per-bounce
queue counts are bit-identical to the all-wavefront pass, for every switch
bounce (1 = the whole pass in one kernel), on the Cornell box, the material
sweep and the textured, alpha-masked small terrain, and in batched
multi-view rendering."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(scene, tail, w, h, spp, max_depth=None, seed=None):
    import torch

    import optix_pt_gb300 as opt
    r = opt.Renderer(scene, tail_bounce=tail)
    r.setupOutputBuffer(w, h)
    if max_depth:
        r.set_max_depth(max_depth)
    if seed is not None:
        r.set_seed(seed)
    r.render(spp, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = r.accum()
    st = r.stats()
    qc = r.queue_counts()
    r.close()
    return s, q, n, st, qc


@pytest.mark.parametrize("name,w,h,spp,depth", [("cornell", 96, 96, 8, None), ("spheres", 160, 90, 2, 12),
                                                 ("terrain_small", 128, 72, 2, 16)])
def test_tail_kernel_is_bit_identical_to_the_wavefront(cuda_dev, name, w, h, spp, depth):
    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural(name)
    base = _render(sc, -1, w, h, spp, depth)
    for tail in (1, 2, 3, 5):
        got = _render(sc, tail, w, h, spp, depth)
        assert np.array_equal(got[0], base[0]) and np.array_equal(got[1], base[1]), (name, tail)
        for k in ("extensionRays", "shadowRays", "pathSamples", "nanSamples"):
            assert got[3][k] == base[3][k], (name, tail, k)
        for a, b in zip(got[4], base[4]):
            assert np.array_equal(a, b), (name, tail)
    assert base[0].sum() > 0


def test_tail_kernel_in_batched_views(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("spheres")
    a = sc.arrays()
    views = [(a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"], 64, 48, 8),
             (a["camEye"], [0.0, 0.5, 0.0], a["camUp"], 50.0, 40, 40, 3)]
    out = []
    for tail in (-1, 3):
        r = opt.Renderer(sc, tail_bounce=tail)
        r.render_batch(views, torch.cuda.current_stream())
        torch.cuda.synchronize()
        out.append([r.batch_view(v) for v in range(len(views))])
        r.close()
    for (s0, q0, n0), (s1, q1, n1) in zip(*out):
        assert n0 == n1 and np.array_equal(s0, s1) and np.array_equal(q0, q1)


def test_tail_kernel_past_the_guided_bounces(cuda_dev):
    """With guiding on, the path-completion kernel takes over only past the
    guided bounces: a tail bounce inside the guided range is raised to the
    guiding maxDepth + 1, or + 2 while the network trains (bounce maxDepth + 1
    then still completes a training path's last record). The renders train
    for their first half and run frozen for the second, so both limits are
    exercised. Online training adds hash-grid gradients with
    atomics, in no fixed order, so two guided renders differ in rounding even
    with the same settings; the renders are therefore compared statistically
    (per-pixel z scores of the difference and the frame mean) with the
    render that has no tail kernel."""
    import torch

    import optix_pt_gb300 as opt
    from gpu_util import pixel_stats
    sc = opt.Scene.procedural("cornell")
    outs = []
    for tail in (-1, 3, 5):
        r = opt.Renderer(sc, spp_batch=16, tail_bounce=tail)
        r.setupOutputBuffer(48, 48)
        r.set_guiding(1)
        r.guiding_options(maxDepth=3, trainSpp=256)
        r.render(512, torch.cuda.current_stream())
        torch.cuda.synchronize()
        s, q, n = r.accum()
        outs.append((s.reshape(-1, 3), q.reshape(-1, 3), n))
        assert r.guide().status()[0] == 0
        r.close()
    for k, tail in ((1, 3), (2, 5)):
        frac, dmean, se, *_ = pixel_stats(outs[k], outs[0])
        print("guided, tail bounce %d vs none: z>3 fraction %.4f, mean diff %.3g (SE %.3g)" % (tail, frac, dmean, se))
        assert frac < 0.01, (tail, frac)
        assert dmean < 4 * se, (tail, dmean, se)
    assert outs[0][0].sum() > 0
