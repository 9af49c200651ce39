"""Batched multi-view rendering: several views of one scene, of uneven
resolution and samples per pixel, in shared wavefront passes.

* View 0 of a batch equals a single-view render of the same view bit for bit
  (same random streams, same summation order).
* The other views are unbiased against independent FP64 oracle renders.
* Guiding trains and samples across the views of a batch.
"""
import numpy as np
import pytest

from gpu_util import pixel_stats
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _basis(eye, target, up, fov, aspect):
    """Camera::setupUvwCoordinatSystem (src/camera.cpp:19-40)."""
    e, t, u = (np.array(v, np.float64) for v in (eye, target, up))
    W = t - e
    W /= np.linalg.norm(W)
    u /= np.linalg.norm(u)
    U = np.cross(u, -W)
    U /= np.linalg.norm(U)
    V = np.cross(-W, U)
    V /= np.linalg.norm(V)
    vl = np.tan(0.5 * np.radians(fov))
    return list((U * vl * aspect).astype(np.float32)), list((V * vl).astype(np.float32)), list(W.astype(np.float32))


def _views(a):
    eye, tgt, up, fov = a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"]
    return [(eye, tgt, up, fov, 64, 64, 24),
            ([0.6, 1.2, 3.2], [0.0, 0.8, 0.0], [0, 1, 0], 55.0, 48, 32, 8),
            ([-0.5, 1.6, 3.0], [0.2, 0.6, -0.5], [0, 1, 0], 35.0, 96, 40, 40)]


def test_batch_view0_matches_single_view(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("cornell")
    views = _views(sc.arrays())
    r = opt.Renderer(sc)
    r.render_batch(views, torch.cuda.current_stream())
    bs, bq, bn = r.batch_view(0)
    single = opt.Renderer(sc)
    single.setupOutputBuffer(64, 64)
    eye, tgt, up, fov = views[0][:4]
    single.setupCamera(eye, tgt, up, fov)
    single.render(24, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = single.accum()
    assert bn == n == 24
    assert np.array_equal(bs, s.reshape(-1, 3)) and np.array_equal(bq, q.reshape(-1, 3))
    r.close()
    single.close()


def test_batch_views_are_unbiased(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("cornell")
    a = sc.arrays()
    views = [v[:6] + (1024,) for v in _views(a)]
    r = opt.Renderer(sc)
    r.render_batch(views, torch.cuda.current_stream())
    lp = r.launch_params()
    orcv = orc.SceneView(sc.struct, 4)
    for k in (1, 2):
        eye, tgt, up, fov, w, h, spp = views[k]
        U, V, W = _basis(eye, tgt, up, fov, w / h)
        cam = list(eye) + U + V + W + list(a["bgColour"])
        cs, cq, _ = orcv.render(cam, w, h, lp.seed, 1 << 20, 256, lp.maxDepth, precision=64)
        g = r.batch_view(k)
        assert g[2] == 1024
        frac, dmean, se, gm, cm, live = pixel_stats(g, (cs, cq, 256))
        print("batch view %d (%dx%d): z>3 fraction %.4f, mean diff %.3g (SE %.3g)" % (k, w, h, frac, dmean, se))
        assert frac < 0.015 and dmean < 4 * se
    r.close()


def test_batch_with_guiding(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("interior_small")
    a = sc.arrays()
    r = opt.Renderer(sc)
    r.set_guiding(1)
    views = [(a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"], 96, 54, 256),
             ([-3.0, 1.2, 2.0], [2.0, 1.0, -1.0], [0, 1, 0], 70.0, 64, 64, 128)]
    st0 = r.stats()
    r.render_batch(views, torch.cuda.current_stream())
    torch.cuda.synchronize()
    status, loss, samples = r.guide().status()
    assert status == 0 and samples > 0
    st1 = r.stats()
    assert st1["pathSamples"] - st0["pathSamples"] == 96 * 54 * 256 + 64 * 64 * 128
    for k in range(2):
        s, q, n = r.batch_view(k)
        assert n == views[k][6] and np.isfinite(s).all() and s.sum() > 0
    r.close()


def test_block_compaction_matches_warp_compaction(cuda_dev):
    """Queue order does not change any path (random streams are keyed by
    pixel, sample and depth): per-block and per-warp appends give the same
    image bit for bit."""
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("spheres")
    out = []
    for comp in (32, 1):
        r = opt.Renderer(sc, compaction=comp, block_size=128)
        r.setupOutputBuffer(160, 90)
        r.render(8, torch.cuda.current_stream())
        torch.cuda.synchronize()
        out.append(r.accum())
        r.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_autotune_measures_every_candidate(cuda_dev):
    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural("cornell")
    best, trials = opt.autotune(sc, 96, 96, 16)
    grid, tails = trials[:18], trials[18:]
    assert len(trials) == 24
    assert {(t["bvhBuilder"], t["leafSize"], t["blockSize"], t["compaction"]) for t in grid} == {
        (tb, tl, b, c) for tb, tl in ((0, 1), (0, 2), (1, 1)) for b in (64, 128, 256) for c in (32, 1)}
    # then the path-completion switch with the grid's best choices
    top = max(grid, key=lambda t: t["samples_per_s"])
    assert [t["tailBounce"] for t in tails] == [0xFFFFFFFF, 3, 4, 5, 6, 8]
    assert all((t["bvhBuilder"], t["leafSize"], t["blockSize"], t["compaction"]) ==
               (top["bvhBuilder"], top["leafSize"], top["blockSize"], top["compaction"]) for t in tails)
    assert all(t["samples_per_s"] > 0 and t["mrays_per_s"] > 0 for t in trials)
    fastest = max(trials, key=lambda t: t["samples_per_s"])
    assert (best["bvhBuilder"], best["leafSize"], best["blockSize"], best["compaction"], best["tailBounce"]) == (
        fastest["bvhBuilder"], fastest["leafSize"], fastest["blockSize"], fastest["compaction"],
        fastest["tailBounce"])
    print("autotune best", best)


def _views_of(scene, shapes):
    a = scene.arrays()
    return [(a["camEye"], a["camTarget"], a["camUp"], a["camFovYDeg"] + 5.0 * i, w, h, spp)
            for i, (w, h, spp) in enumerate(shapes)]


def test_multi_scene_batch_matches_single_scene_batches(cuda_dev):
    """Views of two scenes in one multi-scene batch (one graph launch per pass
    over both scenes): every view equals, bit for bit, the same views of its
    scene rendered as a single-scene batch; with guiding on, both networks
    train without a tensor-core timeout and every view is finite."""
    import torch

    import optix_pt_gb300 as opt
    sa, sb = opt.Scene.procedural("cornell"), opt.Scene.procedural("spheres")
    va = _views_of(sa, [(48, 40, 6), (32, 32, 3)])
    vb = _views_of(sb, [(64, 36, 4), (40, 40, 5), (24, 16, 9)])
    single = []
    for sc, vs in ((sa, va), (sb, vb)):
        r = opt.Renderer(sc)
        r.render_batch(vs, torch.cuda.current_stream())
        torch.cuda.synchronize()
        single.append([r.batch_view(j) for j in range(len(vs))])
        r.close()
    ra, rb = opt.Renderer(sa), opt.Renderer(sb)
    mixed = [(0, va[0]), (1, vb[0]), (1, vb[1]), (0, va[1]), (1, vb[2])]
    where = opt.render_batch_scenes([ra, rb], mixed, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert where == [(0, 0), (1, 0), (1, 1), (0, 1), (1, 2)]
    for k, r in enumerate((ra, rb)):
        for j, (s0, q0, n0) in enumerate(single[k]):
            s1, q1, n1 = r.batch_view(j)
            assert n1 == n0 and np.array_equal(s1, s0) and np.array_equal(q1, q0), (k, j)
    for r in (ra, rb):
        r.set_guiding(1)
    opt.render_batch_scenes([ra, rb], mixed, torch.cuda.current_stream())
    torch.cuda.synchronize()
    for k, r in enumerate((ra, rb)):
        assert r.guide().status()[0] == 0
        for j in range(len(single[k])):
            s, q, n = r.batch_view(j)
            assert n == single[k][j][2] and np.isfinite(s).all() and s.sum() > 0
        r.close()
