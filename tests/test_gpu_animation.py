"""Animated scenes on the GPU: vertex deformation and BVH8 refit.

* The deformation kernel reproduces the host evaluation of a glTF pose bit
  for bit (positions and normals, skinned and rigid shapes).
* A refit with unchanged vertices leaves every BVH8 node bit-identical to
  the freshly collapsed tree.
* After deformation (the animated glTF, and the 327,684-triangle material
  sweep under a non-rigid warp), closest hits through the refit tree are
  bit-identical to the oracle's traversal of a BVH built from scratch over
  the deformed triangles, and occlusion agrees: a refit tree is valid.
* Accumulation restarts on every update (resetSampleCount), and a render of
  the deformed scene follows the oracle's paths with paired random streams.
"""
import numpy as np
import pytest

from gltf_writer import animated_scene
from gpu_util import paired_agreement, rays_towards, render_pair, trace_on_gpu
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def anim_path(tmp_path_factory):
    return animated_scene().save(tmp_path_factory.mktemp("ganim") / "anim.gltf")


def _rays(P, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = P.min(0), P.max(0)
    ext = hi - lo
    return rays_towards(rng, n, (lo - ext, hi + ext), (lo, hi))


def test_deform_matches_host_pose_bit_exact(cuda_dev, anim_path):
    import torch

    import optix_pt_gb300 as opt
    m = opt.GltfModel(anim_path)
    sc = m.scene(0.0, animate=False)
    r = opt.Renderer(sc)
    a = opt.Animator(r, m)
    for t in (0.0, 0.37, 1.0, 1.55, 2.9):
        a.pose(t, torch.cuda.current_stream())
        gp, gn = r.read_vertices(torch.cuda.current_stream())
        hp, hn = m.apply(t)
        assert np.array_equal(gp, hp), (t, np.abs(gp - hp).max())
        assert np.array_equal(gn, hn), (t, np.abs(gn - hn).max())
    r.close()
    m.close()


@pytest.mark.parametrize("name", ["cornell", "spheres", "terrain_small"])
def test_refit_without_motion_is_identity(cuda_dev, name):
    import torch

    import optix_pt_gb300 as opt
    sc = opt.Scene.procedural(name)
    r = opt.Renderer(sc)
    before, order = r.bvh8_nodes()
    r.update_vertices(sc.arrays()["positions"], None, torch.cuda.current_stream())
    torch.cuda.synchronize()
    after, order2 = r.bvh8_nodes()
    assert np.array_equal(order, order2)
    assert np.array_equal(before, after)
    r.close()


def _check_hits(r, scene_now, rays, dev):
    v = orc.SceneView(scene_now.struct, 4)
    g = trace_on_gpu(r, rays, dev)
    c = v.trace(rays)
    bad = (g.view(np.int32) != c.view(np.int32)).any(1)
    assert not bad.any(), "%d of %d rays differ" % (int(bad.sum()), len(rays))
    occ = rays.copy()
    occ[:, 3] = 1e-3
    occ[:, 7] = np.random.default_rng(9).uniform(0.1, 4.0, len(rays)).astype(np.float32)
    go = trace_on_gpu(r, occ, dev, any_hit=True)[:, 3].view(np.int32) >= 0
    co = v.trace(occ, any_hit=True)[:, 3].view(np.int32) >= 0
    assert np.array_equal(go, co)
    return (g[:, 3].view(np.int32) >= 0).mean()


def test_refit_after_animation_hits_exact(cuda_dev, anim_path):
    import torch

    import optix_pt_gb300 as opt
    m = opt.GltfModel(anim_path)
    r = opt.Renderer(m.scene(0.0, animate=False))
    a = opt.Animator(r, m)
    for t in (0.6, 1.4, 2.2):
        a.pose(t, torch.cuda.current_stream())
        torch.cuda.synchronize()
        now = m.scene(t, animate=True)
        frac = _check_hits(r, now, _rays(now.arrays()["positions"], 1 << 15, int(t * 10)), cuda_dev)
        assert frac > 0.2
        assert r.getSampleCount() == 0
    r.close()
    m.close()


def test_refit_after_warp_large_scene(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    from gpu_util import ArrayScene
    sc = opt.Scene.procedural("spheres")
    A = sc.arrays()
    P = A["positions"].astype(np.float64)
    # non-rigid: twist about y, shear, and a ripple
    ang = 0.25 * P[:, 1]
    x = P[:, 0] * np.cos(ang) - P[:, 2] * np.sin(ang)
    z = P[:, 0] * np.sin(ang) + P[:, 2] * np.cos(ang)
    W = np.stack([x + 0.1 * P[:, 1], P[:, 1] + 0.05 * np.sin(3 * P[:, 0]), z], 1).astype(np.float32)
    r = opt.Renderer(sc)
    r.render(2, torch.cuda.current_stream())
    r.update_vertices(W, None, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert r.getSampleCount() == 0
    mats = sc.materials()
    warped = ArrayScene(W, A["triIndices"], A["matIndices"], mats, normals=A["normals"])
    frac = _check_hits(r, warped, _rays(W, 1 << 16, 3), cuda_dev)
    assert frac > 0.2
    r.close()


def test_render_after_deform_follows_oracle(cuda_dev, anim_path):
    """Paired FP32 samples of the deformed renderer against the oracle on the
    same posed scene."""
    import torch

    import optix_pt_gb300 as opt
    m = opt.GltfModel(anim_path)
    r = opt.Renderer(m.scene(0.0, animate=False), spp_batch=2)
    r.setupOutputBuffer(80, 60)
    a = opt.Animator(r, m)
    a.pose(1.25, torch.cuda.current_stream())
    r.render(2, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = r.accum()
    lp = r.launch_params()
    cam = list(lp.eye) + list(lp.U) + list(lp.V) + list(lp.W) + list(lp.bgColour)
    now = m.scene(1.25, animate=True)
    v = orc.SceneView(now.struct, 4)
    cs, cq, cnt = v.render(cam, 80, 60, lp.seed, 0, 2, lp.maxDepth, precision=32)
    fs, fq, _ = orc.SceneView(now.struct, 4, variant="fma").render(cam, 80, 60, lp.seed, 0, 2, lp.maxDepth,
                                                                  precision=32)
    g = s.reshape(-1, 3)
    robust, sensitive, overall = paired_agreement((g,), (cs,), (fs,))
    print("after deform: robust-pixel agreement %.4f, rounding-sensitive pixels %.4f, all pixels %.4f" % (
        robust, sensitive, overall))
    assert robust >= 0.995 and overall >= 0.995, (robust, overall)
    assert sensitive <= 0.05, sensitive
    assert g.sum() > 0
    r.close()
    m.close()
