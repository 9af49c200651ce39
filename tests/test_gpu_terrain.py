"""The terrain workload against the oracle: 9,996,610 triangles (a 2048 x 2048
height field, 20,000 rocks with 30 % glass, 4,000 alpha-masked foliage cards
textured with an sRGB RGBA image, a normal-mapped ground) and its small
variant (50,594 triangles, same materials and textures).

* BVH8 collapse byte-exact against the host build, at full size.
* Closest hits bit-exact, including candidates rejected by the foliage
  texture's alpha (bilinear sRGB sampling must round identically).
* Paired FP32 samples follow the oracle's paths; a high-spp render is
  unbiased against an independent FP64 oracle render.
"""
import numpy as np
import pytest

from gpu_util import paired_agreement, pixel_stats, rays_towards, render_pair, trace_on_gpu
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    import optix_pt_gb300 as opt
    return opt.Scene.procedural("terrain_small")


@pytest.fixture(scope="module")
def full():
    import optix_pt_gb300 as opt
    return opt.Scene.procedural("terrain")


def _alpha_materials(sc):
    m = sc.struct.materials
    return np.array([i for i in range(sc.struct.numMaterials) if m[i].alphaMode == 2], np.int32)  # AM_MASK


def _rays(sc, n, seed):
    """Half from around the camera towards the terrain, half straight-ish
    down from above the canopy (grazing the foliage cards)."""
    rng = np.random.default_rng(seed)
    a = sc.arrays()
    P = a["positions"]
    lo, hi = P.min(0), P.max(0)
    eye = np.array(a["camEye"], np.float32)
    r1 = rays_towards(rng, n // 2, (eye - 20, eye + 20), (lo, hi))
    top_lo = np.array([lo[0], hi[1] + 1, lo[2]], np.float32)
    top_hi = np.array([hi[0], hi[1] + 30, hi[2]], np.float32)
    r2 = rays_towards(rng, n - n // 2, (top_lo, top_hi), (lo, np.array([hi[0], lo[1] + 0.6 * (hi[1] - lo[1]), hi[2]])))
    return np.concatenate([r1, r2])


@pytest.mark.parametrize("which,leaf", [("small", 2), ("small", 3), ("full", 3)])
def test_bvh8_collapse_matches_host(cuda_dev, small, full, which, leaf):
    import optix_pt_gb300 as opt
    sc = small if which == "small" else full
    r = opt.Renderer(sc, leaf_size=leaf, bvh_width=8, bvh_builder="lbvh")
    v = orc.SceneView(sc.struct, leaf)
    hn, ho = v.bvh8(sc.num_triangles)
    gn, go = r.bvh8_nodes()
    assert gn.shape == hn.shape
    assert np.array_equal(gn, hn)
    assert np.array_equal(go, ho)
    r.close()


@pytest.mark.parametrize("which,width,builder", [("small", 8, "lbvh"), ("small", 2, "lbvh"), ("full", 8, "lbvh"),
                                                   ("small", 8, "ploc"), ("full", 8, "ploc")])
def test_closest_hits_bit_exact(cuda_dev, small, full, which, width, builder):
    """Hits are a property of the ray and the scene: the same bits from the
    LBVH- and PLOC-derived trees as from the host's own traversal."""
    import optix_pt_gb300 as opt
    sc = small if which == "small" else full
    r = opt.Renderer(sc, leaf_size=3 if width == 8 else 4, bvh_width=width, bvh_builder=builder)
    v = orc.SceneView(sc.struct, 4)
    rays = _rays(sc, 1 << 17, 21)
    g = trace_on_gpu(r, rays, cuda_dev)
    c = v.trace(rays)
    bad = (g.view(np.int32) != c.view(np.int32)).any(1)
    assert not bad.any(), "%d of %d rays differ" % (int(bad.sum()), len(rays))
    prims = g[:, 3].view(np.int32)
    hit = prims >= 0
    assert hit.mean() > 0.3
    # the rays reach the alpha-masked foliage cards
    mats = sc.arrays()["matIndices"].reshape(-1)
    assert np.isin(mats[prims[hit]], _alpha_materials(sc)).sum() > 40
    r.close()


def test_occlusion_matches(cuda_dev, small):
    import optix_pt_gb300 as opt
    r = opt.Renderer(small)
    v = orc.SceneView(small.struct, 4)
    rays = _rays(small, 1 << 16, 22)
    rays[:, 3] = 1e-3
    rays[:, 7] = np.random.default_rng(4).uniform(1.0, 300.0, len(rays)).astype(np.float32)
    g = trace_on_gpu(r, rays, cuda_dev, any_hit=True)[:, 3].view(np.int32) >= 0
    c = v.trace(rays, any_hit=True)[:, 3].view(np.int32) >= 0
    assert np.array_equal(g, c)
    assert 0.05 < g.mean() < 0.95
    r.close()


@pytest.mark.parametrize("which,w,h,spp", [("small", 160, 90, 2), ("full", 192, 108, 1)])
def test_paired_samples_follow_oracle_paths(cuda_dev, small, full, which, w, h, spp):
    sc = small if which == "small" else full
    g, c, st, cnt, f = render_pair(sc, w, h, spp, spp, 0, 32, batch=spp, classify=True)
    robust, sensitive, overall = paired_agreement(g, c, f)
    print("terrain %s: robust-pixel agreement %.4f, rounding-sensitive pixels %.4f, all pixels %.4f" % (
        which, robust, sensitive, overall))
    assert robust >= 0.995 and overall >= 0.995, (robust, overall)
    assert sensitive <= 0.05, sensitive
    assert abs(int(st["extensionRays"]) - int(cnt[0])) <= 0.02 * int(cnt[0])
    assert abs(int(st["shadowRays"]) - int(cnt[1])) <= 0.02 * max(1, int(cnt[1]))


def test_unbiased_against_fp64(cuda_dev, small):
    g, c, st, cnt = render_pair(small, 96, 54, 1024, 256, 1 << 20, 64)
    frac, dmean, se, gm, cm, live = pixel_stats(g, c)
    assert frac < 0.015, frac
    assert dmean < 4 * se, (dmean, se)
