"""GPU parity through the C ABI: device BSDF vs the reference's golden vectors
and the FP64 oracle; Morton codes, leaf order and BVH topology bit-exact vs the
host build; closest-hit and occlusion results bit-exact vs the host traversal."""
import os

import numpy as np
import pytest

from bsdf_cases import make_fixed_category_queries, make_queries
from conftest import GOLDEN
from gpu_util import ArrayScene, bsdf_on_gpu, material, rays_towards, soup, trace_on_gpu
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _same_branch(*rs):
    """Queries on which every result took the same category and sampling outcome."""
    ok = np.ones(len(rs[0]), bool)
    for r in rs[1:]:
        ok &= (r["category"] == rs[0]["category"]) & (r["ret"] == rs[0]["ret"])
    return ok


def test_bsdf_matches_reference_golden_vectors(cuda_dev):
    """Device FP32 against the reference's own FP32 build (golden vectors),
    field by field in FP32 units in the last place. The device fuses
    multiply-adds and uses CUDA's math functions, the host build neither, so
    the two round differently; the bound is: categories and uniforms consumed
    exact, a stated fraction of bit-identical results, most of the rest within
    16 ULP, and every query beyond that one where the reference's own FP32
    result is itself far from FP64 (the formula is ill-conditioned there):
    the device's deviation from the reference is at most 64x the reference's
    own FP32 error on 99% of those queries."""
    from bsdf_cases import FIELDS, ulp_distance
    g = np.load(os.path.join(GOLDEN, "bsdf_golden.npz"))
    q, ref = g["queries"], g["results"]
    res = bsdf_on_gpu(q, cuda_dev)
    assert np.array_equal(res["category"], ref["category"])
    assert np.array_equal(res["used"], ref["used"])
    assert (res["ret"] == ref["ret"]).mean() > 0.999
    assert np.allclose(res["categoryWeight"], ref["categoryWeight"], rtol=1e-6)
    o64 = orc.bsdf_query(q, precision=64)
    same = _same_branch(res, ref, o64)
    # fraction bit-identical, fraction within 16 ULP (measured on GB300 with margin)
    bars = {"f": (0.60, 0.96), "pdf": (0.50, 0.80), "bsdf": (0.40, 0.76), "dir": (0.12, 0.80)}
    for k in FIELDS:
        u = ulp_distance(res[k][same], ref[k][same])
        ident, near = float((u == 0).mean()), float((u <= 16).mean())
        far = u > 16
        n = int(same.sum())
        dv, rf, o = (np.asarray(x[k][same], np.float64).reshape(n, -1) for x in (res, ref, o64))
        dev_ref = np.linalg.norm(dv - rf, axis=1)      # device vs the reference's FP32 build
        ref_err = np.linalg.norm(rf - o, axis=1)       # the reference's FP32 build vs FP64
        bounded = float((dev_ref[far] <= 64.0 * ref_err[far]).mean()) if far.any() else 1.0
        print("%-4s bit-identical %.4f  <=16 ULP %.4f  beyond: %d, bounded by 64x the reference's own FP32 "
              "error %.4f" % (k, ident, near, int(far.sum()), bounded))
        assert ident >= bars[k][0] and near >= bars[k][1], (k, ident, near)
        assert bounded >= 0.98, (k, bounded)


def test_bsdf_2pow24_queries_vs_fp64_oracle(cuda_dev):
    """The material-sweep BSDF workload: all 2^24 seeded queries (16 chunks)
    evaluated and sampled on the GPU and checked against the FP64 oracle,
    beside the reference's FP32 build (the oracle's FP32 restatement, pinned
    bit for bit to it) on the same queries. The bar is 1e-5 relative to
    FP64 for eval, pdf and sample: the median of every field and the q90 of eval, pdf and sampled
    direction are within it; the sampled BSDF value's q90 and every field's
    fraction of queries over 1e-5 are no worse than the reference's own FP32
    build; and the tail is explained query by query: the queries on which the
    device misses 1e-5 are those on which the reference's FP32 build is
    itself off FP64 (by more than 1e-6), by the same amount (median ratio of
    the two errors <= 1.5)."""
    from bsdf_cases import FIELDS, rel_error
    errs = {k: ([], []) for k in FIELDS}   # device, reference FP32
    agree_cat = checked = 0
    for chunk in range(16):
        q = make_queries(1 << 20, 1000 + chunk) if chunk % 4 else make_fixed_category_queries(1 << 20, 1000 + chunk)
        res = bsdf_on_gpu(q, cuda_dev)
        assert (res["used"] <= 12).all()
        pdf = res["pdf"]
        assert (pdf[np.isfinite(pdf)] >= 0).all()
        assert np.isfinite(res["dir"]).all(1).mean() > 0.999
        o64 = orc.bsdf_query(q, precision=64)
        o32 = orc.bsdf_query(q, precision=32)
        agree_cat += int((res["category"] == o64["category"]).sum())
        checked += len(q)
        same = _same_branch(res, o64, o32)
        for k in FIELDS:
            errs[k][0].append(rel_error(res[k][same], o64[k][same]).astype(np.float32))
            errs[k][1].append(rel_error(o32[k][same], o64[k][same]).astype(np.float32))
    assert checked == 1 << 24
    assert agree_cat / checked > 0.9999
    for k in FIELDS:
        d, r = np.concatenate(errs[k][0]), np.concatenate(errs[k][1])
        med, q90 = float(np.median(d)), float(np.quantile(d, 0.9))
        rq90 = float(np.quantile(r, 0.9))
        over, rover = float((d > 1e-5).mean()), float((r > 1e-5).mean())
        miss = d > 1e-5
        illcond = float((r[miss] > 1e-6).mean()) if miss.any() else 1.0
        # error ratio on the misses (both infinite, e.g. a density only one
        # side finds zero, counts as the same error)
        rat = np.where(np.isinf(d[miss]) & np.isinf(r[miss]), 1.0, d[miss] / np.maximum(r[miss], 1e-30))
        ratio = float(np.median(rat)) if miss.any() else 1.0
        print("%-4s median %.2e q90 %.2e (reference FP32 q90 %.2e)  over 1e-5: %.4f (reference FP32 %.4f)  "
              "misses ill-conditioned %.4f, median error ratio %.2f" % (k, med, q90, rq90, over, rover, illcond,
                                                                      ratio))
        assert med <= 1e-5, (k, med)
        if k != "bsdf":
            assert q90 <= 1e-5, (k, q90)
        else:
            assert q90 <= 1.2 * rq90, (k, q90, rq90)
        assert over <= 1.05 * rover, (k, over, rover)
        assert illcond >= 0.97, (k, illcond)
        assert ratio <= 1.5, (k, ratio)


def _scene_from(arrays_scene, leaf=4, width=8):
    import optix_pt_gb300 as opt
    return opt.Renderer(arrays_scene, leaf_size=leaf, bvh_width=width, bvh_builder="lbvh")


def _scenes():
    import optix_pt_gb300 as opt
    out = [("cornell", opt.Scene.procedural("cornell")), ("spheres", opt.Scene.procedural("spheres"))]
    for n, dup in ((1, False), (2, False), (5000, True), (20000, False)):
        P, I = soup(n, 17 + n, dup)
        out.append(("soup%d" % n, ArrayScene(P, I, np.zeros(n, np.int32), [material()])))
    return out


@pytest.mark.parametrize("leaf", [1, 4])
def test_morton_codes_leaf_order_and_topology(cuda_dev, leaf):
    for name, sc in _scenes():
        r = _scene_from(sc, leaf)
        v = orc.SceneView(sc.struct, leaf)
        codes, order, nodes, used, leaves = v.bvh(sc.num_triangles)
        gcodes, gorder = r.bvh_leaf_order()
        assert np.array_equal(gcodes, codes), name
        assert np.array_equal(gorder, order), name
        gnodes = r.bvh_nodes()
        assert np.array_equal(gnodes, nodes), name
        st = r.stats()
        assert (st["bvhNodes"], st["bvhLeaves"]) == (used, leaves), name
        r.close()


@pytest.mark.parametrize("leaf", [1, 3, 4])
def test_bvh8_collapse_matches_host(cuda_dev, leaf):
    """The compressed 8-wide BVH, byte for byte: node records (quantised
    boxes, slots, child and triangle bases) and the triangle order."""
    for name, sc in _scenes():
        r = _scene_from(sc, leaf, 8)
        v = orc.SceneView(sc.struct, leaf)
        hn, ho = v.bvh8(sc.num_triangles)
        gn, go = r.bvh8_nodes()
        assert gn.shape == hn.shape, (name, gn.shape, hn.shape)
        assert np.array_equal(gn, hn), "%s: %d node records differ" % (name, int((gn != hn).any(1).sum()))
        assert np.array_equal(go, ho), name
        assert r.stats()["bvh8Nodes"] == len(hn)
        r.close()


@pytest.mark.parametrize("width", [8, 2])
def test_closest_hit_bit_exact(cuda_dev, width):
    rng = np.random.default_rng(7)
    for name, sc in _scenes():
        r = _scene_from(sc, 4 if width == 2 else 3, width)
        v = orc.SceneView(sc.struct, 4)
        a = sc.arrays()["positions"] if hasattr(sc, "arrays") else sc.P
        lo, hi = a.min(0), a.max(0)
        pad = (hi - lo) * 0.3 + 1e-3
        rays = rays_towards(rng, 1 << 16, (lo - pad, hi + pad), (lo, hi))
        g = trace_on_gpu(r, rays, cuda_dev)
        c = v.trace(rays)
        assert np.array_equal(g.view(np.int32), c.view(np.int32)), \
            "%s: %d of %d rays differ" % (name, int((g.view(np.int32) != c.view(np.int32)).any(1).sum()), len(rays))
        if sc.num_triangles >= 36:
            assert (g[:, 3].view(np.int32) >= 0).mean() > 0.2, name
        r.close()


@pytest.mark.parametrize("width", [8, 2])
def test_occlusion_bit_exact(cuda_dev, width):
    rng = np.random.default_rng(8)
    for name, sc in _scenes()[:3]:
        r = _scene_from(sc, 3, width)
        v = orc.SceneView(sc.struct, 4)
        a = sc.arrays()["positions"] if hasattr(sc, "arrays") else sc.P
        lo, hi = a.min(0), a.max(0)
        rays = rays_towards(rng, 1 << 15, (lo, hi), (lo, hi), tmin=1e-4, tmax=1.0)
        rays[:, 7] = rng.uniform(0.01, float(np.linalg.norm(hi - lo)), len(rays))
        g = trace_on_gpu(r, rays, cuda_dev, any_hit=True)[:, 3].view(np.int32) >= 0
        c = v.trace(rays, any_hit=True)[:, 3].view(np.int32) >= 0
        assert np.array_equal(g, c), name
        r.close()


def test_alpha_mask_and_blend(cuda_dev):
    """Alpha-tested candidates (cu/device_programs.cu:108-166): MASK ignores
    alpha < cutoff, BLEND ignores xi > alpha; results equal the oracle's."""
    n = 6000
    P, I = soup(n, 99, scale=0.3)
    mats = [material(), material(alphaMode=2, alphaCutoff=0.5), material(alphaMode=1)]
    mats[1].baseColour[3] = 0.3   # masked out
    mats[2].baseColour[3] = 0.5   # blended
    M = (np.arange(n) % 3).astype(np.int32)
    sc = ArrayScene(P, I, M, mats)
    r = _scene_from(sc)
    v = orc.SceneView(sc.struct, 4)
    rng = np.random.default_rng(5)
    rays = rays_towards(rng, 1 << 15, (-2, 2), (-1, 1))
    for any_hit in (False, True):
        g = trace_on_gpu(r, rays, cuda_dev, any_hit)
        c = v.trace(rays, any_hit)
        if any_hit:
            # an occlusion query returns the first accepted triangle it finds,
            # which depends on the tree; only "occluded or not" is canonical
            assert np.array_equal(g[:, 3].view(np.int32) >= 0, c[:, 3].view(np.int32) >= 0)
        else:
            assert np.array_equal(g.view(np.int32), c.view(np.int32))
        prims = g[:, 3].view(np.int32)
        assert not np.isin(prims[prims >= 0] % 3, [1]).any()   # masked material never hit
    r.close()


def test_empty_and_tiny_scenes(cuda_dev):
    P, I = soup(1, 3)
    sc = ArrayScene(P, I, np.zeros(1, np.int32), [material()])
    r = _scene_from(sc)
    rays = rays_towards(np.random.default_rng(1), 256, (-2, 2), (-1, 1))
    g = trace_on_gpu(r, rays, cuda_dev)
    c = orc.SceneView(sc.struct, 4).trace(rays)
    assert np.array_equal(g.view(np.int32), c.view(np.int32))
    r.close()
