"""Traversal faults are counted, never silent.

A ray's walk can go wrong in two ways: a node group is dropped because the
traversal stack is full, or the walk is cut short by its node budget. Both are
counted in optpt_stats (traversalStackOverflows, traversalBudgetExhausted);
every GPU test checks both are zero on the renderers it closes (conftest).
The 8-wide BVH's stack cannot overflow at all: it holds at most one group per
tree level, and optpt_create refuses trees of more than 64 levels (bvh8Levels
in the stats). The reference's OptiX traversal reports neither
(cu/device_programs.cu:63).

Here: a deliberately deep, clustered soup (a caterpillar of 32 Morton
clusters, each a run of 4,096 equal codes: binary LBVH depth 42) that the
64-entry stacks of both BVH widths must survive with hits bit-exact against
the host traversal; and a renderer with a tiny node budget, whose cut-short
walks must show up in the counter.
"""
import numpy as np
import pytest

from gpu_util import ArrayScene, material, rays_towards, trace_on_gpu
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def deep_soup(per_cluster=4096, seed=3):
    """Clusters of tiny triangles at the Morton cells with a single set bit
    (30 cells: bit b of one axis) plus the two corner cells, so that every
    bit of the 30-bit code splits one cluster off the chain, and each
    cluster's equal codes add log2(per_cluster) index-split levels."""
    rng = np.random.default_rng(seed)
    cells = [(0, 0, 0), (1023, 1023, 1023)]
    for a in range(3):
        for b in range(10):
            c = [0, 0, 0]
            c[a] = 1 << b
            cells.append(tuple(c))
    P = []
    for c in cells:
        cen = np.array(c, np.float64) + 0.5
        base = cen + rng.uniform(-0.3, 0.3, (per_cluster, 3))      # inside the cluster's Morton cell
        P.append((base[:, None, :] + rng.uniform(-0.05, 0.05, (per_cluster, 3, 3))).reshape(-1, 3))
    P = np.concatenate(P).astype(np.float32)
    n = len(P) // 3
    return P, np.arange(3 * n, dtype=np.int32).reshape(n, 3), np.array(cells, np.float32) + 0.5


def binary_depth(nodes):
    """Depth of the host LBVH from its (ref0, ref1, count0, count1) records."""
    depth, best, stack = {0: 1}, 1, [0]
    while stack:
        x = stack.pop()
        for s in range(2):
            ref, cnt = nodes[x][s], nodes[x][2 + s]
            if cnt == 0 and ref >= 0:
                depth[ref] = depth[x] + 1
                best = max(best, depth[ref])
                stack.append(ref)
    return best


def _light():
    from optix_pt_gb300 import _ffi
    L = _ffi.Light()
    L.type = 0
    L.radiance[:] = [5e5, 5e5, 5e5]
    L.p0[:] = [300.0, 700.0, 200.0]
    return L


def _scene():
    P, I, centres = deep_soup()
    # the camera looks along the chain from just outside the corner cluster,
    # so camera and shadow rays walk the deepest paths of the tree
    sc = ArrayScene(P, I, np.zeros(len(I), np.int32), [material()], lights=[_light()],
                    cam=((-1.2, -0.9, -1.4), (2.0, 2.0, 2.0), (0.0, 1.0, 0.0), 25.0), max_depth=6)
    return sc, centres


def _rays_at_clusters(rng, centres, n):
    """Rays from random points around the box towards random clusters (most
    end deep in the tree), plus rays that graze the chain."""
    tgt = centres[rng.integers(0, len(centres), n)] + rng.uniform(-0.3, 0.3, (n, 3))
    org = rng.uniform(-100.0, 1130.0, (n, 3))
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = org
    rays[:, 4:7] = d
    rays[:, 7] = 1e16
    return np.concatenate([rays, rays_towards(rng, n // 4, (-50, 1100), (0, 1024))])


@pytest.mark.parametrize("width,builder", [(8, "lbvh"), (8, "ploc"), (2, "lbvh")])
def test_deep_clustered_soup_needs_no_fault(cuda_dev, width, builder):
    import torch

    import optix_pt_gb300 as opt
    sc, centres = _scene()
    v = orc.SceneView(sc.struct, 1)
    nodes = v.bvh(sc.num_triangles)[2]
    assert binary_depth(nodes) >= 40          # deep enough to matter for a 64-entry stack
    r = opt.Renderer(sc, leaf_size=1, bvh_width=width, bvh_builder=builder)
    rng = np.random.default_rng(21)
    rays = _rays_at_clusters(rng, centres, 1 << 16)
    for any_hit in (False, True):
        g = trace_on_gpu(r, rays, cuda_dev, any_hit)
        c = v.trace(rays, any_hit)
        if any_hit:
            assert np.array_equal(g[:, 3].view(np.int32) >= 0, c[:, 3].view(np.int32) >= 0)
        else:
            assert np.array_equal(g.view(np.int32), c.view(np.int32))
            assert (g[:, 3].view(np.int32) >= 0).mean() > 0.5
    # the wavefront kernels (closest hit + shadow rays) over the same tree
    r.setupOutputBuffer(96, 96)
    r.render(4, torch.cuda.current_stream())
    torch.cuda.synchronize()
    st = r.stats()
    assert st["extensionRays"] > 0 and st["shadowRays"] > 0
    assert st["traversalStackOverflows"] == 0 and st["traversalBudgetExhausted"] == 0
    if width == 8:
        assert 0 < st["bvh8Levels"] <= 64
    r.close()


def test_node_budget_exhaustion_is_counted(cuda_dev):
    """With a budget of 3 nodes per ray, walks that need more are cut short;
    each one is counted, and those rays' results may differ from the host's."""
    import optix_pt_gb300 as opt
    sc, centres = _scene()
    r = opt.Renderer(sc, leaf_size=1, node_budget=3)
    r.expect_traversal_faults = True
    rng = np.random.default_rng(22)
    rays = _rays_at_clusters(rng, centres, 4096)
    g = trace_on_gpu(r, rays, cuda_dev)
    st = r.stats()
    assert st["traversalStackOverflows"] == 0
    assert 0 < st["traversalBudgetExhausted"] <= len(rays)
    c = orc.SceneView(sc.struct, 1).trace(rays)
    assert not np.array_equal(g.view(np.int32), c.view(np.int32))
    r.close()
    # the default budget: no walk is cut short on the same rays
    r = opt.Renderer(sc, leaf_size=1)
    g = trace_on_gpu(r, rays, cuda_dev)
    assert np.array_equal(g.view(np.int32), c.view(np.int32))
    assert r.stats()["traversalBudgetExhausted"] == 0
    r.close()
