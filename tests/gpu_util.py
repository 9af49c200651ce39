"""Helpers for the GPU parity tests: device buffers through torch, seeded rays,
and scene structs built from numpy arrays."""
import ctypes

import numpy as np


def to_dev(arr, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr)).to(dev)


def bsdf_on_gpu(q, dev):
    import torch

    import optix_pt_gb300 as opt
    qb = np.ascontiguousarray(q).view(np.uint8)
    qd = torch.from_numpy(qb.copy()).to(dev)
    rd = torch.zeros(len(q) * opt.BSDF_RESULT.itemsize, dtype=torch.uint8, device=dev)
    opt.bsdf_batch(qd.data_ptr(), rd.data_ptr(), len(q), torch.cuda.current_stream())
    torch.cuda.synchronize()
    return rd.cpu().numpy().view(opt.BSDF_RESULT)


def rays_towards(rng, n, origin_box, target_box, tmin=0.0, tmax=1e16):
    o = rng.uniform(origin_box[0], origin_box[1], (n, 3))
    t = rng.uniform(target_box[0], target_box[1], (n, 3))
    d = t - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def trace_on_gpu(renderer, rays, dev, any_hit=False):
    import torch
    rd = to_dev(rays, dev)
    hd = torch.zeros((len(rays), 4), dtype=torch.float32, device=dev)
    renderer.trace(rd.data_ptr(), hd.data_ptr(), len(rays), any_hit, torch.cuda.current_stream())
    torch.cuda.synchronize()
    return hd.cpu().numpy()


class ArrayScene:
    """An optpt_scene over numpy arrays (kept alive by this object)."""

    def __init__(self, positions, tri_indices, mat_indices, materials, lights=(), normals=None, tex_coords=None,
                 cam=((0, 0, 3), (0, 0, 0), (0, 1, 0), 40.0), res=(64, 64), bg=(0, 0, 0), max_depth=8):
        from optix_pt_gb300 import _ffi
        self.P = np.ascontiguousarray(positions, np.float32)
        self.I = np.ascontiguousarray(tri_indices, np.int32)
        self.M = np.ascontiguousarray(mat_indices, np.int32)
        self.N = None if normals is None else np.ascontiguousarray(normals, np.float32)
        self.T = None if tex_coords is None else np.ascontiguousarray(tex_coords, np.float32)
        self.mats = (_ffi.MaterialData * len(materials))(*materials)
        self.lights = (_ffi.Light * max(1, len(lights)))(*lights)
        s = _ffi.SceneStruct()
        fp = ctypes.POINTER(ctypes.c_float)
        ip = ctypes.POINTER(ctypes.c_int32)
        s.positions = self.P.ctypes.data_as(fp)
        s.numVertices = len(self.P)
        s.normals = self.N.ctypes.data_as(fp) if self.N is not None else None
        s.texCoords = self.T.ctypes.data_as(fp) if self.T is not None else None
        s.triIndices = self.I.ctypes.data_as(ip)
        s.numTriangles = len(self.I)
        s.matIndices = self.M.ctypes.data_as(ip)
        s.materials = ctypes.cast(self.mats, ctypes.POINTER(_ffi.MaterialData))
        s.numMaterials = len(materials)
        s.lights = ctypes.cast(self.lights, ctypes.POINTER(_ffi.Light))
        s.numLights = len(lights)
        s.camEye[:], s.camTarget[:], s.camUp[:] = cam[0], cam[1], cam[2]
        s.camFovYDeg = cam[3]
        s.resX, s.resY = res
        s.bgColour[:] = bg
        s.maxDepth = max_depth
        self.struct = s
        self.num_triangles = len(self.I)


def material(rgb=(0.5, 0.5, 0.5), **kw):
    from optix_pt_gb300 import _ffi
    m = _ffi.MaterialData()
    for name in ("baseColourTexture", "normalTexture", "metallicRoughnessTexture", "emissiveTexture",
                 "sheenColourTexture", "sheenRoughnessTexture"):
        setattr(m, name, -1)
    for tf in ("baseColourTexTf", "normalTexTf", "metallicRoughnessTexTf", "emissiveTexTf", "sheenColourTexTf",
               "sheenRoughnessTexTf"):
        getattr(m, tf).scale[:] = [1.0, 1.0]
    m.baseColour[:] = [rgb[0], rgb[1], rgb[2], 1.0]
    m.alphaCutoff = 0.5
    m.ior = 1.5
    m.roughness = 1.0
    for k, v in kw.items():
        if k in ("emission", "sheenColour"):
            getattr(m, k)[:] = v
        else:
            setattr(m, k, v)
    return m


def soup(n, seed, dup=False, scale=0.15):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, (n, 3))
    if dup:
        c[n // 2:] = c[: n - n // 2]
    P = (c[:, None, :] + rng.normal(scale=scale, size=(n, 3, 3))).reshape(-1, 3).astype(np.float32)
    I = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    return P, I


def render_pair(scene, w, h, spp_gpu, spp_cpu, cpu_base, precision, batch=None, classify=False, **renderer_kw):
    """GPU render (sample indices from 0) and an oracle render of the same
    frame (sample indices from cpu_base): ((sum, sumsq, n) GPU, (sum, sumsq,
    n) oracle, GPU stats, oracle ray counts). classify=True appends a fifth
    item, the same oracle render from the oracle's build with fused
    multiply-adds (a second FP32 rounding of the same paths), for
    paired_agreement."""
    import torch

    import optix_pt_gb300 as opt
    from oracle import oracle as orc
    r = opt.Renderer(scene, spp_batch=batch or 0, **renderer_kw)
    r.setupOutputBuffer(w, h)
    r.render(spp_gpu, torch.cuda.current_stream())
    torch.cuda.synchronize()
    s, q, n = r.accum()
    lp = r.launch_params()
    cam = list(lp.eye) + list(lp.U) + list(lp.V) + list(lp.W) + list(lp.bgColour)
    v = orc.SceneView(scene.struct, 4)
    cs, cq, cnt = v.render(cam, w, h, lp.seed, cpu_base, spp_cpu, lp.maxDepth, precision=precision)
    st = r.stats()
    r.close()
    out = (s.reshape(-1, 3), q.reshape(-1, 3), n), (cs, cq, spp_cpu), st, cnt
    if classify:
        vf = orc.SceneView(scene.struct, 4, variant="fma")
        fs, fq, _ = vf.render(cam, w, h, lp.seed, cpu_base, spp_cpu, lp.maxDepth, precision=precision)
        out = out + ((fs, fq, spp_cpu),)
    return out


def paired_agreement(g, c, f, rtol=1e-4, atol=1e-5):
    """Pixels of a paired render (same random streams) on which the GPU and
    the FP32 oracle agree, split by whether the path is robust to FP32
    rounding: a pixel is rounding-sensitive when the oracle's two FP32 builds
    (without and with fused multiply-adds) already disagree on it. Returns
    (agreement on robust pixels, fraction of rounding-sensitive pixels,
    agreement on all pixels)."""
    def close(a, b):
        return (np.abs(a - b) <= rtol * np.maximum(1.0, np.abs(b)) + atol).all(1)
    robust = close(f[0], c[0])
    agree = close(g[0], c[0])
    return float(agree[robust].mean()), float(1.0 - robust.mean()), float(agree.mean())


def pixel_stats(g, c):
    """Per-pixel z scores of two independent Monte Carlo estimates: (fraction
    of live pixels with z > 3, |frame mean difference|, its standard error,
    GPU means, oracle means, live mask)."""
    (gs, gq, gn), (cs, cq, cn) = g, c
    gm, cm = gs / gn, cs / cn
    gv = np.maximum(gq / gn - gm ** 2, 0) / gn
    cv = np.maximum(cq / cn - cm ** 2, 0) / cn
    var = gv + cv
    live = var > 0
    z = np.zeros_like(gm)
    z[live] = np.abs(gm - cm)[live] / np.sqrt(var[live])
    frac = float((z[live] > 3.0).mean()) if live.any() else 0.0
    se = np.sqrt(var.sum()) / var.size
    return frac, abs(gm.mean() - cm.mean()), se, gm, cm, live


def tile_stats(g, c, w, tile=8):
    """z scores of tile means (tile x tile pixels) of two independent
    estimates of a frame whose rows are `w` pixels wide: averaging over a
    tile makes the means closer to Gaussian and their variance estimates
    steadier than per pixel, so the 3-sigma rate is the one a bias would
    lift. Returns the fraction of tile channels with z > 3."""
    (gs, gq, gn), (cs, cq, cn) = g, c
    gm, cm = gs / gn, cs / cn
    gv = np.maximum(gq / gn - gm ** 2, 0) / gn
    cv = np.maximum(cq / cn - cm ** 2, 0) / cn
    h = gm.shape[0] // w
    th, tw = h // tile, w // tile

    def tiles(a):
        a = a.reshape(h, w, 3)[:th * tile, :tw * tile]
        return a.reshape(th, tile, tw, tile, 3).sum((1, 3))

    n = tile * tile
    d = (tiles(gm) - tiles(cm)) / n
    var = (tiles(gv) + tiles(cv)) / (n * n)
    live = var > 0
    z = np.abs(d[live]) / np.sqrt(var[live])
    return float((z > 3.0).mean()) if z.size else 0.0
