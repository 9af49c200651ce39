"""Seeded generators of BSDF queries, shared by the fixture script and the tests.

The distribution follows the material-sweep BSDF oracle workload: wo and wi
uniform on the sphere, roughness U(0.02, 1), metallic and transmission drawn
from {0, U(0,1), 1}, ior U(1.0, 2.4), sheen U(0, 1); plus coat, specular,
subsurface and emissive cases so that every branch of the reference's
categorisation and sampling code is reached.
"""
import numpy as np

from oracle.abi import BSDF_QUERY, NXS


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _tri(rng, n):
    """Each entry 0, U(0,1) or 1 with equal odds."""
    pick = rng.integers(0, 3, size=n)
    u = rng.random(n)
    return np.where(pick == 0, 0.0, np.where(pick == 1, u, 1.0)).astype(np.float32)


def make_queries(n, seed):
    rng = np.random.default_rng(seed)
    q = np.zeros(n, dtype=BSDF_QUERY)
    q["baseColour"] = rng.random((n, 3))
    q["metallic"] = _tri(rng, n)
    q["transmissionWeight"] = _tri(rng, n)
    rough = rng.uniform(0.02, 1.0, n)
    rough[rng.random(n) < 0.08] = 0.0            # specular (roughness 0) branches
    q["roughness"] = rough
    q["ior"] = rng.uniform(1.0, 2.4, n)
    q["specular"] = np.where(rng.random(n) < 0.5, 1.0, np.where(rng.random(n) < 0.5, 0.0, rng.random(n)))
    q["subsurfaceWeight"] = np.where(rng.random(n) < 0.8, 0.0, _tri(rng, n))
    has_coat = rng.random(n) < 0.2
    q["coatWeight"] = np.where(has_coat, rng.random(n), 0.0)
    q["coatRoughness"] = np.where(rng.random(n) < 0.15, 0.0, rng.uniform(0.02, 1.0, n))
    has_sheen = rng.random(n) < 0.3
    q["sheenColour"] = np.where(has_sheen[:, None], rng.random((n, 3)), 0.0)
    sr = rng.uniform(0.02, 1.0, n)
    q["sheenRoughnessMat"] = sr
    q["sheenRoughness"] = np.where(rng.random(n) < 0.1, 0.0, sr * rng.uniform(0.5, 1.0, n))
    emissive = rng.random(n) < 0.03
    q["emission"] = np.where(emissive[:, None], rng.uniform(0.0, 20.0, (n, 3)), 0.0)
    q["category"] = 0
    q["n"] = _unit(rng, n)
    q["wo"] = _unit(rng, n)
    q["wi"] = _unit(rng, n)
    q["xs"] = rng.random((n, NXS), dtype=np.float32)
    # Strictly inside (0, 1): the reference's cuRAND uniforms never return 0.
    q["xs"] = np.clip(q["xs"], np.float32(2 ** -24), np.float32(1.0))
    return q


def make_fixed_category_queries(n, seed):
    """Queries whose MaterialData.category is precomputed on the host
    (material_params.h:187-223), so categoriseMaterial returns it unchanged."""
    q = make_queries(n, seed)
    rng = np.random.default_rng(seed + 1)
    M, D, O, T, Df, Lb, Sp = 1, 2, 8, 16, 64, 1024, 2048
    choices = np.array([M, M | Sp, D | T, D | T | Sp, D | O | Df, D | O | Df | Lb], dtype=np.uint32)
    cat = choices[rng.integers(0, len(choices), n)]
    q["category"] = cat
    q["roughness"] = np.where((cat & Sp) != 0, 0.0, np.maximum(q["roughness"], 0.02))
    q["roughness"] = np.where((cat & Lb) != 0, 0.0, q["roughness"])
    return q


def agreement(q, a, b):
    """Agreement metrics between two BSDF result arrays for the same queries.

    FP32 evaluation of the reference's formulas is ill-conditioned in known
    places (GGX at roughness ~0.02 samples a lobe ~1e-4 rad wide, Oren-Nayar
    evaluates tan(acos(1e-5)) for back-facing directions), so the metrics are
    taken where they are meaningful:
      f_rel      eval, both directions above the surface (n.v, n.l > 0.05)
      dir_abs    sampled direction, absolute component error
      weight_rel bsdf |n.l| / pdf, the throughput factor the integrator uses
      pdf_rel, bsdf_rel  for roughness >= 0.1, above the surface
    Each entry is (q99, q99.9) of the relative (or absolute) error.
    """
    n = q["n"].astype(np.float64)
    nv = np.einsum("ij,ij->i", n, q["wo"])
    nl = np.einsum("ij,ij->i", n, q["wi"])
    good = (nv > 0.05) & (nl > 0.05)
    rough = (q["roughness"] >= 0.1) & (q["coatRoughness"] >= 0.1) & (q["sheenRoughnessMat"] >= 0.1)

    def rel(x, y, floor=1e-30):
        x = np.asarray(x, np.float64).reshape(len(q), -1)
        y = np.asarray(y, np.float64).reshape(len(q), -1)
        fin = np.isfinite(x) & np.isfinite(y)
        return np.abs(x - y) / np.maximum(np.abs(x), floor), fin

    def qs(v):
        return (float(np.quantile(v, 0.99)), float(np.quantile(v, 0.999))) if v.size else (0.0, 0.0)

    def weight(r):
        c = np.abs(np.einsum("ij,ij->i", n, np.asarray(r["dir"], np.float64)))
        p = np.asarray(r["pdf"], np.float64)
        return np.asarray(r["bsdf"], np.float64) * c[:, None] / np.where(p == 0, np.inf, p)[:, None]

    out = {}
    r, fin = rel(a["f"], b["f"])
    out["f_rel"] = qs(r[fin & good[:, None]])
    out["dir_abs"] = qs(np.abs(np.asarray(a["dir"], np.float64) - np.asarray(b["dir"], np.float64)).max(1))
    r, fin = rel(weight(a), weight(b), 1e-6)
    out["weight_rel"] = qs(r[fin])
    for k in ("pdf", "bsdf"):
        r, fin = rel(a[k], b[k])
        out[k + "_rel"] = qs(r[fin & (good & rough)[:, None]])
    return out


# Envelope of FP32 evaluation against FP64 (measured on the reference's own
# FP32 build vs the FP64 restatement, with margin): (q99, q99.9) bounds.
FP32_ENVELOPE = {
    "f_rel": (1e-4, 1e-3),
    "dir_abs": (2e-4, 2e-3),
    "weight_rel": (5e-4, 1e-2),
    "pdf_rel": (3e-3, 2e-2),
    "bsdf_rel": (3e-3, 2e-2),
}


def within(metrics, envelope=FP32_ENVELOPE):
    bad = {k: v for k, v in metrics.items() if v[0] > envelope[k][0] or v[1] > envelope[k][1]}
    return not bad, bad


# ---------------------------------------------------------------- FP32 against FP64, query by query
FIELDS = ("f", "pdf", "bsdf", "dir")


def rel_error(x, y):
    """Norm-relative error |x - y| / |y| of each query's vector (or scalar)
    field; 0 where both are zero, inf where only y is zero or either is NaN."""
    x = np.asarray(x, np.float64).reshape(len(x), -1)
    y = np.asarray(y, np.float64).reshape(len(y), -1)
    d = np.linalg.norm(x - y, axis=1)
    den = np.linalg.norm(y, axis=1)
    r = np.where(den > 0, d / np.where(den > 0, den, 1.0), np.where(d > 0, np.inf, 0.0))
    return np.nan_to_num(r, nan=np.inf)


def ulp_distance(x, y):
    """Largest distance in FP32 units in the last place over a query's
    components (0 = bit-identical; NaN pairs count as identical)."""
    def key(v):
        b = np.asarray(v, np.float32).reshape(len(v), -1).view(np.int32).astype(np.int64)
        return np.where(b < 0, -(b & 0x7FFFFFFF), b)
    a, b = key(x), key(y)
    both_nan = np.isnan(np.asarray(x, np.float32).reshape(len(x), -1)) & \
        np.isnan(np.asarray(y, np.float32).reshape(len(y), -1))
    return np.where(both_nan, 0, np.abs(a - b)).max(1)
