"""CPU oracle of the learned path-guiding network (test infrastructure only).

The reference has no learned guiding: this is a restatement of the method the
GPU implements, used to check its forward pass and gradients.

* Multiresolution hash-grid encoding (Mueller et al., "Instant Neural Graphics
  Primitives", SIGGRAPH 2022): 16 levels x 2 features, 2^19 entries per level,
  dense indexing where (res + 1)^3 fits the table, else the spatial hash
  x + (y * 2654435761 ^ z * 805459861) (mod 2^19); trilinear weights.
* MLP 64 -> 64 -> 64 -> 64 -> 64 -> 64 (ReLU, no biases; a constant-1 input),
  BF16 operands with FP32 accumulation: every matrix operand is rounded to
  BF16 (round to nearest even) exactly where the tensor-core kernels round.
* Output: 8 von Mises-Fisher lobes (mu = normalise(raw), kappa =
  exp(clamp(raw, -3, 5.5)), weights = softmax(logits)); loss -c log q(wi) with
  c = min(weight, 16 x mean positive weight) / sum of weights (Dong et al., "Neural Parametric
  Mixtures for Path Guiding", SIGGRAPH 2023), gradient in closed form.

`gradients(..., use_bf16=False)` gives the exact FP64 gradient of the same loss,
which `finite_difference_check` pins against central differences.
"""
import numpy as np

LEVELS, FEATS, TABLE, WIDTH, LAYERS, LOBES = 16, 2, 1 << 19, 64, 5, 8
IN_NORMAL, IN_WO, IN_ONE = 32, 35, 38
LOG_KAPPA_MIN, LOG_KAPPA_MAX = -3.0, 5.5
WEIGHT_CAP = 16.0
OUT_SELECT, SELECT_MIN, SELECT_SPAN = 40, 0.02, 0.96


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def corners(levels_res, levels_dense, lo, inv_ext, pos):
    """Per level and corner: table entries (n, 16, 8) and weights (n, 16, 8)."""
    p = np.clip((pos.astype(np.float32) - lo.astype(np.float32)) * inv_ext.astype(np.float32), np.float32(0),
                np.float32(0.99999994))
    n = len(pos)
    ent = np.zeros((n, LEVELS, 8), np.int64)
    wts = np.zeros((n, LEVELS, 8), np.float32)
    for l in range(LEVELS):
        r = np.float32(levels_res[l])
        g = p * r
        f = np.floor(g)
        t = g - f
        fi = f.astype(np.uint64)
        res1 = np.uint64(int(r) + 1)
        for c in range(8):
            bx, by, bz = c & 1, (c >> 1) & 1, (c >> 2) & 1
            x, y, z = fi[:, 0] + np.uint64(bx), fi[:, 1] + np.uint64(by), fi[:, 2] + np.uint64(bz)
            wx = t[:, 0] if bx else np.float32(1) - t[:, 0]
            wy = t[:, 1] if by else np.float32(1) - t[:, 1]
            wz = t[:, 2] if bz else np.float32(1) - t[:, 2]
            wts[:, l, c] = (wx * wy) * wz
            if levels_dense[l]:
                e = x + res1 * (y + res1 * z)
            else:
                m = np.uint64(0xFFFFFFFF)
                e = (x + (((y * np.uint64(2654435761)) & m) ^ ((z * np.uint64(805459861)) & m))) & np.uint64(
                    TABLE - 1)
            ent[:, l, c] = e.astype(np.int64)
    return ent, wts


def encode(hash_params, ent, wts, n, wo, dtype=np.float32):
    """Network inputs (n, 64) (FP32 as the kernels form them, or FP64)."""
    h = hash_params.reshape(LEVELS, TABLE, FEATS)
    x = np.zeros((len(n), WIDTH), np.float64)
    for l in range(LEVELS):
        v = h[l][ent[:, l, :]]                     # (n, 8, 2)
        x[:, 2 * l:2 * l + 2] = (wts[:, l, :, None].astype(np.float64) * v).sum(1)
    x[:, IN_NORMAL:IN_NORMAL + 3] = n
    x[:, IN_WO:IN_WO + 3] = wo
    x[:, IN_ONE] = 1.0
    return x.astype(dtype)


def forward(mlp, x0, use_bf16=True):
    """Activations X_0..X_4 (inputs of each layer) and the outputs Z_4."""
    W = mlp.reshape(LAYERS, WIDTH, WIDTH)
    rnd = bf16 if use_bf16 else (lambda a: a.astype(np.float64))
    xs = [rnd(x0)]
    for l in range(LAYERS):
        z = (xs[-1].astype(np.float64) @ rnd(W[l]).astype(np.float64).T)
        z = z.astype(np.float32) if use_bf16 else z
        if l < LAYERS - 1:
            xs.append(rnd(np.maximum(z, 0)))
    return xs, z


def decode(o):
    o = o.astype(np.float64)
    logits = o[:, 4::5][:, :LOBES]
    w = np.exp(logits - logits.max(1, keepdims=True))
    w /= w.sum(1, keepdims=True)
    raw = np.stack([o[:, 5 * k:5 * k + 3] for k in range(LOBES)], 1)  # (n, 8, 3)
    ln = np.linalg.norm(raw, axis=2, keepdims=True)
    mu = raw / np.maximum(ln, 1e-300)
    lk = o[:, 3::5][:, :LOBES]
    kap = np.exp(np.clip(lk, LOG_KAPPA_MIN, LOG_KAPPA_MAX))
    return w, mu, kap, raw, ln, lk


def vmf_pdf(mu, kap, wi):
    t = (mu * wi[:, None, :]).sum(2)
    norm = np.where(kap < 1e-4, 0.25 / np.pi, kap / (2 * np.pi * -np.expm1(-2 * kap)))
    return norm * np.exp(kap * (t - 1)), t


def select_prob(o):
    """Probability of sampling the mixture instead of the BSDF (output 40)."""
    return SELECT_MIN + SELECT_SPAN / (1.0 + np.exp(-o[:, OUT_SELECT].astype(np.float64)))


def mixture_pdf(o, wi):
    w, mu, kap, *_ = decode(o)
    v, _ = vmf_pdf(mu, kap, wi)
    return (w * v).sum(1)


def loss_and_dout(o, wi, c, pb, whole_target=True):
    """Sum over samples of -c log(a q(wi) + (1 - a) pb) (the one-sample MIS
    proposal's density) and its gradient w.r.t. the outputs. The selection
    output always follows that loss; with whole_target the lobe outputs
    follow -c log q instead (the mixture learns the whole target)."""
    w, mu, kap, raw, ln, lk = decode(o)
    v, t = vmf_pdf(mu, kap, wi)
    q = np.maximum((w * v).sum(1), 1e-30)
    a = select_prob(o)
    mix = np.maximum(a * q + (1 - a) * pb, 1e-30)
    loss = float((-c * np.log(mix)).sum())
    r = w * v / q[:, None]
    d = np.zeros((len(o), WIDTH), np.float64)
    sg = (a - SELECT_MIN) / SELECT_SPAN
    d[:, OUT_SELECT] = -c * (q - pb) / mix * SELECT_SPAN * sg * (1 - sg)
    cc = (c if whole_target else c * a * q / mix)[:, None]
    d[:, 4:5 * LOBES:5] = cc * (w - r)
    dlogc = np.where(kap < 1e-3, (2.0 / 3.0) * kap, 1.0 / kap - 2.0 / np.expm1(2 * kap))
    dk = -cc * r * (dlogc + t - 1)
    inside = (lk > LOG_KAPPA_MIN) & (lk < LOG_KAPPA_MAX)
    d[:, 3:5 * LOBES:5] = np.where(inside, dk * kap, 0.0)
    dmu = (-cc * r * kap)[:, :, None] * wi[:, None, :]
    dm = (dmu - (dmu * mu).sum(2, keepdims=True) * mu) / np.maximum(ln, 1e-300)
    for k in range(LOBES):
        d[:, 5 * k:5 * k + 3] = dm[:, k]
    return loss, d


def infer(mlp, hash_params, geom, queries):
    """Network outputs (n, 64) for queries (n, 12) = (pos, -, n, -, wo, -), as
    the inference kernel computes them: hash features from the FP16 copy of
    the table, BF16 operands."""
    res, dense, lo, inv_ext = geom
    q = np.asarray(queries, np.float32).reshape(-1, 12)
    ent, wts = corners(res, dense, lo, inv_ext, q[:, 0:3])
    h16 = hash_params.astype(np.float16).astype(np.float32)
    x0 = encode(h16, ent, wts, q[:, 4:7], q[:, 8:11])
    return forward(mlp, x0, True)[1]


def unpack(packed):
    """(n, 48) float16 packed mixtures -> weights (n, 8), mu (n, 8, 3), kappa
    (n, 8); the selection probability is column 40 (`unpack_select`)."""
    h = np.asarray(packed).view(np.float16).reshape(-1, 48).astype(np.float64)
    mu = h[:, :32].reshape(-1, LOBES, 4)[:, :, :3]
    mu = mu / np.maximum(np.linalg.norm(mu, axis=2, keepdims=True), 1e-6)
    kap = h[:, :32].reshape(-1, LOBES, 4)[:, :, 3]
    w = h[:, 32:40]
    w = w / w.sum(1, keepdims=True)
    return w, mu, kap


def unpack_select(packed):
    return np.asarray(packed).view(np.float16).reshape(-1, 48)[:, 40].astype(np.float64)


def gradients(mlp, hash_params, geom, samples, use_bf16=True):
    """(loss, dMLP (5, 64, 64), dHash (LEVELS * TABLE * 2,)) of a batch.

    samples: (n, 16) float32 = (pos, weight, n, -, wo, pb, wi, -), pb = the
    BSDF lobe's density at wi."""
    res, dense, lo, inv_ext = geom
    s = np.asarray(samples, np.float32).reshape(-1, 16)
    wgt = s[:, 3].astype(np.float64)
    ok = np.isfinite(wgt) & (wgt > 0)
    total = wgt[ok].sum()
    cap = np.float32(WEIGHT_CAP * total / max(ok.sum(), 1))   # heavy-tail cap, as the kernel applies it
    c = np.where(ok, np.minimum(s[:, 3], cap).astype(np.float64) / total if total > 0 else 0.0, 0.0)
    ent, wts = corners(res, dense, lo, inv_ext, s[:, 0:3])
    x0 = encode(hash_params, ent, wts, s[:, 4:7], s[:, 8:11], np.float32 if use_bf16 else np.float64)
    xs, z = forward(mlp, x0, use_bf16)
    W = mlp.reshape(LAYERS, WIDTH, WIDTH)
    loss, d = loss_and_dout(z, s[:, 12:15].astype(np.float64), c, np.maximum(s[:, 11], 0).astype(np.float64))
    rnd = bf16 if use_bf16 else (lambda a: a.astype(np.float64))
    dW = np.zeros((LAYERS, WIDTH, WIDTH))
    dz = rnd(d.astype(np.float32)) if use_bf16 else d
    for l in range(LAYERS - 1, -1, -1):
        dW[l] = dz.astype(np.float64).T @ xs[l].astype(np.float64)
        dx = dz.astype(np.float64) @ rnd(W[l]).astype(np.float64)
        if use_bf16:
            dx = dx.astype(np.float32)
        if l > 0:
            dzn = np.where(xs[l] > 0, dx, 0.0)
            dz = rnd(dzn.astype(np.float32)) if use_bf16 else dzn
    dH = np.zeros(LEVELS * TABLE * FEATS)
    for l in range(LEVELS):
        for f in range(FEATS):
            contrib = wts[:, l, :].astype(np.float64) * dx[:, 2 * l + f, None]
            np.add.at(dH, ((l * TABLE + ent[:, l, :]) * FEATS + f).ravel(), contrib.ravel())
    return loss, dW, dH


def finite_difference_check(seed=0, n=6, eps=1e-5, pb_scale=1.0):
    """Max relative error of the analytic FP64 output gradient against
    central differences of the loss, on random outputs and directions.
    With pb_scale = 0 the lobe gradients are those of -c log q, the
    whole-target lobe loss."""
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, WIDTH))
    o[:, 3::5] = rng.uniform(-2, 5, size=(n, 13))[:, :13]
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    c = rng.uniform(0.5, 2.0, n)
    pb = rng.uniform(0.0, 1.0, n) * pb_scale
    _, d = loss_and_dout(o, wi, c, pb, whole_target=False)
    worst = 0.0
    for i in range(n):
        for j in range(5 * LOBES + 1):
            op, om = o.copy(), o.copy()
            op[i, j] += eps
            om[i, j] -= eps
            fd = (loss_and_dout(op, wi, c, pb, False)[0] - loss_and_dout(om, wi, c, pb, False)[0]) / (2 * eps)
            worst = max(worst, abs(fd - d[i, j]) / max(1e-4, abs(fd) + abs(d[i, j])))
    return worst
