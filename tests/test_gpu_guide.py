"""Learned path guiding on the tensor cores.

* tcgen05 operand layouts: a 128x64x64 K-major MMA and a 64x64x128 MN-major
  MMA (the weight-gradient shape) against FP32 products of the same BF16
  values.
* The network's inference (mixture densities) and its gradients (loss,
  weight and hash-table gradients) against the CPU oracle, which rounds to
  BF16 where the kernels do; tolerances are relative.
* Online training on a synthetic directional target.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(rng, shape):
    x = rng.standard_normal(shape).astype(np.float32)
    bits = (x.view(np.uint32) + 0x8000) >> 16          # round to nearest (ties away)
    return bits.astype(np.uint16), (bits.astype(np.uint32) << 16).view(np.float32)


def test_tcgen05_operand_layouts(cuda_dev):
    import torch

    import optix_pt_gb300 as opt
    rng = np.random.default_rng(3)
    (A, a), (B, b), (G, g), (X, x) = (_bf16(rng, s) for s in ((128, 64), (64, 64), (128, 64), (128, 64)))
    dev = [torch.from_numpy(v.view(np.int16)).to(cuda_dev) for v in (A, B, G, X)]
    c = torch.zeros((128, 64), dtype=torch.float32, device=cuda_dev)
    dw = torch.zeros((128, 64), dtype=torch.float32, device=cuda_dev)
    st = torch.zeros(1, dtype=torch.int32, device=cuda_dev)
    opt.check(opt.lib.optpt_tc_selftest(*[d.data_ptr() for d in dev], c.data_ptr(), dw.data_ptr(), st.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st.item() == 0
    c, dw = c.cpu().numpy(), dw.cpu().numpy()
    ref_c = a.astype(np.float64) @ b.astype(np.float64).T
    ref_dw = g.astype(np.float64).T @ x.astype(np.float64)
    print("C max err", np.abs(c - ref_c).max())
    # where do the 64 rows of the M = 64 result sit among the 128 TMEM lanes?
    lanes = {}
    for r in range(64):
        d = np.abs(dw - ref_dw[r][None, :]).max(1)
        lanes[r] = int(d.argmin()) if d.min() < 1e-3 * (1 + np.abs(ref_dw[r]).max()) else -1
    print("M=64 row -> lane:", lanes)
    assert np.allclose(c, ref_c, rtol=1e-5, atol=1e-4)
    # M = 64: rows 16q .. 16q + 15 in lanes 32q .. 32q + 15 of each lane quarter
    assert lanes == {r: (r // 16) * 32 + r % 16 for r in range(64)}, lanes
    for r in range(64):
        np.testing.assert_allclose(dw[(r // 16) * 32 + r % 16], ref_dw[r], rtol=1e-5, atol=1e-4)


# ------------------------------------------------------------------ network vs oracle
LO, HI = (-5.0, 0.0, -3.0), (5.0, 4.0, 3.0)


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _queries(rng, n):
    q = np.zeros((n, 12), np.float32)
    q[:, 0:3] = rng.uniform(LO, HI, (n, 3))
    q[:, 4:7] = _unit(rng, n)
    q[:, 8:11] = _unit(rng, n)
    return q


def _samples(rng, n):
    s = np.zeros((n, 16), np.float32)
    s[:, 0:3] = rng.uniform(LO, HI, (n, 3))
    s[:, 3] = rng.exponential(1.0, n)
    s[:, 4:7] = _unit(rng, n)
    s[:, 8:11] = _unit(rng, n)
    s[:, 11] = rng.uniform(0.0, 1.0, n)   # BSDF lobe density at wi
    s[:, 12:15] = _unit(rng, n)
    s[::17, 3] = 0.0          # zero-weight samples contribute nothing
    s[5, 3] = np.nan          # non-finite weights are ignored
    return s


def _guide_with_features(seed):
    import optix_pt_gb300 as opt
    g = opt.Guide(LO, HI, seed=seed)
    mlp, hsh = g.params()
    rng = np.random.default_rng(seed)
    hsh = rng.uniform(-0.5, 0.5, hsh.shape).astype(np.float32)   # features large enough to matter
    g.set_params(hash_params=hsh)
    return g, mlp, hsh


def test_guide_inference_matches_oracle(cuda_dev):
    import torch

    from oracle import guide_oracle as go
    g, mlp, hsh = _guide_with_features(11)
    rng = np.random.default_rng(12)
    n = 1000                                            # 7 full tiles + a ragged one
    q = _queries(rng, n)
    qd = torch.from_numpy(q).to(cuda_dev)
    out = torch.zeros((n, 48), dtype=torch.float16, device=cuda_dev)
    g.infer(qd.data_ptr(), n, out.data_ptr(), torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert g.status()[0] == 0
    w, mu, kap = go.unpack(out.cpu().numpy())
    o = go.infer(mlp, hsh, g.geometry(), q)
    wr, mur, kapr, *_ = go.decode(o)
    dirs = _unit(rng, n)
    p_gpu = (w * go.vmf_pdf(mu, kap, dirs)[0]).sum(1)
    p_ref = (wr * go.vmf_pdf(mur, kapr, dirs)[0]).sum(1)
    rel = np.abs(p_gpu - p_ref) / p_ref
    print("mixture pdf rel err: median %.2e p99 %.2e max %.2e" % (np.median(rel), np.quantile(rel, 0.99), rel.max()))
    assert np.median(rel) <= 1e-4 and np.quantile(rel, 0.99) <= 5e-4
    assert np.abs(w - wr).max() < 1e-2
    assert np.abs(go.unpack_select(out.cpu().numpy()) - go.select_prob(o)).max() < 2e-3
    g.close()


def test_guide_gradients_match_oracle(cuda_dev):
    import torch

    from oracle import guide_oracle as go
    g, mlp, hsh = _guide_with_features(21)
    rng = np.random.default_rng(22)
    n = 1000
    s = _samples(rng, n)
    sd = torch.from_numpy(s).to(cuda_dev)
    cnt = torch.tensor([n], dtype=torch.int32, device=cuda_dev)
    loss, dm, dh = g.gradients(sd.data_ptr(), cnt.data_ptr(), n, torch.cuda.current_stream())
    rloss, rdm, rdh = go.gradients(mlp, hsh, g.geometry(), s)
    print("loss gpu %.6f oracle %.6f" % (loss, rloss))
    assert abs(loss - rloss) <= 1e-3 * abs(rloss)
    dm = dm.reshape(5, 64, 64)
    for l in range(5):
        err = np.linalg.norm(dm[l] - rdm[l]) / np.linalg.norm(rdm[l])
        print("layer %d dW rel err %.2e" % (l, err))
        assert err <= 2e-4, (l, err)
    touched = rdh != 0
    err = np.linalg.norm(dh[touched] - rdh[touched]) / np.linalg.norm(rdh[touched])
    print("hash grad rel err %.2e over %d entries; untouched max %.1e" % (err, touched.sum(), np.abs(dh[~touched]).max()))
    assert err <= 2e-4
    assert np.abs(dh[~touched]).max() == 0.0
    g.close()


def test_guide_training_learns_a_directional_target(cuda_dev):
    """Online training on samples whose weight is a position-dependent lobe
    (towards a fixed point): the learned mixture's density along the target
    direction rises far above the untrained network's."""
    import torch

    import optix_pt_gb300 as opt
    from oracle import guide_oracle as go
    g = opt.Guide(LO, HI, seed=5)
    rng = np.random.default_rng(6)
    target = np.array([4.0, 3.5, 0.0])

    def batch(n):
        s = np.zeros((n, 16), np.float32)
        pos = rng.uniform(LO, HI, (n, 3))
        d = target - pos
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        wi = _unit(rng, n)
        kappa = 20.0
        lobe = kappa / (2 * np.pi * (1 - np.exp(-2 * kappa))) * np.exp(kappa * ((wi * d).sum(1) - 1))
        s[:, 0:3] = pos
        s[:, 3] = lobe * 4 * np.pi            # target / uniform sampling pdf
        s[:, 4:7] = _unit(rng, n)
        s[:, 8:11] = _unit(rng, n)
        s[:, 11] = 1 / (4 * np.pi)           # a uniform "BSDF" to mix with
        s[:, 12:15] = wi
        return s

    def score():
        n = 4096
        q = np.zeros((n, 12), np.float32)
        q[:, 0:3] = rng.uniform(LO, HI, (n, 3))
        q[:, 4:7] = _unit(rng, n)
        q[:, 8:11] = _unit(rng, n)
        d = target - q[:, 0:3]
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        out = torch.zeros((n, 48), dtype=torch.float16, device=cuda_dev)
        g.infer(torch.from_numpy(q).to(cuda_dev).data_ptr(), n, out.data_ptr(), torch.cuda.current_stream())
        torch.cuda.synchronize()
        w, mu, kap = go.unpack(out.cpu().numpy())
        return float(np.mean(np.log((w * go.vmf_pdf(mu, kap, d)[0]).sum(1))))

    before = score()
    n = 1 << 14
    cnt = torch.tensor([n], dtype=torch.int32, device=cuda_dev)
    for _ in range(300):
        sd = torch.from_numpy(batch(n)).to(cuda_dev)
        g.train_step(sd.data_ptr(), cnt.data_ptr(), n, torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert g.status()[0] == 0
    after = score()
    print("mean log proposal density along the target direction: before %.3f after %.3f (uniform %.3f)" % (
        before, after, np.log(1 / (4 * np.pi))))
    assert after > before + 2.0
    assert after > np.log(20 / (2 * np.pi)) - 1.5   # near the target lobe's own peak density (log 1.16)
    g.close()


def _packed(mu, kap, w, select=0.5):
    """Rows of packed mixtures (n, 48) float16 from per-row lobes."""
    n = mu.shape[0]
    lobes = np.zeros((n, 8, 4))
    lobes[:, :, :3] = mu
    lobes[:, :, 3] = kap
    h = np.zeros((n, 48), np.float16)
    h[:, :32] = lobes.reshape(n, 32)
    h[:, 32:40] = w
    h[:, 40] = select
    return h


def test_mixture_sampler_matches_its_density(cuda_dev):
    """The shading kernel's mixture sampler and density (the same device
    functions, through optpt_guide_mixture_eval): the density equals the FP64
    vMF mixture of the decoded halves; the sampled directions follow it
    (per-lobe Kolmogorov-Smirnov test of mu . d against the vMF's own CDF,
    uniform azimuth, and lobe-selection frequencies equal to the weights).
    A guided vertex's one-sample MIS weight is unbiased only if the density
    it evaluates is the one its sampler draws from."""
    import torch

    import optix_pt_gb300 as opt
    from oracle import guide_oracle as go
    rng = np.random.default_rng(21)
    n = 4096
    mu = _unit(rng, n * 8).reshape(n, 8, 3) * rng.uniform(0.5, 2.0, (n, 8, 1))
    kap = np.exp(rng.uniform(-3.0, 5.5, (n, 8)))
    w = rng.uniform(0.0, 1.0, (n, 8))
    h = _packed(mu, kap, w)
    mix = torch.from_numpy(h.view(np.int16)).to(cuda_dev)
    wd, mud, kapd = go.unpack(h)
    dirs = _unit(rng, n)
    dp = torch.from_numpy(np.concatenate([dirs, np.zeros((n, 1))], 1).astype(np.float32)).to(cuda_dev)
    opt.Guide.mixture_eval(mix.data_ptr(), n, None, dp.data_ptr(), torch.cuda.current_stream())
    xi = torch.from_numpy(rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)).to(cuda_dev)
    ds = torch.zeros((n, 4), dtype=torch.float32, device=cuda_dev)
    opt.Guide.mixture_eval(mix.data_ptr(), n, xi.data_ptr(), ds.data_ptr(), torch.cuda.current_stream())
    torch.cuda.synchronize()
    for d, got in ((dirs, dp.cpu().numpy()[:, 3]), (ds.cpu().numpy()[:, :3].astype(np.float64), ds.cpu().numpy()[:, 3])):
        ref = (wd * go.vmf_pdf(mud, kapd, d)[0]).sum(1)
        ok = ref > 1e-30
        rel = np.abs(got[ok] - ref[ok]) / ref[ok]
        print("mixture density rel err: median %.2e max %.2e" % (np.median(rel), rel.max()))
        assert np.median(rel) < 2e-6 and rel.max() < 1e-4
    assert np.abs(np.linalg.norm(ds.cpu().numpy()[:, :3], axis=1) - 1).max() < 1e-5

    # one-lobe mixtures: mu . d against F(t) = (exp(k (t - 1)) - exp(-2 k)) / (1 - exp(-2 k))
    R = 1 << 16
    for k in (0.05, 1.0, 10.0, 200.0):
        m = _unit(rng, 1)
        mu1 = np.zeros((R, 8, 3))
        mu1[:, 0] = m
        mu1[:, 1:, 2] = 1.0
        w1 = np.zeros((R, 8))
        w1[:, 0] = 1.0
        h1 = _packed(mu1, np.full((R, 8), k), w1)
        kd = float(h1[0, 3])
        mix1 = torch.from_numpy(h1.view(np.int16)).to(cuda_dev)
        xi1 = torch.from_numpy(rng.uniform(0.0, 1.0, (R, 3)).astype(np.float32)).to(cuda_dev)
        out = torch.zeros((R, 4), dtype=torch.float32, device=cuda_dev)
        opt.Guide.mixture_eval(mix1.data_ptr(), R, xi1.data_ptr(), out.data_ptr(), torch.cuda.current_stream())
        torch.cuda.synchronize()
        d = out.cpu().numpy()[:, :3].astype(np.float64)
        mh = go.unpack(h1[:1])[1][0, 0]
        t = np.clip(d @ mh, -1.0, 1.0)
        ts = np.sort(t)
        cdf = (np.exp(kd * (ts - 1)) - np.exp(-2 * kd)) / -np.expm1(-2 * kd)
        ks = max(np.abs(cdf - np.arange(1, R + 1) / R).max(), np.abs(cdf - np.arange(R) / R).max())
        # azimuth about mu: uniform
        a = np.cross(mh, [0.0, 0.0, 1.0] if abs(mh[2]) < 0.9 else [1.0, 0.0, 0.0])
        a /= np.linalg.norm(a)
        b = np.cross(mh, a)
        phi = np.sort((np.arctan2(d @ b, d @ a) + np.pi) / (2 * np.pi))
        ks_phi = np.abs(phi - (np.arange(R) + 0.5) / R).max()
        print("kappa %g: KS(mu.d) %.4f, KS(azimuth) %.4f" % (kd, ks, ks_phi))
        assert ks < 1.95 / np.sqrt(R) and ks_phi < 1.95 / np.sqrt(R), (kd, ks, ks_phi)

    # lobe selection: eight peaked, well separated lobes; the nearest lobe of
    # each draw is the one selected
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0.577, 0.577, 0.577], [-0.577, -0.577, 0.577]])
    wsel = rng.uniform(0.2, 1.0, 8)
    h2 = _packed(np.broadcast_to(axes, (R, 8, 3)), np.full((R, 8), 200.0), np.broadcast_to(wsel, (R, 8)))
    mix2 = torch.from_numpy(h2.view(np.int16)).to(cuda_dev)
    xi2 = torch.from_numpy(rng.uniform(0.0, 1.0, (R, 3)).astype(np.float32)).to(cuda_dev)
    out = torch.zeros((R, 4), dtype=torch.float32, device=cuda_dev)
    opt.Guide.mixture_eval(mix2.data_ptr(), R, xi2.data_ptr(), out.data_ptr(), torch.cuda.current_stream())
    torch.cuda.synchronize()
    wd2, mud2, _ = go.unpack(h2[:1])
    lobe = np.argmax(out.cpu().numpy()[:, :3].astype(np.float64) @ mud2[0].T, axis=1)
    counts = np.bincount(lobe, minlength=8)
    expect = wd2[0] * R
    chi2 = float(((counts - expect) ** 2 / expect).sum())
    print("lobe selection chi2 %.2f (7 dof)" % chi2)
    assert chi2 < 24.3   # p = 0.001 for 7 degrees of freedom
