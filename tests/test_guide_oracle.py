"""The guiding oracle pins its own gradient: the closed-form output gradient
of -c log q against central differences, and the FP64 backward pass (weight
and hash-table gradients) against finite differences of the FP64 loss."""
import numpy as np

from oracle import guide_oracle as go


def test_output_gradient_matches_finite_differences():
    for seed in range(3):
        assert go.finite_difference_check(seed) < 1e-4
        assert go.finite_difference_check(seed, pb_scale=0.0) < 1e-4   # the whole-target lobe loss


def _geom():
    res = np.floor(16.0 * (256.0 / 16.0) ** (np.arange(16) / 15.0)).astype(np.float32)
    dense = ((res + 1) ** 3 <= (1 << 19)).astype(np.uint32)
    return res, dense, np.zeros(3, np.float32), np.full(3, 0.1, np.float32)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(4)
    n = 8
    s = np.zeros((n, 16), np.float32)
    s[:, 0:3] = rng.uniform(0, 10, (n, 3))
    s[:, 3] = rng.uniform(0.5, 1.5, n)
    for a in (4, 8, 12):
        v = rng.normal(size=(n, 3))
        s[:, a:a + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    mlp = rng.normal(scale=0.3, size=5 * 64 * 64)
    hsh = np.zeros(16 * (1 << 19) * 2)
    geom = _geom()
    ent, _ = go.corners(*geom, s[:, 0:3])
    for l in range(16):                      # give the touched entries values
        for f in range(2):
            hsh[((l * (1 << 19) + ent[:, l, :]) * 2 + f).ravel()] = rng.uniform(-0.5, 0.5, ent[:, l, :].size)
    loss, dW, dH = go.gradients(mlp, hsh, geom, s, use_bf16=False)
    eps = 1e-6
    for idx in [(0, 3, 38), (2, 10, 5), (4, 3, 7), (4, 9, 12), (1, 0, 0)]:
        flat = np.ravel_multi_index(idx, (5, 64, 64))
        mp, mm = mlp.copy(), mlp.copy()
        mp[flat] += eps
        mm[flat] -= eps
        fd = (go.gradients(mp, hsh, geom, s, use_bf16=False)[0] - go.gradients(mm, hsh, geom, s, use_bf16=False)[0]) / (2 * eps)
        assert abs(fd - dW[idx]) <= 1e-5 + 1e-4 * abs(fd), (idx, fd, dW[idx])
    touched = np.flatnonzero(dH)
    for flat in touched[:: max(1, len(touched) // 6)][:6]:
        hp, hm = hsh.copy(), hsh.copy()
        hp[flat] += eps
        hm[flat] -= eps
        fd = (go.gradients(mlp, hp, geom, s, use_bf16=False)[0] - go.gradients(mlp, hm, geom, s, use_bf16=False)[0]) / (2 * eps)
        assert abs(fd - dH[flat]) <= 1e-5 + 1e-4 * abs(fd), (flat, fd, dH[flat])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -3.3, 65504.0], np.float32)
    assert np.array_equal(go.bf16(x), np.array([1.0, 1.0, 1.015625, -3.296875, 65536.0], np.float32))
