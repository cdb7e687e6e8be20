"""CPU checks of the learned warm start's oracle (oracle/mlp.py): its gradients against finite
differences, the BF16 rounding, and the invariances of the descriptors."""
import math

import numpy as np
import pytest


def _params(rng, scale=1.0):
    return {"W1": rng.standard_normal((64, 128)) * math.sqrt(2 / 64) * scale,
            "b1": rng.standard_normal(128) * 0.1, "W2": rng.standard_normal((128, 128)) * math.sqrt(2 / 128) * scale,
            "b2": rng.standard_normal(128) * 0.1, "w3": rng.standard_normal(128) * math.sqrt(1 / 128),
            "b3": np.array([0.05])}


def test_bf16_rounding_is_nearest_even():
    from oracle.mlp import bf16
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    assert bf16(np.float32(1 + 2 ** -8)) == 1.0
    assert bf16(np.float32(1 + 3 * 2 ** -8)) == 1 + 2 ** -6
    assert bf16(np.float32(-2.5)) == -2.5
    x = np.random.default_rng(0).standard_normal(1000)
    r = bf16(x)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8 + 1e-30)


def test_oracle_gradients_match_finite_differences():
    from oracle.mlp import forward_backward
    rng = np.random.default_rng(1)
    p = _params(rng)
    x = rng.standard_normal((37, 64))
    t = rng.standard_normal(37)
    mask = np.ones(37)
    mask[-3:] = 0
    loss, g, _ = forward_backward(p, x, t, mask, rounding=False)
    eps = 1e-6
    for name, idx in (("W1", (3, 17)), ("W1", (60, 127)), ("b1", (5,)), ("W2", (0, 0)),
                      ("W2", (77, 12)), ("b2", (100,)), ("w3", (64,)), ("b3", (0,))):
        q = {k: v.copy() for k, v in p.items()}
        q[name][idx] += eps
        lp, _, _ = forward_backward(q, x, t, mask, rounding=False)
        q[name][idx] -= 2 * eps
        lm, _, _ = forward_backward(q, x, t, mask, rounding=False)
        assert g[name][idx] == pytest.approx((lp - lm) / (2 * eps), rel=1e-5, abs=1e-9), name


def test_rounded_gradients_stay_close_to_exact():
    from oracle.mlp import forward_backward
    rng = np.random.default_rng(2)
    p = _params(rng)
    x = rng.standard_normal((256, 64))
    t = rng.standard_normal(256)
    l1, g1, _ = forward_backward(p, x, t, rounding=True)
    l0, g0, _ = forward_backward(p, x, t, rounding=False)
    assert l1 == pytest.approx(l0, rel=2e-2)
    for k in g0:
        assert np.max(np.abs(g1[k] - g0[k])) <= 3e-2 * np.max(np.abs(g0[k])), k


def test_descriptors_are_rotation_and_permutation_invariant():
    from oracle.mlp import descriptors
    rng = np.random.default_rng(3)
    cell = np.array([200.0, 200.0, 200.0])  # images far away: an isolated cluster
    atoms = rng.uniform(-4, 4, (9, 3))
    pts = rng.uniform(-3, 3, (20, 3))
    d0 = descriptors(pts, atoms, cell)
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    d1 = descriptors(pts @ q.T, atoms @ q.T, cell)
    np.testing.assert_allclose(d1, d0, rtol=1e-10, atol=1e-12)
    d2 = descriptors(pts, atoms[::-1], cell)
    np.testing.assert_allclose(d2, d0, rtol=1e-12, atol=1e-14)
    assert d0.shape == (20, 64) and np.all(d0 >= 0)
    # l = 0 feature of radial n is the sum of the radial Gaussians times Y_00
    from oracle.mlp import MU, SIGMA, R_CUT
    r = np.linalg.norm(pts[0] - atoms, axis=1)
    fc = np.where(r < R_CUT, 0.5 * (np.cos(np.pi * r / R_CUT) + 1), 0.0)
    g = np.exp(-(r[:, None] - MU[None, :]) ** 2 / (2 * SIGMA ** 2)) * fc[:, None]
    np.testing.assert_allclose(d0[0, 0::4], g.sum(0) * 0.282094791773878, rtol=1e-12)


def test_periodic_descriptors_see_images():
    from oracle.mlp import descriptors
    cell = np.array([6.0, 6.0, 6.0])
    atoms = np.array([[0.0, 0.0, 0.0]])
    # the point at (2.9, 0, 0) and (-3.1, 0, 0) are the same point of the periodic cell
    d = descriptors(np.array([[2.9, 0.0, 0.0], [-3.1, 0.0, 0.0]]), atoms, cell)
    np.testing.assert_allclose(d[0], d[1], rtol=1e-12)
