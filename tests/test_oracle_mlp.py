"""The CPU restatement of the surrogate network checks itself (no GPU).

Its analytic gradient against central finite differences, the bfloat16 rounding against
known values, and the pose features against their definitions.
"""
import numpy as np

from oracle import mlp


def random_params(rng, scale=1.0):
    p = np.zeros(mlp.N_PARAMS)
    for k, (o, n) in mlp.OFF.items():
        fan = mlp.N_IN if k in ("W1", "b1") else mlp.H
        p[o:o + n] = rng.uniform(-1, 1, n) * scale / np.sqrt(fan)
    return p


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = random_params(rng)
    X = rng.normal(size=(6, mlp.N_IN))
    y = rng.normal(size=6)
    _, g = mlp.loss_grad(p, X, y)
    idx = np.concatenate([rng.choice(n, 4, replace=False) + o for o, n in mlp.OFF.values() if n > 1] +
                         [np.array([mlp.OFF["b5"][0]])])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        num = (mlp.loss_grad(pp, X, y)[0] - mlp.loss_grad(pm, X, y)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 * max(1.0, abs(num)), (i, num, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.140625, 1e-3], np.float32)
    r = mlp.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even
    assert r[2] == 1.0 + 2 ** -7            # above the tie -> up
    assert r[3] == -2.5 and r[4] == 3.140625
    assert abs(r[5] - 1e-3) <= 2 ** -8 * 1e-3


def test_features_definition():
    rng = np.random.default_rng(5)
    q = rng.normal(size=(3, 3)) * 5
    Fa = mlp.frame(*q)
    assert np.allclose(Fa @ Fa.T, np.eye(3), atol=1e-12) and np.linalg.det(Fa) > 0
    # rotate the same points: the relative quaternion is that rotation expressed in a's frame
    ang = 0.7
    ax = np.array([1.0, 2.0, -0.5])
    ax /= np.linalg.norm(ax)
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    Rm = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
    Fb = mlp.frame(*(q @ Rm.T))
    x = mlp.features(Fa, [1.0, 2.0, 3.0], Fb, [11.0, 2.0, 3.0], 100.0)
    assert np.allclose(x[:3] / mlp.POS_SCALE, Fa @ np.array([10.0, 0, 0]))
    assert np.isclose(x[3], mlp.INV_SCALE / 10.0)
    w = x[4]
    assert np.isclose(np.linalg.norm(x[4:]), 1.0) and w >= 0
    assert np.isclose(2 * np.arccos(min(1.0, w)), ang, atol=1e-9)
    # minimum image
    x2 = mlp.features(Fa, [1.0, 2.0, 3.0], Fb, [99.0, 2.0, 3.0], 100.0)
    assert np.isclose(x2[3], mlp.INV_SCALE / 2.0)
