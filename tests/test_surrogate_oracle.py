"""CPU checks of the surrogate's FP64 reference (spherical harmonics, MLP gradients)."""
import math

import numpy as np

from oracle import surrogate_ref as S


def test_spher_harmon_known_values():
    """tests/kernel/test_wigner_angular_suite.m:55-60: Y00 and Y10 closed forms."""
    th = np.array([0, np.pi / 2, np.pi])
    ph = np.array([0, np.pi / 3, np.pi / 7])
    assert np.allclose(S.spher_harmon(0, 0, th, ph), np.ones(3) / math.sqrt(4 * math.pi), atol=1e-14, rtol=1e-14)
    assert np.allclose(S.spher_harmon(1, 0, th, ph), math.sqrt(3 / (4 * math.pi)) * np.cos(th), atol=1e-14)


def test_spher_harmon_condon_shortley():
    th, ph = 0.7, 1.3
    y11 = -math.sqrt(3 / (8 * math.pi)) * math.sin(th) * np.exp(1j * ph)
    y22 = 0.25 * math.sqrt(15 / (2 * math.pi)) * math.sin(th) ** 2 * np.exp(2j * ph)
    y21 = -math.sqrt(15 / (8 * math.pi)) * math.sin(th) * math.cos(th) * np.exp(1j * ph)
    assert abs(S.spher_harmon(1, 1, th, ph) - y11) < 1e-14
    assert abs(S.spher_harmon(2, 2, th, ph) - y22) < 1e-14
    assert abs(S.spher_harmon(2, 1, th, ph) - y21) < 1e-14
    # Y_{l,-m} = (-1)^m conj(Y_lm)
    assert abs(S.spher_harmon(2, -1, th, ph) + np.conj(y21)) < 1e-14


def test_features_orthonormal():
    """Real features: Re/Im of orthonormal Y_lm, so <f_i f_j> = delta_ij / 2 for m > 0."""
    lmax = 6
    nb, ng = 80, 160
    x, wx = np.polynomial.legendre.leggauss(nb)
    be, ga = np.meshgrid(np.arccos(x), 2 * np.pi * np.arange(ng) / ng, indexing='ij')
    w = np.repeat(wx, ng) * (2 * np.pi / ng)
    F = S.sh_features(be.ravel(), ga.ravel(), lmax)
    assert F.shape[1] == (lmax + 1) ** 2
    G = (F * w[:, None]).T @ F
    scale = np.ones(F.shape[1])
    f = 0
    for l in range(lmax + 1):
        f += 1
        for m in range(1, l + 1):
            scale[f:f + 2] = 0.5
            f += 2
    assert np.abs(G - np.diag(scale)).max() < 1e-12


def test_bf16_rounding():
    a = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159265, 0.0], np.float32)
    r = S.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even
    assert r[2] == 1.0 + 2 ** -7                  # tie to even (upwards)
    assert abs(r[3] + 3.140625) < 1e-12
    assert r[4] == 0.0


def test_mlp_gradient_finite_difference():
    rng = np.random.default_rng(0)
    shapes = S.layer_shapes(9, 12, 2, 5)
    npar = sum(o * i + o for o, i in shapes)
    p = rng.normal(0, 0.4, npar)
    X = rng.normal(size=(7, 9))
    T = rng.normal(size=(7, 5))
    loss, g = S.forward_backward(p, shapes, X, T, round_weights=False)
    for idx in rng.choice(npar, 25, replace=False):
        e = np.zeros(npar)
        e[idx] = 1e-6
        lp, _ = S.forward_backward(p + e, shapes, X, T, round_weights=False)
        lm, _ = S.forward_backward(p - e, shapes, X, T, round_weights=False)
        assert abs((lp - lm) / 2e-6 - g[idx]) < 1e-7 * max(1.0, abs(g[idx]))
