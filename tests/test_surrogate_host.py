"""The surrogate's CPU side: the FP64 MLP oracle's gradient against finite
differences, its training target (the plain 64-orientation integral)
against the closed-form plate and ball, and the weights file."""
import os

import numpy as np
import pytest

from oracle import oracle as O


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    P = rng.normal(size=O.mlp_param_count()) * 0.2
    X = rng.normal(size=(6, 8))
    X[:, 7] = 0.0
    T = rng.normal(size=(6, 8))
    _, g, _ = O.mlp_loss_grad(P, X, T, quant=False)
    h = 1e-6
    for i in rng.choice(len(P), 40, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (O.mlp_loss_grad(Pp, X, T, False)[0] - O.mlp_loss_grad(Pm, X, T, False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), 1e-3)


def test_oracle_forward_is_the_feature_mlp():
    """The FP64 oracle's unquantised forward pass is the MLP over the 28
    features of each sample (x, then d_i d_j and n_i n_j for i <= j, then
    d_i n_j), restated here in NumPy."""
    rng = np.random.default_rng(3)
    P = rng.normal(size=O.mlp_param_count()) * 0.3
    X = rng.normal(size=(9, 8))
    X[:, 7] = 0.0
    _, _, Y = O.mlp_loss_grad(P, X, np.zeros((9, 8)), quant=False)
    d, n = X[:, :3], X[:, 3:6]
    iu = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    F = np.concatenate([X[:, :7], np.stack([d[:, i] * d[:, j] for i, j in iu], 1),
                        np.stack([n[:, i] * n[:, j] for i, j in iu], 1),
                        np.stack([d[:, i] * n[:, j] for i in range(3) for j in range(3)], 1)], 1)
    assert F.shape == (9, 28)
    gelu = lambda z: 0.5 * z * (1.0 + np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))
    o = 0
    W1 = P[o:o + 64 * 28].reshape(64, 28); o += 64 * 28
    b1 = P[o:o + 64]; o += 64
    W2 = P[o:o + 64 * 64].reshape(64, 64); o += 64 * 64
    b2 = P[o:o + 64]; o += 64
    W3 = P[o:o + 64 * 64].reshape(64, 64); o += 64 * 64
    b3 = P[o:o + 64]; o += 64
    W4 = P[o:o + 8 * 64].reshape(8, 64); o += 8 * 64
    b4 = P[o:o + 8]
    h = gelu(F @ W1.T + b1)
    h = gelu(h @ W2.T + b2)
    h = gelu(h @ W3.T + b3)
    ref = h @ W4.T + b4
    np.testing.assert_allclose(Y, ref, rtol=1e-12, atol=1e-12)


def test_target_is_the_exact_plate_and_ball():
    """64 orientations integrate the degree-4 integrand exactly: the target
    equals the closed forms (sigma2 = 0, Gaussian factored out)."""
    rng = np.random.default_rng(1)
    iu = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for _ in range(20):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        R = np.eye(3) - 2 * np.outer(d, d)
        m, p = R @ n, (np.eye(3) - np.outer(n, n)) @ d
        plate = (0.5 - p @ p / 8) * (np.eye(3) - np.outer(m, m)) - 0.25 * np.outer(R @ p, R @ p)
        ball = (1 / 3 - 1 / 15) * np.eye(3) - (2 / 15) * np.outer(d, d)
        np.testing.assert_allclose(O.surrogate_target(d, n, 1), [plate[i, j] for i, j in iu], atol=1e-14)
        np.testing.assert_allclose(O.surrogate_target(d, n, 0), [ball[i, j] for i, j in iu], atol=1e-14)


def test_weights_file_roundtrip_and_checksum(tmp_path):
    from tiralib_gb300 import surrogate as S
    p = S.init_params(3)
    assert p.size == S.param_count() == O.mlp_param_count() == 64 * 28 + 64 + 2 * (64 * 64 + 64) + 8 * 64 + 8
    W4 = p[64 * 28 + 64 + 2 * (64 * 64 + 64):][:512].reshape(8, 64)
    assert np.all(W4[6:] == 0) and np.any(W4[:6] != 0)
    f = os.path.join(tmp_path, "net.bin")
    S.save(f, p, "sigma2 = 0, power 1")
    q, note = S.load(f)
    assert np.array_equal(p, q) and note == "sigma2 = 0, power 1"
    blob = bytearray(open(f, "rb").read())
    blob[-5] ^= 0x40
    open(f, "wb").write(bytes(blob))
    with pytest.raises(ValueError, match="checksum"):
        S.load(f)
