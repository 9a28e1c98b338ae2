"""The surrogate on the GPU: its training samples against the oracle's plain
integral, its training kernels' gradients against the FP64 CPU MLP, its
tensor-core inference against the oracle forward, training, and the 3D
vote with the plate by the network, the exact closed form and the plain
64-orientation integral."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    from tiralib_gb300 import surrogate
    return surrogate


@pytest.fixture(scope="module")
def trained(S):
    """A network trained briefly (the tests use it for its behaviour, not
    for the accuracy of a full training run)."""
    X, T = S.samples(1 << 18, seed=11)
    p = S.init_params(0)
    hist = S.train(p, X, T, batch=4096, steps=4000, lr=3e-3)
    return p, hist


def test_samples_are_the_plain_integral(S):
    X, T = S.samples(3000, seed=5)
    np.testing.assert_allclose(np.linalg.norm(X[:, :3], axis=1), 1.0, atol=1e-5)
    np.testing.assert_allclose(np.linalg.norm(X[:, 3:6], axis=1), 1.0, atol=1e-5)
    assert set(np.unique(X[:, 6])) <= {0.0, 1.0} and 0.3 < X[:, 6].mean() < 0.7
    ref = np.array([O.surrogate_target(x[:3], x[3:6], int(x[6])) for x in X[:400]])
    np.testing.assert_allclose(T[:400, :6], ref, rtol=0, atol=2e-6)
    assert np.all(T[:, 6:] == 0) and np.all(X[:, 7] == 0)
    # canonical inputs: plate n_z >= 0 and d.n >= 0; ball n = e_z and d_z >= 0
    pl = X[:, 6] == 1.0
    assert np.all(X[pl, 5] >= 0) and np.all((X[pl, :3] * X[pl, 3:6]).sum(1) >= -1e-7)
    assert np.all(X[~pl, 3:6] == np.array([0, 0, 1], np.float32)) and np.all(X[~pl, 2] >= 0)


def test_training_gradient_matches_fp64_mlp(S):
    rng = np.random.default_rng(2)
    p = S.init_params(4) + rng.normal(0, 0.02, S.param_count()).astype(np.float32)
    p[S.layout()[-1][1] + 6:] = 0.0
    X, T = S.samples(256, seed=9)
    g, loss = S.grad(p, X, T)
    # quant 2: the forward pass with the packed-BF16 GELU the GPU trains with
    loss_ref, g_ref, _ = O.mlp_loss_grad(p.astype(np.float64), X, T, quant=2)
    assert loss == pytest.approx(loss_ref, rel=1e-3)
    # FP32 accumulation and rare flips of a bf16 rounding against the FP64 oracle
    assert np.linalg.norm(g - g_ref) <= 2e-3 * np.linalg.norm(g_ref)
    for name, off, shape in S.layout():
        n = int(np.prod(shape))
        blk, ref = g[off:off + n], g_ref[off:off + n]
        assert np.linalg.norm(blk - ref) <= 5e-3 * max(np.linalg.norm(ref), 1e-8), name


def test_tensor_core_inference_matches_fp64_forward(S):
    p = S.init_params(7)
    X, T = S.samples(5000, seed=3)
    # warp-level mma.sync, FP32 GELU
    Y = S.evaluate(p, X, engine="mma", gelu="fp32")
    _, _, Yref = O.mlp_loss_grad(p.astype(np.float64), X, T, quant=1)
    err = np.abs(Y[:, :6] - Yref[:, :6])
    scale = np.abs(Yref[:, :6]).max()
    assert np.median(err) <= 2e-3 * scale and err.max() <= 3e-2 * scale
    # tcgen05 with the FP32 GELU: the same products and roundings as mma.sync;
    # only the FP32 summation order inside the tensor core may differ
    Ytc = S.evaluate(p, X, engine="tcgen05", gelu="fp32")
    assert np.abs(Ytc[:, :6] - Y[:, :6]).max() <= 1e-3 * scale
    assert np.all(Ytc[:, 6:] == 0)
    # tcgen05 with the packed-BF16 GELU against the oracle's emulation of it
    Yb = S.evaluate(p, X, engine="tcgen05", gelu="bf16")
    _, _, Yref2 = O.mlp_loss_grad(p.astype(np.float64), X, T, quant=2)
    err = np.abs(Yb[:, :6] - Yref2[:, :6])
    assert np.median(err) <= 2e-3 * scale and err.max() <= 3e-2 * scale


def test_tcgen05_inference_ragged_sizes(S):
    """Sample counts that are not multiples of the 128-row tile, and more
    tiles than CTAs (each CTA loops over tiles)."""
    p = S.init_params(5)
    for n in (1, 127, 129, 1000, 200_003):
        X, T = S.samples(n, seed=n)
        Y = S.evaluate(p, X)
        _, _, Yref = O.mlp_loss_grad(p.astype(np.float64), X[:4000], T[:4000], quant=2)
        scale = np.abs(Yref[:, :6]).max()
        err = np.abs(Y[:4000, :6] - Yref[:, :6])
        assert np.isfinite(Y).all()
        assert np.median(err) <= 2e-3 * scale and err.max() <= 3e-2 * scale, n


def test_tcgen05_wait_that_runs_out_returns_an_error(S):
    """Each layer of the tensor-core network waits for its MMAs on an
    mbarrier for a bounded number of polls.  With a bound of zero polls every
    wait runs out at once: the kernel stops at the next layer, waits for the
    MMAs still in flight with the full bound, releases its tensor memory and
    reports the timeout, so the call raises and the context stays usable.
    The next call with the default bound gives the same outputs, bit for bit,
    as the call before the failure."""
    from tiralib_gb300 import TvgbError
    p = S.init_params(3)
    X, _ = S.samples(20_000, seed=4)
    Y0 = S.evaluate(p, X)
    with pytest.raises(TvgbError, match="timed out"):
        S.evaluate(p, X, wait_limit=0)
    Y1 = S.evaluate(p, X)
    np.testing.assert_array_equal(Y0, Y1)


def test_training_reduces_the_loss(S, trained):
    p, hist = trained
    assert np.all(np.isfinite(hist))
    assert hist[-50:].mean() < 0.1 * hist[:10].mean()
    X, T = S.samples(20000, seed=77)       # held-out pairs
    Y = S.evaluate(p, X)
    rel = np.linalg.norm(Y[:, :6] - T[:, :6]) / np.linalg.norm(T[:, :6])
    print(f"held-out relative error of the briefly trained network: {rel:.3g}")
    assert rel < 0.08


def _field(seed, shape=(20, 22, 24)):
    import tiralib_gb300 as tv
    rng = np.random.default_rng(seed)
    vol = rng.normal(size=shape).astype(np.float32)
    return tv.structure_tensor3(vol, 1.0, mode="same", layout="mat3")


@pytest.mark.parametrize("ball", [False, True])
def test_closed_and_plain64_modes_are_the_exact_vote(S, ball):
    import tiralib_gb300 as tv
    F = _field(1)
    closed, _, _, _ = S.vote3(F, 2.0, mode="closed", ball=ball)
    plain, _, _, _ = S.vote3(F, 2.0, mode="plain64", ball=ball)
    ref, _, _ = tv.vote3(F, 2.0, 0.0, samples=20, ball=ball)
    u = [0, 1, 2, 4, 5, 8]
    scale = np.abs(ref.reshape(-1, 9)[:, u]).max()
    assert np.abs(closed - ref).max() <= 1e-5 * scale
    assert np.abs(plain - ref).max() <= 1e-5 * scale


def test_surrogate_vote_and_its_judge(S, trained):
    import tiralib_gb300 as tv
    p, _ = trained
    F = _field(2)
    exact, _, _, _ = S.vote3(F, 2.0, mode="closed", ball=True)
    # tol = 0: every CTA fails the judge and is voted exactly
    strict, _, _, st = S.vote3(F, 2.0, params=p, mode="surrogate", tol=0.0, ball=True)
    assert st[0] > 0 and st[1] == st[0]
    assert np.abs(strict - exact).max() <= 1e-5 * np.abs(exact).max()
    # a loose tolerance keeps the network's plate everywhere
    loose, _, _, st = S.vote3(F, 2.0, params=p, mode="surrogate", tol=1e9, ball=True)
    assert st[1] == 0
    rel = np.linalg.norm(loose - exact) / np.linalg.norm(exact)
    print(f"surrogate vote relative error (briefly trained network): {rel:.3g}")
    assert rel < 0.05
    # without the network the mode is refused
    with pytest.raises(tv.TvgbError):
        S.vote3(F, 2.0, params=None, mode="surrogate")


def _kernel_ms(fn, name):
    """Library-timed duration (ms) of the named kernel over one call of fn."""
    import ctypes
    import tiralib_gb300 as tv
    lib = tv.lib()
    buf = ctypes.create_string_buffer(1 << 14)
    lib.tvgb_profile_enable(1)
    lib.tvgb_profile_read(buf, len(buf))
    out = fn()
    lib.tvgb_profile_read(buf, len(buf))
    lib.tvgb_profile_enable(0)
    for line in buf.value.decode().splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[0] == name:
            return float(parts[2]) / int(parts[1]), out
    raise AssertionError(f"{name} was not launched")


def test_what_the_trained_network_gains(S):
    """The learned plate vote against the method it stands in for, the plain
    64-orientation integral, in the same kernel skeleton: speed of each, and
    the network's vote error against the exact vote, trained and untrained.
    On GB300 the network's 192 GELUs per pair (tanh on the MUFU pipe, 16 per
    SM clock) cost about what the plain integral's ~1600 FP32 operations per
    pair cost on the FMA pipe, so the measured speed ratio is near 1; the
    test records it and bounds it from below."""
    import torch
    dev = torch.device("cuda:0")
    X, T = S.samples(1 << 22, seed=4, device=dev)
    trained = S.init_params(0)
    S.train(trained, X, T, batch=8192, steps=20000, lr=3e-3)
    untrained = S.init_params(0)
    F = _field(3, shape=(32, 40, 48))
    exact, _, _, _ = S.vote3(F, 4.0, mode="closed")
    S.vote3(F, 4.0, mode="plain64")                                   # warm-up
    S.vote3(F, 4.0, params=trained, mode="surrogate", tol=float("inf"))
    t_plain, (plain, _, _, _) = _kernel_ms(lambda: S.vote3(F, 4.0, mode="plain64"), "k_vote3_sur_plain64")
    t_net, (net, _, _, st) = _kernel_ms(lambda: S.vote3(F, 4.0, params=trained, mode="surrogate",
                                                       tol=float("inf")), "k_vote3_surtc")
    raw, _, _, _ = S.vote3(F, 4.0, params=untrained, mode="surrogate", tol=float("inf"))
    nrm = np.linalg.norm(exact)
    e_plain = np.linalg.norm(plain - exact) / nrm
    e_net = np.linalg.norm(net - exact) / nrm
    e_raw = np.linalg.norm(raw - exact) / nrm
    print(f"plain64 {t_plain:.2f} ms (err {e_plain:.1e}), network {t_net:.2f} ms (err {e_net:.1e}, untrained "
          f"{e_raw:.1e}): speed ratio {t_plain / t_net:.2f}")
    assert st[1] == 0                       # no judge: every plate by the network
    assert e_plain < 1e-5
    assert e_net < 2e-2 and e_net < 0.1 * e_raw
    assert t_plain / t_net > 0.5
