"""GPU consumers of a voted 2D field against the reference's own outputs
(tests/golden/reconstruct_reference.npz: tiralib's reconstruct.py and
metrics.py run on the same fields) and the oracle: stick saliency, Otsu's
threshold, saliency thresholding with closing + hole filling, SIMF, and the
parameter sweep / differential-evolution search of optimize_tk."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g(golden):
    return golden("reconstruct_reference.npz")


@pytest.fixture(scope="module")
def tv():
    import tiralib_gb300
    return tiralib_gb300


def near_threshold(s, thr):
    return np.abs(s.astype(np.float64) - thr) <= 1e-5 * max(float(s.max()), 1e-30)


def test_stick_saliency_matches_reference(tv, g):
    from tiralib_gb300 import reconstruct as R
    H, W = g["V"].shape[:2]
    s = R.stick_saliency(g["V"].reshape(H, W, 2, 2))
    assert s.shape == (H, W) and s.dtype == np.float32
    np.testing.assert_allclose(s, g["saliency"], rtol=0, atol=2e-6 * float(g["saliency"].max()))


def test_otsu_threshold_matches_reference(tv, g):
    from tiralib_gb300 import reconstruct as R
    assert R._otsu_threshold(g["saliency"].ravel()) == pytest.approx(float(g["otsu"]), rel=1e-12, abs=0)
    assert R._otsu_threshold(np.zeros(10, np.float32)) == 0.0
    v = np.random.default_rng(0).gamma(2.0, 1.0, 100000).astype(np.float32)
    assert R._otsu_threshold(v) == pytest.approx(O.otsu_threshold(v), rel=1e-12)


@pytest.mark.parametrize("key,kw", [("mask_otsu", {}), ("mask_fill_r0", {"fill": True}),
                                    ("mask_fill_r2", {"fill": True, "close_radius": 2})])
def test_saliency_threshold_matches_reference(tv, g, key, kw):
    from tiralib_gb300 import reconstruct as R
    H, W = g["V"].shape[:2]
    V = g["V"].reshape(H, W, 2, 2)
    m = R.saliency_threshold(V, **kw)
    assert m.dtype == bool and m.shape == (H, W)
    diff = m != g[key]
    # only pixels whose saliency sits at the threshold may differ (FP32 closed form vs LAPACK)
    assert not diff.any() or near_threshold(g["saliency"], float(g["otsu"])).any()
    if not kw:
        assert not (diff & ~near_threshold(g["saliency"], float(g["otsu"]))).any()


def test_saliency_fixed_threshold(tv, g):
    from tiralib_gb300 import reconstruct as R
    H, W = g["V"].shape[:2]
    thr = float(np.median(g["saliency"]))
    m = R.saliency_threshold(g["V"].reshape(H, W, 2, 2), threshold=thr)
    assert not ((m != g["mask_fixed"]) & ~near_threshold(g["saliency"], thr)).any()


def test_fill_matches_scipy_on_random_masks(tv):
    """closing + hole filling on fields whose saliency is a chosen random mask."""
    from tiralib_gb300 import reconstruct as R
    from scipy.ndimage import binary_closing, binary_fill_holes
    rng = np.random.default_rng(5)
    for H, W, r in [(37, 51, 0), (64, 64, 1), (100, 77, 3), (130, 140, 2)]:
        mask = rng.random((H, W)) < 0.45
        F = np.zeros((H, W, 4), np.float32)
        F[..., 0] = mask.astype(np.float32)          # [[1, 0], [0, 0]]: saliency 1 where set, else 0
        got = R.saliency_threshold(F, fill=True, threshold=0.5, close_radius=r)
        b = mask
        if r:
            b = binary_closing(b, structure=np.ones((2 * r + 1, 2 * r + 1), bool))
        assert np.array_equal(got, binary_fill_holes(b)), (H, W, r)


def test_simf_matches_reference(tv, g):
    from tiralib_gb300 import metrics as M
    H, W = g["V"].shape[:2]
    G = g["G"].reshape(H, W, 2, 2)
    V = g["V"].reshape(H, W, 2, 2)
    assert M.simf(G, V) == pytest.approx(O.simf(G, V), rel=1e-5)
    assert M.simf(G, G) == pytest.approx(0.0, abs=1e-6 * float(np.abs(G).max()))
    assert M.simf(G, np.zeros_like(G)) == pytest.approx(O.simf(G, np.zeros_like(G)), rel=1e-6)


def test_sweep_matches_reference(tv, g):
    from tiralib_gb300 import optimize as OP
    H, W = g["I"].shape[:2]
    vals, fields = OP.tk_sweep(g["G"], g["I"], g["sweep_params"], return_fields=True)
    ref = g["sweep_simf"]
    assert np.all(np.abs(vals - ref) <= 1e-4 * np.maximum(np.abs(ref), 1e-3))
    # each swept field is the plain 2D vote with that candidate's window
    for k, (s1, s2, pw) in enumerate(g["sweep_params"]):
        w = OP.w_from_sigma(s1, s2)
        one = np.empty_like(g["I"])
        tv.tensorvote(one, g["I"], s1, s2, int(pw), w, H, W, True, True, 20)
        np.testing.assert_allclose(fields[k].reshape(H, W, 4), one, rtol=0, atol=1e-5 * float(np.abs(one).max()))


def test_optimize_tk_finds_the_generating_parameters(tv, g):
    """G was voted with (3, 1, 1): differential evolution over a narrow box
    must find an objective near 0, batched and not."""
    from tiralib_gb300 import optimize as OP
    bounds = [(2.0, 4.0), (0.0, 2.0), (1, 2)]
    for batched in (False, True):
        s1, s2, pw, field, fun = OP.optimize_tk(g["G"], g["I"], bounds=bounds, seed=1, batched=batched, maxiter=30,
                                                popsize=8, polish=False)
        assert fun < 0.2 * float(g["sweep_simf"][0])
        assert fun == pytest.approx(OP.tk_sweep(g["G"], g["I"], [[s1, s2, pw]])[0], rel=1e-6, abs=1e-9)
        assert field.shape == g["G"].shape[:2] + (2, 2)
