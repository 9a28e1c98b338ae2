"""GPU parity of the 2D vote through the drop-in modules that mirror the
reference's pybind11 extensions (tensorvote_tk / tensorvote_atv) and its
cuda_wrappers.py, against the reference NumPy implementation and the
reference C++ CPU path (tests/golden)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module")
def mods():
    from tiralib_gb300 import cuda_wrappers, tensorvote_atv, tensorvote_tk
    return tensorvote_tk, tensorvote_atv, cuda_wrappers


@pytest.mark.parametrize("field", ["stick", "ball", "mixed"])
@pytest.mark.parametrize("s1,s2,p,N", [(5.0, 0.0, 1, 20), (5.0, 2.0, 1, 20), (5.0, 2.0, 3, 20), (3.0, 1.0, 1, 0)])
def test_tk_matches_numpy_reference(mods, golden, field, s1, s2, p, N):
    """python/tira/tests/test_cpu_gpu.py:132: max|d| / max|cpu| < 1e-4."""
    tk, _, cw = mods
    g = golden("tv2_numpy_reference.npz")
    flat = g[f"in_{field}"]
    out = cw.tk_vote2_cuda(flat.reshape(24, 24, 2, 2).astype(np.float64), s1, s2, p, True, N)
    assert rel(out.reshape(24, 24, 4), g[f"tk_{field}_{s1}_{s2}_{p}_{N}"]) < 1e-4
    # prebuilt-table path equals the standard path (test_cpu_gpu.py:129)
    w = cw._w_from_sigma(s1, s2)
    nb = cw._build_nb_numpy(s1, s2, p, N if N > 0 else 10, w)
    pre = cw.tk_vote2_cuda_prebuilt_flat(flat, nb, s1, s2, p, True, N if N > 0 else 10)
    assert np.abs(pre - out).max() < 1e-5
    assert np.abs(out[..., 0, 1] - out[..., 1, 0]).max() < 1e-5


@pytest.mark.parametrize("field", ["stick", "ball", "mixed"])
def test_atv_matches_numpy_reference(mods, golden, field):
    _, _, cw = mods
    g = golden("tv2_numpy_reference.npz")
    out = cw.atv_vote2_cuda(g[f"in_{field}"].reshape(24, 24, 2, 2).astype(np.float64), 3.0)
    assert rel(out.reshape(24, 24, 4), g[f"atv_{field}_3.0"]) < 1e-4


CPP_CASES = {
    "tk_s2_p1_n10": dict(sigma1=2.0, sigma2=0.0, power=1, w=13, samples=10),
    "tk_s2_p2_n20_sig2": dict(sigma1=2.0, sigma2=1.0, power=2, w=13, samples=20),
    "tk_stick_only": dict(sigma1=1.5, sigma2=0.0, power=1, w=9, samples=10, plate=False),
    "tk_plate_only": dict(sigma1=1.5, sigma2=0.0, power=1, w=9, samples=10, stick=False),
}


@pytest.mark.parametrize("case", sorted(CPP_CASES))
def test_tk_matches_reference_cpp(mods, golden, case):
    tk, _, _ = mods
    g = golden("tv2_cpp_reference.npz")
    kw = CPP_CASES[case]
    out = tk.tensorvote_tk(g["in"], kw["sigma1"], kw["sigma2"], kw["power"], kw["w"], kw.get("stick", True),
                           kw.get("plate", True), kw["samples"])
    assert rel(out, g[case]) < 1e-4


def test_atv_matches_reference_cpp(mods, golden):
    _, atv, _ = mods
    g = golden("tv2_cpp_reference.npz")
    out = atv.tensorvote_atv(g["in"], 2.0, 13)
    assert rel(out, g["atv_s2"]) < 1e-4


def test_tk_ragged_sizes_against_oracle(mods):
    tk, _, _ = mods
    rng = np.random.default_rng(4)
    for H, W in [(1, 50), (37, 3), (70, 45)]:
        A = rng.normal(size=(H, W, 2, 2)).astype(np.float32)
        F = (A @ np.swapaxes(A, -1, -2)).reshape(H, W, 4).astype(np.float32)
        out = tk.tensorvote_tk(F, 3.0, 0.5, 2, 0, True, True, 20)
        ref = O.tensorvote2(F, 3.0, 0.5, 2, 19, samples=20)
        assert rel(out, ref) < 1e-4


def test_tk_large_images_against_oracle(mods):
    """The staged kernel on images of many CTAs (640 x 800 at power 2,
    1024 x 960 at power 1), against the oracle."""
    tk, _, _ = mods
    rng = np.random.default_rng(7)
    for (H, W), p in [((800, 640), 2), ((960, 1024), 1)]:
        A = rng.normal(size=(H, W, 2, 2)).astype(np.float32)
        F = (A @ np.swapaxes(A, -1, -2)).reshape(H, W, 4).astype(np.float32)
        out = tk.tensorvote_tk(F, 3.0, 0.0, p, 0, True, True, 20)
        ref = O.tensorvote2(F, 3.0, 0.0, p, 19, samples=20)
        assert rel(out, ref) < 1e-4, (H, W, p)
