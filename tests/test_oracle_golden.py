"""Pin the CPU oracle (oracle/tvoracle_*.c) to the reference's own outputs.

The fixtures in tests/golden/ come from tiralib's C++ CPU functions compiled
from the reference sources and from its NumPy 2D implementation
(tests/golden/make_golden.py).  Everything here runs on the CPU.
"""
import numpy as np
import pytest

from oracle import oracle as O

UNIQUE9 = [0, 1, 2, 4, 5, 8]   # the entries eigen.h reads back from a glm::mat3


def rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.lib()


TV3_CASES = {
    "tk_s15_n20": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=20),
    "tk_s15_n3": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=3),
    "tk_s15_n2": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=2),
    "tk_s2_p2_n20_sig2": dict(sigma1=2.0, sigma2=1.0, w=7, power=2, samples=20),
    "tk_analytic": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=0),
    "tk_stick_only": dict(sigma1=2.0, sigma2=0.0, w=7, power=1, samples=20, plate=False),
    "tk_plate_only": dict(sigma1=2.0, sigma2=0.0, w=7, power=1, samples=20, stick=False),
    "atv_s15": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=20, is_atv=True),
}


@pytest.mark.parametrize("case", sorted(TV3_CASES))
def test_tensorvote3_matches_reference_cpu(golden, case):
    g = golden("tv3_cpp_reference.npz")
    T = g["in"].reshape(8, 9, 10, 3, 3)
    out = O.tensorvote3(T, **TV3_CASES[case]).reshape(-1, 9)[:, UNIQUE9]
    ref = g[case].reshape(-1, 9)[:, UNIQUE9]
    assert rel(out, ref) < 1e-5


def test_tensorvote3_output_symmetric():
    rng = np.random.default_rng(0)
    A = rng.normal(size=(5, 5, 5, 3, 3)).astype(np.float32)
    T = (A @ np.swapaxes(A, -1, -2)).astype(np.float32)
    out = O.tensorvote3(T, 1.0, 0.0, 5, 1, samples=20)
    assert np.array_equal(out, np.swapaxes(out, -1, -2))


def test_plate_riemann_rule_exact_for_three_or_more_samples(golden):
    """power=1: the plate integrand is a trig polynomial of degree 4 in the
    orientation angle, so every S >= 3 rule gives the same value (S=2 does not)."""
    g = golden("tv3_cpp_reference.npz")
    a, b, c = (g[k].reshape(-1, 9) for k in ("tk_s15_n20", "tk_s15_n3", "tk_s15_n2"))
    assert rel(b, a) < 1e-5
    assert rel(c, a) > 1e-3


TV2_CASES = {
    "tk_s2_p1_n10": dict(sigma1=2.0, sigma2=0.0, power=1, w=13, samples=10),
    "tk_s2_p2_n20_sig2": dict(sigma1=2.0, sigma2=1.0, power=2, w=13, samples=20),
    "tk_stick_only": dict(sigma1=1.5, sigma2=0.0, power=1, w=9, samples=10, plate=False),
    "tk_plate_only": dict(sigma1=1.5, sigma2=0.0, power=1, w=9, samples=10, stick=False),
    "atv_s2": dict(sigma1=2.0, sigma2=0.0, power=1, w=13, samples=10, is_atv=True),
}


@pytest.mark.parametrize("case", sorted(TV2_CASES))
def test_tensorvote2_matches_reference_cpu(golden, case):
    g = golden("tv2_cpp_reference.npz")
    out = O.tensorvote2(g["in"], **TV2_CASES[case])
    assert rel(out, g[case]) < 1e-5


def test_neighbors2d_table_matches_reference(golden):
    g = golden("tv2_cpp_reference.npz")
    nb = O.build_neighbors2d(7, 2.0, 0.5, 2, 10)
    ref = g["nb_w7"]
    assert nb.dtype.itemsize == 48
    for f in nb.dtype.names:
        np.testing.assert_allclose(nb[f], ref[f], rtol=0, atol=1e-6)


@pytest.mark.parametrize("field", ["stick", "ball", "mixed"])
@pytest.mark.parametrize("s1,s2,p,N", [(5.0, 0.0, 1, 20), (5.0, 2.0, 1, 20), (5.0, 2.0, 3, 20), (3.0, 1.0, 1, 0)])
def test_tensorvote2_matches_numpy_reference(golden, field, s1, s2, p, N):
    """The reference's own bar between its NumPy and CUDA 2D paths:
    max|d| / max|ref| < 1e-4 (python/tira/tests/test_cpu_gpu.py:132).  N=0 is
    the NumPy closed-form plate; the sampled rule with 10 samples is exact for
    power 1."""
    g = golden("tv2_numpy_reference.npz")
    w = 2 * int(3 * max(s1, s2)) + 1
    out = O.tensorvote2(g[f"in_{field}"], s1, s2, p, w, samples=N if N > 0 else 10)
    assert rel(out, g[f"tk_{field}_{s1}_{s2}_{p}_{N}"]) < 1e-4


@pytest.mark.parametrize("field", ["stick", "ball", "mixed"])
def test_atv2_matches_numpy_reference(golden, field):
    g = golden("tv2_numpy_reference.npz")
    out = O.tensorvote2(g[f"in_{field}"], 3.0, 0.0, 1, 19, is_atv=True)
    assert rel(out, g[f"atv_{field}_3.0"]) < 1e-4


def test_eigen3_matches_reference(golden):
    g = golden("eigen_cpp_reference.npz")
    m9 = g["m9"]
    ev = O.evals3(m9)
    scale = np.maximum(np.abs(g["evals3"]).max(axis=1, keepdims=True), 1e-30)
    assert (np.abs(ev - g["evals3"]) / scale).max() < 1e-5
    vec = O.evecs3cart(m9, g["evals3"])
    ref = g["evecs3cart"]
    # eigenvectors up to sign
    dots = np.abs(np.einsum("nij,nij->ni", vec, ref))
    assert (1.0 - dots).max() < 1e-5
    sph = O.evecs3spherical(m9, g["evals3"])
    assert np.abs(sph - g["evecs3sph"]).max() < 1e-4


def test_eigen2_matches_reference(golden):
    g = golden("eigen_cpp_reference.npz")
    ev = O.evals2(g["m4"])
    scale = np.maximum(np.abs(g["evals2"]).max(axis=1, keepdims=True), 1.0)
    assert (np.abs(ev - g["evals2"]) / scale).max() < 1e-5
    th = O.evecs2polar(g["m4"], g["evals2"])
    assert np.abs(th - g["evecs2"]).max() < 1e-5


def test_eigen3_fp64_jacobi_reconstructs():
    rng = np.random.default_rng(4)
    A = rng.normal(size=(200, 3, 3))
    M = A @ np.swapaxes(A, 1, 2)
    s6 = M.reshape(-1, 9)[:, UNIQUE9]
    ev, vec = O.eig3_f64(s6)
    R = np.einsum("nki,nk,nkj->nij", vec, ev, vec)
    assert np.abs(R - M).max() < 1e-12 * np.abs(M).max() * 100
    assert np.all(np.diff(ev, axis=1) >= 0)


def test_filters_match_reference(golden):
    g = golden("filter_cpp_reference.npz")
    for k in g.files:
        if k.startswith("g1d_"):
            _, s, K = k.split("_")
            np.testing.assert_allclose(O.gaussian1d(int(K), float(s)), g[k], rtol=1e-6, atol=1e-8)
    out = O.gaussian_convolve3(g["vol"], 1.5, 1.0, 2.0)
    assert out.shape == g["conv3_15_10_20"].shape
    assert rel(out, g["conv3_15_10_20"]) < 1e-6
    out = O.gaussian_convolve2(g["img"], 1.0)
    assert out.shape == g["conv2_1"].shape
    assert rel(out, g["conv2_1"]) < 1e-6


def test_gradient_is_volume_gradient_rule():
    """volume<T>::gradient (tira/volume.h:974): central difference inside,
    one-sided at the faces, unit spacing -- numpy's edge_order=1 rule."""
    rng = np.random.default_rng(5)
    v = rng.normal(size=(6, 7, 8)).astype(np.float32)
    for axis, np_axis in ((0, 2), (1, 1), (2, 0)):
        np.testing.assert_allclose(O.gradient3(v, axis), np.gradient(v.astype(np.float64), axis=np_axis),
                                   rtol=1e-6, atol=1e-6)


def test_structure_tensor3_valid_matches_reference_blur():
    """structure tensor = gradient outer product, blurred per component with
    gaussian_convolve3 (valid): assemble it from the pinned pieces."""
    rng = np.random.default_rng(6)
    v = rng.normal(size=(14, 15, 16)).astype(np.float32)
    st = O.structure_tensor3(v, 1.5, 0)
    g = [O.gradient3(v, a) for a in range(3)]
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for c, (a, b) in enumerate(pairs):
        ref = O.gaussian_convolve3(g[a] * g[b], 1.5, 1.5, 1.5)
        assert st[c].shape == ref.shape
        assert rel(st[c], ref) < 1e-6
    same = O.structure_tensor3(v, 1.5, 1)
    assert same.shape == (6, 14, 15, 16)
    R = O.lib().or_ksize3(1.5) // 2
    assert rel(same[:, R:-R, R:-R, R:-R], st) < 1e-6


def test_fp64_oracle_close_to_fp32_reference(golden):
    """The FP64 precision oracle and the FP32 reference restatement agree to
    FP32 rounding on well-conditioned random tensors."""
    g = golden("tv3_cpp_reference.npz")
    T = g["in"].reshape(8, 9, 10, 3, 3)
    f64 = O.tensorvote3_f64(T, 1.5, 0.0, 5, 1).reshape(-1, 6)
    ref = g["tk_s15_n20"].reshape(-1, 9)[:, UNIQUE9]
    assert rel(ref, f64) < 1e-4


def test_consumers_match_reference(golden):
    """The oracle's restatement of reconstruct.py / metrics.py against the
    reference's own outputs (tests/golden/reconstruct_reference.npz)."""
    g = golden("reconstruct_reference.npz")
    H, W = g["V"].shape[:2]
    V = g["V"].reshape(H, W, 2, 2)
    s = O.stick_saliency(V)
    np.testing.assert_allclose(s, g["saliency"], rtol=0, atol=1e-6 * float(g["saliency"].max()))
    assert abs(O.otsu_threshold(g["saliency"].ravel()) - float(g["otsu"])) < 1e-12
    sal = g["saliency"]
    assert np.array_equal(sal > float(g["otsu"]), g["mask_otsu"])
    assert np.array_equal(O.saliency_threshold(V, fill=True), g["mask_fill_r0"]) or \
        np.abs(s - float(g["otsu"])).min() < 1e-6
    assert np.array_equal(O.saliency_threshold(V, fill=True, close_radius=2), g["mask_fill_r2"]) or \
        np.abs(s - float(g["otsu"])).min() < 1e-6
    G = g["G"].reshape(H, W, 2, 2)
    I = g["I"]
    for (s1, s2, pw), ref in zip(g["sweep_params"], g["sweep_simf"]):
        w = 2 * int(3 * max(s1, s2)) + 1
        B = O.tensorvote2(I, s1, s2, int(pw), w, samples=20).reshape(H, W, 2, 2)
        assert abs(O.simf(G, B) - ref) <= 1e-5 * max(abs(ref), 1e-3)
