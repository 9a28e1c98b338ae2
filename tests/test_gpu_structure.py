"""GPU parity of the separable Gaussian filters and the fused structure
tensor against the reference's outputs (tests/golden, filter.h compiled
unmodified) and the CPU oracle (gradient, outer product, blur)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module")
def tv():
    import tiralib_gb300
    return tiralib_gb300


def test_gaussian_filter3d_matches_reference(tv, golden):
    g = golden("filter_cpp_reference.npz")
    out = tv.gaussian_filter3d(g["vol"], sigma_w=1.5, sigma_h=1.0, sigma_d=2.0)
    assert out.shape == g["conv3_15_10_20"].shape
    assert rel(out, g["conv3_15_10_20"]) < 1e-6


def test_gaussian_convolve2_matches_reference(tv, golden):
    g = golden("filter_cpp_reference.npz")
    out = tv.gaussian_convolve2(g["img"], 1.0)
    assert out.shape == g["conv2_1"].shape
    assert rel(out, g["conv2_1"]) < 1e-6


@pytest.mark.parametrize("mode", ["valid", "same"])
@pytest.mark.parametrize("shape,sigma", [((20, 22, 24), 1.5), ((15, 40, 33), 1.0), ((30, 17, 70), 2.0)])
def test_structure_tensor3_matches_oracle(tv, mode, shape, sigma):
    rng = np.random.default_rng(sum(shape))
    v = rng.normal(size=shape).astype(np.float32)
    out = tv.structure_tensor3(v, sigma, mode=mode, layout="planes")
    ref = O.structure_tensor3(v, sigma, 0 if mode == "valid" else 1)
    assert out.shape == ref.shape
    assert rel(out, ref) < 1e-5


# every fixed-tap kernel (K = 3 .. 13) and the any-K kernel (K = 15, 25);
# deep volumes so that several z chunks meet inside the volume
@pytest.mark.parametrize("sigma", [0.3, 0.7, 1.7, 2.5, 4.0])
@pytest.mark.parametrize("mode", ["valid", "same"])
def test_structure_tensor3_tap_counts(tv, sigma, mode):
    rng = np.random.default_rng(int(sigma * 10))
    v = rng.normal(size=(90, 37, 45)).astype(np.float32)
    out = tv.structure_tensor3(v, sigma, mode=mode, layout="planes")
    ref = O.structure_tensor3(v, sigma, 0 if mode == "valid" else 1)
    assert out.shape == ref.shape
    assert rel(out, ref) < 1e-5


def test_structure_tensor3_layouts_agree(tv):
    rng = np.random.default_rng(1)
    v = rng.normal(size=(12, 13, 14)).astype(np.float32)
    p = tv.structure_tensor3(v, 1.0, layout="planes")
    s = tv.structure_tensor3(v, 1.0, layout="sym6")
    m = tv.structure_tensor3(v, 1.0, layout="mat3")
    np.testing.assert_array_equal(np.moveaxis(p, 0, -1), s)
    np.testing.assert_array_equal(m.reshape(-1, 9)[:, [0, 1, 2, 4, 5, 8]], s.reshape(-1, 6))


@pytest.mark.parametrize("mode", ["valid", "same"])
def test_structure_tensor2_matches_oracle(tv, mode):
    rng = np.random.default_rng(2)
    img = rng.normal(size=(50, 61)).astype(np.float32)
    out = tv.structure_tensor2(img, 1.0, mode=mode)
    ref = O.structure_tensor2(img, 1.0, 0 if mode == "valid" else 1)
    assert out.shape == ref.shape
    assert rel(out, ref) < 1e-5


def test_pipeline3_matches_chained_oracle(tv):
    rng = np.random.default_rng(3)
    v = rng.normal(size=(16, 18, 20)).astype(np.float32)
    out, ev, vec = tv.pipeline3(v, 1.0, 2.0, w=9, samples=20, st_mode="same", out_layout="mat3",
                                evecs="cartesian")
    st = O.structure_tensor3(v, 1.0, 1)                      # (6, s0, s1, s2)
    s6 = np.moveaxis(st, 0, -1)
    m9 = s6[..., [0, 1, 2, 1, 3, 4, 2, 4, 5]].reshape(16, 18, 20, 3, 3)
    ref = O.tensorvote3(m9, 2.0, 0.0, 9, 1, samples=20)
    u = [0, 1, 2, 4, 5, 8]
    assert rel(out.reshape(-1, 9)[:, u], ref.reshape(-1, 9)[:, u]) < 1e-4
    ref_ev = O.evals3(out.reshape(-1, 9))
    assert (np.abs(ev.reshape(-1, 3) - ref_ev).max(axis=1) / np.abs(ref_ev).max(axis=1)).max() < 1e-5


def _profiled(tv, fn):
    """Run fn with the library's kernel timing on; the kernel names that ran."""
    import ctypes
    L = tv.lib()
    buf = ctypes.create_string_buffer(1 << 14)
    L.tvgb_profile_enable(1)
    L.tvgb_profile_read(buf, len(buf))
    out = fn()
    L.tvgb_profile_read(buf, len(buf))
    L.tvgb_profile_enable(0)
    return out, {line.split()[0] for line in buf.value.decode().strip().splitlines() if line.strip()}


@pytest.mark.parametrize("mode", ["valid", "same"])
@pytest.mark.parametrize("sigma", [0.3, 0.7, 1.0, 1.5, 1.7, 2.0])      # 3, 5, 7, 9, 11, 13 taps
@pytest.mark.parametrize("shape", [(21, 22, 24), (9, 70, 64), (40, 17, 36), (6, 8, 32)])
def test_structure_tensor3_tma_kernel_matches_oracle(tv, mode, sigma, shape):
    """Volumes whose rows are 16-byte multiples (s2 % 4 == 0) take the
    TMA-staged kernel (k_st3_tma): every tap count of the fixed-tap
    kernels, both output modes, faces in every axis, several CTAs in x and
    y, fewer planes than taps; against the oracle's restatement of
    volume::gradient + the separable Gaussian (filter.h)."""
    K = int(np.ceil(6 * sigma)) | 1
    if mode == "valid" and min(shape) < K:
        pytest.skip("valid output empty: the volume is smaller than the window")
    rng = np.random.default_rng(sum(shape) + int(10 * sigma))
    v = rng.normal(size=shape).astype(np.float32)
    out, ran = _profiled(tv, lambda: tv.structure_tensor3(v, sigma, mode=mode, layout="planes"))
    assert "k_st3_tma" in ran
    ref = O.structure_tensor3(v, sigma, 0 if mode == "valid" else 1)
    assert out.shape == ref.shape
    assert rel(out, ref) < 1e-5


def test_structure_tensor3_tma_kernel_layouts(tv):
    """The TMA kernel's three output layouts hold the same numbers, and the
    rows that are not 16-byte multiples take the other kernel."""
    rng = np.random.default_rng(3)
    v = rng.normal(size=(13, 19, 28)).astype(np.float32)
    (p, ran) = _profiled(tv, lambda: tv.structure_tensor3(v, 1.5, layout="planes"))
    assert "k_st3_tma" in ran
    s6 = tv.structure_tensor3(v, 1.5, layout="sym6")
    m = tv.structure_tensor3(v, 1.5, layout="mat3")
    np.testing.assert_array_equal(np.moveaxis(p, 0, -1), s6)
    m9 = m.reshape(-1, 9)
    np.testing.assert_array_equal(m9[:, [0, 1, 2, 4, 5, 8]], s6.reshape(-1, 6))
    np.testing.assert_array_equal(m9[:, [3, 6, 7]], m9[:, [1, 2, 5]])
    _, ran = _profiled(tv, lambda: tv.structure_tensor3(v[:, :, :27].copy(), 1.5))
    assert "k_st3_tma" not in ran and "k_st3" in ran
