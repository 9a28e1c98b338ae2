"""CPU-side checks of the product library: it builds for sm_103a, loads,
exports every entry point declared in include/tvgb.h, and its host-only
functions agree with the reference (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tv():
    import tiralib_gb300
    from tiralib_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from tiralib_gb300 import build
        build.build()
    return tiralib_gb300


def declared_symbols():
    src = open(os.path.join(REPO, "include", "tvgb.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|double|const char\*|unsigned long long)\s+(tvgb_\w+)\(", src, re.M)))


def test_library_exports_every_declared_symbol(tv):
    names = declared_symbols()
    assert len(names) >= 18
    L = ctypes.CDLL(tv._lib.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(tv._lib.SIGNATURES)


def test_library_is_built_for_sm_103a_only(tv):
    data = open(tv._lib.LIB_PATH, "rb").read()
    assert b"sm_103a" in data


def test_neighbors2d_table_matches_reference(tv, golden):
    g = golden("tv2_cpp_reference.npz")
    nb = tv.build_neighbors2d(7, 2.0, 0.5, 2, 10)
    ref = g["nb_w7"]
    assert nb.dtype.itemsize == 48 and nb.size == ref.size
    for f in nb.dtype.names:
        np.testing.assert_allclose(nb[f], ref[f], rtol=0, atol=2e-6)


def test_neighbors3d_table_matches_reference(tv, golden):
    """tvgb_build_neighbors3d against the reference's cpu::build_neighbors3d
    (tensorvote.h:1411), bit for bit, including sigma = 0 rows."""
    g = golden("nb3_cpp_reference.npz")
    for key in g.files:
        w, s1, s2 = key.split("_")[1:]
        nb = tv.build_neighbors3d(int(w[1:]), float(s1), float(s2))
        ref = g[key]
        assert nb.dtype.itemsize == 32 and nb.size == ref.size
        for f in nb.dtype.names:
            np.testing.assert_array_equal(nb[f], ref[f], err_msg=f"{key}.{f}")


def test_tensorvote3_rejects_a_negative_device(tv):
    """The reference's negative device index selects its CPU path
    (eigen.h:897); this library has none and says so instead of running on
    whatever device is current."""
    T = np.zeros((2, 2, 2, 9), np.float32)
    out = np.zeros_like(T)
    with pytest.raises(tv.TvgbError, match="CPU path"):
        tv.tensorvote3(T, out, 2, 2, 2, 1.0, 0.0, 3, 1, device=-1)


def test_sticknorm3_matches_oracle(tv):
    from oracle import oracle as O
    for args in [(4.0, 0.0, 1), (2.0, 1.0, 3), (6.0, 0.5, 2)]:
        assert abs(tv.sticknorm3(*args) - O.sticknorm3(*args)) <= 1e-6 * O.sticknorm3(*args)


def test_errors_are_raised_not_swallowed(tv):
    with pytest.raises(tv.TvgbError):
        tv._lib.call("tvgb_build_neighbors2d", -1, 1.0, 0.0, 1, 1, 1, 1, None, None)
    msg = tv._lib.lib().tvgb_last_error().decode()
    assert "count is NULL" in msg or "w must be" in msg


def test_cuda_wrappers_table_matches_reference_numpy_table(tv):
    """_build_nb_numpy follows the reference helper's recipe; its entries agree
    with the reference C++ table to float precision."""
    from tiralib_gb300 import cuda_wrappers as cw
    a = cw._build_nb_numpy(2.0, 0.5, 2, 10, 7)
    b = tv.build_neighbors2d(7, 2.0, 0.5, 2, 10)
    for f in a.dtype.names:
        np.testing.assert_allclose(a[f], b[f], rtol=1e-5, atol=1e-6)


def test_empty_inputs_give_empty_outputs(tv):
    """An empty field, volume or batch returns empty outputs; the library
    returns before it touches a pointer or the GPU."""
    o, e, v = tv.vote3(np.zeros((0, 4, 4, 3, 3), np.float32), 1.0, w=5, evals=True, evecs="cartesian")
    assert o.shape == (0, 4, 4, 3, 3) and e.shape == (0, 4, 4, 3) and v.shape == (0, 4, 4, 3, 3)
    assert tv.structure_tensor3(np.zeros((0, 8, 8), np.float32), 1.0).shape == (6, 0, 8, 8)
    assert tv.structure_tensor2(np.zeros((0, 5), np.float32), 1.0).shape == (0, 5, 4)
    o, e, v = tv.pipeline3(np.zeros((0, 8, 8), np.float32), 1.0, 2.0, w=5)
    assert o.shape == (6, 0, 8, 8) and e.shape == (0, 8, 8, 3) and v.shape == (0, 8, 8, 3, 3)
    e, v, nref = tv.eig3(np.zeros((0, 9), np.float32))
    assert e.shape == (0, 3) and v.shape == (0, 3, 3) and nref == 0
    assert tv.evals3_symmetric(np.zeros((0, 9), np.float32)).shape == (0, 3)
    assert tv.evals2_symmetric(np.zeros((0, 4), np.float32)).shape == (0, 2)
    out = np.zeros((0, 5, 4), np.float32)
    tv.tensorvote(out, np.zeros((0, 5, 4), np.float32), 1.0, 0.0, 1, 5, 0, 5)


def test_inputs_smaller_than_the_window_raise(tv):
    """A valid convolution of an input smaller than its window is refused by
    the library with its own message (argument checks run before any GPU
    work)."""
    cases = [
        (lambda: tv.gaussian_convolve2(np.zeros((3, 6), np.float32), 1.0), "smaller than the window"),
        (lambda: tv.gaussian_filter3d(np.zeros((4, 20, 20), np.float32)), "smaller than the window"),
        (lambda: tv.structure_tensor3(np.zeros((4, 20, 20), np.float32), 1.0, mode="valid"), "smaller than"),
        (lambda: tv.structure_tensor2(np.zeros((3, 20), np.float32), 1.0, mode="valid"), "smaller than"),
        (lambda: tv.pipeline3(np.zeros((4, 20, 20), np.float32), 1.0, 2.0, w=5, st_mode="valid"), "smaller than"),
    ]
    for fn, msg in cases:
        with pytest.raises(tv.TvgbError, match=msg):
            fn()
    with pytest.raises(tv.TvgbError, match="must be odd"):
        tv.vote3(np.zeros((0, 4, 4, 3, 3), np.float32), 1.0, w=4)   # arguments are checked even when empty
