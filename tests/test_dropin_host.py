"""Host-side checks of the drop-in modules that mirror the reference's
pybind11 extensions (tensorvote_tk / tensorvote_atv): their argument
validation raises the reference's messages before any GPU work, so these run
without a GPU."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def mods():
    from tiralib_gb300 import cuda_wrappers, tensorvote_atv, tensorvote_tk
    return tensorvote_tk, tensorvote_atv, cuda_wrappers


def test_validation_messages(mods):
    tk, atv, _ = mods
    with pytest.raises(RuntimeError, match=r"shape \(H, W, 4\)"):
        tk.tensorvote_tk(np.zeros((4, 4, 3), np.float32), 1.0)
    with pytest.raises(RuntimeError, match="sigma1 must be > 0"):
        tk.tensorvote_tk(np.zeros((4, 4, 4), np.float32), 0.0)
    with pytest.raises(RuntimeError, match="sigma must be > 0"):
        atv.tensorvote_atv(np.zeros((4, 4, 4), np.float32), 0.0)
    with pytest.raises(RuntimeError, match="positive odd"):
        tk.tensorvote_tk_prebuilt(np.zeros((4, 4, 4), np.float32), b"", 0, 4, 1.0)

