"""Host-side checks of the drop-in modules that mirror the reference's
pybind11 extensions (tensorvote_tk / tensorvote_atv) and its consumers
(optimize.py, reconstruct.py): argument validation and host-side rules, all
before any GPU work, so these run without a GPU."""
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



def test_consumer_host_logic():
    """The consumers' host-side rules (tiralib's optimize.py / reconstruct.py):
    the search window from the sigmas, the power rounding, the deferred
    methods, and argument errors raised before any GPU work."""
    from tiralib_gb300 import optimize, reconstruct
    for s1, s2 in [(1.0, 0.0), (3.0, 1.0), (0.2, 0.1), (5.5, 7.2), (10.0, 0.0)]:
        w = 2 * int(3 * max(s1, s2)) + 1                       # optimize.py:9
        w = max(w, 3)
        assert optimize.w_from_sigma(s1, s2) == (w + 1 if w % 2 == 0 else w)
        assert optimize.w_from_sigma(s1, s2) % 2 == 1
    assert [optimize._round_power(p) for p in (0.2, 1.4, 1.6, 29.5)] == [1, 1, 2, 30]
    for fn in (reconstruct.levelset_reconstruct, reconstruct.sympr_reconstruct):
        with pytest.raises(NotImplementedError):
            fn(np.zeros((4, 4, 2, 2), np.float32))
    with pytest.raises(ValueError, match="unknown threshold method"):
        reconstruct.saliency_threshold(np.zeros((4, 4, 2, 2), np.float32), threshold="mean")
    with pytest.raises(ValueError, match="tk_sweep"):
        optimize.tk_sweep(np.zeros((4, 5, 2, 2), np.float32), np.zeros((4, 4, 2, 2), np.float32), [(1.0, 0.0, 1)])
