"""Drop-in for the reference's pybind11 module `tensorvote_atv`
(python/tira/cuda_ext/tensorvote_atv.cu:52-137): same name, arguments,
defaults, validation messages and (H, W, 4) float32 layout; the vote runs in
libtvgb (2D ATV, tvgb_tensorvote with is_atv = 1).
"""
import numpy as np

from . import api


def tensorvote_atv(field, sigma, w=0, stick=True, plate=True, samples=10):
    f = np.ascontiguousarray(field, dtype=np.float32)
    if f.ndim != 3 or f.shape[2] != 4:
        raise RuntimeError("field must have shape (H, W, 4)")
    H, W = f.shape[:2]
    if H <= 0 or W <= 0:
        raise RuntimeError("field must have positive H and W")
    if sigma <= 0.0:
        raise RuntimeError("sigma must be > 0")
    if w <= 0:
        w = 2 * int(np.float32(3.0) * np.float32(sigma)) + 1
        if w < 3:
            w = 3
    if w % 2 == 0:
        w += 1
    out = np.zeros((H, W, 4), np.float32)
    # sigma2 and power are unused by ATV (tensorvote_atv.cu:103-107)
    api.tensorvote(out, f, float(sigma), 0.0, 1, int(w), H, W, bool(stick), bool(plate), int(samples), True)
    return out
