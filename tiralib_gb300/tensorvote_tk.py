"""Drop-in for the reference's pybind11 module `tensorvote_tk`
(python/tira/cuda_ext/tensorvote_tk.cu:206-253): same function names,
argument names, defaults, validation messages and (H, W, 4) float32 layout.
The work runs in libtvgb (2D TK vote, tvgb_tensorvote / _prebuilt).
"""
import numpy as np

from . import api

_NB_ITEMSIZE = api.NB2_DTYPE.itemsize   # 48


def _field(field):
    f = np.ascontiguousarray(field, dtype=np.float32)
    if f.ndim != 3 or f.shape[2] != 4:
        raise RuntimeError("field must have shape (H, W, 4)")
    if f.shape[0] <= 0 or f.shape[1] <= 0:
        raise RuntimeError("field must have positive H and W")
    return f


def tensorvote_tk(field, sigma1, sigma2=0.0, power=1, w=0, stick=True, plate=True, samples=20):
    """CUDA TK tensor voting on a 2D tensor field (tensorvote_tk.cu:62-137)."""
    f = _field(field)
    if sigma1 <= 0.0:
        raise RuntimeError("sigma1 must be > 0")
    if power < 1:
        power = 1
    if w <= 0:
        sigmax = sigma2 if sigma2 > sigma1 else sigma1
        w = 2 * int(np.float32(3.0) * np.float32(sigmax)) + 1
        if w < 3:
            w = 3
    if w % 2 == 0:
        w += 1
    H, W = f.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    api.tensorvote(out, f, float(sigma1), float(sigma2), int(power), int(w), H, W, bool(stick), bool(plate),
                   int(samples), False)
    return out


def tensorvote_tk_prebuilt(field, nb_buf, nb_count, w, sigma1, sigma2=0.0, power=1, stick=True, plate=True,
                           samples=20):
    """TK voting with a pre-built neighbour table (48 bytes/entry)
    (tensorvote_tk.cu:149-203)."""
    f = _field(field)
    if sigma1 <= 0.0:
        raise RuntimeError("sigma1 must be > 0")
    if power < 1:
        power = 1
    if w <= 0 or w % 2 == 0:
        raise RuntimeError("w must be a positive odd integer")
    raw = np.ascontiguousarray(np.frombuffer(memoryview(nb_buf).tobytes(), dtype=np.uint8))
    if raw.size != int(nb_count) * _NB_ITEMSIZE:
        raise RuntimeError("nb_buf byte size does not match nb_count * sizeof(Neighbor2D) (48)")
    H, W = f.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    api.tensorvote_prebuilt(out, f, raw, int(nb_count), float(sigma1), float(sigma2), int(power), int(w), H, W,
                            bool(stick), bool(plate), int(samples))
    return out
