"""Tensor-field comparison on the GPU (tiralib's
python/tira/tensors_lib/metrics.py: simf, the objective of its parameter
sweeps), via tvgb_simf2.  Fields: (H, W, 2, 2) / (H, W, 4) float32 NumPy
arrays or CUDA torch tensors."""
import ctypes

from . import api as _api
from .reconstruct import _field4


def simf(A, B):
    """metrics.py:37: mean over pixels of ||A - alpha B||_F, alpha = <A,B> / <B,B>."""
    FA, sa = _field4(A)
    FB, sb = _field4(B)
    if sa != sb:
        raise ValueError(f"simf: shapes differ ({sa} vs {sb})")
    out = ctypes.c_double(0.0)
    _api.call("tvgb_simf2", _api._ptr(FA), _api._ptr(FB), sa[0] * sa[1], ctypes.byref(out),
              _api._stream_for(FA, FB))
    return float(out.value)
