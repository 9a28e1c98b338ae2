"""Binary reconstruction from a voted 2D tensor field, on the GPU.

Drop-in for tiralib's python/tira/tensors_lib/reconstruct.py: the same
functions, arguments and results, computed by libtvgb (tvgb_stick_saliency2,
tvgb_otsu_threshold, tvgb_saliency_threshold2).  Fields are (H, W, 2, 2)
(or (H, W, 4) [a, b, b, c]) NumPy arrays or CUDA torch tensors, float32 on
the device (float64 input is converted).  The level-set and SymPR methods
are stubs in the reference too (reconstruct.py:117-144) and raise here.
"""
import ctypes

import numpy as np

from . import api as _api


def _field4(T):
    """(H, W, 2, 2) or (H, W, 4) -> contiguous float32 (H, W, 4) view, and (H, W)."""
    if _api._is_torch(T):
        H, W = T.shape[:2]
        T = _api._check_f32(T.reshape(H, W, 4).contiguous(), "T")
        return T, (H, W)
    T = np.asarray(T)
    H, W = T.shape[:2]
    return np.ascontiguousarray(T.reshape(H, W, 4), dtype=np.float32), (H, W)


def stick_saliency(T):
    """reconstruct.py:14: per-pixel |lambda|max - |lambda|min (float32, (H, W))."""
    F, (H, W) = _field4(T)
    out = _api._empty_like_kind(F, (H, W))
    _api.call("tvgb_stick_saliency2", _api._ptr(F), H * W, _api._ptr(out), _api._stream_for(F, out))
    return out


def _otsu_threshold(values):
    """reconstruct.py:34: Otsu's threshold of non-negative values (256-bin histogram over [0, max])."""
    v = _api._check_f32(values.reshape(-1) if _api._is_torch(values) else np.asarray(values).ravel(), "values")
    thr = ctypes.c_double(0.0)
    _api.call("tvgb_otsu_threshold", _api._ptr(v), int(_api._numel(v)), ctypes.byref(thr), _api._stream_for(v))
    return float(thr.value)


def saliency_threshold(T, fill=False, threshold="otsu", close_radius=0):
    """reconstruct.py:66: bool mask of saliency > threshold ("otsu" or a
    number); with fill=True, closed by a (2 close_radius + 1)^2 square and
    hole-filled (scipy.ndimage.binary_closing + binary_fill_holes)."""
    F, (H, W) = _field4(T)
    use_otsu = isinstance(threshold, str)
    if use_otsu and threshold != "otsu":
        raise ValueError(f"unknown threshold method {threshold!r}")
    if _api._is_torch(F):
        import torch
        mask = torch.empty((H, W), dtype=torch.uint8, device=F.device)
    else:
        mask = np.empty((H, W), np.uint8)
    used = ctypes.c_double(0.0)
    _api.call("tvgb_saliency_threshold2", _api._ptr(F), H, W, int(bool(fill)), int(use_otsu),
              0.0 if use_otsu else float(threshold), int(close_radius if fill else 0), _api._ptr(mask),
              ctypes.byref(used), _api._stream_for(F))
    return mask.bool() if _api._is_torch(mask) else mask.astype(bool)


def levelset_reconstruct(T, **kwargs):
    """Deferred in the reference (reconstruct.py:117): not implemented."""
    raise NotImplementedError("levelset_reconstruct is deferred in tiralib as well")


def sympr_reconstruct(T, **kwargs):
    """Deferred in the reference (reconstruct.py:131): not implemented."""
    raise NotImplementedError("sympr_reconstruct is deferred in tiralib as well")
