"""Counterpart of python/tira/tensors_lib/cuda_wrappers.py on libtvgb.

Same public names and conventions (field layouts, N -> samples mapping,
_build_nb_numpy's table, _NB_DTYPE).  One deliberate difference: the
reference silently falls back to its NumPy implementation when its CUDA
extension is missing (cuda_wrappers.py:44-56, 248-251); here a missing
library raises instead, so a result always comes from the GPU path.
"""
import math

import numpy as np

from . import tensorvote_atv as _cuda_atv_mod
from . import tensorvote_tk as _cuda_tk_mod
from .api import NB2_DTYPE as _NB_DTYPE  # noqa: F401  (48-byte tira::Neighbor2D)

CUDA_TK_AVAILABLE = True
CUDA_ATV_AVAILABLE = True

_TV_EPSILON = 1e-12


def _w_from_sigma(sigma1, sigma2):
    """Window rule of python/tira/tensors_lib/optimize.py:9-15."""
    sigmax = max(float(sigma1), float(sigma2))
    pad = int(3 * sigmax)
    w = 2 * pad + 1
    if w < 3:
        w = 3
    if w % 2 == 0:
        w += 1
    return w


def _build_nb_numpy(sigma1, sigma2, power, samples, w):
    """Neighbor2D table with vectorised NumPy, following the same recipe as
    the reference helper (cuda_wrappers.py:76-188): FP64 plate accumulation
    over `samples` orientations with Riemann weight pi / samples."""
    hw = w // 2
    dv_g, du_g = np.meshgrid(np.arange(-hw, hw + 1, dtype=np.int32), np.arange(-hw, hw + 1, dtype=np.int32),
                             indexing="ij")
    dv, du = dv_g.ravel(), du_g.ravel()
    duf, dvf = du.astype(np.float32), dv.astype(np.float32)
    l2 = duf ** 2 + dvf ** 2
    L = np.sqrt(l2)
    nz = L > 0.0
    dx = np.where(nz, duf / np.where(nz, L, 1.0), 0.0).astype(np.float32)
    dy = np.where(nz, dvf / np.where(nz, L, 1.0), 0.0).astype(np.float32)
    c1 = (np.exp(-(l2 / sigma1 ** 2)) if sigma1 > 0 else np.where(l2 > _TV_EPSILON, 0.0, 1.0)).astype(np.float32)
    c2 = (np.exp(-(l2 / sigma2 ** 2)) if sigma2 > 0 else np.where(l2 > _TV_EPSILON, 0.0, 1.0)).astype(np.float32)
    Ra = (1.0 - 2.0 * dx * dx).astype(np.float32)
    Rb = (-2.0 * dx * dy).astype(np.float32)
    Rc = (1.0 - 2.0 * dy * dy).astype(np.float32)
    n = du.size
    acc = np.zeros((3, n))
    eta_s = (2 ** (2 * power) * math.factorial(power) ** 2) / (np.pi * math.factorial(2 * power) * (sigma1 ** 2 + sigma2 ** 2))
    if samples > 0:
        for i in range(samples):
            th = i * np.pi / samples
            qx, qy = np.cos(th), np.sin(th)
            qTd = qx * dx.astype(np.float64) + qy * dy.astype(np.float64)
            t2 = qTd * qTd
            D = c1.astype(np.float64) * (1.0 - t2) ** power + c2.astype(np.float64) * t2 ** power
            Rqx = Ra.astype(np.float64) * qx + Rb.astype(np.float64) * qy
            Rqy = Rb.astype(np.float64) * qx + Rc.astype(np.float64) * qy
            f = eta_s * D
            acc[0] += f * Rqx * Rqx
            acc[1] += f * Rqx * Rqy
            acc[2] += f * Rqy * Rqy
        acc *= np.pi / samples
    nb = np.empty(n, dtype=_NB_DTYPE)
    nb["du"], nb["dv"], nb["dx"], nb["dy"], nb["c1"], nb["c2"] = du, dv, dx, dy, c1, c2
    nb["Ra"], nb["Rb"], nb["Rc"] = Ra, Rb, Rc
    nb["Va"], nb["Vb"], nb["Vc"] = acc.astype(np.float32)
    return np.ascontiguousarray(nb)


def _field_to_flat4(field):
    """(H, W, 2, 2) -> (H, W, 4) float32 [T00, T01, T10, T11]."""
    H, W = field.shape[:2]
    flat = np.empty((H, W, 4), np.float32)
    flat[..., 0] = field[..., 0, 0]
    flat[..., 1] = field[..., 0, 1]
    flat[..., 2] = field[..., 1, 0]
    flat[..., 3] = field[..., 1, 1]
    return flat


def _flat4_to_field(flat, out_dtype=np.float64):
    H, W = flat.shape[:2]
    field = np.empty((H, W, 2, 2), dtype=out_dtype)
    field[..., 0, 0] = flat[..., 0]
    field[..., 0, 1] = flat[..., 1]
    field[..., 1, 0] = flat[..., 2]
    field[..., 1, 1] = flat[..., 3]
    return field


def _samples(plate, N):
    # N = 0 (closed-form plate in NumPy) maps to 10 samples, as the reference does
    if plate:
        return max(1, int(N)) if N > 0 else 10
    return 1


def tk_vote2_cuda_flat(flat_in, H, W, sigma1, sigma2=0.0, power=1, plate=True, N=20, out_dtype=np.float64):
    flat_out = _cuda_tk_mod.tensorvote_tk(flat_in, float(sigma1), float(sigma2), int(power), 0, True, bool(plate),
                                          _samples(plate, N))
    return _flat4_to_field(flat_out, out_dtype=out_dtype)


def tk_vote2_cuda_prebuilt_flat(flat_in, nb, sigma1, sigma2=0.0, power=1, plate=True, N=20, out_dtype=np.float64):
    w = _w_from_sigma(sigma1, sigma2)
    nb_bytes = np.frombuffer(nb.tobytes(), dtype=np.uint8)
    flat_out = _cuda_tk_mod.tensorvote_tk_prebuilt(flat_in, nb_bytes, int(len(nb)), int(w), float(sigma1),
                                                   float(sigma2), int(power), True, bool(plate), _samples(plate, N))
    return _flat4_to_field(flat_out, out_dtype=out_dtype)


def tk_vote2_cuda(field, sigma1, sigma2=0.0, power=1, plate=True, N=20):
    """Counterpart of ts.tk_vote2(field, sigma1, sigma2, power, plate, N) on the GPU."""
    flat_out = _cuda_tk_mod.tensorvote_tk(_field_to_flat4(field), float(sigma1), float(sigma2), int(power), 0, True,
                                          bool(plate), _samples(plate, N))
    return _flat4_to_field(flat_out, out_dtype=field.dtype)


def atv_vote2_cuda(field, sigma):
    """Counterpart of ts.atv_vote2(field, sigma) on the GPU."""
    flat_out = _cuda_atv_mod.tensorvote_atv(_field_to_flat4(field), float(sigma))
    return _flat4_to_field(flat_out, out_dtype=field.dtype)
