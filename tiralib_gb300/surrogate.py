"""The learned plate / ball vote (MLP surrogate) on the GPU.

The network, 28 -> 64 -> 64 -> 64 -> 6 with GELU, maps the features of
(offset direction d = o / |o|, plate normal n, flag: 1 plate / 0 ball) --
the seven inputs and the degree-2 monomials d_i d_j, n_i n_j, d_i n_j -- to
the angular part of the unit-scale plate or ball vote at offset o
(sigma2 = 0, power 1; the Gaussian exp(-|o|^2 / sigma^2) is applied
analytically, so the direction is all the network needs).  Sample rows (X)
hold the seven raw inputs (8 floats); the features are formed in the
kernels.  Everything runs in libtvgb:

  samples(n, seed)          training pairs from the plain 64-orientation integral
  train(params, X, T, ...)  quantisation-aware training by its own kernels
  grad(params, X, T)        one forward + backward pass (for gradient checks)
  evaluate(params, X)       inference on the tensor cores (BF16, FP32 accumulate)
  vote3(field, ...)         3D vote with the plate / ball by the network, the
                            exact closed form or the plain integral
  save / load               a versioned weights file with a checksum

Arrays are NumPy (host) or CUDA torch tensors, float32.
"""
import ctypes
import hashlib
import struct

import numpy as np

from . import api as _api
from ._lib import Vote3Params

PLATE_SURROGATE, PLATE_CLOSED, PLATE_PLAIN64 = 0, 1, 2
_MODES = {"surrogate": PLATE_SURROGATE, "closed": PLATE_CLOSED, "plain64": PLATE_PLAIN64}

_MAGIC = b"TVGBSUR1"
_VERSION = 2          # 2: the 28-feature first layer (1: seven raw inputs)


def param_count():
    return int(_api._lib.lib().tvgb_surrogate_param_count())


def layout():
    """(name, offset, shape) of each parameter block in the flat vector."""
    out, off = [], 0
    for name, shape in (("W1", (64, 28)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64, 64)),
                        ("b3", (64,)), ("W4", (8, 64)), ("b4", (8,))):
        out.append((name, off, shape))
        off += int(np.prod(shape))
    return out


def init_params(seed=0):
    """Glorot-uniform weights, zero biases; the padded output rows are zero."""
    rng = np.random.default_rng(seed)
    p = np.zeros(param_count(), np.float32)
    for name, off, shape in layout():
        if name.startswith("W"):
            fan_out, fan_in = shape
            fan_out = 6 if name == "W4" else fan_out
            lim = np.sqrt(6.0 / (fan_in + fan_out))
            w = rng.uniform(-lim, lim, shape).astype(np.float32)
            if name == "W4":
                w[6:, :] = 0.0
            p[off:off + w.size] = w.ravel()
    return p


def samples(n, seed=0, device=None):
    """(X, T): n x 8 inputs and targets from the plain orientation integral,
    generated on the GPU (NumPy arrays, or CUDA tensors on `device`)."""
    if device is not None:
        import torch
        X = torch.empty((n, 8), dtype=torch.float32, device=device)
        T = torch.empty((n, 8), dtype=torch.float32, device=device)
    else:
        X = np.empty((n, 8), np.float32)
        T = np.empty((n, 8), np.float32)
    _api.call("tvgb_surrogate_samples", n, seed, _api._ptr(X), _api._ptr(T), _api._stream_for(X, T))
    return X, T


def grad(params, X, T):
    """(gradient, loss) of one forward + backward pass over all rows of X."""
    p = _api._check_f32(params, "params")
    X = _api._check_f32(X, "X")
    T = _api._check_f32(T, "T")
    B = int(X.shape[0])
    g = _api._empty_like_kind(p, (param_count(),))
    loss = ctypes.c_float(0.0)
    _api.call("tvgb_surrogate_grad", _api._ptr(p), _api._ptr(X), _api._ptr(T), B, _api._ptr(g), ctypes.byref(loss),
              _api._stream_for(p, X, T))
    return g, float(loss.value)


def train(params, X, T, batch=8192, steps=2000, lr=2e-3, history=True):
    """Adam on the network in place (params: a float32 array or CUDA tensor);
    returns the per-step loss (NumPy) when history is set."""
    p = params if _api._is_torch(params) else params
    if not _api._is_torch(p):
        if p.dtype != np.float32 or not p.flags.c_contiguous:
            raise ValueError("params must be a contiguous float32 array (updated in place)")
    X = _api._check_f32(X, "X")
    T = _api._check_f32(T, "T")
    hist = np.empty(steps, np.float32) if history else None
    _api.call("tvgb_surrogate_train", _api._ptr(p), _api._ptr(X), _api._ptr(T), int(X.shape[0]), int(batch),
              int(steps), float(lr), None if hist is None else hist.ctypes.data_as(ctypes.c_void_p),
              _api._stream_for(p, X, T))
    return hist


_GELU = {"fp32": 0, "bf16": 1}


def evaluate(params, X, engine="tcgen05", gelu="bf16", wait_limit=None):
    """The network's outputs (n x 8, 6 used) on the tensor cores.  engine
    "tcgen05" (tensor memory; gelu "bf16", the packed arithmetic the network
    is trained with and the vote uses, or "fp32") or "mma" (warp-level
    mma.sync, GELU in FP32; a cross-check of the tcgen05 path).  wait_limit
    (tcgen05 only) bounds each layer's wait for its MMAs in mbarrier polls;
    None is the library's default, and a wait that runs out raises TvgbError."""
    X = _api._check_f32(X, "X")
    Y = _api._empty_like_kind(X, (int(X.shape[0]), 8))
    P = _api._ptr(_api._check_f32(params, "params"))
    if engine == "tcgen05":
        _api.call("tvgb_surrogate_eval_tc_limit", P, _api._ptr(X), int(X.shape[0]), _api._ptr(Y), _GELU[gelu],
                  -1 if wait_limit is None else int(wait_limit), _api._stream_for(X, Y))
    elif engine == "mma":
        if gelu != "fp32":
            raise ValueError("the mma engine computes the GELU in FP32 only")
        _api.call("tvgb_surrogate_eval", P, _api._ptr(X), int(X.shape[0]), _api._ptr(Y), _api._stream_for(X, Y))
    else:
        raise ValueError(f"engine must be 'tcgen05' or 'mma', not {engine!r}")
    return Y


def vote3(field, sigma, params=None, mode="surrogate", tol=1e-3, w=0, stick=True, plate=True, ball=False,
          parity=True, layout="mat3", out_layout="mat3", evals=False, evecs=None):
    """3D TK vote (power 1, sigma2 = 0) with the plate / ball vote by `mode`:
    "surrogate" (the network, judged per CTA against the exact plate of 32
    of its receivers, normwise, with tolerance tol), "closed" (exact closed
    form) or "plain64" (the plain
    64-orientation integral).  Returns (voted field, evals, evecs, stats)
    with stats = (CTAs, CTAs recomputed exactly)."""
    field = _api._check_f32(field, "field")
    L = _api.LAYOUTS[layout]
    dims = tuple(field.shape[1:4]) if L == _api.LAYOUT_SYM6_PLANES else tuple(field.shape[:3])
    OL = _api.LAYOUTS[out_layout]
    oshape = (6,) + dims if OL == _api.LAYOUT_SYM6_PLANES else (dims + (6,) if OL == _api.LAYOUT_SYM6 else dims + (3, 3))
    o = _api._empty_like_kind(field, oshape)
    ev = _api._empty_like_kind(field, dims + (3,)) if evals else None
    fmt = _api.EVECS[evecs]
    vec = None
    if fmt == _api.EVEC_CARTESIAN:
        vec = _api._empty_like_kind(field, dims + (3, 3))
    elif fmt == _api.EVEC_SPHERICAL:
        vec = _api._empty_like_kind(field, dims + (6,))
    p = Vote3Params(float(sigma), 0.0, int(w), 1, 0, int(stick), int(plate), int(ball), 0, int(parity))
    stats = (ctypes.c_ulonglong * 2)()
    net = None if params is None else _api._check_f32(params, "params")
    _api.call("tvgb_vote3_surrogate", _api._ptr(field), L, dims[0], dims[1], dims[2], ctypes.byref(p),
              _api._ptr(net), _MODES[mode], float(tol), _api._ptr(o), OL, _api._ptr(ev), _api._ptr(vec), fmt, stats,
              _api._stream_for(field, o, ev, vec))
    return o, ev, vec, (int(stats[0]), int(stats[1]))


def save(path, params, meta=""):
    """Weights file: magic, version, parameter count, SHA-256 of the float32
    payload, a UTF-8 note, then the payload."""
    p = np.ascontiguousarray(params if not _api._is_torch(params) else params.cpu().numpy(), np.float32)
    if p.size != param_count():
        raise ValueError(f"expected {param_count()} parameters, got {p.size}")
    payload = p.tobytes()
    note = meta.encode("utf-8")
    with open(path, "wb") as f:
        f.write(_MAGIC + struct.pack("<III", _VERSION, p.size, len(note)) + hashlib.sha256(payload).digest() + note
                + payload)


def load(path):
    """Read a weights file written by save(); checks magic, size and checksum.
    Returns (params, note)."""
    with open(path, "rb") as f:
        blob = f.read()
    if blob[:8] != _MAGIC:
        raise ValueError(f"{path}: not a surrogate weights file")
    version, count, nlen = struct.unpack("<III", blob[8:20])
    if version != _VERSION or count != param_count():
        raise ValueError(f"{path}: unsupported version {version} or size {count}")
    digest = blob[20:52]
    note = blob[52:52 + nlen].decode("utf-8")
    payload = blob[52 + nlen:]
    if len(payload) != 4 * count or hashlib.sha256(payload).digest() != digest:
        raise ValueError(f"{path}: corrupt weights (size or checksum)")
    return np.frombuffer(payload, np.float32).copy(), note
