"""Python host API over libtvgb, mirroring tiralib's entry points for the
tensor-voting path.

Arrays may be NumPy arrays (host memory: the library stages them to the GPU
and copies results back) or torch CUDA tensors (device memory: work is
queued on torch's current stream, nothing is copied).  Names, argument order
and meaning follow the reference:

  tensorvote3            tira::cuda::tensorvote3      tira/functions/tensorvote.h:2817
  tensorvote             tira::cuda::tensorvote       tensorvote.h:2201
  tensorvote_prebuilt    tira::cuda::tensorvote_prebuilt  tensorvote.h:2237
  build_neighbors2d      tira::cpu::build_neighbors2d tensorvote.h:1223
  build_neighbors3d      tira::cpu::build_neighbors3d tensorvote.h:1411
  evals3_symmetric       tira::cuda::evals3_symmetric eigen.h:896
  evecs3spherical_symmetric                           eigen.h:945
  evals2_symmetric / evecs2polar_symmetric            eigen.h:769 / :828
  gaussian_filter3d      tira::cuda::gaussian_filter3d filter.h:401
  gaussian_convolve2     tira::cuda::gaussian_convolve2 filter.h:305

plus the fused entry points of this library (eig3, structure_tensor3/2,
vote3, pipeline3).  Errors raise TvgbError (the reference prints CUDA errors
and continues; its pybind layer raises RuntimeError on bad arguments, which
TvgbError subclasses).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (EIG_PARITY, EIG_PRECISE, EVEC_CARTESIAN, EVEC_NONE, EVEC_SPHERICAL, LAYOUT_MAT3,
                   LAYOUT_SYM6, LAYOUT_SYM6_PLANES, TvgbError, Vote3Params, call)

try:  # torch is optional for host-only use
    import torch
except Exception:  # pragma: no cover
    torch = None

LAYOUTS = {"mat3": LAYOUT_MAT3, "sym6": LAYOUT_SYM6, "planes": LAYOUT_SYM6_PLANES}
EVECS = {None: EVEC_NONE, "none": EVEC_NONE, "cartesian": EVEC_CARTESIAN, "spherical": EVEC_SPHERICAL}

NB2_DTYPE = np.dtype([
    ("du", np.int32), ("dv", np.int32),
    ("dx", np.float32), ("dy", np.float32),
    ("c1", np.float32), ("c2", np.float32),
    ("Ra", np.float32), ("Rb", np.float32), ("Rc", np.float32),
    ("Va", np.float32), ("Vb", np.float32), ("Vc", np.float32),
])  # tira::Neighbor2D, 48 bytes (tensorvote.h:776)

NB3_DTYPE = np.dtype([
    ("du", np.int32), ("dv", np.int32), ("dw", np.int32),
    ("d", np.float32, (3,)),
    ("c1", np.float32), ("c2", np.float32),
])  # tira::Neighbor3D, 32 bytes (tensorvote.h:1147)


# ----------------------------------------------------------------- array helpers

def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


def _check_f32(a, name):
    if _is_torch(a):
        if a.dtype != torch.float32:
            raise TypeError(f"{name} must be float32")
        if not a.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
        if not a.is_cuda:
            raise ValueError(f"{name}: torch tensors must be on a CUDA device (use NumPy for host arrays)")
        return a
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a


def _ptr(a):
    if a is None:
        return None
    if _is_torch(a):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)


def _stream_for(*arrays):
    for a in arrays:
        if _is_torch(a) and a.is_cuda:
            return ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    return None


def _empty_like_kind(ref, shape):
    if _is_torch(ref):
        return torch.empty(shape, dtype=torch.float32, device=ref.device)
    return np.empty(shape, np.float32)


def _zeros_like_kind(ref, shape):
    if _is_torch(ref):
        return torch.zeros(shape, dtype=torch.float32, device=ref.device)
    return np.zeros(shape, np.float32)


def _numel(a):
    return a.numel() if _is_torch(a) else a.size


# ----------------------------------------------------------------- eigen

def evals3_symmetric(mats, n=None, device=0):
    """Eigenvalues (ascending) of n glm::mat3 tensors -> new (n, 3) array,
    on the host for host input and on the device for device input, as the
    reference (eigen.h:896)."""
    mats = _check_f32(mats, "mats")
    n = _numel(mats) // 9 if n is None else int(n)
    out = _empty_like_kind(mats, (n, 3))
    call("tvgb_evals3_symmetric", _ptr(mats), n, _ptr(out), _stream_for(mats))
    return out


def evecs3spherical_symmetric(mats, lambdas, n=None, device=0):
    """(theta, phi) of the three eigenvectors -> new (n, 6) array (eigen.h:945)."""
    mats = _check_f32(mats, "mats")
    lambdas = _check_f32(lambdas, "lambdas")
    n = _numel(mats) // 9 if n is None else int(n)
    out = _empty_like_kind(mats, (n, 6))
    call("tvgb_evecs3spherical_symmetric", _ptr(mats), _ptr(lambdas), n, _ptr(out), _stream_for(mats, lambdas))
    return out


def evals2_symmetric(mats, n=None, device=0):
    """Eigenvalues (ascending) of n 2x2 tensors [a,b,b,c] -> new (n, 2) (eigen.h:769)."""
    mats = _check_f32(mats, "mats")
    n = _numel(mats) // 4 if n is None else int(n)
    out = _empty_like_kind(mats, (n, 2))
    call("tvgb_evals2_symmetric", _ptr(mats), n, _ptr(out), _stream_for(mats))
    return out


def evecs2polar_symmetric(mats, evals, n=None, device=0):
    """Eigenvector angles theta0, theta1 -> new (n, 2) (eigen.h:828)."""
    mats = _check_f32(mats, "mats")
    evals = _check_f32(evals, "evals")
    n = _numel(mats) // 4 if n is None else int(n)
    out = _empty_like_kind(mats, (n, 2))
    call("tvgb_evecs2polar_symmetric", _ptr(mats), _ptr(evals), n, _ptr(out), _stream_for(mats, evals))
    return out


def eig3(mats, layout="mat3", evecs="cartesian", precise=False, want_evals=True):
    """Fused 3x3 solve.  layout: 'mat3' (n,9) | 'sym6' (n,6) | 'planes' (6,n).
    evecs: None | 'cartesian' (n,3,3 rows e0,e1,e2) | 'spherical' (n,6).
    Returns (evals (n,3) or None, evecs or None, number refined in FP64)."""
    mats = _check_f32(mats, "mats")
    L = LAYOUTS[layout]
    n = _numel(mats) // (9 if L == LAYOUT_MAT3 else 6)
    ev = _empty_like_kind(mats, (n, 3)) if want_evals else None
    fmt = EVECS[evecs]
    vec = None
    if fmt == EVEC_CARTESIAN:
        vec = _empty_like_kind(mats, (n, 3, 3))
    elif fmt == EVEC_SPHERICAL:
        vec = _empty_like_kind(mats, (n, 6))
    nref = ctypes.c_size_t(0)
    call("tvgb_eig3", _ptr(mats), L, n, _ptr(ev), _ptr(vec), fmt, EIG_PRECISE if precise else EIG_PARITY,
         ctypes.byref(nref) if precise else None, _stream_for(mats))
    return ev, vec, int(nref.value)


# ----------------------------------------------------------------- filters / structure tensor

def gaussian_filter3d(source, width=None, height=None, depth=None, sigma_w=1.0, sigma_h=1.0, sigma_d=1.0):
    """Valid separable Gaussian of one scalar volume (filter.h:401).  source
    is (depth, height, width) (width fastest).  Returns the new volume."""
    source = _check_f32(source, "source")
    if width is None:
        depth, height, width = source.shape
    dims = (ctypes.c_uint * 3)()
    k = [int(np.ceil(np.float32(6.0) * np.float32(s))) | 1 for s in (sigma_w, sigma_h, sigma_d)]
    out = _empty_like_kind(source, _valid(depth - k[2] + 1, height - k[1] + 1, width - k[0] + 1))
    call("tvgb_gaussian_filter3d", _ptr(source), width, height, depth, sigma_w, sigma_h, sigma_d, _ptr(out),
         dims, _stream_for(source))
    return out


def gaussian_convolve2(source, sigma1, sigma2=None):
    """Valid separable 2D Gaussian (filter.h:305), window (unsigned)(6 sigma).
    source (height, width); sigma1 along width, sigma2 along height."""
    source = _check_f32(source, "source")
    sigma2 = sigma1 if sigma2 is None else sigma2
    sy, sx = source.shape
    kw, kh = int(np.float32(6.0) * np.float32(sigma1)), int(np.float32(6.0) * np.float32(sigma2))
    out = _empty_like_kind(source, _valid(sy - kh + 1, sx - kw + 1))
    dims = (ctypes.c_uint * 2)()
    call("tvgb_gaussian_convolve2", _ptr(source), sx, sy, sigma1, sigma2, _ptr(out), dims, _stream_for(source))
    return out


def _valid(*dims):
    """Output extent of a valid convolution, clamped at 0 so that an input
    smaller than the window reaches the library, which reports it."""
    return tuple(max(int(d), 0) for d in dims)


def _ksize3(sigma):
    k = int(np.ceil(np.float32(6.0) * np.float32(sigma)))
    return k + 1 if k % 2 == 0 else k


def structure_tensor3(volume, sigma, mode="same", layout="planes"):
    """Gradient -> outer product -> separable Gaussian of a (s0,s1,s2) volume.
    mode 'valid' (the reference's gaussian_filter3d) or 'same'.
    layout 'planes' -> (6, s0', s1', s2'); 'sym6' -> (s0',s1',s2',6); 'mat3' -> (...,3,3)."""
    volume = _check_f32(volume, "volume")
    s0, s1, s2 = volume.shape
    m = 0 if mode == "valid" else 1
    K = _ksize3(sigma)
    d = _valid(s0 - K + 1, s1 - K + 1, s2 - K + 1) if m == 0 else (s0, s1, s2)
    L = LAYOUTS[layout]
    shape = (6,) + d if L == LAYOUT_SYM6_PLANES else (d + (6,) if L == LAYOUT_SYM6 else d + (3, 3))
    out = _empty_like_kind(volume, shape)
    dims = (ctypes.c_uint * 3)()
    call("tvgb_structure_tensor3", _ptr(volume), s0, s1, s2, sigma, m, _ptr(out), L, dims, _stream_for(volume))
    return out


def structure_tensor2(image, sigma, mode="same"):
    """np.gradient(edge_order=2) -> [a,b,b,c] -> gaussian_convolve2 per
    component.  Returns (s0', s1', 4)."""
    image = _check_f32(image, "image")
    s0, s1 = image.shape
    m = 0 if mode == "valid" else 1
    K = int(np.float32(6.0) * np.float32(sigma))
    d = _valid(s0 - K + 1, s1 - K + 1) if m == 0 else (s0, s1)
    out = _empty_like_kind(image, d + (4,))
    dims = (ctypes.c_uint * 2)()
    call("tvgb_structure_tensor2", _ptr(image), s0, s1, sigma, m, _ptr(out), dims, _stream_for(image))
    return out


# ----------------------------------------------------------------- voting

def tensorvote3(input_field, output_field, s0, s1, s2, sigma, sigma2, w, power, device=0, stick=True, plate=True,
                samples=20, is_atv=False):
    """tira::cuda::tensorvote3 (tensorvote.h:2817): input/output are n
    glm::mat3 (9 floats per voxel); output_field is written in place."""
    input_field = _check_f32(input_field, "input_field")
    if not (_is_torch(output_field) or (isinstance(output_field, np.ndarray) and output_field.dtype == np.float32
                                        and output_field.flags.c_contiguous)):
        raise TypeError("output_field must be a C-contiguous float32 array or CUDA tensor")
    call("tvgb_tensorvote3", _ptr(input_field), _ptr(output_field), s0, s1, s2, sigma, sigma2, w, power, device,
         int(stick), int(plate), samples, int(is_atv), _stream_for(input_field, output_field))
    return output_field


def tensorvote(t_out, t_in, sigma1, sigma2, power, w, shape0, shape1, stick=True, plate=True, samples=10,
               is_atv=False, debug=False):
    """tira::cuda::tensorvote (tensorvote.h:2201): 2D TK / ATV on [a,b,b,c]."""
    t_in = _check_f32(t_in, "t_in")
    call("tvgb_tensorvote", _ptr(t_out), _ptr(t_in), sigma1, sigma2, int(power), w, shape0, shape1, int(stick),
         int(plate), samples, int(is_atv), _stream_for(t_in, t_out))
    return t_out


def tensorvote_prebuilt(t_out, t_in, host_nb, nb_count, sigma1, sigma2, power, w, shape0, shape1, stick=True,
                        plate=True, samples=10):
    """tira::cuda::tensorvote_prebuilt (tensorvote.h:2237): 2D TK with a
    caller-built Neighbor2D table (NB2_DTYPE records)."""
    t_in = _check_f32(t_in, "t_in")
    nb = np.ascontiguousarray(host_nb)
    call("tvgb_tensorvote_prebuilt", _ptr(t_out), _ptr(t_in), ctypes.c_void_p(nb.ctypes.data), int(nb_count), sigma1,
         sigma2, int(power), w, shape0, shape1, int(stick), int(plate), samples, _stream_for(t_in, t_out))
    return t_out


def build_neighbors2d(w, sigma1, sigma2, power, samples, stick=True, plate=True):
    """tira::cpu::build_neighbors2d (tensorvote.h:1223) -> NB2_DTYPE array."""
    out = np.zeros(max(w, 0) ** 2, NB2_DTYPE)
    cnt = ctypes.c_int(0)
    call("tvgb_build_neighbors2d", int(w), sigma1, sigma2, power, samples, int(stick), int(plate),
         ctypes.c_void_p(out.ctypes.data), ctypes.byref(cnt))
    return out[: cnt.value]


def build_neighbors3d(w, sigma1, sigma2=0.0):
    """tira::cpu::build_neighbors3d (tensorvote.h:1411; sigma = (sigma1,
    sigma2)) -> NB3_DTYPE array of w**3 records, dw outermost."""
    out = np.zeros(max(w, 0) ** 3, NB3_DTYPE)
    cnt = ctypes.c_int(0)
    call("tvgb_build_neighbors3d", int(w), sigma1, sigma2, ctypes.c_void_p(out.ctypes.data), ctypes.byref(cnt))
    return out[: cnt.value]


def sticknorm3(sigma1, sigma2, power):
    return _lib.lib().tvgb_sticknorm3(sigma1, sigma2, power)


def make_params(sigma1, sigma2=0.0, w=0, power=1, samples=20, stick=True, plate=True, ball=False, is_atv=False,
                parity=True):
    return Vote3Params(float(sigma1), float(sigma2), int(w), int(power), int(samples), int(stick), int(plate),
                       int(ball), int(is_atv), int(parity))


def vote3(field, sigma1, sigma2=0.0, w=0, power=1, samples=20, stick=True, plate=True, ball=False, is_atv=False,
          parity=True, layout="mat3", out_layout="mat3", evals=False, evecs=None, out=True):
    """Extended 3D vote (tvgb_vote3).  field: (s0,s1,s2,3,3) / (s0,s1,s2,6) /
    (6,s0,s1,s2) per `layout`.  Returns (voted field, evals, evecs)."""
    field = _check_f32(field, "field")
    L = LAYOUTS[layout]
    dims = tuple(field.shape[1:4]) if L == LAYOUT_SYM6_PLANES else tuple(field.shape[:3])
    s0, s1, s2 = dims
    OL = LAYOUTS[out_layout]
    oshape = (6,) + dims if OL == LAYOUT_SYM6_PLANES else (dims + (6,) if OL == LAYOUT_SYM6 else dims + (3, 3))
    o = _empty_like_kind(field, oshape) if out else None
    ev = _empty_like_kind(field, dims + (3,)) if evals else None
    fmt = EVECS[evecs]
    vec = None
    if fmt == EVEC_CARTESIAN:
        vec = _empty_like_kind(field, dims + (3, 3))
    elif fmt == EVEC_SPHERICAL:
        vec = _empty_like_kind(field, dims + (6,))
    p = make_params(sigma1, sigma2, w, power, samples, stick, plate, ball, is_atv, parity)
    call("tvgb_vote3", _ptr(field), L, s0, s1, s2, ctypes.byref(p), _ptr(o), OL, _ptr(ev), _ptr(vec), fmt,
         _stream_for(field))
    return o, ev, vec


def pipeline3(volume, sigma_st, sigma1, sigma2=0.0, w=0, power=1, samples=20, st_mode="same", stick=True,
              plate=True, ball=False, parity=True, out_layout="planes", out=True, evals=True, evecs="cartesian",
              outputs=None, is_atv=False):
    """Structure tensor -> vote -> fused eigendecomposition of a scalar
    volume (tvgb_pipeline3).  `outputs` may pass preallocated
    (out, evals, evecs) arrays (host or device).  Returns that triple."""
    volume = _check_f32(volume, "volume")
    s0, s1, s2 = volume.shape
    m = 0 if st_mode == "valid" else 1
    K = _ksize3(sigma_st)
    dims = _valid(s0 - K + 1, s1 - K + 1, s2 - K + 1) if m == 0 else (s0, s1, s2)
    OL = LAYOUTS[out_layout]
    fmt = EVECS[evecs]
    if outputs is None:
        oshape = (6,) + dims if OL == LAYOUT_SYM6_PLANES else (dims + (6,) if OL == LAYOUT_SYM6 else dims + (3, 3))
        o = _empty_like_kind(volume, oshape) if out else None
        ev = _empty_like_kind(volume, dims + (3,)) if evals else None
        vec = None
        if fmt == EVEC_CARTESIAN:
            vec = _empty_like_kind(volume, dims + (3, 3))
        elif fmt == EVEC_SPHERICAL:
            vec = _empty_like_kind(volume, dims + (6,))
    else:
        o, ev, vec = outputs
    p = make_params(sigma1, sigma2, w, power, samples, stick, plate, ball, is_atv, parity)
    odims = (ctypes.c_uint * 3)()
    call("tvgb_pipeline3", _ptr(volume), s0, s1, s2, sigma_st, m, ctypes.byref(p), _ptr(o), OL, _ptr(ev), _ptr(vec),
         fmt, odims, _stream_for(volume, o, ev, vec))
    return o, ev, vec


def launch_count():
    """Kernel launches issued by libtvgb in this process."""
    return int(_lib.lib().tvgb_launch_count())


def memory_stats(reset_peak=False):
    """(bytes, peak bytes) of device memory libtvgb holds in its own
    temporaries (tvgb_memory_stats); caller arrays are not counted."""
    cur, peak = ctypes.c_ulonglong(0), ctypes.c_ulonglong(0)
    call("tvgb_memory_stats", ctypes.byref(cur), ctypes.byref(peak), int(bool(reset_peak)))
    return int(cur.value), int(peak.value)


__all__ = [
    "TvgbError", "NB2_DTYPE", "evals3_symmetric", "evecs3spherical_symmetric", "evals2_symmetric",
    "evecs2polar_symmetric", "eig3", "gaussian_filter3d", "gaussian_convolve2", "structure_tensor3",
    "structure_tensor2", "tensorvote3", "tensorvote", "tensorvote_prebuilt", "build_neighbors2d", "build_neighbors3d",
    "NB3_DTYPE", "sticknorm3",
    "make_params", "vote3", "pipeline3", "launch_count", "memory_stats",
]
