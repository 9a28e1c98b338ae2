"""NumPy bindings of the CPU oracle (oracle/tvoracle_*.c) and, where it was
built in this checkout, of the reference's own CPU code (oracle/_ref).

TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this module as the checker / the timed CPU reference.
The product package (tiralib_gb300) never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtvoracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libtiraref.so")

_P = ctypes.c_void_p
_U = ctypes.c_uint
_I = ctypes.c_int
_F = ctypes.c_float
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_LL = ctypes.c_longlong


def build(reference_root=None):
    """Compile the oracle (always) and the reference CPU library (when the
    reference checkout is given and present)."""
    subprocess.check_call([os.path.join(HERE, "build_oracle.sh")])
    if reference_root and os.path.isdir(reference_root):
        subprocess.check_call([os.path.join(HERE, "build_ref.sh"), reference_root])


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class _Lib:
    def __init__(self, path, sigs):
        self.path = path
        self.lib = ctypes.CDLL(path)
        for name, (res, args) in sigs.items():
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args


_ORACLE_SIGS = {
    "or_mlp_param_count": (_I, []),
    "or_mlp_loss_grad": (_D, [_P, _P, _P, _I, _I, _P, _P]),
    "or_surrogate_target": (None, [_P, _P, _I, _P]),
    "or_evals2": (None, [_P, _SZ, _P]),
    "or_evecs2polar": (None, [_P, _P, _SZ, _P]),
    "or_evals3": (None, [_P, _SZ, _P]),
    "or_evecs3spherical": (None, [_P, _P, _SZ, _P]),
    "or_evecs3cart": (None, [_P, _P, _SZ, _P]),
    "or_eig3_f64_batch": (None, [_P, _SZ, _P, _P]),
    "or_eig3_batch_threads": (None, [_P, _SZ, _P, _P, _I]),
    "or_ksize3": (_U, [_F]),
    "or_ksize2": (_U, [_F]),
    "or_gaussian1d": (None, [_U, _F, _P]),
    "or_gaussian_convolve3": (None, [_P, _U, _U, _U, _F, _F, _F, _P, _P]),
    "or_gaussian_convolve2": (None, [_P, _U, _U, _F, _P, _P]),
    "or_gradient3": (None, [_P, _U, _U, _U, _I, _P]),
    "or_structure_tensor3": (None, [_P, _U, _U, _U, _F, _I, _P, _P]),
    "or_structure_tensor2": (None, [_P, _U, _U, _F, _I, _P, _P]),
    "or_sticknorm3": (_F, [_F, _F, _U]),
    "or_tensorvote3": (None, [_P, _P, _U, _U, _U, _F, _F, _U, _U, _I, _I, _U, _I]),
    "or_tensorvote3_sel": (None, [_P, _P, _U, _U, _U, _F, _F, _U, _U, _I, _I, _U, _I, _P, _LL, _I]),
    "or_tensorvote3_f64": (None, [_P, _P, _U, _U, _U, _D, _D, _U, _U, _I, _I, _I, _P, _LL, _I]),
    "or_build_neighbors2d": (_I, [_I, _F, _F, _U, _U, _I, _I, _P]),
    "or_tensorvote2": (None, [_P, _P, _F, _F, _I, _U, _U, _U, _I, _I, _U, _I]),
    "or_tensorvote2_prebuilt": (None, [_P, _P, _P, _I, _F, _F, _I, _U, _U, _U, _I, _I, _U]),
}

_REF_SIGS = {
    "ref_evals3": (None, [_P, _SZ, _P]),
    "ref_evecs3spherical": (None, [_P, _P, _SZ, _P]),
    "ref_evecs3cart": (None, [_P, _P, _SZ, _P]),
    "ref_evals2": (None, [_P, _SZ, _P]),
    "ref_evecs2polar": (None, [_P, _P, _SZ, _P]),
    "ref_gaussian1d": (None, [_U, _F, _P]),
    "ref_gaussian_convolve3": (None, [_P, _U, _U, _U, _F, _F, _F, _P, _P]),
    "ref_gaussian_convolve2": (None, [_P, _U, _U, _F, _P, _P]),
    "ref_build_neighbors2d": (_I, [_I, _F, _F, _U, _U, _I, _I, _P]),
    "ref_sizeof_neighbor2d": (_I, []),
    "ref_build_neighbors3d": (_I, [_I, _F, _F, _P]),
    "ref_sizeof_neighbor3d": (_I, []),
    "ref_tensorvote2": (None, [_P, _P, _F, _F, _I, _U, _U, _U, _I, _I, _U, _I]),
    "ref_tensorvote3": (None, [_P, _P, _U, _U, _U, _F, _F, _U, _U, _I, _I, _U, _I]),
    "ref_sticknorm3": (_D, [_F, _F, _U]),
}

_oracle = None
_ref = None


def lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(LIB_PATH):
            build()
        _oracle = _Lib(LIB_PATH, _ORACLE_SIGS).lib
    return _oracle


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        _ref = _Lib(REF_PATH, _REF_SIGS).lib
    return _ref


# ---------------------------------------------------------------- eigen

def evals3(m9, use_ref=False):
    m9 = _f32(m9).reshape(-1, 9)
    out = np.empty((m9.shape[0], 3), np.float32)
    (ref().ref_evals3 if use_ref else lib().or_evals3)(_ptr(m9), m9.shape[0], _ptr(out))
    return out


def evecs3spherical(m9, ev3, use_ref=False):
    m9 = _f32(m9).reshape(-1, 9)
    ev3 = _f32(ev3).reshape(-1, 3)
    out = np.empty((m9.shape[0], 6), np.float32)
    (ref().ref_evecs3spherical if use_ref else lib().or_evecs3spherical)(_ptr(m9), _ptr(ev3), m9.shape[0], _ptr(out))
    return out


def evecs3cart(m9, ev3, use_ref=False):
    m9 = _f32(m9).reshape(-1, 9)
    ev3 = _f32(ev3).reshape(-1, 3)
    out = np.empty((m9.shape[0], 3, 3), np.float32)
    (ref().ref_evecs3cart if use_ref else lib().or_evecs3cart)(_ptr(m9), _ptr(ev3), m9.shape[0], _ptr(out))
    return out


def evals2(m4, use_ref=False):
    m4 = _f32(m4).reshape(-1, 4)
    out = np.empty((m4.shape[0], 2), np.float32)
    (ref().ref_evals2 if use_ref else lib().or_evals2)(_ptr(m4), m4.shape[0], _ptr(out))
    return out


def evecs2polar(m4, ev2, use_ref=False):
    m4 = _f32(m4).reshape(-1, 4)
    ev2 = _f32(ev2).reshape(-1, 2)
    out = np.empty((m4.shape[0], 2), np.float32)
    (ref().ref_evecs2polar if use_ref else lib().or_evecs2polar)(_ptr(m4), _ptr(ev2), m4.shape[0], _ptr(out))
    return out


def eig3_threads(m9, threads):
    """eigen.h's FP32 solve (eigenvalues + cartesian eigenvectors) over a
    batch, OpenMP over matrices."""
    m9 = _f32(m9).reshape(-1, 9)
    ev = np.empty((m9.shape[0], 3), np.float32)
    vec = np.empty((m9.shape[0], 3, 3), np.float32)
    lib().or_eig3_batch_threads(_ptr(m9), m9.shape[0], _ptr(ev), _ptr(vec), threads)
    return ev, vec


def eig3_f64(s6):
    """FP64 Jacobi: s6 (n, 6) xx,xy,xz,yy,yz,zz -> (evals (n,3), evecs (n,3,3) rows)."""
    s6 = np.ascontiguousarray(s6, dtype=np.float64).reshape(-1, 6)
    ev = np.empty((s6.shape[0], 3))
    vec = np.empty((s6.shape[0], 3, 3))
    lib().or_eig3_f64_batch(_ptr(s6), s6.shape[0], _ptr(ev), _ptr(vec))
    return ev, vec


# ---------------------------------------------------------------- filter

def gaussian1d(ksize, sigma, use_ref=False):
    out = np.empty(ksize, np.float32)
    (ref().ref_gaussian1d if use_ref else lib().or_gaussian1d)(ksize, sigma, _ptr(out))
    return out


def gaussian_convolve3(vol, sw, sh, sd, use_ref=False):
    """vol indexed [z, y, x]; returns the valid convolution [z', y', x']."""
    vol = _f32(vol)
    sz, sy, sx = vol.shape
    out = np.empty(vol.size, np.float32)
    dims = np.zeros(3, np.uint32)
    (ref().ref_gaussian_convolve3 if use_ref else lib().or_gaussian_convolve3)(
        _ptr(vol), sx, sy, sz, sw, sh, sd, _ptr(out), _ptr(dims))
    ox, oy, oz = (int(d) for d in dims)
    return out[: ox * oy * oz].reshape(oz, oy, ox)


def gaussian_convolve2(img, sigma, use_ref=False):
    img = _f32(img)
    sy, sx = img.shape
    out = np.empty(img.size, np.float32)
    dims = np.zeros(2, np.uint32)
    (ref().ref_gaussian_convolve2 if use_ref else lib().or_gaussian_convolve2)(
        _ptr(img), sx, sy, sigma, _ptr(out), _ptr(dims))
    ox, oy = (int(d) for d in dims)
    return out[: ox * oy].reshape(oy, ox)


def gradient3(vol, axis):
    vol = _f32(vol)
    out = np.empty_like(vol)
    s0, s1, s2 = vol.shape
    lib().or_gradient3(_ptr(vol), s0, s1, s2, axis, _ptr(out))
    return out


def structure_tensor3(vol, sigma, mode):
    """-> (6, s0', s1', s2') component planes xx, xy, xz, yy, yz, zz."""
    vol = _f32(vol)
    s0, s1, s2 = vol.shape
    K = lib().or_ksize3(sigma)
    R = K // 2
    if mode == 0:
        n_out = (s0 - 2 * R) * (s1 - 2 * R) * (s2 - 2 * R)
    else:
        n_out = s0 * s1 * s2
    out = np.empty(6 * n_out, np.float32)
    dims = np.zeros(3, np.uint32)
    lib().or_structure_tensor3(_ptr(vol), s0, s1, s2, sigma, mode, _ptr(out), _ptr(dims))
    return out.reshape(6, int(dims[0]), int(dims[1]), int(dims[2]))


def structure_tensor2(img, sigma, mode):
    """-> (s0', s1', 4) [a, b, b, c]."""
    img = _f32(img)
    s0, s1 = img.shape
    out = np.empty((s0 * s1 * 4,), np.float32)
    dims = np.zeros(2, np.uint32)
    lib().or_structure_tensor2(_ptr(img), s0, s1, sigma, mode, _ptr(out), _ptr(dims))
    oy, ox = int(dims[0]), int(dims[1])
    return out[: oy * ox * 4].reshape(oy, ox, 4)


# ---------------------------------------------------------------- voting

def sticknorm3(s1, s2, p, use_ref=False):
    return (ref().ref_sticknorm3 if use_ref else lib().or_sticknorm3)(s1, s2, p)


def tensorvote3(in9, sigma1, sigma2, w, power, stick=True, plate=True, samples=20, is_atv=False,
                use_ref=False):
    """in9 (s0, s1, s2, 3, 3) float32 -> (s0, s1, s2, 3, 3) float32."""
    in9 = _f32(in9)
    s0, s1, s2 = in9.shape[:3]
    out = np.zeros_like(in9)
    fn = ref().ref_tensorvote3 if use_ref else lib().or_tensorvote3
    fn(_ptr(in9), _ptr(out), s0, s1, s2, sigma1, sigma2, w, power, int(stick), int(plate), samples, int(is_atv))
    return out


def tensorvote3_receivers(in9, receivers, sigma1, sigma2, w, power, stick=True, plate=True, samples=20,
                          is_atv=False, threads=1):
    """Vote only the listed flat receiver indices (OpenMP over receivers)."""
    in9 = _f32(in9)
    s0, s1, s2 = in9.shape[:3]
    out = np.zeros_like(in9)
    rec = np.ascontiguousarray(receivers, dtype=np.int64)
    lib().or_tensorvote3_sel(_ptr(in9), _ptr(out), s0, s1, s2, sigma1, sigma2, w, power, int(stick), int(plate),
                             samples, int(is_atv), _ptr(rec), rec.size, threads)
    return out


def tensorvote3_f64(in9, sigma1, sigma2, w, power, stick=True, plate=True, ball=False, receivers=None, threads=1):
    """FP64 precision oracle -> (s0, s1, s2, 6) float64 (xx, xy, xz, yy, yz, zz)."""
    in9 = _f32(in9)
    s0, s1, s2 = in9.shape[:3]
    out = np.zeros((s0, s1, s2, 6))
    rec = None if receivers is None else np.ascontiguousarray(receivers, dtype=np.int64)
    lib().or_tensorvote3_f64(_ptr(in9), _ptr(out), s0, s1, s2, sigma1, sigma2, w, power, int(stick), int(plate),
                             int(ball), _ptr(rec) if rec is not None else None, 0 if rec is None else rec.size, threads)
    return out


NB2_DTYPE = np.dtype([
    ("du", np.int32), ("dv", np.int32),
    ("dx", np.float32), ("dy", np.float32),
    ("c1", np.float32), ("c2", np.float32),
    ("Ra", np.float32), ("Rb", np.float32), ("Rc", np.float32),
    ("Va", np.float32), ("Vb", np.float32), ("Vc", np.float32),
])

NB3_DTYPE = np.dtype([
    ("du", np.int32), ("dv", np.int32), ("dw", np.int32),
    ("d", np.float32, (3,)),
    ("c1", np.float32), ("c2", np.float32),
])


def build_neighbors2d(w, s1, s2, power, samples, stick=True, plate=True, use_ref=False):
    out = np.zeros(w * w, NB2_DTYPE)
    fn = ref().ref_build_neighbors2d if use_ref else lib().or_build_neighbors2d
    n = fn(w, s1, s2, power, samples, int(stick), int(plate), _ptr(out))
    return out[:n]


def build_neighbors3d_ref(w, s1, s2):
    """The compiled reference's tira::cpu::build_neighbors3d table (fixtures only)."""
    assert ref().ref_sizeof_neighbor3d() == NB3_DTYPE.itemsize
    out = np.zeros(w ** 3, NB3_DTYPE)
    n = ref().ref_build_neighbors3d(w, s1, s2, _ptr(out))
    return out[:n]


def tensorvote2(in4, sigma1, sigma2, power, w, stick=True, plate=True, samples=10, is_atv=False, use_ref=False):
    """in4 (s0, s1, 4) [a, b, b, c] float32 -> same layout."""
    in4 = _f32(in4)
    s0, s1 = in4.shape[:2]
    out = np.zeros_like(in4)
    fn = ref().ref_tensorvote2 if use_ref else lib().or_tensorvote2
    fn(_ptr(out), _ptr(in4), sigma1, sigma2, power, w, s0, s1, int(stick), int(plate), samples, int(is_atv))
    return out


def tensorvote2_prebuilt(in4, nb, sigma1, sigma2, power, w, stick=True, plate=True, samples=10):
    in4 = _f32(in4)
    nb = np.ascontiguousarray(nb, NB2_DTYPE)
    s0, s1 = in4.shape[:2]
    out = np.zeros_like(in4)
    lib().or_tensorvote2_prebuilt(_ptr(out), _ptr(in4), _ptr(nb), nb.size, sigma1, sigma2, power, w, s0, s1,
                                  int(stick), int(plate), samples)
    return out


# ---------------------------------------------------------------- consumers of a voted 2D field
# NumPy / SciPy restatements of python/tira/tensors_lib/reconstruct.py and
# metrics.py (the reference is itself NumPy; these are the checker's copy of
# its rules, pinned against tests/golden/reconstruct_reference.npz).

def stick_saliency(T):
    """reconstruct.py:14: |lambda|max - |lambda|min per pixel of (H, W, 2, 2)."""
    mags = np.sort(np.abs(np.linalg.eigvalsh(T)), axis=-1)
    return mags[..., 1] - mags[..., 0]


def otsu_threshold(values):
    """reconstruct.py:34: Otsu on a 256-bin histogram over [0, max]."""
    vmax = float(values.max())
    if vmax <= 0:
        return 0.0
    hist, edges = np.histogram(values, bins=256, range=(0.0, vmax))
    hist = hist.astype(np.float64)
    if hist.sum() == 0:
        return 0.0
    centers = (edges[:-1] + edges[1:]) / 2.0
    w0 = np.cumsum(hist)
    w1 = hist.sum() - w0
    cum = np.cumsum(hist * centers)
    with np.errstate(divide="ignore", invalid="ignore"):
        mu0 = np.where(w0 > 0, cum / w0, 0.0)
        mu1 = np.where(w1 > 0, (cum[-1] - cum) / w1, 0.0)
    return float(centers[np.argmax(w0 * w1 * (mu0 - mu1) ** 2)])


def saliency_threshold(T, fill=False, threshold="otsu", close_radius=0):
    """reconstruct.py:66: saliency > threshold, optionally closed and hole-filled."""
    from scipy.ndimage import binary_closing, binary_fill_holes
    s = stick_saliency(T)
    thr = otsu_threshold(s.ravel()) if threshold == "otsu" else float(threshold)
    b = s > thr
    if not fill:
        return b
    if close_radius > 0:
        b = binary_closing(b, structure=np.ones((2 * close_radius + 1,) * 2, bool))
    return binary_fill_holes(b)


def simf(A, B):
    """metrics.py:37: mean over pixels of ||A - alpha B||_F, alpha = <A,B>/<B,B>."""
    A = np.asarray(A, np.float64)
    B = np.asarray(B, np.float64)
    den = np.sum(B * B)
    alpha = 0.0 if den < 1e-8 else np.sum(A * B) / den
    return float(np.mean(np.linalg.norm(A - alpha * B, axis=(-2, -1))))


# ---------------------------------------------------------------- plate / ball surrogate (tvoracle_mlp.c)

def mlp_param_count():
    return int(lib().or_mlp_param_count())


def mlp_loss_grad(params, X, T, quant=True):
    """FP64 loss and gradient of the surrogate MLP over a batch: X (B, 8)
    inputs, T (B, 8) targets (first 6 used).  quant: False (exact), True / 1
    (BF16 weights and layer inputs, GELU exact then rounded) or 2 (as 1 with
    the GELU in packed BF16 arithmetic, as the GPU trains and votes).
    Returns (loss, grad, Y)."""
    P = np.ascontiguousarray(params, np.float64)
    X = np.ascontiguousarray(X, np.float64).reshape(-1, 8)
    T = np.ascontiguousarray(T, np.float64).reshape(-1, 8)
    g = np.zeros(mlp_param_count())
    Y = np.zeros_like(T)
    loss = lib().or_mlp_loss_grad(_ptr(P), _ptr(X), _ptr(T), X.shape[0], int(quant), _ptr(g), _ptr(Y))
    return float(loss), g, Y


def surrogate_target(direction, normal, plate):
    """The plain orientation integral (64 orientations; sigma2 = 0, power 1,
    Gaussian factored out) for one offset direction and plate normal:
    (xx, xy, xz, yy, yz, zz)."""
    d = np.ascontiguousarray(direction, np.float64)
    nn = np.ascontiguousarray(normal, np.float64)
    F = np.zeros(6)
    lib().or_surrogate_target(_ptr(d), _ptr(nn), int(plate), _ptr(F))
    return F
