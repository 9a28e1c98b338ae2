"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the tiralib reference tree is available:

    python tests/golden/make_golden.py [<path to the tiralib checkout> [nb3]]

The path defaults to $TIRALIB_REFERENCE, else a `reference` directory beside
this repository; `nb3` regenerates only the Neighbor3D tables.

Three reference sources are used, and nothing else:
  * tiralib's own C++ CPU functions, compiled unmodified by oracle/build_ref.sh
    (glm / Boost replaced by the stand-ins in oracle/shim) -> oracle/_ref;
  * tiralib's NumPy 2D implementation python/tira/tensors.py (tk_vote2 at
    tensors.py:265, atv_vote2 at tensors.py:164), imported with its unused
    plotting / skeleton dependencies stubbed out;
  * tiralib's field consumers python/tira/tensors_lib/reconstruct.py
    (stick_saliency, _otsu_threshold, saliency_threshold) and metrics.py
    (simf), imported as they are (NumPy / SciPy only).
The field generators follow the reference tests' recipes
(python/tira/tests/test_cpu_gpu.py:41-75, test_cuda_vs_python.py:48-91,
test_analytical_vs_numerical.py:19-36) at smaller sizes so the fixtures
stay small.  Outputs: one .npz per group.
"""
import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402


def load_reference_module(ref_root, rel, name):
    spec = importlib.util.spec_from_file_location(name, os.path.join(ref_root, rel))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_reference_tensors(ref_root):
    """Import python/tira/tensors.py with its optional imports stubbed."""
    pkg = types.ModuleType("tensors_lib")
    pkg.__path__ = []
    sys.modules["tensors_lib"] = pkg
    for sub in ("phantoms", "noise", "metrics", "plots"):
        m = types.ModuleType("tensors_lib." + sub)
        sys.modules["tensors_lib." + sub] = m
        setattr(pkg, sub, m)
    sk = types.ModuleType("skimage")
    skm = types.ModuleType("skimage.morphology")
    skm.skeletonize = lambda *a, **k: None
    sk.morphology = skm
    sys.modules["skimage"] = sk
    sys.modules["skimage.morphology"] = skm
    path = os.path.join(ref_root, "python", "tira", "tensors.py")
    spec = importlib.util.spec_from_file_location("tira_ref_tensors", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# field generators after the reference tests' recipes ------------------------

def stick_field(H, W, seed):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, np.pi, (H, W)); l1 = rng.uniform(0.5, 1.0, (H, W))
    vx, vy = np.cos(ang), np.sin(ang)
    T = np.zeros((H, W, 2, 2))
    T[..., 0, 0] = l1 * vx * vx; T[..., 0, 1] = l1 * vx * vy; T[..., 1, 0] = l1 * vx * vy; T[..., 1, 1] = l1 * vy * vy
    return T


def ball_field(H, W, seed):
    rng = np.random.default_rng(seed)
    lam = rng.uniform(0.3, 1.0, (H, W))
    T = np.zeros((H, W, 2, 2)); T[..., 0, 0] = lam; T[..., 1, 1] = lam
    return T


def mixed_field(H, W, seed):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, np.pi, (H, W)); l1 = rng.uniform(0.5, 1.0, (H, W)); l0 = rng.uniform(0.0, 0.4, (H, W))
    vx, vy = np.cos(ang), np.sin(ang)
    T = np.zeros((H, W, 2, 2))
    T[..., 0, 0] = l0 + (l1 - l0) * vx * vx; T[..., 0, 1] = (l1 - l0) * vx * vy
    T[..., 1, 0] = T[..., 0, 1]; T[..., 1, 1] = l0 + (l1 - l0) * vy * vy
    return T


def random_spd3(shape, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=shape + (3, 3))
    return (scale * (A @ np.swapaxes(A, -1, -2))).astype(np.float32)


def flat4(T):
    H, W = T.shape[:2]
    return np.ascontiguousarray(T.reshape(H, W, 4), dtype=np.float32)


def main(ref_root):
    O.build(ref_root)
    assert O.ref_available(), "reference CPU library did not build"
    ts = load_reference_tensors(ref_root)

    # --- 2D: the reference NumPy implementation (FP64) ---------------------
    fx = {}
    cases = [(5.0, 0.0, 1, 20), (5.0, 2.0, 1, 20), (5.0, 2.0, 3, 20), (3.0, 1.0, 1, 0)]
    fields = {"stick": stick_field(24, 24, 0), "ball": ball_field(24, 24, 0), "mixed": mixed_field(24, 24, 0)}
    for fname, T in fields.items():
        T32 = T.astype(np.float32).astype(np.float64)      # the float32 field both sides see
        fx[f"in_{fname}"] = flat4(T32)
        for (s1, s2, p, N) in cases:
            out = ts.tk_vote2(T32, sigma1=s1, sigma2=s2, power=p, plate=True, N=N)
            fx[f"tk_{fname}_{s1}_{s2}_{p}_{N}"] = out.reshape(24, 24, 4)
        fx[f"atv_{fname}_3.0"] = ts.atv_vote2(T32, sigma=3.0).reshape(24, 24, 4)
    np.savez_compressed(os.path.join(HERE, "tv2_numpy_reference.npz"), **fx)

    # --- 2D: the reference C++ CPU path -------------------------------------
    fx = {}
    F = flat4(mixed_field(20, 22, 7))
    fx["in"] = F
    for key, kw in {
        "tk_s2_p1_n10": dict(sigma1=2.0, sigma2=0.0, power=1, w=13, samples=10),
        "tk_s2_p2_n20_sig2": dict(sigma1=2.0, sigma2=1.0, power=2, w=13, samples=20),
        "tk_stick_only": dict(sigma1=1.5, sigma2=0.0, power=1, w=9, samples=10, plate=False),
        "tk_plate_only": dict(sigma1=1.5, sigma2=0.0, power=1, w=9, samples=10, stick=False),
        "atv_s2": dict(sigma1=2.0, sigma2=0.0, power=1, w=13, samples=10, is_atv=True),
    }.items():
        fx[key] = O.tensorvote2(F, use_ref=True, **kw)
    fx["nb_w7"] = O.build_neighbors2d(7, 2.0, 0.5, 2, 10, use_ref=True)
    np.savez_compressed(os.path.join(HERE, "tv2_cpp_reference.npz"), **fx)

    # --- 3D: the reference C++ CPU path (tira::cpu::tensorvote3) -----------
    fx = {}
    T = random_spd3((8, 9, 10), 11)
    fx["in"] = T.reshape(8, 9, 10, 9)
    for key, kw in {
        "tk_s15_n20": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=20),
        "tk_s15_n3": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=3),
        "tk_s15_n2": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=2),
        "tk_s2_p2_n20_sig2": dict(sigma1=2.0, sigma2=1.0, w=7, power=2, samples=20),
        "tk_analytic": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=0),
        "tk_stick_only": dict(sigma1=2.0, sigma2=0.0, w=7, power=1, samples=20, plate=False),
        "tk_plate_only": dict(sigma1=2.0, sigma2=0.0, w=7, power=1, samples=20, stick=False),
        "atv_s15": dict(sigma1=1.5, sigma2=0.0, w=5, power=1, samples=20, is_atv=True),
    }.items():
        out = O.tensorvote3(T, use_ref=True, **kw)
        fx[key] = out.reshape(8, 9, 10, 9)
    np.savez_compressed(os.path.join(HERE, "tv3_cpp_reference.npz"), **fx)

    # --- eigen (tira/functions/eigen.h) -------------------------------------
    fx = {}
    rng = np.random.default_rng(3)
    M = random_spd3((1500,), 5)
    M[:50] = 0.0
    M[:50, [0, 1, 2], [0, 1, 2]] = rng.normal(size=(50, 3))      # diagonal branch
    M[50:100] = np.eye(3, dtype=np.float32) * rng.uniform(0.5, 2, (50, 1, 1)).astype(np.float32)  # isotropic
    Q, _ = np.linalg.qr(rng.normal(size=(200, 3, 3)))
    lam = np.sort(rng.uniform(-2, 2, (200, 3)), axis=1)
    M[100:300] = (Q * lam[:, None, :]) @ np.swapaxes(Q, 1, 2)    # indefinite
    M9 = M.reshape(-1, 9).astype(np.float32)
    fx["m9"] = M9
    fx["evals3"] = O.evals3(M9, use_ref=True)
    fx["evecs3sph"] = O.evecs3spherical(M9, fx["evals3"], use_ref=True)
    fx["evecs3cart"] = O.evecs3cart(M9, fx["evals3"], use_ref=True)
    B = rng.normal(size=(1000, 2, 2)).astype(np.float32)
    B = (B @ np.swapaxes(B, 1, 2)).reshape(-1, 4)
    B[:20] = 0.0
    fx["m4"] = B
    fx["evals2"] = O.evals2(B, use_ref=True)
    fx["evecs2"] = O.evecs2polar(B, fx["evals2"], use_ref=True)
    np.savez_compressed(os.path.join(HERE, "eigen_cpp_reference.npz"), **fx)

    # --- separable Gaussian (tira/functions/filter.h) -----------------------
    fx = {}
    for s in (1.0, 1.5, 2.0):
        K3 = int(np.ceil(6 * s)) | 1
        fx[f"g1d_{s}_{K3}"] = O.gaussian1d(K3, s, use_ref=True)
    vol = np.random.default_rng(9).normal(size=(18, 20, 22)).astype(np.float32)
    fx["vol"] = vol
    fx["conv3_15_10_20"] = O.gaussian_convolve3(vol, 1.5, 1.0, 2.0, use_ref=True)
    img = np.random.default_rng(10).normal(size=(30, 40)).astype(np.float32)
    fx["img"] = img
    fx["conv2_1"] = O.gaussian_convolve2(img, 1.0, use_ref=True)
    np.savez_compressed(os.path.join(HERE, "filter_cpp_reference.npz"), **fx)

    # --- consumers of a voted 2D field (reconstruct.py, metrics.py) ---------
    rec = load_reference_module(ref_root, "python/tira/tensors_lib/reconstruct.py", "tira_ref_reconstruct")
    met = load_reference_module(ref_root, "python/tira/tensors_lib/metrics.py", "tira_ref_metrics")
    fx = {}
    rng = np.random.default_rng(21)
    H, W = 40, 44
    img = np.zeros((H, W))
    yy, xx = np.mgrid[0:H, 0:W]
    for _ in range(4):                       # a few rings and bars: closed curves give holes to fill
        cy, cx, r = rng.uniform(8, 32), rng.uniform(8, 36), rng.uniform(4, 9)
        img[np.abs(np.hypot(yy - cy, xx - cx) - r) < 1.0] = 1.0
    img[5:7, 3:40] = 1.0
    img += rng.normal(0, 0.05, img.shape)
    gy, gx = np.gradient(img)
    T = np.stack([np.stack([gx * gx, gx * gy], -1), np.stack([gx * gy, gy * gy], -1)], -2)
    T32 = T.astype(np.float32)
    I = flat4(T32.astype(np.float64)).reshape(H, W, 4)
    fx["I"] = I
    V = O.tensorvote2(I, sigma1=2.0, sigma2=0.0, power=1, w=13, samples=20, use_ref=True)
    V = V.reshape(H, W, 2, 2).astype(np.float32)
    fx["V"] = V.reshape(H, W, 4)
    fx["saliency"] = rec.stick_saliency(V)
    fx["otsu"] = np.float64(rec._otsu_threshold(fx["saliency"].ravel()))
    fx["mask_otsu"] = rec.saliency_threshold(V)
    fx["mask_fixed"] = rec.saliency_threshold(V, threshold=float(np.median(fx["saliency"])))
    fx["mask_fill_r0"] = rec.saliency_threshold(V, fill=True)
    fx["mask_fill_r2"] = rec.saliency_threshold(V, fill=True, close_radius=2)
    # the sweep's objective: simf of a target against votes of the field at several parameter sets
    G = O.tensorvote2(I, sigma1=3.0, sigma2=1.0, power=1, w=19, samples=20, use_ref=True)
    G = G.reshape(H, W, 2, 2).astype(np.float32)
    fx["G"] = G.reshape(H, W, 4)
    params = np.array([[1.5, 0.0, 1], [3.0, 1.0, 1], [2.5, 0.5, 2], [4.2, 3.0, 3]], np.float64)
    fx["sweep_params"] = params
    vals = []
    for s1, s2, pw in params:
        w = 2 * int(3 * max(s1, s2)) + 1
        B = O.tensorvote2(I, sigma1=s1, sigma2=s2, power=int(pw), w=w, samples=20, use_ref=True)
        vals.append(met.simf(G, B.reshape(H, W, 2, 2).astype(np.float32)))
    fx["sweep_simf"] = np.array(vals, np.float64)
    np.savez_compressed(os.path.join(HERE, "reconstruct_reference.npz"), **fx)
    make_neighbors3d(ref_root)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


def make_neighbors3d(ref_root):
    """tira::Neighbor3D tables from the reference's cpu::build_neighbors3d
    (tensorvote.h:1411), for the library's host-side table builder."""
    O.build(ref_root)
    assert O.ref_available(), "reference CPU library did not build"
    fx = {}
    for (w, s1, s2) in [(5, 1.5, 0.0), (7, 2.0, 0.5), (9, 0.0, 1.0)]:
        fx[f"nb3_w{w}_{s1}_{s2}"] = O.build_neighbors3d_ref(w, s1, s2)
    np.savez_compressed(os.path.join(HERE, "nb3_cpp_reference.npz"), **fx)


def reference_root(argv):
    """The tiralib checkout: the first argument, else $TIRALIB_REFERENCE, else
    a `reference` directory beside this repository."""
    if len(argv) > 1:
        return argv[1]
    env = os.environ.get("TIRALIB_REFERENCE")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")


if __name__ == "__main__":
    root = reference_root(sys.argv[:2])
    if len(sys.argv) > 2 and sys.argv[2] == "nb3":
        make_neighbors3d(root)
    else:
        main(root)
