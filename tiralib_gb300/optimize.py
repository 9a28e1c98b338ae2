"""TK parameter search on the GPU (tiralib's
python/tira/tensors_lib/optimize.py:256 optimize_tk).

The objective of optimize_tk is SIMF(G, TK(I; sigma1, sigma2, power)): one 2D
vote per candidate.  `tk_sweep` evaluates any number of candidates in one
libtvgb call (tvgb_tensorvote_sweep: the input field is solved once, each
candidate gets its own window and neighbour table, its vote and its SIMF).
`optimize_tk` runs SciPy's differential evolution with the reference's
settings on that objective; with batched=True a whole generation is scored
in one sweep call (differential_evolution(vectorized=True), which updates
the population once per generation).
"""
import ctypes

import numpy as np

from . import api as _api
from .reconstruct import _field4


def w_from_sigma(sigma1, sigma2):
    """optimize.py:9: 2 int(3 max(sigma1, sigma2)) + 1, at least 3, odd."""
    w = 2 * int(3 * max(float(sigma1), float(sigma2))) + 1
    w = max(w, 3)
    return w + 1 if w % 2 == 0 else w


def tk_sweep(G, I, params, samples=20, plate=True, return_fields=False):
    """SIMF(G, TK vote of I) for each row (sigma1, sigma2, power) of params.
    Returns a float64 array (K,), and the (K, H, W, 2, 2) voted fields when
    return_fields is set."""
    FI, (H, W) = _field4(I)
    FG, sg = _field4(G)
    if sg != (H, W):
        raise ValueError(f"tk_sweep: G is {sg}, I is {(H, W)}")
    P = np.ascontiguousarray(np.atleast_2d(np.asarray(params, np.float64)).reshape(-1, 3))
    K = P.shape[0]
    out = np.empty(K, np.float64)
    fields = None
    if return_fields:
        fields = _api._empty_like_kind(FI, (K, H, W, 2, 2))
    _api.call("tvgb_tensorvote_sweep", _api._ptr(FI), _api._ptr(FG), H, W, P.ctypes.data_as(ctypes.c_void_p), K,
              int(samples), int(bool(plate)), out.ctypes.data_as(ctypes.c_void_p), _api._ptr(fields),
              _api._stream_for(FI, FG))
    return (out, fields) if return_fields else out


def _round_power(p):
    return max(1, int(round(float(p))))


def optimize_tk(G, I, bounds=None, seed=42, cuda=True, batched=False, maxiter=500, popsize=15, tol=1e-5,
                polish=True):
    """optimize.py:256: minimise SIMF(G, TK(I; sigma1, sigma2, power)) over
    bounds [(sigma1), (sigma2), (power)] by differential evolution.  Returns
    (sigma1, sigma2, power, voted field (H, W, 2, 2), objective).  The vote
    always runs on the GPU (`cuda` is accepted for the reference's signature);
    the plate uses 20 samples, as the reference's CUDA path."""
    from scipy.optimize import differential_evolution
    del cuda
    if bounds is None:
        bounds = [(1.0, 30.0), (0.0, 20.0), (1, 30)]

    def score(X):
        X = np.atleast_2d(X)
        ok = np.all(np.isfinite(X), axis=1)
        res = np.full(X.shape[0], np.inf)
        if ok.any():
            P = np.stack([X[ok, 0], X[ok, 1], [_round_power(p) for p in X[ok, 2]]], axis=1)
            v = tk_sweep(G, I, P)
            v[~np.isfinite(v)] = np.inf
            res[ok] = v
        return res

    if batched:
        res = differential_evolution(lambda X: score(X.T), bounds=bounds, seed=seed, maxiter=maxiter,
                                     popsize=popsize, tol=tol, polish=polish, vectorized=True, updating="deferred")
    else:
        res = differential_evolution(lambda x: float(score(x)[0]), bounds=bounds, seed=seed, maxiter=maxiter,
                                     popsize=popsize, tol=tol, polish=polish)
    s1, s2, pw = float(res.x[0]), float(res.x[1]), _round_power(res.x[2])
    _, fields = tk_sweep(G, I, [[s1, s2, pw]], return_fields=True)
    return s1, s2, pw, fields[0], float(res.fun)
