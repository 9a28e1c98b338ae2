"""GPU parity of the batched eigensolvers (libtvgb, C ABI) against the
reference's outputs (tests/golden, from tira/functions/eigen.h compiled
unmodified) and the CPU oracle; precise mode against the FP64 oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

UNIQUE9 = [0, 1, 2, 4, 5, 8]


@pytest.fixture(scope="module")
def tv():
    import tiralib_gb300
    return tiralib_gb300


def evals_rel(got, ref):
    scale = np.maximum(np.abs(ref).max(axis=1, keepdims=True), 1e-30)
    return float((np.abs(got - ref) / scale).max())


def test_evals3_matches_reference(tv, golden):
    g = golden("eigen_cpp_reference.npz")
    ev = tv.evals3_symmetric(g["m9"])
    assert evals_rel(ev, g["evals3"]) < 1e-4   # the parity bar (FP32, FMA vs host libm)


def test_evecs3spherical_matches_reference(tv, golden):
    g = golden("eigen_cpp_reference.npz")
    sph = tv.evecs3spherical_symmetric(g["m9"], g["evals3"])
    # compare as unit vectors (the angles wrap at +-pi)
    def to_vec(s):
        th, ph = s[:, 0::2], s[:, 1::2]
        return np.stack([np.cos(th) * np.sin(ph), np.sin(th) * np.sin(ph), np.cos(ph)], axis=-1)
    a, b = to_vec(sph.astype(np.float64)), to_vec(g["evecs3sph"].astype(np.float64))
    dots = np.abs((a * b).sum(-1))
    assert (1.0 - dots).max() < 1e-5


@pytest.mark.parametrize("layout", ["mat3", "sym6", "planes"])
@pytest.mark.parametrize("fmt", ["cartesian", "spherical", None])
def test_eig3_fused_matches_oracle(tv, layout, fmt):
    rng = np.random.default_rng(1)
    n = 5000 + 37                      # ragged last tile
    A = rng.normal(size=(n, 3, 3)).astype(np.float32)
    M = (A @ np.swapaxes(A, 1, 2)).astype(np.float32)
    m9 = M.reshape(n, 9)
    if layout == "mat3":
        inp = m9
    elif layout == "sym6":
        inp = np.ascontiguousarray(m9[:, UNIQUE9])
    else:
        inp = np.ascontiguousarray(m9[:, UNIQUE9].T)
    ev, vec, _ = tv.eig3(inp, layout=layout, evecs=fmt)
    ref_ev = O.evals3(m9)
    assert evals_rel(ev, ref_ev) < 1e-4
    if fmt == "cartesian":
        ref = O.evecs3cart(m9, ref_ev)
        dots = np.abs(np.einsum("nij,nij->ni", vec, ref))
        assert (1.0 - dots).max() < 1e-4
    elif fmt == "spherical":
        ref = O.evecs3spherical(m9, ref_ev)
        assert np.abs(np.cos(vec) - np.cos(ref)).max() < 1e-3


@pytest.mark.parametrize("precise", [False, True])
@pytest.mark.parametrize("layout", ["mat3", "sym6", "planes"])
def test_eig3_many_tiles_per_block(tv, layout, precise):
    """2^20 + 37 tensors: every block of the grid-stride solver works through
    several tiles, each staged while the previous one is solved (the AoS
    layouts), ending with a ragged tile."""
    rng = np.random.default_rng(11)
    n = (1 << 20) + 37
    A = rng.normal(size=(n, 3, 3)).astype(np.float32)
    M = (A @ np.swapaxes(A, 1, 2)).astype(np.float32)
    m9 = M.reshape(n, 9)
    if layout == "mat3":
        inp = m9
    elif layout == "sym6":
        inp = np.ascontiguousarray(m9[:, UNIQUE9])
    else:
        inp = np.ascontiguousarray(m9[:, UNIQUE9].T)
    ev, vec, _ = tv.eig3(inp, layout=layout, evecs="cartesian", precise=precise)
    ref_ev = O.evals3(m9)
    assert evals_rel(ev, ref_ev) < 1e-4
    ref = O.evecs3cart(m9, ref_ev)
    lam = ref_ev.astype(np.float64)
    scale = np.abs(lam).max(axis=1)
    sep = np.minimum(lam[:, 1] - lam[:, 0], lam[:, 2] - lam[:, 1]) > 1e-2 * scale   # well separated
    dots = np.abs(np.einsum("nij,nij->ni", vec[sep], ref[sep]))
    assert sep.sum() > n // 2
    assert (1.0 - dots).max() < 1e-4


def test_eig3_empty_and_device(tv):
    import torch
    ev, vec, _ = tv.eig3(np.zeros((0, 9), np.float32))
    assert ev.shape == (0, 3)
    rng = np.random.default_rng(2)
    A = rng.normal(size=(300, 3, 3)).astype(np.float32)
    M = (A @ np.swapaxes(A, 1, 2)).reshape(300, 9).astype(np.float32)
    d_ev, d_vec, _ = tv.eig3(torch.from_numpy(M).cuda())
    torch.cuda.synchronize()
    h_ev, h_vec, _ = tv.eig3(M)
    np.testing.assert_array_equal(d_ev.cpu().numpy(), h_ev)
    np.testing.assert_array_equal(d_vec.cpu().numpy(), h_vec)


def synthetic_c3(n, seed):
    """Q diag(l) Q^T with Haar Q, log-uniform l in [1e-6, 1e3], 10 % with a
    pair within 1e-6 relative and 1 % fully degenerate."""
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, 3, 3))
    Q, R = np.linalg.qr(G)
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    lam = 10.0 ** rng.uniform(-6, 3, (n, 3))
    k = rng.uniform(size=n)
    pair = k < 0.10
    lam[pair, 1] = lam[pair, 0] * (1 + rng.uniform(-1e-6, 1e-6, pair.sum()))
    full = k > 0.99
    lam[full, 1] = lam[full, 0]
    lam[full, 2] = lam[full, 0]
    M = (Q * lam[:, None, :]) @ np.swapaxes(Q, 1, 2)
    return M.astype(np.float32)


def test_eig3_precise_refines_near_degenerate_pairs(tv):
    n = 20000
    M = synthetic_c3(n, 3)
    m9 = M.reshape(n, 9)
    ev_p, vec_p, nref = tv.eig3(m9, precise=True)
    ev_r, vec_r, _ = tv.eig3(m9, precise=False)
    assert 0 < nref < n
    ref_ev, ref_vec = O.eig3_f64(m9[:, UNIQUE9].astype(np.float64))
    scale = np.abs(ref_ev).max(axis=1, keepdims=True)
    err_p = np.abs(ev_p - ref_ev) / scale
    err_r = np.abs(ev_r - ref_ev) / scale
    # normwise eigenvalue error stays at FP32 level in both modes
    assert err_p.max() < 1e-5
    # backward error of the precise frame: ||A V - V L|| / ||A||
    A64 = M.astype(np.float64)
    V = vec_p.astype(np.float64)                       # rows e0, e1, e2
    res = np.einsum("nij,nkj->nki", A64, V) - ev_p[:, :, None] * V
    bw = np.linalg.norm(res.reshape(n, -1), axis=1) / np.linalg.norm(A64.reshape(n, -1), axis=1)
    orth = np.abs(np.einsum("nij,nkj->nik", V, V) - np.eye(3)).max(axis=(1, 2))
    assert np.median(bw) < 1e-6 and bw.max() < 1e-4
    assert orth.max() < 1e-5
    # the refined tensors' frames are at least as orthogonal as the parity solve's
    Vr = vec_r.astype(np.float64)
    orth_r = np.abs(np.einsum("nij,nkj->nik", Vr, Vr) - np.eye(3)).max(axis=(1, 2))
    assert orth.max() <= max(orth_r.max(), 1e-5)
    # eigenvectors of near-degenerate pairs: the float32 input determines
    # them (FP64 resolves gaps far below FP32 rounding); the FP64 refinement
    # recovers them, the FP32 closed form cannot
    gaps = np.diff(ref_ev, axis=1) / scale
    gmin = np.full(ref_ev.shape, np.inf)
    gmin[:, :2] = np.minimum(gmin[:, :2], gaps)
    gmin[:, 1:] = np.minimum(gmin[:, 1:], gaps)
    near = (gmin > 1e-7) & (gmin <= 1e-3)
    assert near.sum() > 100

    def angles(vec):
        v = vec.astype(np.float64)
        v /= np.linalg.norm(v, axis=2, keepdims=True)
        dot = np.abs(np.einsum("nij,nij->ni", v, ref_vec))
        return np.arctan2(np.linalg.norm(np.cross(v, ref_vec), axis=2), dot)[near]

    ang_p, ang_r = angles(vec_p), angles(vec_r)
    print(f"near-degenerate eigenvector angle: precise median {np.median(ang_p):.3g} max {ang_p.max():.3g}; "
          f"parity median {np.median(ang_r):.3g} max {ang_r.max():.3g} (n = {near.sum()})")
    assert np.median(ang_p) < 1e-5
    assert np.quantile(ang_p, 0.99) < 1e-3
    assert np.median(ang_p) < 1e-2 * np.median(ang_r)
    del err_r


def test_eig2_matches_reference(tv, golden):
    g = golden("eigen_cpp_reference.npz")
    ev = tv.evals2_symmetric(g["m4"])
    scale = np.maximum(np.abs(g["evals2"]).max(axis=1, keepdims=True), 1.0)
    assert (np.abs(ev - g["evals2"]) / scale).max() < 1e-5
    th = tv.evecs2polar_symmetric(g["m4"], g["evals2"])
    d = np.abs(th - g["evecs2"])
    d = np.minimum(d, np.abs(d - 2 * np.pi))
    assert d.max() < 1e-4


@pytest.mark.parametrize("precise", [False, True])
def test_eig3_streamed_host_batch_equals_device_batch(tv, precise):
    """A large batch in host memory runs chunk by chunk, its copies
    overlapped with the solve on a ring of streams; the results and the
    refined count equal those of the same batch solved in device memory
    (the last chunk is ragged)."""
    import torch
    rng = np.random.default_rng(11)
    n = (1 << 23) + 12345
    Q, _ = np.linalg.qr(rng.normal(size=(4096, 3, 3)))
    lam = rng.uniform(-2, 2, size=(4096, 3))
    lam[::7, 1] = lam[::7, 0] * (1 + 1e-6)          # near-degenerate pairs
    base = (Q * lam[:, None, :]) @ np.swapaxes(Q, 1, 2)
    M = base[rng.integers(0, 4096, size=n)].astype(np.float32).reshape(n, 9)
    M += rng.normal(scale=1e-3, size=(n, 1)).astype(np.float32) * np.eye(3, dtype=np.float32).reshape(1, 9)
    ev_h, vec_h, nr_h = tv.eig3(M, layout="mat3", evecs="cartesian", precise=precise)
    Md = torch.from_numpy(M).cuda()
    ev_d, vec_d, nr_d = tv.eig3(Md, layout="mat3", evecs="cartesian", precise=precise)
    np.testing.assert_array_equal(ev_h, ev_d.cpu().numpy())
    np.testing.assert_array_equal(vec_h, vec_d.cpu().numpy())
    assert nr_h == nr_d
    if precise:
        assert nr_h > 0
