"""GPU parity of the 3D vote (libtvgb through its C ABI) against the
reference's own CPU outputs (tests/golden/tv3_cpp_reference.npz), the CPU
oracle and the FP64 precision oracle.

Tolerance: max |gpu - ref| / max |ref| < 1e-4 on the six unique entries, the
reference's own CPU/GPU bar (python/tira/tests/test_cpu_gpu.py:132).
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

UNIQUE9 = [0, 1, 2, 4, 5, 8]
TOL = 1e-4


@pytest.fixture(scope="module")
def tv():
    import tiralib_gb300
    return tiralib_gb300


def rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


def u6(x):
    return np.asarray(x).reshape(-1, 9)[:, UNIQUE9]


def oracle_vote3(T, *args, **kw):
    """The oracle over every receiver, spread over the host's cores."""
    n = int(np.prod(T.shape[:3]))
    return O.tensorvote3_receivers(T, np.arange(n), *args, threads=os.cpu_count() or 1, **kw)


def spd_field(shape, seed):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=shape + (3, 3))
    return (A @ np.swapaxes(A, -1, -2)).astype(np.float32)


GOLDEN_CASES = {
    "tk_s15_n20": dict(sigma=1.5, sigma2=0.0, w=5, power=1, samples=20),
    "tk_s15_n3": dict(sigma=1.5, sigma2=0.0, w=5, power=1, samples=3),
    "tk_s15_n2": dict(sigma=1.5, sigma2=0.0, w=5, power=1, samples=2),          # literal 2-point rule
    "tk_s2_p2_n20_sig2": dict(sigma=2.0, sigma2=1.0, w=7, power=2, samples=20),
    "tk_analytic": dict(sigma=1.5, sigma2=0.0, w=5, power=1, samples=0),
    "tk_stick_only": dict(sigma=2.0, sigma2=0.0, w=7, power=1, samples=20, plate=False),
    "tk_plate_only": dict(sigma=2.0, sigma2=0.0, w=7, power=1, samples=20, stick=False),
    "atv_s15": dict(sigma=1.5, sigma2=0.0, w=5, power=1, samples=20, is_atv=True),
}


@pytest.mark.parametrize("case", sorted(GOLDEN_CASES))
def test_tensorvote3_matches_reference_golden(tv, golden, case):
    g = golden("tv3_cpp_reference.npz")
    T = np.ascontiguousarray(g["in"])                       # (8, 9, 10, 9) glm::mat3
    out = np.zeros_like(T)
    kw = dict(GOLDEN_CASES[case])
    tv.tensorvote3(T, out, 8, 9, 10, kw.pop("sigma"), kw.pop("sigma2"), kw.pop("w"), kw.pop("power"), 0, **kw)
    assert rel(u6(out), u6(g[case])) < TOL
    # symmetric output, as the reference GPU kernels write it
    o = out.reshape(-1, 3, 3)
    assert np.array_equal(o, np.swapaxes(o, 1, 2))


@pytest.mark.parametrize("shape,sigma,w,samples", [
    ((13, 17, 19), 2.0, 9, 20),      # ragged in every axis
    ((1, 40, 35), 1.0, 3, 0),        # single plane, closed-form plate
    ((33, 9, 20), 1.5, 7, 3),        # minimal exact sample count
    ((5, 6, 40), 3.0, 19, 64),       # window larger than the volume
    ((20, 24, 36), 2.0, 13, 20),     # several CTAs in every axis
])
def test_vote3_fast_path_matches_oracle(tv, shape, sigma, w, samples):
    T = spd_field(shape, sum(shape) + w)
    out, _, _ = tv.vote3(T, sigma, 0.0, w=w, power=1, samples=samples)
    ref = oracle_vote3(T, sigma, 0.0, w, 1, samples=samples)
    assert rel(u6(out), u6(ref)) < TOL


@pytest.mark.parametrize("shape,sigma,w", [
    ((13, 17, 19), 2.0, 9),          # ragged in every axis
    ((1, 40, 35), 1.0, 3),           # single plane
    ((5, 6, 40), 3.0, 19),           # window larger than the volume
    ((20, 24, 36), 2.0, 13),         # several CTAs in every axis
])
def test_vote3_atv_fast_path_matches_oracle(tv, shape, sigma, w):
    """ATV (tensorvote.h:710) on the tiled kernel's stick / plate / ball terms
    against the oracle's restatement of the reference's per-pair ATV, both
    through the parity entry point (eigen.h voters with the spherical round
    trip) and the extended one."""
    T = spd_field(shape, sum(shape) + 3 * w)
    ref = oracle_vote3(T, sigma, 0.0, w, 1, is_atv=True)
    out = np.zeros_like(T)
    tv.tensorvote3(T, out, *shape, sigma, 0.0, w, 1, 0, True, True, 20, True)
    assert rel(u6(out), u6(ref)) < TOL
    out2, _, _ = tv.vote3(T, sigma, 0.0, w=w, is_atv=True)
    assert rel(u6(out2), u6(ref)) < TOL


def test_vote3_sigma2_and_power3(tv):
    T = spd_field((9, 11, 12), 5)
    out, _, _ = tv.vote3(T, 2.0, 1.5, w=9, power=3, samples=7)
    ref = oracle_vote3(T, 2.0, 1.5, 9, 3, samples=7)
    assert rel(u6(out), u6(ref)) < TOL
    out, _, _ = tv.vote3(T, 2.0, 1.5, w=9, power=1, samples=20)
    ref = oracle_vote3(T, 2.0, 1.5, 9, 1, samples=20)
    assert rel(u6(out), u6(ref)) < TOL


def test_vote3_input_layouts_agree(tv):
    T = spd_field((7, 8, 9), 6)
    m9 = T.reshape(7, 8, 9, 9)
    s6 = np.ascontiguousarray(m9[..., UNIQUE9])
    planes = np.ascontiguousarray(np.moveaxis(s6, -1, 0))
    a, _, _ = tv.vote3(T, 1.5, w=7, layout="mat3", out_layout="sym6")
    b, _, _ = tv.vote3(s6, 1.5, w=7, layout="sym6", out_layout="sym6")
    c, _, _ = tv.vote3(planes, 1.5, w=7, layout="planes", out_layout="planes")
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, np.moveaxis(c, 0, -1))


def test_vote3_fused_eigen_matches_oracle(tv):
    T = spd_field((10, 11, 12), 7)
    out, ev, vec = tv.vote3(T, 2.0, w=9, evals=True, evecs="cartesian")
    m9 = out.reshape(-1, 9)
    ref_ev = O.evals3(m9)
    scale = np.abs(ref_ev).max(axis=1, keepdims=True)
    assert (np.abs(ev.reshape(-1, 3) - ref_ev) / scale).max() < 1e-5
    ref_vec = O.evecs3cart(m9, ref_ev)
    dots = np.abs(np.einsum("nij,nij->ni", vec.reshape(-1, 3, 3), ref_vec))
    assert (1 - dots).max() < 1e-4


def test_vote3_device_arrays_and_stream(tv):
    import torch
    T = spd_field((12, 13, 14), 8)
    host, _, _ = tv.vote3(T, 1.5, w=7)
    d = torch.from_numpy(T).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dev, _, _ = tv.vote3(d, 1.5, w=7)
    s.synchronize()
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


def test_vote3_ball_against_fp64_oracle(tv):
    """The ball term has no reference counterpart: it is checked against the
    FP64 restatement (lambda0 x mean of unit stick votes over the sphere)."""
    T = spd_field((9, 10, 11), 9)
    out, _, _ = tv.vote3(T, 1.5, w=7, stick=False, plate=False, ball=True, parity=False)
    ref = O.tensorvote3_f64(T, 1.5, 0.0, 7, 1, stick=False, plate=False, ball=True)
    assert rel(u6(out), ref.reshape(-1, 6)) < 1e-5
    out2, _, _ = tv.vote3(T, 1.5, w=7, power=2, stick=False, plate=False, ball=True, parity=False)
    ref2 = O.tensorvote3_f64(T, 1.5, 0.0, 7, 2, stick=False, plate=False, ball=True)
    assert rel(u6(out2), ref2.reshape(-1, 6)) < 1e-5


def test_vote3_precise_voters_against_fp64_oracle(tv):
    T = spd_field((11, 12, 13), 10)
    out, _, _ = tv.vote3(T, 2.0, w=9, parity=False)
    ref = O.tensorvote3_f64(T, 2.0, 0.0, 9, 1)
    assert rel(u6(out), ref.reshape(-1, 6)) < 2e-5


def test_vote3_linear_in_scale(tv):
    """Doubling the field doubles the vote exactly (power-of-two scaling)."""
    T = spd_field((8, 9, 10), 11)
    a, _, _ = tv.vote3(T, 1.5, w=7)
    b, _, _ = tv.vote3(2.0 * T, 1.5, w=7)
    np.testing.assert_array_equal(2.0 * a, b)


def test_vote3_rejects_bad_arguments(tv):
    T = spd_field((4, 4, 4), 12)
    with pytest.raises(tv.TvgbError):
        tv.vote3(T, 1.0, w=4)            # even window
    with pytest.raises(tv.TvgbError):
        tv.vote3(T, 0.0, 0.0, w=5)       # both sigmas zero
    out = np.zeros_like(T)
    with pytest.raises(tv.TvgbError):
        tv.tensorvote3(T, out, 4, 4, 4, 1.0, 0.0, 6, 1)


def test_repeated_host_calls_reuse_the_library_pool():
    """Host-array calls stage through the library's own memory pool, which
    keeps freed memory for the next call; results are unchanged from call to
    call, the library's live temporaries return to zero, and the cached
    memory can be handed back to the driver."""
    import tiralib_gb300 as tv
    rng = np.random.default_rng(5)
    A = rng.normal(size=(18, 20, 22, 3, 3))
    T = (A @ np.swapaxes(A, -1, -2)).astype(np.float32)
    first, ev1, _ = tv.vote3(T, 2.0, 0.0, w=9, evals=True)
    again, ev2, _ = tv.vote3(T, 2.0, 0.0, w=9, evals=True)
    np.testing.assert_array_equal(first, again)
    np.testing.assert_array_equal(ev1, ev2)
    assert tv.memory_stats()[0] == 0
    assert tv.lib().tvgb_release_cached_memory() == 0
    third, _, _ = tv.vote3(T, 2.0, 0.0, w=9)
    np.testing.assert_array_equal(first, third)


@pytest.mark.parametrize("out_layout,evecs", [("planes", "cartesian"), ("mat3", "spherical")])
def test_pipeline3_host_outputs_in_slabs_equal_device_outputs(out_layout, evecs):
    """Large volumes with host outputs vote in z-slabs, each slab copied to
    the host while the next one votes; the results equal those written to
    device outputs bit for bit (slab edges fall on the kernel's own receiver
    groups)."""
    import torch
    import tiralib_gb300 as tv
    rng = np.random.default_rng(8)
    shape = (164, 160, 168)                       # 4.4 M voxels: above the slab threshold
    vol = rng.normal(size=shape).astype(np.float32)
    kw = dict(sigma_st=1.5, sigma1=2.0, w=9, samples=20, st_mode="same", out_layout=out_layout, evecs=evecs)
    o_h, ev_h, vec_h = tv.pipeline3(vol, **kw)
    o_d, ev_d, vec_d = tv.pipeline3(torch.from_numpy(vol).cuda(), **kw)
    np.testing.assert_array_equal(o_h, o_d.cpu().numpy())
    np.testing.assert_array_equal(ev_h, ev_d.cpu().numpy())
    np.testing.assert_array_equal(vec_h, vec_d.cpu().numpy())


def test_vote3_host_outputs_in_slabs_equal_device_outputs():
    """tvgb_vote3 (behind tira::cuda::tensorvote3's drop-in) with host
    arrays of a large field votes in z-slabs with the copies overlapped; the
    results equal those written to device arrays bit for bit."""
    import torch
    import tiralib_gb300 as tv
    rng = np.random.default_rng(9)
    shape = (164, 160, 168)
    A = rng.normal(size=(4096, 3, 3)).astype(np.float32)
    T = (A @ np.swapaxes(A, -1, -2))[rng.integers(0, 4096, size=int(np.prod(shape)))].reshape(shape + (3, 3))
    T = np.ascontiguousarray(T, np.float32)
    kw = dict(w=9, samples=20, layout="mat3", out_layout="mat3", evals=True, evecs="spherical")
    o_h, ev_h, vec_h = tv.vote3(T, 2.0, 0.0, **kw)
    o_d, ev_d, vec_d = tv.vote3(torch.from_numpy(T).cuda(), 2.0, 0.0, **kw)
    np.testing.assert_array_equal(o_h, o_d.cpu().numpy())
    np.testing.assert_array_equal(ev_h, ev_d.cpu().numpy())
    np.testing.assert_array_equal(vec_h, vec_d.cpu().numpy())


@pytest.mark.parametrize("parity", [True, False])
def test_vote3_with_no_terms_gives_the_zero_tensors_eigendecomposition(parity):
    """stick = plate = ball = 0 with eigen outputs requested: the voted field
    is zero and every receiver gets the zero tensor's eigendecomposition (the
    same the eigensolver gives it: eigenvalues 0, the identity frame), not
    whatever the arrays held before."""
    import torch
    import tiralib_gb300 as tv
    dev = torch.device("cuda:0")
    T = torch.from_numpy(spd_field((5, 6, 7), 4)).to(dev)
    out, ev, vec = tv.vote3(T, 1.5, w=5, stick=False, plate=False, ball=False, parity=parity, out_layout="sym6",
                            evals=True, evecs="cartesian")
    torch.cuda.synchronize()
    assert float(out.abs().max()) == 0.0
    assert float(ev.abs().max()) == 0.0
    ref = O.evecs3cart(np.zeros((1, 9), np.float32), np.zeros((1, 3), np.float32))[0]
    np.testing.assert_array_equal(vec.cpu().numpy().reshape(-1, 3, 3), np.broadcast_to(ref, (5 * 6 * 7, 3, 3)))
