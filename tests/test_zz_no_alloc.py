"""The allocation-free 3D vote entry point, called through the C ABI.

tvgb_vote3_noalloc exists for callers that may not allocate device memory
while they run (a real-time host loop or plugin callback where allocation is
forbidden, or a process whose device memory belongs to another allocator):
it keeps its voter-record scratch in a fixed device array instead of
allocating.  These tests check that it gives the same voted field and
eigenvalues as the allocating entry point (tvgb_vote3) on two calls in a row
of different sizes (the shared array keeps the previous call's contents), and
that sizes beyond its maximum and host arrays are refused with a clear error.
This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_VOXELS = 1 << 19


def spd_field(shape, seed):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=shape + (3, 3))
    return (A @ np.swapaxes(A, -1, -2)).astype(np.float32)


def rel(a, b):
    a = np.asarray(a, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def _call(L, field, dims, params, out, ev, stream):
    return L.tvgb_vote3_noalloc(ctypes.c_void_p(field.data_ptr()), 9, dims[0], dims[1], dims[2], ctypes.byref(params),
                                ctypes.c_void_p(out.data_ptr()), 6, ctypes.c_void_p(ev.data_ptr()), None, 0,
                                ctypes.c_void_p(stream))


def test_noalloc_vote_matches_allocating_entry_point():
    import torch
    import tiralib_gb300 as tv
    from tiralib_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    params = tv.make_params(2.0, 0.0, w=9, power=1, samples=20, stick=True, plate=True)
    # two calls in a row, different sizes: the second must not see the first's records
    for shape, seed in (((24, 28, 30), 1), ((12, 40, 17), 2)):
        T = spd_field(shape, seed)
        t_dev = torch.from_numpy(T).to(dev)
        ref_out, ref_ev, _ = tv.vote3(t_dev, 2.0, 0.0, w=9, power=1, samples=20, layout="mat3", out_layout="sym6",
                                      evals=True)
        out = torch.full(shape + (6,), float("nan"), device=dev)
        ev = torch.full(shape + (3,), float("nan"), device=dev)
        rc = _call(L, t_dev, shape, params, out, ev, stream)
        torch.cuda.synchronize()
        assert rc == 0, L.tvgb_last_error().decode()
        got, got_ev = out.cpu().numpy(), ev.cpu().numpy()
        assert np.isfinite(got).all() and np.isfinite(got_ev).all()
        assert rel(got, ref_out.cpu().numpy()) < 1e-4
        assert rel(got_ev, ref_ev.cpu().numpy()) < 1e-4


def test_noalloc_vote_refuses_oversize_and_host_arrays():
    import torch
    import tiralib_gb300 as tv
    from tiralib_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda:0")
    params = tv.make_params(2.0, 0.0, w=9)
    big = (81, 81, 81)                      # 531441 > 524288 voxels
    assert big[0] * big[1] * big[2] > MAX_VOXELS
    t_dev = torch.zeros(big + (3, 3), device=dev)
    out = torch.empty(big + (6,), device=dev)
    ev = torch.empty(big + (3,), device=dev)
    rc = _call(L, t_dev, big, params, out, ev, 0)
    assert rc == 1
    assert "maximum" in L.tvgb_last_error().decode()
    host = spd_field((4, 4, 4), 3)
    out_h = np.zeros((4, 4, 4, 6), np.float32)
    rc = L.tvgb_vote3_noalloc(ctypes.c_void_p(host.ctypes.data), 9, 4, 4, 4, ctypes.byref(params),
                              ctypes.c_void_p(out_h.ctypes.data), 6, None, None, 0, None)
    assert rc == 1
    assert "device memory" in L.tvgb_last_error().decode()


def test_noalloc_vote_with_no_terms_writes_eigen_outputs():
    """With no term voting, the allocation-free entry point still fills the
    requested eigenvalue array (the zero tensor's eigenvalues), as the
    allocating entry point does."""
    import torch
    import tiralib_gb300 as tv
    from tiralib_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    shape = (6, 7, 8)
    t_dev = torch.from_numpy(spd_field(shape, 5)).to(dev)
    params = tv.make_params(2.0, 0.0, w=5, stick=False, plate=False, ball=False)
    out = torch.full(shape + (6,), float("nan"), device=dev)
    ev = torch.full(shape + (3,), float("nan"), device=dev)
    rc = _call(L, t_dev, shape, params, out, ev, stream)
    torch.cuda.synchronize()
    assert rc == 0, L.tvgb_last_error().decode()
    ref_out, ref_ev, _ = tv.vote3(t_dev, 2.0, w=5, stick=False, plate=False, out_layout="sym6", evals=True)
    torch.cuda.synchronize()
    assert torch.equal(out, ref_out) and torch.equal(ev, ref_ev)
    assert float(ev.abs().max()) == 0.0
