"""A C++ program written against tiralib's entry points (tests/cpp), built
with the header shims and run on the GPU; its outputs are checked against
the CPU oracle."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_cpp_caller_through_shims(tmp_path):
    from test_shim_build import build_shim_check
    exe = build_shim_check(str(tmp_path))
    out = os.path.join(str(tmp_path), "out.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    n = 6 * 7 * 8
    raw = np.fromfile(out, np.float32)
    T = raw[:9 * n].reshape(6, 7, 8, 3, 3)
    voted = raw[9 * n:18 * n]
    ev = raw[18 * n:21 * n].reshape(n, 3)
    vol = raw[21 * n:21 * n + 12 * 13 * 14].reshape(12, 13, 14)
    blurred = raw[21 * n + 12 * 13 * 14:]
    ref = O.tensorvote3(T, 1.5, 0.0, 5, 1, samples=20)
    u = [0, 1, 2, 4, 5, 8]
    a, b = voted.reshape(-1, 9)[:, u], ref.reshape(-1, 9)[:, u]
    assert np.abs(a - b).max() / np.abs(b).max() < 1e-4
    ref_ev = O.evals3(voted.reshape(-1, 9))
    assert (np.abs(ev - ref_ev).max(axis=1) / np.abs(ref_ev).max(axis=1)).max() < 1e-4
    ref_blur = O.gaussian_convolve3(vol, 1.0, 1.0, 1.0)
    assert blurred.size == ref_blur.size
    assert np.abs(blurred - ref_blur.ravel()).max() < 1e-5 * np.abs(ref_blur).max() + 1e-7
