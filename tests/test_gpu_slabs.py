"""The z-slab decomposition on the GPU: slab by slab, the 3D path gives the
whole volume's voted tensors and eigenpairs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("parts", [2, 3, 5])
def test_gpu_slabs_reproduce_pipeline3(parts):
    import tiralib_gb300 as tv
    from tiralib_gb300 import slabs
    vol = np.random.default_rng(parts).normal(size=(41, 20, 23)).astype(np.float32)
    out, ev, vec = tv.pipeline3(vol, 1.0, 2.0, w=0, samples=20, out_layout="planes", evecs="cartesian")
    got = [slabs.pipeline3_slab(vol, z0, z1, 1.0, 2.0) for z0, z1 in slabs.partition(41, parts)]
    o = np.concatenate([g[0] for g in got], axis=1)
    e = np.concatenate([g[1] for g in got])
    scale = np.abs(out).max()
    assert np.abs(o - out).max() <= 1e-6 * scale
    assert np.abs(e - ev).max() <= 1e-5 * np.abs(ev).max()
