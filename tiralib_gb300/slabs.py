"""z-slab decomposition of the 3D path (structure tensor -> vote -> eigen).

The path has no reduction: each output voxel depends on the input volume
within a fixed distance, so the volume splits along z (the slow axis) into
slabs that ranks (or one GPU, slab by slab) process independently.  A slab
that owns output planes [z0, z1) needs:
  * the structure tensor on planes [z0 - hw, z1 + hw) (hw = w // 2: the
    vote's reach), clipped to the volume;
  * hence the input volume on [z0 - hw - r, z1 + hw + r), r = K // 2 + 1
    (the blur's half-width plus the gradient's one plane), clipped;
within that input the structure tensor is computed in "same" mode, and the
planes it gets wrong (within r of a cut that is not the volume's own edge)
are never used.  The result on [z0, z1) equals the full-volume result: the
same voters, summed in the same order.
"""
import numpy as np


def ksize3(sigma):
    """Taps of the 3D structure tensor's Gaussian (filter.h:405-410)."""
    k = int(np.ceil(6.0 * np.float32(sigma)))
    return k if k % 2 else k + 1


def vote_window(sigma1, sigma2=0.0, w=0):
    if w:
        return int(w)
    sm = max(float(np.float32(sigma1)), float(np.float32(sigma2)))
    w = 2 * int(np.float32(3.0) * np.float32(sm)) + 1
    w = max(w, 3)
    return w if w % 2 else w + 1


def partition(nz, parts):
    """Owned plane ranges [z0, z1) of `parts` near-equal slabs (empty ones
    when parts > nz)."""
    bounds = [nz * i // parts for i in range(parts + 1)]
    return [(bounds[i], bounds[i + 1]) for i in range(parts)]


def halo_ranges(nz, z0, z1, sigma_st, sigma1, sigma2=0.0, w=0):
    """For owned planes [z0, z1): (in_lo, in_hi) of the input volume to read,
    (st_lo, st_hi) of the structure tensor the vote needs, both absolute
    plane indices clipped to [0, nz)."""
    hw = vote_window(sigma1, sigma2, w) // 2
    r = ksize3(sigma_st) // 2 + 1
    st_lo, st_hi = max(0, z0 - hw), min(nz, z1 + hw)
    in_lo, in_hi = max(0, st_lo - r), min(nz, st_hi + r)
    return (in_lo, in_hi), (st_lo, st_hi)


def pipeline3_slab(volume, z0, z1, sigma_st, sigma1, sigma2=0.0, w=0, samples=20, ball=False, parity=True,
                   evecs="cartesian"):
    """The 3D path for owned planes [z0, z1) of `volume` ((nz, ny, nx), NumPy
    or CUDA torch): (voted planes (6, z1 - z0, ny, nx), eigenvalues,
    eigenvectors) equal to those planes of the whole-volume result."""
    from . import api
    nz = int(volume.shape[0])
    (in_lo, in_hi), (st_lo, st_hi) = halo_ranges(nz, z0, z1, sigma_st, sigma1, sigma2, w)
    sub = volume[in_lo:in_hi]
    if api._is_torch(sub):
        sub = sub.contiguous()
    st = api.structure_tensor3(sub, sigma_st, mode="same", layout="planes")
    st = st[:, st_lo - in_lo:st_hi - in_lo]
    st = st.contiguous() if api._is_torch(st) else np.ascontiguousarray(st)
    out, ev, vec = api.vote3(st, sigma1, sigma2, w=vote_window(sigma1, sigma2, w), samples=samples, ball=ball,
                             parity=parity, layout="planes", out_layout="planes", evals=True, evecs=evecs)
    a, b = z0 - st_lo, z1 - st_lo
    return out[:, a:b], ev[a:b], vec[a:b]
