"""z-slab decomposition of the 3D path, on the CPU with the oracle: the
halo rules give each slab exactly the whole-volume result for its planes,
in one process and across two gloo ranks (the N > 1 path's host logic)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tiralib_gb300 import slabs

SIG_ST, SIG, SAMPLES = 1.0, 1.5, 3          # K = 7 (r = 4), w = 9 (hw = 4); 3 samples: the exact plate rule


def oracle_path(vol):
    """structure tensor (same size) -> TK stick + plate vote, as mat3 (z, y, x, 3, 3)."""
    st = O.structure_tensor3(vol, SIG_ST, 1)
    s6 = np.moveaxis(st, 0, -1)
    m9 = np.ascontiguousarray(s6[..., [0, 1, 2, 1, 3, 4, 2, 4, 5]].reshape(s6.shape[:3] + (3, 3)))
    return O.tensorvote3(m9, SIG, 0.0, slabs.vote_window(SIG), 1, samples=SAMPLES)


def oracle_slab(vol, z0, z1):
    nz = vol.shape[0]
    (in_lo, in_hi), (st_lo, st_hi) = slabs.halo_ranges(nz, z0, z1, SIG_ST, SIG)
    st = O.structure_tensor3(vol[in_lo:in_hi], SIG_ST, 1)[:, st_lo - in_lo:st_hi - in_lo]
    s6 = np.moveaxis(st, 0, -1)
    m9 = np.ascontiguousarray(s6[..., [0, 1, 2, 1, 3, 4, 2, 4, 5]].reshape(s6.shape[:3] + (3, 3)))
    out = O.tensorvote3(m9, SIG, 0.0, slabs.vote_window(SIG), 1, samples=SAMPLES)
    return out[z0 - st_lo:z1 - st_lo]


def volume(nz=30, ny=9, nx=10, seed=0):
    return np.random.default_rng(seed).normal(size=(nz, ny, nx)).astype(np.float32)


def test_partition_covers_every_plane_once():
    for nz, parts in [(10, 3), (7, 7), (5, 8), (256, 6)]:
        p = slabs.partition(nz, parts)
        assert len(p) == parts
        assert p[0][0] == 0 and p[-1][1] == nz
        assert all(a[1] == b[0] for a, b in zip(p, p[1:]))
        assert all(z1 >= z0 for z0, z1 in p)


def test_halo_ranges():
    (il, ih), (sl, sh) = slabs.halo_ranges(100, 40, 60, 1.5, 4.0)   # K = 9 -> r = 5, w = 25 -> hw = 12
    assert (sl, sh) == (28, 72) and (il, ih) == (23, 77)
    (il, ih), (sl, sh) = slabs.halo_ranges(100, 0, 10, 1.5, 4.0)
    assert (sl, sh) == (0, 22) and (il, ih) == (0, 27)


def test_slabs_reproduce_the_whole_volume():
    vol = volume()
    full = oracle_path(vol)
    parts = [oracle_slab(vol, z0, z1) for z0, z1 in slabs.partition(vol.shape[0], 3)]
    assert np.array_equal(np.concatenate(parts), full)


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    vol = volume()                                   # every rank builds the same seeded volume
    z0, z1 = slabs.partition(vol.shape[0], world)[rank]
    mine = oracle_slab(vol, z0, z1)
    got = [None] * world
    dist.all_gather_object(got, (z0, z1, mine))
    if rank == 0:
        got.sort(key=lambda t: t[0])
        q.put(np.concatenate([t[2] for t in got]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_whole_volume():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    result = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert np.array_equal(result, oracle_path(volume()))
