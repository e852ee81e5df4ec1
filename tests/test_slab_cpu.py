"""The z-slab split of the deshade (ambient_image_processor_gb300/slab.py) on the CPU.

The host logic (partition, halo exchange after every iteration, the v_z halo for the
divergence, the two all-to-all transpositions between slabs and z pencils) runs over
real torch.distributed ranks (gloo, world sizes 2 and 3) with the oracle standing in
for the GPU (tests/slab_oracle_backend.py).  The loop's u and v must equal the
oracle's single-volume loop bit for bit, and l must equal a one-rank run of the same
backend bit for bit (and the oracle's FP64 Poisson integration to rounding)."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch

import oracle
from ambient_image_processor_gb300 import slab
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
from slab_oracle_backend import OracleSlabBackend

SHAPE = (13, 10, 12)  # D, H, W: uneven slabs for 2 and 3 ranks, one halo plane each side
ITERATIONS = 12


def _volume():
    return np.log(tissue_phantom_3d(*SHAPE, seed=4)).astype(np.float32)


def _assemble(results, key):
    return np.concatenate([np.asarray(r[key]) for r in results], axis=0)


def _single_volume(f):
    u, vx, vy, vz = oracle.tgv2_deshade(f, 1.0, 2.0, 1.0, ITERATIONS, dtype=np.float32)
    geo = slab.SlabGeometry(f.shape[2], f.shape[1], f.shape[0], 1, 0)
    (res,) = slab.run_emulated([slab.deshade_rank(geo, OracleSlabBackend(geo),
                                                  torch.from_numpy(f), ITERATIONS)])
    return u, vx, vy, vz, res[4].numpy()


def test_partition():
    assert slab.split_evenly(13, 3) == [(0, 5), (5, 9), (9, 13)]
    g = slab.SlabGeometry(12, 10, 13, 3, 1)
    assert (g.z_range, g.below, g.above, g.local_depth, g.local_z_range) == \
        ((5, 9), 1, 1, 6, (4, 10))
    assert slab.SlabGeometry(12, 10, 13, 3, 0).local_depth == 6  # 5 own + 1 halo
    assert [slab.SlabGeometry(12, 10, 13, 3, r).column_range() for r in range(3)] == \
        [(0, 48), (48, 84), (84, 120)]
    with pytest.raises(ValueError):
        slab.SlabGeometry(12, 10, 5, 3, 0).check()  # fewer than two planes per rank
    assert slab.field_count(slab.HALO_FIELDS) == 4  # ubar and the three vbar


@pytest.mark.parametrize("dropped", [slab.FIELD_UBAR, 1 << 6, 1 << 7, 1 << 8])
def test_every_halo_field_is_needed(dropped, monkeypatch):
    """Leaving one of ubar, vbar_x, vbar_y, vbar_z out of the halo exchange changes
    the result: the exchange is the one the loop needs, not more or less."""
    monkeypatch.setattr(slab, "HALO_FIELDS", slab.HALO_FIELDS & ~dropped)
    f = _volume()
    u = _single_volume(f)[0]
    D, H, W = f.shape
    gens = []
    for r in range(2):
        geo = slab.SlabGeometry(W, H, D, 2, r)
        gens.append(slab.deshade_rank(geo, OracleSlabBackend(geo),
                                      torch.from_numpy(slab.local_input(f, geo)), ITERATIONS))
    res = slab.run_emulated(gens)
    assert not np.array_equal(np.concatenate([x[0].numpy() for x in res]), u)


@pytest.mark.parametrize("ranks", [2, 3, 4])
def test_emulated_ranks_equal_the_single_volume(ranks):
    f = _volume()
    u, vx, vy, vz, l1 = _single_volume(f)
    D, H, W = f.shape
    gens = []
    for r in range(ranks):
        geo = slab.SlabGeometry(W, H, D, ranks, r)
        gens.append(slab.deshade_rank(geo, OracleSlabBackend(geo),
                                      torch.from_numpy(slab.local_input(f, geo)), ITERATIONS))
    res = slab.run_emulated(gens)
    got = [np.concatenate([x[k].numpy() for x in res]) for k in range(6)]
    for a, b in zip(got[:4], (u, vx, vy, vz)):
        assert np.array_equal(a, b)
    assert np.array_equal(got[4], l1)
    assert np.array_equal(got[5], got[0] - got[4])


def test_single_rank_poisson_matches_the_oracle():
    f = _volume()
    u, vx, vy, vz, l1 = _single_volume(f)
    ref = oracle.integrate_poisson_dct(vx.astype(np.float64), vy.astype(np.float64),
                                       vz.astype(np.float64))
    assert np.abs(l1 - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def _worker(rank, ranks, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ranks)
    try:
        f = _volume()
        D, H, W = f.shape
        geo = slab.SlabGeometry(W, H, D, ranks, rank)
        gen = slab.deshade_rank(geo, OracleSlabBackend(geo),
                                torch.from_numpy(slab.local_input(f, geo)), ITERATIONS)
        res = slab.run_distributed(gen, rank, ranks)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"),
                 **{k: t.numpy() for k, t in zip(("u", "vx", "vy", "vz", "l", "r"), res)})
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("ranks", [2, 3])
def test_gloo_ranks_equal_the_single_volume(ranks):
    import torch.multiprocessing as mp
    f = _volume()
    u, vx, vy, vz, l1 = _single_volume(f)
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_worker, args=(ranks, _free_port(), d), nprocs=ranks, join=True)
        parts = [dict(np.load(os.path.join(d, f"rank{r}.npz"))) for r in range(ranks)]
    for key, ref in (("u", u), ("vx", vx), ("vy", vy), ("vz", vz), ("l", l1)):
        assert np.array_equal(_assemble(parts, key), ref), key
