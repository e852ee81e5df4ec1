"""The z-slab split on one GPU: every rank's slab is a context of its own on this
GPU, and the driver runs the ranks in lock step in one process (slab.run_emulated),
handing halo planes and pencils from one rank's device buffers to another's.  No
kernel waits on another rank's.  u, v, l and r must equal the single-volume deshade
(tgvdct_tgv2_run_dev and tgvdct_poisson_integrate_dev on the whole volume) bit for
bit: the split moves only exact copies of values."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300 import slab
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu


def _whole(f, iterations, eigen, data=pkg.DATA_L1):
    import torch
    D, H, W = f.shape
    prm = pkg.default_params(width=W, height=H, depth=D, iteration_count=iterations,
                             poisson_eigen=eigen, data_term=data)
    u, vx, vy, vz, l = (torch.empty_like(f) for _ in range(5))
    with pkg.Context(prm) as ctx:
        ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr())
        ctx.poisson_integrate_dev(vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), l.data_ptr())
        torch.cuda.synchronize()
        ctx.check_device_error()
    return u, vx, vy, vz, l


@pytest.mark.parametrize("shape,ranks,iterations,eigen,data", [
    ((24, 40, 48), 2, 60, pkg.EIGEN_REFERENCE, pkg.DATA_L1),
    ((31, 36, 44), 3, 45, pkg.EIGEN_ACCURATE, pkg.DATA_L1),
    ((64, 96, 128), 4, 40, pkg.EIGEN_REFERENCE, pkg.DATA_L1),
    # a width that rules out TMA: the register-staged fused kernel on every slab
    ((20, 30, 42), 2, 35, pkg.EIGEN_REFERENCE, pkg.DATA_L1),
    ((40, 24, 32), 5, 30, pkg.EIGEN_ACCURATE, pkg.DATA_L2),
])
def test_emulated_ranks_equal_the_single_volume(gpu_lib, shape, ranks, iterations, eigen,
                                                data):
    import torch
    D, H, W = shape
    f = torch.from_numpy(np.log(tissue_phantom_3d(D, H, W, seed=6))).cuda()
    ref = _whole(f, iterations, eigen, data)
    prm = pkg.default_params(width=W, height=H, depth=D, poisson_eigen=eigen, data_term=data)
    backends, gens = [], []
    for r in range(ranks):
        geo = slab.SlabGeometry(W, H, D, ranks, r)
        be = slab.CudaSlabBackend(prm, geo)
        backends.append(be)
        gens.append(slab.deshade_rank(geo, be, slab.local_input(f, geo), iterations))
    try:
        res = slab.run_emulated(gens)
        torch.cuda.synchronize()
        for be in backends:
            be.ctx.check_device_error()
    finally:
        for be in backends:
            be.close()
    for k, name in enumerate(("u", "v_x", "v_y", "v_z", "l")):
        got = torch.cat([x[k] for x in res])
        assert torch.equal(got, ref[k]), name
    r = torch.cat([x[5] for x in res])
    assert torch.equal(r, ref[0] - ref[4])
