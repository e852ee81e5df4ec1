"""Failure handling on the host, without faulting the GPU: a device allocation that
cannot succeed returns TGVDCT_ERR_OOM and leaves the library usable, and a NaN in the
input runs to the end with the NaN confined to its neighbourhood."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu


def test_state_allocation_failure_is_reported_and_recoverable(gpu_lib):
    # 2048^3 voxels: about 1.2 TB of loop state, more than the device holds
    with pytest.raises(pkg.TgvdctError) as e:
        pkg.Context(pkg.default_params(width=2048, height=2048, depth=2048))
    assert e.value.status == pkg.ERR_OOM
    assert "cudaMalloc" in str(e.value)
    f = tissue_phantom_3d(8, 12, 16, seed=3)
    u, *_ = pkg.tgv2_l1_deshade_launch(f, 1.0, 10)
    assert np.isfinite(u).all()


def test_nan_input_stays_local(gpu_lib):
    """The stencils move information at most two voxels per iteration (the dual step
    reads ubar one voxel away, the primal step reads p and q one voxel away), so after
    K iterations a NaN at one voxel cannot reach voxels more than 2K away."""
    f = tissue_phantom_3d(24, 32, 40, seed=4)
    g = f.copy()
    g[12, 16, 20] = np.nan
    K = 4
    u_clean, *_ = pkg.tgv2_l1_deshade_launch(f, 1.0, K)
    u_nan, vx, vy, vz = pkg.tgv2_l1_deshade_launch(g, 1.0, K)
    z, y, x = np.indices(f.shape)
    far = np.maximum.reduce([abs(z - 12), abs(y - 16), abs(x - 20)]) > 2 * K
    assert np.array_equal(u_nan[far], u_clean[far])
    assert np.isnan(u_nan[12, 16, 20])
    assert np.isfinite(vx[far]).all()
