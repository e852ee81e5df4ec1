"""tgvdct_integrate_poisson_noalloc_dev: the Poisson integration that allocates nothing.

It exists for callers that may not allocate device memory while they run — a host
application whose memory manager owns the GPU, a pipeline whose footprint is fixed
in advance, a latency-critical loop in which cudaMalloc/cudaFree would synchronise
the device.  Its scratch is a static device array inside the library, shared by
every call.  This test calls it through the C ABI twice in a row and checks each
result against the allocating entry point's, within the DCT tolerance used by the
other parity tests.  The file sorts last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL_DCT = 1e-5  # as in test_parity_gpu.py
NOALLOC_MAX_VOXELS = 1 << 21  # TGVDCT_NOALLOC_MAX_VOXELS in include/tgvdct.h


def _noalloc(vx, vy, vz, shape, out, stream=None, eigen=None):
    d, h, w = shape
    return pkg.lib().tgvdct_integrate_poisson_noalloc_dev(
        vx.data_ptr(), vy.data_ptr(), vz.data_ptr() if vz is not None else None, w, h, d,
        pkg.DCT_FP32, pkg.EIGEN_REFERENCE if eigen is None else eigen, out.data_ptr(), stream)


def test_two_calls_in_a_row_match_the_allocating_entry_point(gpu_lib):
    import torch

    rng = np.random.default_rng(123)
    shape = (12, 20, 24)
    fields = [[rng.standard_normal(shape).astype(np.float32) for _ in range(3)] for _ in range(2)]
    expected = [pkg.TGVDeshadeProcessor.integrate_image_gradients_poisson_cosine_transform(*v)
                for v in fields]
    dev = [[torch.from_numpy(a).cuda() for a in v] for v in fields]
    outs = [torch.empty(shape, dtype=torch.float32, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    # two calls back to back on one stream, the second with different data
    assert _noalloc(*dev[0], shape, outs[0]) == pkg.OK
    assert _noalloc(*dev[1], shape, outs[1]) == pkg.OK
    torch.cuda.synchronize()
    for out, ref in zip(outs, expected):
        assert rel_l2(out.cpu().numpy(), ref) < TOL_DCT


def test_depth_one_and_shape_change(gpu_lib):
    import torch

    rng = np.random.default_rng(7)
    shape = (1, 40, 36)
    vx, vy = (rng.standard_normal(shape).astype(np.float32) for _ in range(2))
    ref = pkg.TGVDeshadeProcessor.integrate_image_gradients_poisson_cosine_transform(vx, vy, None)
    dvx, dvy = torch.from_numpy(vx).cuda(), torch.from_numpy(vy).cuda()
    out = torch.empty_like(dvx)
    assert _noalloc(dvx, dvy, None, shape, out) == pkg.OK
    torch.cuda.synchronize()
    assert rel_l2(out.cpu().numpy(), ref) < TOL_DCT


def test_rejects_volumes_beyond_the_static_scratch(gpu_lib):
    lib = pkg.lib()
    # too many voxels, and one side beyond the largest cosine table
    for w, h, d in ((256, 256, 64), (512, 8, 8)):
        st = lib.tgvdct_integrate_poisson_noalloc_dev(ctypes.c_void_p(16), ctypes.c_void_p(16),
                                                      ctypes.c_void_p(16), w, h, d, pkg.DCT_FP32,
                                                      pkg.EIGEN_REFERENCE, ctypes.c_void_p(16),
                                                      None)
        assert st == pkg.ERR_BAD_ARG
        assert b"TGVDCT_NOALLOC_MAX" in lib.tgvdct_last_error()


@pytest.mark.parametrize("shape", [(32, 256, 256), (256, 256, 32)])
@pytest.mark.parametrize("eigen", ["reference", "accurate"])
def test_largest_volumes_with_a_256_side(gpu_lib, shape, eigen):
    """At TGVDCT_NOALLOC_MAX_VOXELS with a side of 256 the volumes fill the static
    scratch and the cosine tables use their full rows."""
    import torch

    mode = pkg.EIGEN_REFERENCE if eigen == "reference" else pkg.EIGEN_ACCURATE
    assert int(np.prod(shape)) == NOALLOC_MAX_VOXELS
    rng = np.random.default_rng(11)
    v = [rng.standard_normal(shape).astype(np.float32) for _ in range(3)]
    ref = pkg.TGVDeshadeProcessor.integrate_image_gradients_poisson_cosine_transform(
        *v, poisson_eigen=mode)
    dev = [torch.from_numpy(a).cuda() for a in v]
    outs = [torch.empty(shape, dtype=torch.float32, device="cuda") for _ in range(2)]
    for out in outs:
        assert _noalloc(*dev, shape, out, eigen=mode) == pkg.OK
    torch.cuda.synchronize()
    for out in outs:
        assert rel_l2(out.cpu().numpy(), ref) < TOL_DCT


def test_a_call_leaves_free_device_memory_unchanged(gpu_lib):
    """After a first call (which loads the library's device code and does the
    set-up), a call changes the device's free memory by nothing."""
    import torch

    shape = (64, 64, 64)
    rng = np.random.default_rng(5)
    dev = [torch.from_numpy(rng.standard_normal(shape).astype(np.float32)).cuda()
           for _ in range(3)]
    out = torch.empty(shape, dtype=torch.float32, device="cuda")
    assert _noalloc(*dev, shape, out) == pkg.OK
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for eigen in (pkg.EIGEN_REFERENCE, pkg.EIGEN_ACCURATE):
        assert _noalloc(*dev, shape, out, eigen=eigen) == pkg.OK
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
