"""The persistent single-plane kernel (TGVDCT_KERNEL_PERSISTENT_PLANE, the automatic
choice for a single plane whose state fits in 96 MB) against the per-launch two-pass
kernels: the same device functions, so the results must be bit-identical, across
geometries, data terms, dual precisions, iteration counts that are not a multiple of
the launch chunk, callbacks that end a launch early, and a domain mask (which takes
the two-pass kernels)."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import rectangles_ellipses_2d

pytestmark = pytest.mark.gpu


def _run(f, kernel, iterations, *, geometry=pkg.GEOMETRY_2D, data=pkg.DATA_L1,
         precision=pkg.STATE_FP32, paint=0, calls=None, mask=None, tau=None):
    import torch
    H, W = f.shape
    prm = pkg.default_params(width=W, height=H, depth=1, iteration_count=iterations,
                             geometry=geometry, data_term=data, state_precision=precision,
                             iteration_kernel=kernel, paint_iteration_interval=paint)
    if tau is not None:
        prm.tau = prm.sigma = tau
    ft = torch.from_numpy(f).cuda()
    u, vx, vy, vz = (torch.empty_like(ft) for _ in range(4))
    cb = None
    if calls is not None:
        def fn(it, count, *_):
            calls.append(it)
            return 0
        cb = pkg.CALLBACK(fn)
    with pkg.Context(prm) as ctx:
        if mask is not None:
            m = torch.from_numpy(mask).cuda()
            ctx.set_domain_mask_dev(m.data_ptr())
        ctx.run_dev(ft.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr(),
                    callback=cb)
        torch.cuda.synchronize()
        ctx.check_device_error()
    return u, vx, vy, vz


def _same(a, b):
    import torch
    return all(torch.equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("shape,geometry,data,precision,iterations", [
    ((512, 512), pkg.GEOMETRY_2D, pkg.DATA_L1, pkg.STATE_FP32, 1000),
    ((257, 131), pkg.GEOMETRY_3D, pkg.DATA_L1, pkg.STATE_FP32, 77),
    ((96, 80), pkg.GEOMETRY_2D, pkg.DATA_L2, pkg.STATE_FP32, 45),
    ((300, 200), pkg.GEOMETRY_2D, pkg.DATA_L1, pkg.STATE_FX16_DUAL, 64),
    ((130, 64), pkg.GEOMETRY_3D, pkg.DATA_L2, pkg.STATE_BF16_DUAL, 33),
    ((3, 1000), pkg.GEOMETRY_2D, pkg.DATA_L1, pkg.STATE_FP32, 50),  # 3 rows: 3 blocks
    ((2000, 7), pkg.GEOMETRY_2D, pkg.DATA_L1, pkg.STATE_FP32, 50),  # thin: 13 px per row
])
def test_persistent_plane_equals_two_pass(gpu_lib, shape, geometry, data, precision,
                                          iterations):
    f = rectangles_ellipses_2d(*shape, seed=sum(shape))
    tau = 1.0 / np.sqrt(12.0) if shape == (512, 512) else None
    a = _run(f, pkg.KERNEL_PERSISTENT_PLANE, iterations, geometry=geometry, data=data,
             precision=precision, tau=tau)
    b = _run(f, pkg.KERNEL_TWO_PASS, iterations, geometry=geometry, data=data,
             precision=precision, tau=tau)
    assert _same(a, b)


def test_callbacks_end_launches_early(gpu_lib):
    f = rectangles_ellipses_2d(200, 240, seed=3)
    calls_a, calls_b = [], []
    a = _run(f, pkg.KERNEL_PERSISTENT_PLANE, 100, paint=7, calls=calls_a)
    b = _run(f, pkg.KERNEL_TWO_PASS, 100, paint=7, calls=calls_b)
    assert calls_a == calls_b == list(range(7, 100, 7))
    assert _same(a, b)


def test_automatic_choice_is_the_persistent_kernel_for_small_planes(gpu_lib):
    f = rectangles_ellipses_2d(160, 176, seed=5)
    a = _run(f, pkg.KERNEL_AUTO, 90)
    b = _run(f, pkg.KERNEL_TWO_PASS, 90)
    assert _same(a, b)


def test_domain_mask_takes_the_two_pass_kernels(gpu_lib):
    f = rectangles_ellipses_2d(128, 144, seed=9)
    mask = np.ones_like(f)
    mask[40:90, 30:100] = 0.0
    a = _run(f, pkg.KERNEL_PERSISTENT_PLANE, 60, mask=mask)
    b = _run(f, pkg.KERNEL_TWO_PASS, 60, mask=mask)
    assert _same(a, b)
