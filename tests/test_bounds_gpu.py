"""The bounds-checking build (libtgvdct_checked.so: every instrumented kernel checks
the indices it is about to use and records the first bad one instead of making the
access).  compute-sanitizer is not available on these GPUs; the checked library plus
small and odd shapes stands in for it.  Each path must record nothing and give exactly the
normal library's results."""
import ctypes

import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu


def _first_bad(L):
    w = ctypes.c_uint64(0)
    assert L.tgvdct_bounds_check(ctypes.byref(w)) == pkg.OK, L.tgvdct_last_error()
    return w.value


def _process(L, f, mask=None, **kw):
    w, h, d = pkg._dims(f)
    p = pkg.default_params(width=w, height=h, depth=d, iteration_count=25, **kw)
    u, l, r = (np.empty_like(f) for _ in range(3))
    if mask is None:
        st = L.tgvdct_process_tgv2_l1(ctypes.byref(p), f, None, 0, 0, 1, pkg.CALLBACK(), None,
                                      u, l, r)
    else:
        st = L.tgvdct_process_tgv2_l1_masked(ctypes.byref(p), f, mask, 0, 1, 1, pkg.CALLBACK(),
                                             None, u, l, r)
    assert st == pkg.OK, L.tgvdct_last_error()
    return u, l, r


SHAPES = [
    ((13, 24, 32), {}),                                           # fused TMA kernel
    ((9, 17, 30), {}),                                            # register-staged (width 30)
    ((11, 20, 36), {"iteration_kernel": pkg.KERNEL_TWO_PASS}),
    ((7, 9, 12), {"state_precision": pkg.STATE_BF16_DUAL}),       # 16-bit duals, small
    ((1, 33, 47), {"geometry": pkg.GEOMETRY_2D}),                 # 2-D (two-pass)
    ((1, 40, 64), {"geometry": pkg.GEOMETRY_2D, "iteration_kernel": pkg.KERNEL_FUSED}),
    ((5, 8, 8), {}),
    # shifted passes: edge blocks only, then blocks without boundary tests as well
    ((13, 24, 32), {"iteration_kernel": pkg.KERNEL_FUSED_SHIFTED}),
    ((6, 30, 100), {"iteration_kernel": pkg.KERNEL_FUSED_SHIFTED, "z_chunk": 2}),
]


@pytest.mark.parametrize("shape,kw", SHAPES)
def test_deshade_paths_stay_in_bounds(gpu_lib, shape, kw):
    Lc, L = pkg.lib_checked(), pkg.lib()
    f = tissue_phantom_3d(*shape, seed=13).astype(np.float32)  # the calls take the log
    if shape[0] == 1:
        f = np.ascontiguousarray(f[0])
    assert _first_bad(Lc) == 0
    got = _process(Lc, f, **kw)
    assert _first_bad(Lc) == 0
    for a, b in zip(got, _process(L, f, **kw)):
        assert np.array_equal(a, b, equal_nan=True) and np.isfinite(a).any()


def test_masked_and_downsampled_paths_stay_in_bounds(gpu_lib):
    Lc, L = pkg.lib_checked(), pkg.lib()
    f = tissue_phantom_3d(12, 20, 28, seed=14).astype(np.float32)
    m = (np.indices(f.shape).sum(axis=0) % 7 != 0).astype(np.float32)
    got = _process(Lc, f, mask=m)
    assert _first_bad(Lc) == 0
    for a, b in zip(got, _process(L, f, mask=m)):
        assert np.array_equal(a, b, equal_nan=True) and np.isfinite(a).any()
    # the masked shifted passes, on blocks away from every face as well
    g = tissue_phantom_3d(10, 30, 100, seed=15).astype(np.float32)
    gm = (np.indices(g.shape).sum(axis=0) % 7 != 0).astype(np.float32)
    gm[:, :, :20] = 0.0
    kw = {"iteration_kernel": pkg.KERNEL_FUSED_SHIFTED, "z_chunk": 3}
    got = _process(Lc, g, mask=gm, **kw)
    assert _first_bad(Lc) == 0
    for a, b in zip(got, _process(L, g, mask=gm, **kw)):
        assert np.array_equal(a, b, equal_nan=True) and np.isfinite(a).any()
    alpha = np.array([1.0, 2.0], np.float32)
    outs = []
    for lib in (Lc, L):
        u, l, r, dv = (np.empty_like(f) for _ in range(4))
        st = lib.tgvdct_process_tgvk_l1_downsampled(
            f, m.ctypes.data_as(ctypes.c_void_p), 28, 20, 12, 0.6, 1.0, 2, alpha, 15, 1, 1, 0, 0,
            pkg.CALLBACK(), None, u, l, r, dv.ctypes.data_as(ctypes.c_void_p))
        assert st == pkg.OK
        outs.append((u, l, r, dv))
    assert _first_bad(Lc) == 0
    for a, b in zip(*outs):
        assert np.array_equal(a, b, equal_nan=True) and np.isfinite(a).any()


@pytest.mark.parametrize("kernel", [pkg.KERNEL_AUTO, pkg.KERNEL_FUSED_SHIFTED])
@pytest.mark.parametrize("shape", [(10, 12, 16), (40, 40, 40), (21, 19, 44)])
def test_reverse_mode_stays_in_bounds(gpu_lib, shape, kernel):
    """The reverse sweep: one-voxel adjoint kernels at the small shape, the z-marching
    projection pass at the larger ones; with shifted passes as the iteration kernel the
    fused adjoint pass between them (edge tiles with idle rows and columns at 21 x 19 x
    44)."""
    import torch
    Lc = pkg.lib_checked()
    d, h, w = shape
    f = torch.from_numpy(np.log(tissue_phantom_3d(*shape, seed=15))).cuda()
    gu = torch.ones_like(f)
    p = pkg.default_params(width=w, height=h, depth=d, iteration_count=12,
                           iteration_kernel=kernel)
    ctx = ctypes.c_void_p()
    assert Lc.tgvdct_create(ctypes.byref(p), ctypes.byref(ctx)) == pkg.OK
    try:
        u, vx, vy, vz, gf = (torch.empty_like(f) for _ in range(5))
        gp = torch.empty(3, dtype=torch.float64, device="cuda")
        assert Lc.tgvdct_tgv2_forward_checkpointed_dev(ctx, f.data_ptr(), u.data_ptr(),
                                                       vx.data_ptr(), vy.data_ptr(),
                                                       vz.data_ptr(), 5, None) == pkg.OK
        assert Lc.tgvdct_tgv2_backward_dev(ctx, gu.data_ptr(), None, None, None, gf.data_ptr(),
                                           gp.data_ptr(), None) == pkg.OK
        torch.cuda.synchronize()
        assert _first_bad(Lc) == 0
        assert torch.isfinite(gf).all()
    finally:
        Lc.tgvdct_destroy(ctx)
