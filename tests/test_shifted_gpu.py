"""Shifted passes (TGVDCT_KERNEL_FUSED_SHIFTED).

Each pass runs the primal step of one iteration and the dual step of the next, so the
duals run half an iteration ahead between passes; a dual step before a run and a primal
step after it convert the loop state.  The arithmetic of every update is the same
sequence as in the two-pass and fused kernels, so the results must be bit-identical to
theirs: for both parities of a run, every z-chunking, shapes whose blocks all touch the
volume's faces and shapes with blocks that run without boundary tests, both data terms,
callbacks between runs, CUDA graph replays of long runs, the stepping entry point and
the state snapshot, masked runs (frozen voxels outside the domain) and 16-bit duals."""
import ctypes

import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu


def _process(f, kernel, iterations, **kw):
    return pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(
        f, 0.9, 2.0, 1.0, iterations, iteration_kernel=kernel,
        set_negative_values_to_zero=False, **kw)


def _equal(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


# (depth, height, width), z-chunk: depth 2 and 3, single-plane chunks, widths a
# multiple of 4 but not of 32 (edge blocks with idle columns), heights not a multiple
# of 8, and widths / heights with blocks away from every face (no boundary tests)
SHAPES = [((2, 16, 32), 0), ((3, 20, 36), 1), ((9, 26, 100), 2), ((9, 26, 100), 4),
          ((17, 33, 68), 0), ((12, 40, 132), 5)]


@pytest.mark.parametrize("iterations", [2, 3, 4, 7])
@pytest.mark.parametrize("shape,z_chunk", SHAPES)
def test_runs_equal_two_pass(gpu_lib, iterations, shape, z_chunk):
    f = tissue_phantom_3d(*shape, seed=21)
    ref = _process(f, pkg.KERNEL_TWO_PASS, iterations)
    _equal(ref, _process(f, pkg.KERNEL_FUSED_SHIFTED, iterations, z_chunk=z_chunk))


@pytest.mark.parametrize("prec", [pkg.STATE_FX16_DUAL, pkg.STATE_BF16_DUAL])
@pytest.mark.parametrize("iterations", [2, 5])
@pytest.mark.parametrize("shape,z_chunk", [((9, 26, 104), 2), ((12, 40, 136), 0),
                                           ((3, 20, 40), 1)])
def test_16bit_duals_equal_two_pass(gpu_lib, prec, iterations, shape, z_chunk):
    # p, q stored in 16 bits (widths a multiple of 8 for the TMA strides), every update
    # in FP32: the same rounding of the stored duals as the other kernels
    f = tissue_phantom_3d(*shape, seed=28)
    ref = _process(f, pkg.KERNEL_TWO_PASS, iterations, state_precision=prec)
    _equal(ref, _process(f, pkg.KERNEL_FUSED_SHIFTED, iterations, state_precision=prec,
                         z_chunk=z_chunk))
    _equal(ref, _process(f, pkg.KERNEL_FUSED, iterations, state_precision=prec))


# extreme shapes: one row, a width of 4 (one column of TMA alignment), two planes,
# heights and widths that leave a single tile with idle rows and columns
@pytest.mark.parametrize("shape,z_chunk", [((2, 1, 4), 0), ((5, 1, 36), 2), ((3, 9, 4), 1),
                                           ((2, 2, 8), 0), ((40, 3, 12), 7)])
def test_extreme_shapes(gpu_lib, shape, z_chunk):
    f = tissue_phantom_3d(*shape, seed=26)
    ref = _process(f, pkg.KERNEL_TWO_PASS, 9)
    _equal(ref, _process(f, pkg.KERNEL_FUSED_SHIFTED, 9, z_chunk=z_chunk))


def _mask(shape):
    """An off-centre ellipsoid with scattered holes: blocks wholly outside the domain,
    wholly inside, and mixed, and plane ranges trimmed at both ends."""
    d, h, w = shape
    z, y, x = np.indices(shape, dtype=np.float64)
    r = ((z - 0.55 * d) / (0.4 * d)) ** 2 + ((y - 0.45 * h) / (0.45 * h)) ** 2 + \
        ((x - 0.5 * w) / (0.4 * w)) ** 2
    holes = (z * 7 + y * 3 + x) % 11 == 0
    return ((r < 1.0) & ~holes).astype(np.float32) * 2.0  # the domain is mask >= 1


@pytest.mark.parametrize("iterations", [2, 7])
@pytest.mark.parametrize("shape,z_chunk", [((9, 26, 100), 0), ((12, 40, 132), 5),
                                           ((3, 20, 36), 1), ((20, 24, 64), 3)])
def test_masked_runs_equal_two_pass(gpu_lib, iterations, shape, z_chunk):
    f = tissue_phantom_3d(*shape, seed=27)
    m = _mask(shape)
    kw = dict(mask=m, set_negative_values_to_zero=False)
    a = pkg.TGVDeshadeMaskedProcessor.processTGV2L1GPUCuda(
        f, 0.9, 2.0, 1.0, iterations, iteration_kernel=pkg.KERNEL_TWO_PASS, **kw)
    b = pkg.TGVDeshadeMaskedProcessor.processTGV2L1GPUCuda(
        f, 0.9, 2.0, 1.0, iterations, iteration_kernel=pkg.KERNEL_FUSED_SHIFTED,
        z_chunk=z_chunk, **kw)
    _equal(a, b)


@pytest.mark.parametrize("data_term", [pkg.DATA_L1, pkg.DATA_L2])
def test_data_terms_and_long_runs(gpu_lib, data_term):
    # 300 iterations: the first alone, then one graph replay of 299
    f = tissue_phantom_3d(10, 24, 64, seed=22)
    ref = _process(f, pkg.KERNEL_TWO_PASS, 300, data_term=data_term)
    _equal(ref, _process(f, pkg.KERNEL_FUSED_SHIFTED, 300, data_term=data_term))
    _equal(ref, _process(f, pkg.KERNEL_FUSED, 300, data_term=data_term))


def test_callbacks_between_runs(gpu_lib):
    f = tissue_phantom_3d(8, 24, 40, seed=23)
    seen = {}

    def keep(kernel):
        def cb(it, count, u, l, r):
            seen.setdefault(kernel, []).append((it, u.copy(), l.copy(), r.copy()))
            return it == 30
        return cb

    outs = {}
    for kernel in (pkg.KERNEL_TWO_PASS, pkg.KERNEL_FUSED_SHIFTED):
        outs[kernel] = _process(f, kernel, 47, paint_iteration_interval=5,
                                iteration_finished_callback=keep(kernel))
    a, b = seen[pkg.KERNEL_TWO_PASS], seen[pkg.KERNEL_FUSED_SHIFTED]
    assert [s[0] for s in a] == [s[0] for s in b] == [5, 10, 15, 20, 25, 30]
    for x, y in zip(a, b):
        _equal(x[1:], y[1:])
    _equal(outs[pkg.KERNEL_TWO_PASS], outs[pkg.KERNEL_FUSED_SHIFTED])


def _loop_state(kernel, f, steps, **kw):
    """u, v and the launches after tgvdct_tgv2_step_dev calls of the given lengths."""
    import torch
    d, h, w = f.shape
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=1,
                             iteration_kernel=kernel, **kw)
    ft = torch.from_numpy(f).cuda()
    with pkg.Context(prm) as ctx:
        L = pkg.lib()
        assert L.tgvdct_state_init_dev(ctx._ctx, ctypes.c_void_p(ft.data_ptr()), None) == pkg.OK
        launches = []
        for n in steps:
            assert L.tgvdct_tgv2_step_dev(ctx._ctx, n, None) == pkg.OK
            launches.append(ctx.loop_launches())
        buf = torch.zeros((ctx.state_bytes() + 3) // 4, dtype=torch.float32, device="cuda")
        ctx.save_state_dev(buf.data_ptr())
        torch.cuda.synchronize()
        ctx.check_device_error()
        return buf.cpu().numpy(), launches


def test_stepping_and_snapshot_equal_fused(gpu_lib):
    f = np.log(tissue_phantom_3d(7, 18, 44, seed=24)).astype(np.float32)
    steps = [5, 1, 2, 9]
    a, la = _loop_state(pkg.KERNEL_FUSED, f, steps)
    b, lb = _loop_state(pkg.KERNEL_FUSED_SHIFTED, f, steps)
    # the whole snapshot (f, u, v and the current ubar, vbar, p, q) is the same
    assert np.array_equal(a, b)
    assert la == [5, 1, 2, 9]
    assert lb == [6, 1, 3, 10]  # a run of n >= 2 is n + 1 launches


def test_loop_launch_count(gpu_lib):
    import torch
    f = torch.from_numpy(tissue_phantom_3d(6, 16, 32, seed=25)).cuda()
    out = [torch.empty_like(f) for _ in range(4)]
    counts = {}
    for kernel in (pkg.KERNEL_FUSED, pkg.KERNEL_FUSED_SHIFTED, pkg.KERNEL_TWO_PASS):
        prm = pkg.default_params(width=32, height=16, depth=6, iteration_count=300,
                                 iteration_kernel=kernel)
        with pkg.Context(prm) as ctx:
            ctx.run_dev(f.data_ptr(), *(o.data_ptr() for o in out))
            torch.cuda.synchronize()
            counts[kernel] = ctx.loop_launches()
    assert counts[pkg.KERNEL_FUSED] == 300
    assert counts[pkg.KERNEL_TWO_PASS] == 600
    # the first iteration alone, then a graph of 299 (a dual step, 298 shifted passes,
    # a primal step)
    assert counts[pkg.KERNEL_FUSED_SHIFTED] == 1 + 300
    prm = pkg.default_params(width=32, height=16, depth=6, iteration_count=1300,
                             iteration_kernel=pkg.KERNEL_FUSED_SHIFTED)
    with pkg.Context(prm) as ctx:
        for _ in range(2):  # the second run replays the graphs of the first
            ctx.run_dev(f.data_ptr(), *(o.data_ptr() for o in out))
            torch.cuda.synchronize()
            # replays of at most 512 iterations: 1 + (512 + 1) + (512 + 1) + (275 + 1)
            assert ctx.loop_launches() == 1 + 513 + 513 + 276
