"""The down-sampled deshade (tgvk_deshade_downsampled/ in the reference) and its cubic
B-spline resize (resize/ResizeProcessor.cpp through ITK) on the GPU, against the oracle.
The resize runs the same FP64 operation sequence as the oracle and must agree bit for
bit; the deshade agrees within the FP32 loop tolerance of the other deshade tests."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
import oracle
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5  # FP32 GPU loop vs the oracle's FP32 loop (device norm3df/sqrtf vs CPU)


def blob_mask(shape, seed=0):
    d, h, w = shape
    z, y, x = np.meshgrid(np.linspace(-1, 1, d) if d > 1 else np.zeros(1),
                          np.linspace(-1, 1, h), np.linspace(-1, 1, w), indexing="ij")
    m = ((x / 0.8) ** 2 + ((y - 0.1) / 0.75) ** 2 + (z / 0.85) ** 2 < 1).astype(np.float32)
    return m


RESIZES = [
    ((16, 24, 32), (8, 12, 16)),       # factor 1/2: the knots
    ((13, 29, 40), (5, 11, 15)),       # factor 0.37
    ((8, 12, 16), (16, 24, 32)),       # upsampling: two extra samples, then cropped
    ((6, 9, 17), (5, 7, 12)),          # lines short enough for the closed mirror start
    ((1, 37, 50), (1, 23, 30)),        # 2-D
    ((1, 23, 30), (1, 37, 50)),        # 2-D upsampling (the grid grows in depth too)
    ((1, 1, 40), (1, 1, 27)),          # single-sample axes
]


@pytest.mark.parametrize("src,dst", RESIZES)
def test_resize_is_bit_identical_to_the_oracle(gpu_lib, src, dst):
    x = np.random.default_rng(sum(src)).standard_normal(src).astype(np.float32)
    got = pkg.ResizeProcessor.process(x, dst[2], dst[1], dst[0])
    want = oracle.resize_bspline3(x, dst)
    assert got.shape == tuple(dst)
    assert np.array_equal(got, want)


def test_resize_knots_and_constants_at_full_size(gpu_lib):
    """256x256x192 -> 128x128x96 samples the knots: the interpolant equals the data
    there up to the FP64 prefilter's rounding (about 1e-15 absolute, more than a float
    ulp only for values within ~1e-8 of zero); a constant stays exactly 1.0 (the masked
    deshade thresholds the resized mask at 1)."""
    import torch
    x = torch.randn((192, 256, 256), device="cuda", generator=torch.Generator(
        device="cuda").manual_seed(5))
    y = torch.empty((96, 128, 128), device="cuda")
    pkg._check(pkg.lib().tgvdct_resize_bspline3_dev(x.data_ptr(), 256, 256, 192, y.data_ptr(),
                                                     128, 128, 96, None))
    assert float((y - x[::2, ::2, ::2]).abs().max()) < 1e-6
    ones = torch.ones((96, 128, 128), device="cuda")
    up = torch.empty((192, 256, 256), device="cuda")
    pkg._check(pkg.lib().tgvdct_resize_bspline3_dev(ones.data_ptr(), 128, 128, 96, up.data_ptr(),
                                                     256, 256, 192, None))
    assert bool((up == 1).all())


CASES = [
    # (shape, factor, masked-variant?, with mask?)
    ((20, 28, 36), 0.5, True, True),
    ((20, 28, 36), 0.5, True, False),
    ((20, 28, 36), 0.5, False, True),
    ((19, 27, 33), 0.6, False, False),
    ((1, 48, 64), 0.5, True, True),
    ((1, 48, 64), 0.5, False, True),
    ((12, 16, 20), 1.0, True, True),
]


@pytest.mark.parametrize("shape,factor,masked,with_mask", CASES)
def test_downsampled_deshade_matches_the_oracle(gpu_lib, shape, factor, masked, with_mask):
    f = tissue_phantom_3d(*shape, seed=6).reshape(shape)
    if shape[0] == 1:
        f = f[0]
    mask = blob_mask(shape).reshape(f.shape) if with_mask else None
    proc = (pkg.TGVKDeshadeDownsampledProcessor if masked
            else pkg.TGVKDeshadeDownsampledNotMaskedProcessor)
    u, l, r, dv = proc.processTGVKL1Cuda(f, factor, 1.0, 2, [1.0, 2.0], 60, mask=mask,
                                         set_negative_values_to_zero=True,
                                         add_background_back=True, calculate_div_v=True)
    ou, ol, orr, odv = oracle.process_tgvk_l1_downsampled(
        f, factor, 1.0, 2, [1.0, 2.0], 60, mask=mask, set_negative_values_to_zero=True,
        add_background_back=True, not_masked=not masked, calculate_div_v=True)
    for name, a, b in (("u", u, ou), ("l", l, ol), ("r", r, orr), ("div v", dv, odv)):
        assert a.shape == f.shape
        assert rel_l2(a, b) < TOL, name


def test_callback_sees_the_downsampled_images(gpu_lib):
    f = tissue_phantom_3d(16, 20, 24, seed=7)
    seen = []

    def cb(i, count, u, l, r):
        seen.append((i, u.shape, l.shape, r.shape))
        return False

    pkg.TGVKDeshadeDownsampledProcessor.processTGVKL1Cuda(
        f, 0.5, 1.0, 2, [1.0, 2.0], 20, paint_iteration_interval=10,
        iteration_finished_callback=cb)
    assert [s[0] for s in seen] == [10]
    assert all(s[1] == (8, 10, 12) == s[2] == s[3] for s in seen)


def test_orders_other_than_two_are_refused(gpu_lib):
    f = np.ones((8, 8, 8), np.float32)
    with pytest.raises(pkg.TgvdctError) as e:
        pkg.TGVKDeshadeDownsampledProcessor.processTGVKL1Cuda(f, 0.5, 1.0, 3, [1, 2, 3], 5)
    assert e.value.status == pkg.ERR_UNSUPPORTED
    assert "order 3" in str(e.value)


def test_downsampled_program_writes_shading_and_deshaded(gpu_lib, tmp_path):
    """tgvk_deshade_downsampled_application input f order lambda iterations [mask]
    prefix: alpha = (1, 2), the clamp and the add-back, as the reference program."""
    import os
    import subprocess

    from ambient_image_processor_gb300 import build as pkg_build
    from test_refapi_gpu import read_mha, write_mha
    f = tissue_phantom_3d(16, 20, 24, seed=8)
    mask = blob_mask(f.shape)
    write_mha(str(tmp_path / "f.mha"), f)
    write_mha(str(tmp_path / "m.mha"), mask)
    exe = pkg_build.DOWNSAMPLED_CLI
    assert os.path.exists(exe)
    prefix = str(tmp_path / "out")
    r = subprocess.run([exe, str(tmp_path / "f.mha"), "0.5", "2", "1", "40",
                        str(tmp_path / "m.mha"), prefix], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _, ol, orr, _ = oracle.process_tgvk_l1_downsampled(f, 0.5, 1.0, 2, [1.0, 2.0], 40, mask=mask,
                                                       set_negative_values_to_zero=True,
                                                       add_background_back=True)
    assert rel_l2(read_mha(prefix + "_shading.mha"), ol) < TOL
    assert rel_l2(read_mha(prefix + "_deshaded.mha"), orr) < TOL
    r = subprocess.run([exe, str(tmp_path / "f.mha"), "0.5", "3", "1", "40", prefix],
                       capture_output=True, text=True)
    assert r.returncode == 10 + pkg.ERR_UNSUPPORTED and "order 3" in r.stderr
