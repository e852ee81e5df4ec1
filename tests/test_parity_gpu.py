"""CUDA path against the reference's own kernels (golden fixtures) and the CPU oracle.

Tolerances: the FP32 kernels keep the reference's operation order (explicit fmaf
only), so the remaining differences are the rounding of CUDA's norm3df/cospif and
of the FP32 DCT contractions; they are stated per test below."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
import oracle
from ambient_image_processor_gb300.phantoms import rectangles_ellipses_2d, tissue_phantom_3d
from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

TOL_U = 2e-5    # relative L2 of u after <= 60 iterations
TOL_V = 2e-4    # relative L2 of v (small field, larger relative rounding)
TOL_DCT = 1e-5  # FP32 contraction vs the reference's FP64-basis sum


@pytest.mark.parametrize("name", ["deshade3d", "deshade3d_odd", "deshade3d_d1", "deshade3d_h1",
                                  "deshade3d_w1", "deshade3d_tiny"])
def test_deshade3d_vs_reference(gpu_lib, name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, vx, vy, vz = pkg.tgv2_l1_deshade_launch(g["f"], lam, int(it), 0, -1, None, a0, a1)
    assert rel_l2(u, g["u"]) < TOL_U
    for got, key in ((vx, "v_x"), (vy, "v_y"), (vz, "v_z")):
        assert np.abs(got - g[key]).max() < 1e-5 or rel_l2(got, g[key]) < TOL_V, key


@pytest.mark.parametrize("name", ["deshade2d", "deshade2d_odd"])
def test_deshade2d_vs_reference(gpu_lib, name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, vx, vy = pkg.tgv2_l1_deshade_launch_2d(g["f"], lam, int(it), 0, None, a0, a1)
    assert rel_l2(u, g["u"]) < TOL_U
    assert rel_l2(vx, g["v_x"]) < TOL_V and rel_l2(vy, g["v_y"]) < TOL_V


@pytest.mark.parametrize("name", ["denoise_l1", "denoise_l2", "denoise_l2_d1"])
def test_denoise_vs_reference(gpu_lib, name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u = pkg.tgv2_denoise_launch(g["f"], lam, int(it), a0, a1, int(g["data_term"]))
    assert rel_l2(u, g["u"]) < TOL_U


@pytest.mark.parametrize("tag", ["10x12x16", "1x18x24", "5x7x1", "1x1x9", "3x1x1", "4x4x4"])
def test_dct_ops_vs_reference(gpu_lib, tag):
    g = load_golden(f"dct_{tag}_f32")
    x = g["x"]
    assert rel_l2(pkg.cosine_transform_kernel_launch(x), g["cosine_transform"]) < TOL_DCT
    assert rel_l2(pkg.inverse_cosine_transform_kernel_launch(x),
                  g["inverse_cosine_transform"]) < TOL_DCT
    assert rel_l2(pkg.solve_poisson_in_cosine_domain_kernel_launch(x), g["solve_poisson"]) < 1e-6
    d = pkg.divergence_kernel_launch(g["v_x"], g["v_y"], g["v_z"])
    assert np.array_equal(d, g["divergence"])
    l = pkg.TGVDeshadeProcessor.integrate_image_gradients_poisson_cosine_transform(
        g["v_x"], g["v_y"], g["v_z"])
    assert rel_l2(l, g["integrate"]) < TOL_DCT


@pytest.mark.parametrize("name", ["process3d", "process3d_d1"])
def test_process_vs_reference(gpu_lib, name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, l, r = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(g["f"], lam, a0, a1, int(it))
    assert rel_l2(u, g["denoised"]) < TOL_U
    assert rel_l2(l, g["shading"]) < 1e-4
    assert rel_l2(r, g["deshaded"]) < 1e-4


@pytest.mark.parametrize("shape", [(33, 47, 29), (17, 130, 67), (1, 257, 131)])
def test_larger_volumes_vs_oracle(gpu_lib, shape):
    f = tissue_phantom_3d(*shape, seed=3)
    it = 150
    u, vx, vy, vz = pkg.tgv2_l1_deshade_launch(f, 1.0, it, 0, -1, None, 2.0, 1.0)
    ou, ovx, ovy, ovz = oracle.tgv2_deshade(f, 1.0, 2.0, 1.0, it, dtype=np.float32)
    assert rel_l2(u, ou) < 5e-5
    assert rel_l2(vx, ovx) < 5e-4 and rel_l2(vy, ovy) < 5e-4 and rel_l2(vz, ovz) < 5e-4


def test_l2_data_term_vs_oracle(gpu_lib):
    f = tissue_phantom_3d(20, 24, 28, seed=4)
    u = pkg.tgv2_denoise_launch(f, 0.8, 80, 2.0, 1.0, pkg.DATA_L2)
    ou, *_ = oracle.tgv2_deshade(f, 0.8, 2.0, 1.0, 80, data_term="l2", dtype=np.float32)
    assert rel_l2(u, ou) < TOL_U


def test_callback_cadence_and_stop(gpu_lib):
    f = tissue_phantom_3d(10, 16, 20, seed=5)
    seen = []

    def cb(it, count, u, vx, vy, vz):
        seen.append((it, count, u.copy()))
        return it == 20

    u, vx, vy, vz = pkg.tgv2_l1_deshade_launch(f, 1.0, 35, 10, -1, cb, 2.0, 1.0)
    assert [s[0] for s in seen] == [10, 20] and all(s[1] == 35 for s in seen)
    # stopped after iteration index 20, i.e. 21 iterations
    ou, ovx, *_ = oracle.tgv2_deshade(f, 1.0, 2.0, 1.0, 21, dtype=np.float32)
    assert rel_l2(u, ou) < TOL_U and rel_l2(seen[-1][2], ou) < TOL_U
    ou11, *_ = oracle.tgv2_deshade(f, 1.0, 2.0, 1.0, 11, dtype=np.float32)
    assert rel_l2(seen[0][2], ou11) < TOL_U


def test_process_callback_gets_u_l_r(gpu_lib):
    f = tissue_phantom_3d(8, 12, 16, seed=6)
    got = []

    def cb(it, count, u, l, r):
        got.append((it, u, l, r))
        return False

    u, l, r = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(
        f, 1.0, 2.0, 1.0, 25, paint_iteration_interval=12, iteration_finished_callback=cb)
    assert [g[0] for g in got] == [12, 24]
    ou, ol, orr = oracle.process_tgv2_l1(f, 1.0, 2.0, 1.0, 13, dtype=np.float32)
    assert rel_l2(got[0][1], ou) < TOL_U and rel_l2(got[0][2], ol) < 1e-4
    assert rel_l2(got[0][3], orr) < 1e-4


def test_mask_and_add_back(gpu_lib):
    f = tissue_phantom_3d(8, 12, 16, seed=8)
    mask = (np.random.default_rng(0).random(f.shape) > 0.3).astype(np.float32)
    u, l, r = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(f, 1.0, 2.0, 1.0, 30, mask_image=mask,
                                                           add_background_back=True)
    ou, ovx, ovy, ovz = oracle.tgv2_deshade(f, 1.0, 2.0, 1.0, 30, dtype=np.float32)
    ol = oracle.integrate_poisson_dct(ovx, ovy, ovz)
    orr, olm = oracle.deshade_epilogue(ou, ol, mask, True, True)
    assert rel_l2(l, olm) < 1e-4 and rel_l2(r, orr) < 1e-4


def test_log_domain(gpu_lib):
    f = tissue_phantom_3d(10, 14, 18, seed=9)
    u, l, r = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(
        f, 1.0, 2.0, 1.0, 30, set_negative_values_to_zero=False, log_domain=True)
    ou, ol, orr = oracle.process_tgv2_l1(np.log(f), 1.0, 2.0, 1.0, 30,
                                         set_negative_values_to_zero=False, dtype=np.float32)
    assert rel_l2(np.log(u), ou) < 1e-4
    assert rel_l2(np.log(l), ol) < 1e-3
    assert rel_l2(np.log(r), orr) < 1e-4


def test_2d_geometry_differs_from_3d_on_depth_one(gpu_lib):
    # the terminal program runs 2-D images through the 3-D launcher (B_z w = -w on the
    # single slice), which is not the 2-D launcher's result
    f = rectangles_ellipses_2d(20, 24, seed=3)
    u3, vx3, vy3, vz3 = pkg.tgv2_l1_deshade_launch(f[None], 1.0, 30, 0, -1, None, 2.0, 1.0)
    u2, vx2, vy2 = pkg.tgv2_l1_deshade_launch_2d(f, 1.0, 30, 0, None, 2.0, 1.0)
    assert np.abs(u3[0] - u2).max() > 1e-3 and np.abs(vz3).max() > 1e-3


# Relative L2 error of u and r against the FP64 oracle after 100 iterations of a
# 24x32x40 phantom, per state precision (BF16 keeps 8 mantissa bits of p and q; the
# 16-bit fixed point keeps 15 bits of p/alpha1 and q/alpha0).
MIXED_TOL = {pkg.STATE_FP32: 1e-5, pkg.STATE_BF16_DUAL: 5e-3, pkg.STATE_FX16_DUAL: 2e-4}


@pytest.mark.parametrize("prec", [pkg.STATE_FP32, pkg.STATE_BF16_DUAL, pkg.STATE_FX16_DUAL])
def test_state_precision_error_vs_fp64(gpu_lib, prec):
    f = tissue_phantom_3d(24, 32, 40, seed=10)
    u, l, r = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(f, 1.0, 2.0, 1.0, 100,
                                                           state_precision=prec,
                                                           poisson_eigen=pkg.EIGEN_ACCURATE)
    ou, ol, orr = oracle.process_tgv2_l1(f, 1.0, 2.0, 1.0, 100, dtype=np.float64)
    assert rel_l2(u, ou) < MIXED_TOL[prec]
    assert rel_l2(r, orr) < MIXED_TOL[prec]


def test_bad_arguments_raise(gpu_lib):
    with pytest.raises(pkg.TgvdctError):
        pkg.tgv2_l1_deshade_launch(np.zeros((2, 3, 4), np.float32), 1.0, 5, 0, -1, None, 0.0, 1.0)


@pytest.mark.parametrize("prec", [pkg.STATE_FP32, pkg.STATE_FX16_DUAL, pkg.STATE_BF16_DUAL])
@pytest.mark.parametrize("kernel", [pkg.KERNEL_FUSED, pkg.KERNEL_FUSED_REGISTER,
                                    pkg.KERNEL_FUSED_SHIFTED])
@pytest.mark.parametrize("shape,z_chunk,two_d,data_term", [
    ((37, 45, 72), 5, False, pkg.DATA_L1),   # width % 8 == 0: the TMA pipeline
    ((37, 45, 70), 5, False, pkg.DATA_L1),   # width % 4 != 0: register prefetch
    ((19, 8, 64), 0, False, pkg.DATA_L2),
    ((19, 8, 33), 0, False, pkg.DATA_L2),
    ((6, 17, 40), 1, False, pkg.DATA_L1),
    ((1, 50, 40), 0, False, pkg.DATA_L1),
    ((1, 50, 40), 0, True, pkg.DATA_L1),
    ((1, 50, 41), 0, True, pkg.DATA_L1),
    ((4, 1, 9), 1, False, pkg.DATA_L1),
    ((3, 5, 8), 2, False, pkg.DATA_L2),
])
def test_fused_kernels_equal_two_pass(gpu_lib, prec, kernel, shape, z_chunk, two_d, data_term):
    # same update sequence: one pass with on-chip halo recompute (TMA-fed or
    # register-fed) vs two in-place passes, so the results are bit-identical
    f = tissue_phantom_3d(*shape, seed=12)
    if two_d:
        f = f[0]
    kw = dict(state_precision=prec, data_term=data_term, two_d=two_d,
              set_negative_values_to_zero=False)
    a = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(f, 0.9, 2.0, 1.0, 40,
                                                     iteration_kernel=pkg.KERNEL_TWO_PASS, **kw)
    b = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(f, 0.9, 2.0, 1.0, 40,
                                                     iteration_kernel=kernel,
                                                     z_chunk=z_chunk, **kw)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


# Tensor-core DCT modes against the reference's FP64 results.  BF16x3 keeps ~16
# significant bits per product; one TF32 product keeps ~11.
TC_TOL = {pkg.DCT_BF16X3: 3e-5, pkg.DCT_TF32: 3e-3}


@pytest.mark.parametrize("mode", [pkg.DCT_BF16X3, pkg.DCT_TF32])
@pytest.mark.parametrize("tag", ["10x12x16", "1x18x24", "5x7x1", "1x1x9", "3x1x1", "4x4x4"])
def test_tensor_core_dct_vs_fp64_reference(gpu_lib, mode, tag):
    g = load_golden(f"dct_{tag}_f64")
    x = g["x"].astype(np.float32)
    tol = TC_TOL[mode]
    assert rel_l2(pkg.cosine_transform_kernel_launch(x, mode), g["cosine_transform"]) < tol
    assert rel_l2(pkg.inverse_cosine_transform_kernel_launch(x, mode),
                  g["inverse_cosine_transform"]) < tol
    l = pkg.TGVDeshadeProcessor.integrate_image_gradients_poisson_cosine_transform(
        g["v_x"], g["v_y"], g["v_z"], dct_mode=mode, poisson_eigen=pkg.EIGEN_ACCURATE)
    # l is a smoothed difference of v: its error is bounded relative to v, not to l
    vmax = max(np.abs(g[k]).max() for k in ("v_x", "v_y", "v_z"))
    assert rel_l2(l, g["integrate"]) < 4 * tol or np.abs(l - g["integrate"]).max() < tol * vmax


@pytest.mark.parametrize("mode", [pkg.DCT_FP32, pkg.DCT_BF16X3, pkg.DCT_TF32])
@pytest.mark.parametrize("shape", [(40, 72, 136), (1, 200, 256), (256, 16, 24)])
def test_dct_round_trip_and_vs_oracle(gpu_lib, mode, shape):
    rng = np.random.default_rng(5)
    x = rng.standard_normal(shape).astype(np.float32)
    y = pkg.inverse_cosine_transform_kernel_launch(pkg.cosine_transform_kernel_launch(x, mode),
                                                   mode)
    assert rel_l2(y, x) < (2e-5 if mode != pkg.DCT_TF32 else 5e-3)
    ref = oracle.cosine_transform(x.astype(np.float64))
    assert rel_l2(pkg.cosine_transform_kernel_launch(x, mode), ref) < (
        1e-6 if mode == pkg.DCT_FP32 else TC_TOL[mode])
