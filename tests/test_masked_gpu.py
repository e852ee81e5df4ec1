"""The masked deshade on the GPU (tgv_deshade_masked/ in the reference) against the
reference's own masked kernels (golden fixtures) and the oracle."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
import oracle
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

MASKED = ["masked3d", "masked3d_odd", "masked2d", "masked2d_back"]
TOL = 1e-5  # FP32 GPU vs the reference's FP32 kernels (device norm3df/sqrtf vs CPU)


def ellipsoid_mask(shape, seed=0):
    rng = np.random.default_rng(seed)
    d, h, w = shape
    z, y, x = np.meshgrid(np.linspace(-1, 1, d) if d > 1 else np.zeros(1),
                          np.linspace(-1, 1, h), np.linspace(-1, 1, w), indexing="ij")
    m = (((x - 0.2) / 0.85) ** 2 + (y / 0.7) ** 2 + ((z + 0.1) / 0.9) ** 2 < 1).astype(np.float32)
    m[rng.random(m.shape) < 0.02] = 0.0  # holes inside the domain
    return m


@pytest.mark.parametrize("name", MASKED)
def test_masked_loop_matches_reference(gpu_lib, name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, vx, vy, vz = pkg.tgv2_l1_deshade_masked_launch(g["f"], g["mask"], lam, int(it), a0, a1)
    assert rel_l2(u, g["u"]) < TOL
    for got, key in ((vx, "v_x"), (vy, "v_y"), (vz, "v_z")):
        assert rel_l2(got, g[key]) < TOL
    out = g["mask"] < 1  # outside the domain nothing moves
    assert np.array_equal(u[out], g["f"][out])
    assert not np.any(vx[out]) and not np.any(vy[out]) and not np.any(vz[out])


@pytest.mark.parametrize("name", MASKED)
def test_masked_processor_matches_reference(gpu_lib, name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, l, r = pkg.TGVDeshadeMaskedProcessor.processTGV2L1GPUCuda(
        g["f"], lam, a0, a1, int(it), mask=g["mask"], set_negative_values_to_zero=True,
        add_background_back=bool(g["add_background_back"]))
    assert rel_l2(u, g["denoised"]) < TOL
    assert rel_l2(l, g["shading"]) < 1e-4  # l is small: relative error of a small field
    assert rel_l2(r, g["deshaded"]) < TOL


@pytest.mark.parametrize("shape", [(12, 24, 64), (9, 17, 62), (1, 40, 48)])
@pytest.mark.parametrize("precision", [pkg.STATE_FP32, pkg.STATE_FX16_DUAL])
def test_masked_kernels_agree_and_match_oracle(gpu_lib, shape, precision):
    """TMA fused (width multiple of 4), its two-pass fallback (width 62) and the
    two-pass kernels give the same bits under a domain mask; FP32 matches the oracle."""
    import torch
    f = np.log(tissue_phantom_3d(*shape, seed=23)).astype(np.float32)
    m = ellipsoid_mask(shape, 3)
    d, h, w = shape
    geometry = pkg.GEOMETRY_2D if d == 1 else pkg.GEOMETRY_3D
    ft, mt = torch.from_numpy(f).cuda(), torch.from_numpy(m).cuda()
    outs = {}
    for kernel in (pkg.KERNEL_FUSED, pkg.KERNEL_TWO_PASS):
        prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=45,
                                 geometry=geometry, state_precision=precision,
                                 iteration_kernel=kernel, z_chunk=5)
        u, vx, vy, vz = (torch.empty_like(ft) for _ in range(4))
        with pkg.Context(prm) as ctx:
            ctx.set_domain_mask_dev(mt.data_ptr())
            ctx.run_dev(ft.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(),
                        vz.data_ptr() if d > 1 else None)
            torch.cuda.synchronize()
            ctx.check_device_error()
        outs[kernel] = [t.cpu().numpy() for t in (u, vx, vy)]
    for a, b in zip(outs[pkg.KERNEL_FUSED], outs[pkg.KERNEL_TWO_PASS]):
        assert np.array_equal(a, b)
    if precision == pkg.STATE_FP32:
        ou, ovx, ovy, _ = oracle.tgv2_deshade_masked(f, m, 1.0, 2.0, 1.0, 45, dtype=np.float32)
        u, vx, vy = outs[pkg.KERNEL_FUSED]
        assert rel_l2(u, ou) < TOL and rel_l2(vx, ovx) < TOL and rel_l2(vy, ovy) < TOL


def test_all_ones_mask_is_the_unmasked_loop(gpu_lib):
    g = load_golden("deshade3d")
    lam, a0, a1, it = g["params"]
    u, vx, vy, vz = pkg.tgv2_l1_deshade_masked_launch(g["f"], np.ones_like(g["f"]), lam, int(it),
                                                      a0, a1)
    u2, vx2, vy2, vz2 = pkg.tgv2_l1_deshade_launch(g["f"], lam, int(it), alpha0=a0, alpha1=a1)
    for a, b in ((u, u2), (vx, vx2), (vy, vy2), (vz, vz2)):
        assert np.array_equal(a, b)


def test_empty_mask_changes_nothing(gpu_lib):
    f = tissue_phantom_3d(6, 10, 16, seed=7)
    u, vx, vy, vz = pkg.tgv2_l1_deshade_masked_launch(f, np.zeros_like(f), 1.0, 20, 2.0, 1.0)
    assert np.array_equal(u, f)
    assert not (vx.any() or vy.any() or vz.any())


def test_masked_context_matches_host_call_and_refuses_reverse_mode(gpu_lib):
    import torch
    shape = (10, 16, 32)
    f = tissue_phantom_3d(*shape, seed=8)
    m = ellipsoid_mask(shape, 4)
    d, h, w = shape
    hu, hl, hr = pkg.TGVDeshadeMaskedProcessor.processTGV2L1GPUCuda(
        f, 1.0, 2.0, 1.0, 30, mask=m, add_background_back=True)
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=30)
    ft, mt = torch.from_numpy(f).cuda(), torch.from_numpy(m).cuda()
    u, l, r = (torch.empty_like(ft) for _ in range(3))
    with pkg.Context(prm) as ctx:
        ctx.set_domain_mask_dev(mt.data_ptr())
        ctx.process_dev(ft.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                        set_negative_values_to_zero=True, add_background_back=True)
        torch.cuda.synchronize()
        assert np.array_equal(u.cpu().numpy(), hu)
        assert np.array_equal(l.cpu().numpy(), hl)
        assert np.array_equal(r.cpu().numpy(), hr)
        with pytest.raises(pkg.TgvdctError):
            ctx.process_dev(ft.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                            mask_ptr=mt.data_ptr())
        with pytest.raises(pkg.TgvdctError):
            ctx.forward_checkpointed_dev(ft.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                                         r.data_ptr(), 10)
        ctx.set_domain_mask_dev(None)  # cleared: the unmasked loop again
        ctx.process_dev(ft.data_ptr(), u.data_ptr(), l.data_ptr(), r.data_ptr(),
                        set_negative_values_to_zero=True)
        torch.cuda.synchronize()
    pu, _, _ = pkg.TGVDeshadeProcessor.processTGV2L1GPUCuda(f, 1.0, 2.0, 1.0, 30)
    assert np.array_equal(u.cpu().numpy(), pu)


def test_masked_callback_gets_masked_deshade(gpu_lib):
    g = load_golden("masked3d")
    lam, a0, a1, it = g["params"]
    seen = []

    def cb(i, count, u, l, r):
        seen.append((i, u.copy(), l.copy(), r.copy()))
        return False

    fu, fl, fr = pkg.TGVDeshadeMaskedProcessor.processTGV2L1GPUCuda(
        g["f"], lam, a0, a1, int(it), paint_iteration_interval=int(it) - 1,
        iteration_finished_callback=cb, mask=g["mask"])
    # called after iteration index it-1, i.e. on the final state: the callback's
    # on-device deshade equals the returned one
    assert [s[0] for s in seen] == [int(it) - 1]
    _, u, l, r = seen[0]
    assert np.array_equal(u, fu) and np.array_equal(l, fl) and np.array_equal(r, fr)
    out = g["mask"] == 0
    assert not np.any(r[out]) and not np.any(l[out])


def test_blocks_outside_the_domain_are_skipped_exactly(gpu_lib):
    """A domain in one sub-box: most blocks of the fused kernel have no voxel in it and
    leave at once (per-block flags).  The result is the two-pass kernels' bits and the
    oracle's, also after set_params changes the z-chunk (the flags are rebuilt)."""
    import torch
    shape = (20, 40, 96)
    d, h, w = shape
    f = np.log(tissue_phantom_3d(*shape, seed=29)).astype(np.float32)
    m = np.zeros(shape, np.float32)
    m[3:9, 10:20, 40:70] = 1.0  # 12 of the 75 blocks at z-chunk 4 touch it
    ft, mt = torch.from_numpy(f).cuda(), torch.from_numpy(m).cuda()

    def run(kernel, z_chunk, z_chunk_after=None):
        prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=40,
                                 iteration_kernel=kernel, z_chunk=z_chunk)
        u, vx, vy, vz = (torch.empty_like(ft) for _ in range(4))
        with pkg.Context(prm) as ctx:
            ctx.set_domain_mask_dev(mt.data_ptr())
            if z_chunk_after is not None:
                prm.z_chunk = z_chunk_after
                ctx.set_params(prm)
            ctx.run_dev(ft.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr())
            torch.cuda.synchronize()
            ctx.check_device_error()
        return [t.cpu().numpy() for t in (u, vx, vy, vz)]

    ref = run(pkg.KERNEL_TWO_PASS, 0)
    for got in (run(pkg.KERNEL_FUSED, 4), run(pkg.KERNEL_FUSED, 4, z_chunk_after=7),
                run(pkg.KERNEL_FUSED, 0)):
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    ou, ovx, ovy, ovz = oracle.tgv2_deshade_masked(f, m, 1.0, 2.0, 1.0, 40, dtype=np.float32)
    assert rel_l2(ref[0], ou) < TOL and rel_l2(ref[1], ovx) < TOL
    out = m < 1
    assert np.array_equal(ref[0][out], f[out])
