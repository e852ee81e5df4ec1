"""The CUDA reverse mode against the FP64 unrolled oracle gradient and against
central finite differences of the CUDA forward loop."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
import oracle
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _tensors(*arrays):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in arrays]


@pytest.mark.parametrize("alphas", [(2.0, 1.0), (0.01, 0.05)])
@pytest.mark.parametrize("shape,data_term,K,every", [
    ((6, 10, 12), pkg.DATA_L1, 15, 4),
    ((7, 9, 16), pkg.DATA_L2, 12, 5),
    ((1, 20, 24), pkg.DATA_L1, 16, 16),
    ((1, 20, 24), pkg.DATA_L2, 9, 2),
])
def test_adjoint_matches_fp64_oracle(gpu_lib, alphas, shape, data_term, K, every):
    import torch
    from ambient_image_processor_gb300.autograd import tgv_denoise

    rng = np.random.default_rng(3)
    f = np.log(tissue_phantom_3d(*shape, seed=13, noise=0.05))
    target = f + 0.05 * rng.standard_normal(shape)
    cv = [0.01 * rng.standard_normal(shape) for _ in range(3)]
    a0, a1 = alphas
    lam = 1.1
    ft, tt = _tensors(f, target)
    ft.requires_grad_(True)
    p = [torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
         for x in (a0, a1, lam)]
    u, v = tgv_denoise(ft, p[0], p[1], p[2], K, every, data_term)
    loss = 0.5 * ((u - tt) ** 2).sum() + sum((v[c] * _tensors(cv[c])[0]).sum() for c in range(3))
    loss.backward()
    uo = u.detach().cpu().numpy().astype(np.float64)
    # the FP64 oracle's gradient of the same loss at the same point
    _, gf, gp = oracle.tgv2_gradient(f.astype(np.float64), lam, a0, a1, K,
                                     grad_u=uo - target, grad_v=cv,
                                     data_term="l1" if data_term == pkg.DATA_L1 else "l2")
    assert rel_l2(ft.grad.cpu().numpy(), gf) < 1e-3
    got = [p[2].grad.item(), p[0].grad.item(), p[1].grad.item()]  # lambda, alpha0, alpha1
    for g, ref in zip(got, gp):
        assert abs(g - ref) <= 1e-3 * max(abs(ref), 1e-2 * np.abs(gf).sum()), (got, gp)


def test_adjoint_checkpoint_stride_does_not_change_the_gradient(gpu_lib):
    import torch
    from ambient_image_processor_gb300.autograd import tgv_denoise

    f = np.log(tissue_phantom_3d(9, 12, 20, seed=14))
    grads = []
    for every in (1, 3, 7, 30):
        ft = _tensors(f)[0].requires_grad_(True)
        lam = torch.tensor(1.0, device="cuda", requires_grad=True)
        u, v = tgv_denoise(ft, 2.0, 1.0, lam, 30, every)
        (u ** 2).sum().backward()
        grads.append((ft.grad.cpu().numpy(), lam.grad.item()))
    for g, l in grads[1:]:
        assert np.array_equal(g, grads[0][0]) and l == pytest.approx(grads[0][1], rel=1e-6)


def test_adjoint_finite_differences_96cube(gpu_lib):
    """The 96^3 adjoint workload: 5-class phantom with noise 0.05, K = 200, checkpoints
    every 20, loss = 1/2 |u_K - clean|^2, central differences with h = 1e-3.
    Single input voxels are differenced through the FP64 forward loop (the oracle): in
    FP32 the rounding flips a 1e-3 perturbation leaves across the volume are ~10% of a
    single voxel's signal.  The three scalars, and one random direction over all
    voxels, are differenced through the CUDA forward loop (loss summed in FP64).
    The denoiser uses the L2 data term: with the L1 prox the loss has kinks closer
    than h = 1e-3 (test_adjoint_oracle.py checks the L1 adjoint at smaller h)."""
    import torch
    from ambient_image_processor_gb300.autograd import tgv_denoise

    noisy, clean, _ = tissue_phantom_3d(96, 96, 96, bias=False, noise=0.05, rician=False, seed=4,
                                        return_parts=True)
    K, every, h = 200, 20, 1e-3
    a0, a1, lam = 2.0, 1.0, 1.0
    ft, ct = _tensors(noisy, clean)
    ft.requires_grad_(True)
    p = [torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
         for x in (a0, a1, lam)]
    u, _ = tgv_denoise(ft, p[0], p[1], p[2], K, every, pkg.DATA_L2)
    (0.5 * ((u - ct) ** 2).sum()).backward()
    gf = ft.grad.cpu().numpy().astype(np.float64)
    scale = np.sqrt(np.mean(gf ** 2))

    # 16 seeded voxels, FP64 forward
    f64, c64 = noisy.astype(np.float64), clean.astype(np.float64)

    def loss64(fa):
        uu = oracle.tgv2_deshade(fa, lam, a0, a1, K, data_term="l2", dtype=np.float64)[0]
        return 0.5 * float(np.sum((uu - c64) ** 2))

    rng = np.random.default_rng(44)
    for j in rng.choice(noisy.size, 16, replace=False):
        fp, fm = f64.copy(), f64.copy()
        fp.flat[j] += h
        fm.flat[j] -= h
        fd = (loss64(fp) - loss64(fm)) / (2 * h)
        assert abs(fd - gf.flat[j]) <= 1e-3 * max(abs(fd), scale), (j, fd, gf.flat[j])

    # scalars and one random direction, CUDA forward
    prm = pkg.default_params(width=96, height=96, depth=96, iteration_count=K,
                             data_term=pkg.DATA_L2)
    ctx = pkg.Context(prm)
    uo = torch.empty_like(ct)
    vx, vy, vz = (torch.empty_like(ct) for _ in range(3))

    def loss(fa, a0_, a1_, lam_):
        prm.alpha0, prm.alpha1, prm.lambda_ = a0_, a1_, lam_
        ctx.set_params(prm)
        ft2 = _tensors(fa)[0]
        ctx.run_dev(ft2.data_ptr(), uo.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr())
        torch.cuda.synchronize()
        d = uo.double() - ct.double()
        return 0.5 * float((d * d).sum())

    # alpha0, alpha1, lambda: a 1e-3 step switches projections on or off at some voxels,
    # so the h = 1e-3 quotient differs from the derivative by a few 1e-3 (FP64 and FP32
    # alike); the FP64 quotient at h = 1e-6 is the derivative to ~1e-6
    got = [p[2].grad.item(), p[0].grad.item(), p[1].grad.item()]  # lambda, alpha0, alpha1
    base = [lam, a0, a1]

    def loss64p(pv):
        uu = oracle.tgv2_deshade(f64, pv[0], pv[1], pv[2], K, data_term="l2",
                                 dtype=np.float64)[0]
        return 0.5 * float(np.sum((uu - c64) ** 2))

    for k in range(3):
        for hh, tol, fn in ((1e-6, 1e-4, loss64p),
                            (h, 1e-2, lambda pv: loss(noisy, pv[1], pv[2], pv[0]))):
            bp, bm = list(base), list(base)
            bp[k] += hh
            bm[k] -= hh
            fd = (fn(bp) - fn(bm)) / (2 * hh)
            assert abs(fd - got[k]) <= tol * max(abs(fd), 1.0), (k, hh, fd, got[k])
    # one random direction over all voxels (every projection near its switch feels a
    # volume-wide step, so this one goes through FP64 at h = 1e-6 too)
    delta = rng.choice([-1.0, 1.0], size=noisy.shape)
    hh = 1e-6
    fd = (loss64(f64 + hh * delta) - loss64(f64 - hh * delta)) / (2 * hh)
    assert abs(fd - float(np.sum(gf * delta))) <= 1e-4 * abs(fd), (fd, np.sum(gf * delta))


def test_poisson_integration_adjoint_identity(gpu_lib):
    """<g, M B v> = <B^T M g, v> for the integration and its adjoint."""
    import torch
    pkg_ctx = pkg.Context(pkg.default_params(width=32, height=24, depth=16))
    rng = np.random.default_rng(7)
    v = [torch.from_numpy(rng.standard_normal((16, 24, 32)).astype(np.float32)).cuda()
         for _ in range(3)]
    g = torch.from_numpy(rng.standard_normal((16, 24, 32)).astype(np.float32)).cuda()
    l = torch.empty_like(g)
    gv = [torch.empty_like(g) for _ in range(3)]
    pkg_ctx.poisson_integrate_dev(v[0].data_ptr(), v[1].data_ptr(), v[2].data_ptr(), l.data_ptr())
    pkg_ctx.poisson_integrate_adjoint_dev(g.data_ptr(), gv[0].data_ptr(), gv[1].data_ptr(),
                                          gv[2].data_ptr())
    torch.cuda.synchronize()
    lhs = float((g.double() * l.double()).sum())
    rhs = float(sum((a.double() * b.double()).sum() for a, b in zip(gv, v)))
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), 1.0)
    pkg_ctx.close()


def test_deshade_gradient_through_the_shading_field(gpu_lib):
    """Loss on u and l of tgv_deshade; its derivative along a random direction of f
    against the FP64 forward (TGV loop + Poisson-DCT integration) at h = 1e-6."""
    import torch
    from ambient_image_processor_gb300.autograd import tgv_deshade

    shape = (8, 12, 16)
    noisy, clean, _ = tissue_phantom_3d(*shape, bias=True, noise=0.05, rician=False, seed=5,
                                        return_parts=True)
    f = np.log(np.maximum(noisy, 0.05)).astype(np.float64)
    rng = np.random.default_rng(8)
    gu = rng.standard_normal(shape)
    gl = rng.standard_normal(shape)
    K, a0, a1, lam = 40, 2.0, 1.0, 1.0
    ft = _tensors(f)[0].requires_grad_(True)
    u, v, l = tgv_deshade(ft, a0, a1, lam, K, 10, pkg.DATA_L2)
    loss = (u * _tensors(gu)[0]).sum() + (l * _tensors(gl)[0]).sum()
    loss.backward()
    grad = ft.grad.cpu().numpy().astype(np.float64)

    def loss64(fa):
        uu, vx, vy, vz = oracle.tgv2_deshade(fa, lam, a0, a1, K, data_term="l2", dtype=np.float64)
        ll = oracle.integrate_poisson_dct(vx, vy, vz)
        return float(np.sum(uu * gu) + np.sum(ll * gl))

    delta = rng.choice([-1.0, 1.0], size=shape)
    h = 1e-6
    fd = (loss64(f + h * delta) - loss64(f - h * delta)) / (2 * h)
    assert abs(fd - float(np.sum(grad * delta))) <= 1e-4 * abs(fd), (fd, np.sum(grad * delta))


def test_backward_graph_replay_and_rebuild(gpu_lib):
    """The backward sweep is captured as a CUDA graph on a context's first backward and
    replayed after; a new step (lambda) or a new checkpoint stride rebuilds it.  Every
    call must give the gradient a fresh context gives."""
    import torch
    f = torch.from_numpy(np.log(tissue_phantom_3d(10, 12, 16, seed=15))).cuda()
    gu = torch.from_numpy(np.random.default_rng(4).standard_normal((10, 12, 16))
                          .astype(np.float32)).cuda()

    def run(ctx, every):
        u, vx, vy, vz, gf = (torch.empty_like(f) for _ in range(5))
        gp = torch.empty(3, dtype=torch.float64, device="cuda")
        ctx.forward_checkpointed_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(),
                                     vz.data_ptr(), every)
        ctx.backward_dev(gu.data_ptr(), None, None, None, gf.data_ptr(), gp.data_ptr())
        torch.cuda.synchronize()
        ctx.check_device_error()
        return gf.cpu().numpy(), gp.cpu().numpy()

    def fresh(lam, every):
        with pkg.Context(pkg.default_params(width=16, height=12, depth=10, iteration_count=24,
                                            lambda_=lam)) as c:
            return run(c, every)

    ref1, ref2, ref3 = fresh(1.0, 5), fresh(0.7, 5), fresh(0.7, 3)
    with pkg.Context(pkg.default_params(width=16, height=12, depth=10, iteration_count=24,
                                        lambda_=1.0)) as ctx:
        for want, (lam, every) in ((ref1, (1.0, 5)), (ref1, (1.0, 5)), (ref2, (0.7, 5)),
                                   (ref3, (0.7, 3)), (ref3, (0.7, 3))):
            ctx.set_params(pkg.default_params(width=16, height=12, depth=10,
                                              iteration_count=24, lambda_=lam))
            gf, gp = run(ctx, every)
            assert np.array_equal(gf, want[0])
            assert np.allclose(gp, want[1], rtol=1e-9, atol=0)


def _gradient(f, K, every, data_term=pkg.DATA_L1, z_chunk=0, kernel=pkg.KERNEL_AUTO, seed=5):
    """d/df and d/d(lambda, alpha0, alpha1) of <g, u> + <h, v> through the C ABI."""
    import torch
    d, h, w = f.shape
    rng = np.random.default_rng(seed)
    ft = torch.from_numpy(f).cuda()
    g = [torch.from_numpy(rng.standard_normal(f.shape).astype(np.float32)).cuda()
         for _ in range(4)]
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=K, data_term=data_term,
                             z_chunk=z_chunk, iteration_kernel=kernel)
    with pkg.Context(prm) as ctx:
        u, vx, vy, vz, gf = (torch.empty_like(ft) for _ in range(5))
        gp = torch.empty(3, dtype=torch.float64, device="cuda")
        ctx.forward_checkpointed_dev(ft.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(),
                                     vz.data_ptr(), every)
        ctx.backward_dev(*(x.data_ptr() for x in g), gf.data_ptr(), gp.data_ptr())
        torch.cuda.synchronize()
        ctx.check_device_error()
        return gf.cpu().numpy(), gp.cpu().numpy()


# (depth, height, width), z-chunk: edge tiles with idle columns and rows, single-plane
# and two-plane volumes, several z-chunks per column of tiles (each with its first and
# last plane made again by the neighbouring chunk), one plane per chunk
@pytest.mark.parametrize("data_term", [pkg.DATA_L1, pkg.DATA_L2])
@pytest.mark.parametrize("shape,z_chunk", [((9, 12, 20), 0), ((20, 24, 40), 3),
                                           ((13, 17, 70), 5), ((1, 20, 24), 0),
                                           ((2, 9, 33), 1), ((30, 33, 36), 7)])
def test_fused_adjoint_passes_equal_separate_passes(gpu_lib, data_term, shape, z_chunk):
    """With shifted passes as the iteration kernel the reverse sweep runs the fused
    adjoint pass (R3 of one iteration, R1 and R2 of the one before) between a segment's
    first and last iterations; with the two-pass kernels it runs R3.R1 and R2 as separate
    passes, and with a checkpoint at every iteration no fused pass at all.  d/df must be
    bit-identical; the parameter gradients are block sums accumulated in FP64 in launch
    order, so they agree to rounding."""
    f = np.log(tissue_phantom_3d(*shape, seed=16)).astype(np.float32)
    ref = _gradient(f, 11, 11, data_term, z_chunk, pkg.KERNEL_TWO_PASS)
    for every in (1, 2, 11):
        got = _gradient(f, 11, every, data_term, z_chunk, pkg.KERNEL_FUSED_SHIFTED)
        assert np.array_equal(got[0], ref[0])
        assert np.allclose(got[1], ref[1], rtol=1e-5, atol=1e-7 * np.abs(ref[0]).sum())
