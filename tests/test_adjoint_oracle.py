"""The FP64 reverse mode of the oracle (oracle/tgv_adjoint.hpp) against central finite
differences of the FP64 forward loop.  CPU only: this pins the reference gradient the
CUDA adjoint is compared with."""
import numpy as np
import pytest

import oracle
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d


def loss_and_grads(f, lam, a0, a1, K, g, c, data_term):
    u, vx, vy, vz = oracle.tgv2_deshade(f, lam, a0, a1, K, data_term=data_term, dtype=np.float64)
    L = 0.5 * np.sum((u - g) ** 2) + np.sum(c[0] * vx + c[1] * vy + c[2] * vz)
    return L, u


@pytest.mark.parametrize("alphas", [(1.7, 0.6), (0.004, 0.03)])  # second: both projections active
@pytest.mark.parametrize("shape,data_term", [((5, 6, 7), "l1"), ((4, 7, 6), "l2"),
                                             ((1, 9, 8), "l1"), ((1, 9, 8), "l2")])
def test_fp64_adjoint_matches_central_differences(shape, data_term, alphas):
    rng = np.random.default_rng(11)
    f = np.log(tissue_phantom_3d(*shape, seed=21, noise=0.05)).astype(np.float64)
    g = f + 0.05 * rng.standard_normal(shape)
    c = [0.01 * rng.standard_normal(shape) for _ in range(3)]
    (a0, a1), lam, K = alphas, 1.3, 14
    L0, u = loss_and_grads(f, lam, a0, a1, K, g, c, data_term)
    uK, gf, gp = oracle.tgv2_gradient(f, lam, a0, a1, K, grad_u=u - g, grad_v=c,
                                      data_term=data_term)
    assert np.allclose(uK, u, rtol=0, atol=1e-12)
    if alphas[0] < 0.01:
        assert abs(gp[1]) > 1e-3 and abs(gp[2]) > 1e-3  # both projections contribute
    h = 1e-6
    # input voxels
    flat = rng.choice(f.size, 8, replace=False)
    for j in flat:
        fp, fm = f.copy(), f.copy()
        fp.flat[j] += h
        fm.flat[j] -= h
        fd = (loss_and_grads(fp, lam, a0, a1, K, g, c, data_term)[0]
              - loss_and_grads(fm, lam, a0, a1, K, g, c, data_term)[0]) / (2 * h)
        assert abs(fd - gf.flat[j]) <= 1e-6 * max(1.0, abs(fd)), (j, fd, gf.flat[j])
    # lambda, alpha0, alpha1
    base = [lam, a0, a1]
    for k in range(3):
        pp, pm = list(base), list(base)
        pp[k] += h
        pm[k] -= h
        fd = (loss_and_grads(f, *pp, K, g, c, data_term)[0]
              - loss_and_grads(f, *pm, K, g, c, data_term)[0]) / (2 * h)
        assert abs(fd - gp[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gp[k])


def test_fp64_adjoint_scalars_at_200_iterations():
    # K = 200 as in the 96^3 adjoint workload, on a 16^3 phantom; a 1e-3 step crosses
    # projection kinks (quotients off by ~1e-3), h = 1e-6 only rarely (~1e-5)
    noisy, clean, _ = tissue_phantom_3d(16, 16, 16, bias=False, noise=0.05, rician=False, seed=4,
                                        return_parts=True)
    f, c, K = noisy.astype(np.float64), clean.astype(np.float64), 200
    base = [1.0, 0.2, 0.3]  # lambda, alpha0, alpha1: both projections active

    def L(p):
        u = oracle.tgv2_deshade(f, p[0], p[1], p[2], K, data_term="l2", dtype=np.float64)[0]
        return 0.5 * np.sum((u - c) ** 2)

    u = oracle.tgv2_deshade(f, *base, K, data_term="l2", dtype=np.float64)[0]
    _, _, gp = oracle.tgv2_gradient(f, *base, K, grad_u=u - c, data_term="l2")
    assert np.all(np.abs(gp) > 1e-3)
    h = 1e-6
    for k in range(3):
        pp, pm = list(base), list(base)
        pp[k] += h
        pm[k] -= h
        fd = (L(pp) - L(pm)) / (2 * h)
        assert abs(fd - gp[k]) <= 5e-5 * max(abs(fd), 1.0), (k, fd, gp[k])
