"""The TGV2 primal energy (FP64 sums on the device), the energy-based stop, and the
stop request of the loop.  The energy is checked against an FP64 numpy restatement
of the same operators; stopping must leave exactly the state a shorter run gives."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu


def _fwd(a, axis):
    """Forward difference with a zero last slice (the F operator)."""
    out = np.zeros_like(a)
    lo = [slice(None)] * a.ndim
    hi = [slice(None)] * a.ndim
    lo[axis] = slice(0, -1)
    hi[axis] = slice(1, None)
    out[tuple(lo)] = a[tuple(hi)] - a[tuple(lo)]
    return out


def _bwd(a, axis):
    """w[i - e] - w[i], and -w[i] on the first slice (the reference's B operator)."""
    out = -a.copy()
    lo = [slice(None)] * a.ndim
    hi = [slice(None)] * a.ndim
    lo[axis] = slice(0, -1)
    hi[axis] = slice(1, None)
    out[tuple(hi)] += a[tuple(lo)]
    return out


def energy_np(f, u, vx, vy, vz, lam, a0, a1, l1=True):
    f, u, vx, vy = (np.asarray(a, np.float64) for a in (f, u, vx, vy))
    three = vz is not None
    d = u - f
    data = np.abs(d).sum() if l1 else 0.5 * (d * d).sum()
    ax_x, ax_y = u.ndim - 1, u.ndim - 2
    gx, gy = _fwd(u, ax_x) - vx, _fwd(u, ax_y) - vy
    g2 = gx * gx + gy * gy
    exx, eyy = _bwd(vx, ax_x), _bwd(vy, ax_y)
    exy = 0.5 * (_bwd(vy, ax_x) + _bwd(vx, ax_y))
    e2 = exx * exx + eyy * eyy + 2 * exy * exy
    if three:
        vz = np.asarray(vz, np.float64)
        gz = _fwd(u, 0) - vz
        g2 = g2 + gz * gz
        ezz = _bwd(vz, 0)
        exz = 0.5 * (_bwd(vz, ax_x) + _bwd(vx, 0))
        eyz = 0.5 * (_bwd(vz, ax_y) + _bwd(vy, 0))
        e2 = e2 + ezz * ezz + 2 * exz * exz + 2 * eyz * eyz
    first, second = np.sqrt(g2).sum(), np.sqrt(e2).sum()
    return np.array([lam * data, a1 * first, a0 * second, lam * data + a1 * first + a0 * second])


@pytest.mark.parametrize("shape", [(12, 17, 23), (1, 40, 52)])
@pytest.mark.parametrize("data_term", [pkg.DATA_L1, pkg.DATA_L2])
def test_energy_matches_fp64_restatement(gpu_lib, shape, data_term):
    rng = np.random.default_rng(sum(shape) + data_term)
    f, u = (rng.standard_normal(shape).astype(np.float32) for _ in range(2))
    vx, vy, vz = (0.3 * rng.standard_normal(shape).astype(np.float32) for _ in range(3))
    two_d = shape[0] == 1
    if two_d:
        f, u, vx, vy = (a[0] for a in (f, u, vx, vy))
    got = pkg.tgv2_energy(f, u, vx, vy, None if two_d else vz, lambda_=1.3, alpha0=2.0,
                          alpha1=0.7, data_term=data_term)
    want = energy_np(f, u, vx, vy, None if two_d else vz, 1.3, 2.0, 0.7,
                     l1=data_term == pkg.DATA_L1)
    np.testing.assert_allclose(got, want, rtol=1e-6)


def _run(f, iterations, **kw):
    import torch
    d, h, w = f.shape
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=iterations, **kw)
    u, vx, vy, vz = (torch.empty_like(f) for _ in range(4))
    with pkg.Context(prm) as ctx:
        st = ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr())
        torch.cuda.synchronize()
        ctx.check_device_error()
        return st, ctx.iterations_run, ctx.energy_history(), [t.cpu().numpy() for t in
                                                                  (u, vx, vy, vz)]


def test_energy_checks_change_nothing_and_the_energy_falls(gpu_lib):
    import torch
    f = torch.from_numpy(np.log(tissue_phantom_3d(20, 28, 36, seed=9))).cuda()
    _, _, _, plain = _run(f, 200)
    st, n, hist, checked = _run(f, 200, energy_check_interval=10)
    assert st == pkg.OK and n == 200
    assert len(hist) == 19  # after iterations 10, 20, ..., 190
    assert hist[-1] < hist[0]
    for a, b in zip(plain, checked):
        assert np.array_equal(a, b)
    # the last check is the energy of the state after iteration 190
    _, _, _, s191 = _run(f, 191)
    e = pkg.tgv2_energy(f.cpu().numpy(), s191[0], s191[1], s191[2], s191[3])
    assert e[3] == pytest.approx(hist[-1], rel=1e-9)


def test_energy_tolerance_stops_with_the_state_of_a_shorter_run(gpu_lib):
    import torch
    f = torch.from_numpy(np.log(tissue_phantom_3d(16, 24, 32, seed=10))).cuda()
    st, n, hist, stopped = _run(f, 3000, energy_check_interval=20, energy_tolerance=2e-4)
    assert st == pkg.STOPPED and 20 < n < 3000 and n % 20 == 1
    assert abs(hist[-1] - hist[-2]) <= 2e-4 * abs(hist[-1])
    _, m, _, shorter = _run(f, n)
    assert m == n
    for a, b in zip(stopped, shorter):
        assert np.array_equal(a, b)


def test_stop_request(gpu_lib):
    """A request made before a run stops it at once; one made from the callback after
    iteration 20 stops the loop before iteration 21 runs."""
    import torch
    f = torch.from_numpy(np.log(tissue_phantom_3d(12, 16, 20, seed=11))).cuda()
    d, h, w = f.shape
    u, vx, vy, vz = (torch.empty_like(f) for _ in range(4))
    prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=100,
                             paint_iteration_interval=10, callback_on_device=1)
    with pkg.Context(prm) as ctx:
        ctx.request_stop()
        st = ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr())
        assert st == pkg.STOPPED and ctx.iterations_run == 0

        def cb(it, count, a, b, c, e, user):
            if it == 20:
                ctx.request_stop()
            return 0

        cbw = pkg.CALLBACK(cb)
        st = ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(),
                         vz.data_ptr(), callback=cbw)
        torch.cuda.synchronize()
        assert st == pkg.STOPPED and ctx.iterations_run == 21
        got = [t.cpu().numpy() for t in (u, vx, vy, vz)]
        # the next run is not affected
        st = ctx.run_dev(f.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(), vz.data_ptr())
        assert st == pkg.OK and ctx.iterations_run == 100
    _, _, _, ref = _run(f, 21)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
