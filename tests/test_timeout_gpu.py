"""Bounded pipeline waits that run out on the GPU, on purpose and without a fault.

The fused and shifted TMA iteration kernels and the pipelined tensor-core DCT passes
wait on mbarriers for their staged data.  Every such wait is bounded; when one runs out the
kernel raises the context's device error flag, lets its own copies (and tensor-core
operations) in flight finish, and returns, and later launches return at once.  Here
the limit is set to 0 with tgvdct_set_pipeline_wait_limit, so the first wait that
finds its data not yet landed gives up.  The call then reports TGVDCT_ERR_TIMEOUT
through tgvdct_check_device_error, and the same context, with the default limit back,
gives the bits of a fresh context.  No kernel traps, asserts, or spins without limit:
the copies a block drains on its way out land in microseconds, and that drain keeps
its 200 ms bound whatever the consumers' limit is."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import cosine_modes_rhs, tissue_phantom_3d

pytestmark = pytest.mark.gpu

DEFAULT_NS = 200_000_000


def _expect_timeout(ctx):
    with pytest.raises(pkg.TgvdctError) as e:
        ctx.check_device_error()
    assert e.value.status == pkg.ERR_TIMEOUT


def test_iteration_pipeline_wait_runs_out_and_the_context_recovers(gpu_lib):
    import torch
    D, H, W = 48, 64, 64  # widths a multiple of 4: the TMA pipeline runs
    f = torch.from_numpy(np.log(tissue_phantom_3d(D, H, W, seed=8))).cuda()
    prm = pkg.default_params(width=W, height=H, depth=D, iteration_count=40,
                             iteration_kernel=pkg.KERNEL_FUSED)
    out = [torch.empty_like(f) for _ in range(4)]
    ref = [torch.empty_like(f) for _ in range(4)]

    def run(ctx, bufs):
        ctx.run_dev(f.data_ptr(), *(b.data_ptr() for b in bufs))

    with pkg.Context(prm) as ctx:
        ctx.set_pipeline_wait_limit(0)
        run(ctx, out)
        _expect_timeout(ctx)
        ctx.check_device_error()  # the flag was cleared by the report
        ctx.set_pipeline_wait_limit(DEFAULT_NS)
        run(ctx, out)
        torch.cuda.synchronize()
        ctx.check_device_error()
    with pkg.Context(prm) as fresh:
        run(fresh, ref)
        torch.cuda.synchronize()
        fresh.check_device_error()
    for a, b in zip(out, ref):
        assert torch.equal(a, b)


def test_shifted_pass_wait_runs_out_and_the_context_recovers(gpu_lib):
    """The shifted passes (p, q ring and u, f, v ring): five iterations through the
    stepping entry point are one dual step, four shifted passes and one primal step, so
    the first kernel that waits on a pipeline is a shifted pass.  Its waits give up, its
    producer drains both rings, and the context then reproduces a fresh one's state."""
    import ctypes
    import torch
    D, H, W = 40, 48, 64
    f = torch.from_numpy(np.log(tissue_phantom_3d(D, H, W, seed=9))).cuda()
    prm = pkg.default_params(width=W, height=H, depth=D, iteration_count=1,
                             iteration_kernel=pkg.KERNEL_FUSED_SHIFTED)
    L = pkg.lib()

    def run(ctx):
        assert L.tgvdct_state_init_dev(ctx._ctx, ctypes.c_void_p(f.data_ptr()), None) == pkg.OK
        assert L.tgvdct_tgv2_step_dev(ctx._ctx, 5, None) == pkg.OK
        assert ctx.loop_launches() == 6

    def snapshot(ctx):
        buf = torch.zeros((ctx.state_bytes() + 3) // 4, dtype=torch.float32, device="cuda")
        ctx.save_state_dev(buf.data_ptr())
        torch.cuda.synchronize()
        return buf

    with pkg.Context(prm) as ctx:
        ctx.set_pipeline_wait_limit(0)
        run(ctx)
        _expect_timeout(ctx)
        ctx.check_device_error()  # cleared by the report
        ctx.set_pipeline_wait_limit(DEFAULT_NS)
        run(ctx)
        torch.cuda.synchronize()
        ctx.check_device_error()
        got = snapshot(ctx)
    with pkg.Context(prm) as fresh:
        run(fresh)
        torch.cuda.synchronize()
        fresh.check_device_error()
        ref = snapshot(fresh)
    assert torch.equal(got, ref)


@pytest.mark.parametrize("mode", [pkg.DCT_BF16X3, pkg.DCT_TF32])
def test_tensor_core_dct_wait_runs_out_and_the_context_recovers(gpu_lib, mode):
    import torch
    n = 64
    rhs = torch.from_numpy(cosine_modes_rhs(n, n, n, seed=3)).cuda()
    prm = pkg.default_params(width=n, height=n, depth=n, dct_mode=mode,
                             poisson_eigen=pkg.EIGEN_ACCURATE)
    out, ref = torch.empty_like(rhs), torch.empty_like(rhs)
    with pkg.Context(prm) as ctx:
        ctx.poisson_solve_dev(rhs.data_ptr(), out.data_ptr())  # builds the plan
        torch.cuda.synchronize()
        ctx.check_device_error()
        ctx.set_pipeline_wait_limit(0)
        ctx.poisson_solve_dev(rhs.data_ptr(), out.data_ptr())
        _expect_timeout(ctx)
        ctx.set_pipeline_wait_limit(DEFAULT_NS)
        ctx.poisson_solve_dev(rhs.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        ctx.check_device_error()
    with pkg.Context(prm) as fresh:
        fresh.poisson_solve_dev(rhs.data_ptr(), ref.data_ptr())
        torch.cuda.synchronize()
        fresh.check_device_error()
    assert torch.equal(out, ref)
