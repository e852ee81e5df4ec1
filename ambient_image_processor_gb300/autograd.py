"""PyTorch autograd over the CUDA TGV2 loop and its hand-written reverse mode.

``tgv_denoise(f, alpha0, alpha1, lam, iterations)`` runs the TGV2 primal-dual loop
(the reference's tgv2_l1_deshade_launch / tgv2_l2_launch iteration, 3-D operators)
on a CUDA tensor and returns (u, v): the denoised image and the bias gradient
field.  ``tgv_deshade`` adds the shading field l, the DCT Poisson integration of v
(TGVDeshadeProcessor.cpp:386-408), differentiated through its adjoint B^T M.  Gradients flow to f and to alpha0, alpha1 and lambda (pass them as
tensors with requires_grad) for bilevel parameter learning.  The forward keeps a
checkpoint of the full state every ``checkpoint_every`` iterations; backward
recomputes each segment from its checkpoint and runs the adjoint iteration (the
transposed difference operators and the Jacobians of the projections and of the
prox) from the last iteration to the first.  All compute runs in libtgvdct; torch
provides device memory and the stream.
"""
from __future__ import annotations

import torch

from . import DATA_L1, DCT_FP32, EIGEN_REFERENCE, Context, default_params


def _as_float(x):
    return float(x.detach().item()) if isinstance(x, torch.Tensor) else float(x)


class TGVDenoiseFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, alpha0, alpha1, lam, iterations, checkpoint_every, data_term):
        if not f.is_cuda:
            raise ValueError("f must be a CUDA tensor")
        f = f.detach().contiguous().to(torch.float32)
        shape = tuple(f.shape)
        vol = f if f.dim() == 3 else f.reshape((1,) + shape)
        d, h, w = vol.shape
        prm = default_params(width=w, height=h, depth=d, lambda_=_as_float(lam),
                             alpha0=_as_float(alpha0), alpha1=_as_float(alpha1),
                             iteration_count=int(iterations), data_term=int(data_term))
        tgv = Context(prm)
        u = torch.empty_like(vol)
        v = torch.empty((3,) + tuple(vol.shape), dtype=torch.float32, device=vol.device)
        stream = torch.cuda.current_stream(vol.device).cuda_stream
        tgv.forward_checkpointed_dev(vol.data_ptr(), u.data_ptr(), v[0].data_ptr(),
                                     v[1].data_ptr(), v[2].data_ptr(), int(checkpoint_every),
                                     stream)
        ctx.tgv = tgv
        ctx.shape = shape
        ctx.vol_shape = tuple(vol.shape)
        ctx.param_like = [p if isinstance(p, torch.Tensor) else None for p in (alpha0, alpha1, lam)]
        return u.reshape(shape), v.reshape((3,) + shape)

    @staticmethod
    def backward(ctx, grad_u, grad_v):
        tgv = ctx.tgv
        dev = grad_u.device if grad_u is not None else grad_v.device
        gu = grad_u.contiguous().to(torch.float32).reshape(ctx.vol_shape) if grad_u is not None else None
        gv = grad_v.contiguous().to(torch.float32).reshape((3,) + ctx.vol_shape) if grad_v is not None else None
        gf = torch.empty(ctx.vol_shape, dtype=torch.float32, device=dev)
        gp = torch.empty(3, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        tgv.backward_dev(gu.data_ptr() if gu is not None else None,
                         gv[0].data_ptr() if gv is not None else None,
                         gv[1].data_ptr() if gv is not None else None,
                         gv[2].data_ptr() if gv is not None else None,
                         gf.data_ptr(), gp.data_ptr(), stream)
        outs = []
        # gp: d/dlambda, d/dalpha0, d/dalpha1; inputs: alpha0, alpha1, lam
        for like, g in zip(ctx.param_like, (gp[1], gp[2], gp[0])):
            outs.append(None if like is None else g.to(like.dtype).reshape(like.shape))
        return (gf.reshape(ctx.shape), outs[0], outs[1], outs[2], None, None, None)


def tgv_denoise(f, alpha0=2.0, alpha1=1.0, lam=1.0, iterations=100, checkpoint_every=20,
                data_term=DATA_L1):
    """(u, v) after `iterations` TGV2 iterations from u = ubar = f; differentiable in f,
    alpha0, alpha1 and lam (tensors) through the checkpointed reverse mode."""
    return TGVDenoiseFunction.apply(f, alpha0, alpha1, lam, iterations, checkpoint_every,
                                    data_term)


class PoissonIntegrateFunction(torch.autograd.Function):
    """l = M (B_x v_x + B_y v_y + B_z v_z): the Poisson-DCT integration of v on the GPU;
    backward applies the adjoint B^T M (M, the DCT solve, is symmetric)."""

    @staticmethod
    def forward(ctx, v, dct_mode, poisson_eigen):
        v = v.detach().contiguous().to(torch.float32)
        shape = tuple(v.shape[1:])
        vol = shape if len(shape) == 3 else (1,) + shape
        d, h, w = vol
        prm = default_params(width=w, height=h, depth=d, dct_mode=int(dct_mode),
                             poisson_eigen=int(poisson_eigen))
        tgv = Context(prm)
        vv = v.reshape((3,) + vol)
        l = torch.empty(vol, dtype=torch.float32, device=v.device)
        stream = torch.cuda.current_stream(v.device).cuda_stream
        tgv.poisson_integrate_dev(vv[0].data_ptr(), vv[1].data_ptr(),
                                  vv[2].data_ptr() if d > 1 else None, l.data_ptr(), stream)
        ctx.tgv = tgv
        ctx.vol = vol
        ctx.shape = shape
        return l.reshape(shape)

    @staticmethod
    def backward(ctx, grad_l):
        d = ctx.vol[0]
        gl = grad_l.contiguous().to(torch.float32).reshape(ctx.vol)
        gv = torch.zeros((3,) + ctx.vol, dtype=torch.float32, device=gl.device)
        stream = torch.cuda.current_stream(gl.device).cuda_stream
        ctx.tgv.poisson_integrate_adjoint_dev(gl.data_ptr(), gv[0].data_ptr(), gv[1].data_ptr(),
                                              gv[2].data_ptr() if d > 1 else None, stream)
        return gv.reshape((3,) + ctx.shape), None, None


def tgv_deshade(f, alpha0=2.0, alpha1=1.0, lam=1.0, iterations=100, checkpoint_every=20,
                data_term=DATA_L1, dct_mode=DCT_FP32, poisson_eigen=EIGEN_REFERENCE):
    """(u, v, l): the TGV2 loop and the Poisson-DCT integration of v, differentiable in
    f, alpha0, alpha1 and lam.  The deshaded image is u - l."""
    u, v = tgv_denoise(f, alpha0, alpha1, lam, iterations, checkpoint_every, data_term)
    l = PoissonIntegrateFunction.apply(v, dct_mode, poisson_eigen)
    return u, v, l
