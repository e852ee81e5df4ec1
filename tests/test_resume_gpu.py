"""Checkpoint / resume of the loop state: K1 iterations, a snapshot, a load into a
fresh context and K2 more iterations give the bits of one run of K1 + K2, for each
kernel family and dual storage, and for the masked loop."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d

pytestmark = pytest.mark.gpu

CASES = [
    ((14, 20, 32), {}),                                           # fused TMA kernel
    ((14, 20, 32), {"state_precision": pkg.STATE_FX16_DUAL}),     # 16-bit dual fields
    ((14, 20, 32), {"iteration_kernel": pkg.KERNEL_TWO_PASS}),    # in place
    ((13, 19, 30), {}),                                           # register-staged fused
    ((1, 48, 64), {"geometry": pkg.GEOMETRY_2D}),                 # 2-D
    ((14, 20, 32), {"masked": True}),                             # masked loop
]


@pytest.mark.parametrize("shape,kw", CASES)
def test_resume_equals_one_run(gpu_lib, shape, kw):
    import torch
    kw = dict(kw)
    masked = kw.pop("masked", False)
    f = torch.from_numpy(np.log(tissue_phantom_3d(*shape, seed=12))).cuda()
    d, h, w = shape
    mask = None
    if masked:
        m = np.ones(shape, np.float32)
        m[:, :3, :] = 0
        m[::4, :, ::5] = 0
        mask = torch.from_numpy(m).cuda()
    three = kw.get("geometry", pkg.GEOMETRY_3D) == pkg.GEOMETRY_3D

    def ctx_for(k):
        c = pkg.Context(pkg.default_params(width=w, height=h, depth=d, iteration_count=k, **kw))
        if mask is not None:
            c.set_domain_mask_dev(mask.data_ptr())
        return c

    def outs():
        return [torch.empty_like(f) for _ in range(4)]

    def ptrs(o):
        return [o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(),
                o[3].data_ptr() if three else None]

    whole = outs()
    with ctx_for(70) as c:
        c.run_dev(f.data_ptr(), *ptrs(whole))
    first = outs()
    with ctx_for(30) as a:
        a.run_dev(f.data_ptr(), *ptrs(first))
        snap = torch.empty(a.state_bytes(), dtype=torch.uint8, device="cuda")
        a.save_state_dev(snap.data_ptr())
        torch.cuda.synchronize()
    resumed = outs()
    with ctx_for(40) as b:
        b.load_state_dev(snap.data_ptr())
        st = b.resume_dev(*ptrs(resumed))
        torch.cuda.synchronize()
        b.check_device_error()
        assert st == pkg.OK and b.iterations_run == 40
    for x, y in zip(whole[:4 if three else 3], resumed[:4 if three else 3]):
        assert torch.equal(x, y)
