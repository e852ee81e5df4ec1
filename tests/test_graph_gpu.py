"""Loops replayed as CUDA graphs (chunks with no callback due) give the same bits as
iteration-by-iteration launches."""
import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
from ambient_image_processor_gb300.phantoms import rectangles_ellipses_2d, tissue_phantom_3d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,geometry,kernel", [
    ((1, 64, 96), pkg.GEOMETRY_2D, pkg.KERNEL_AUTO),
    ((10, 24, 32), pkg.GEOMETRY_3D, pkg.KERNEL_AUTO),
    ((9, 17, 30), pkg.GEOMETRY_3D, pkg.KERNEL_AUTO),
    ((8, 16, 32), pkg.GEOMETRY_3D, pkg.KERNEL_TWO_PASS),
])
def test_graph_replay_matches_single_launches(gpu_lib, shape, geometry, kernel):
    import torch
    f = (rectangles_ellipses_2d(shape[1], shape[2], seed=3)[None] if shape[0] == 1
         else tissue_phantom_3d(*shape, seed=3))
    d, h, w = shape
    its = 100  # 1 single + 3 graph chunks of 32 + 3 single iterations
    ft = torch.from_numpy(np.ascontiguousarray(f, np.float32)).cuda()
    outs = []
    for paint in (0, 1):  # 1: a device callback after every iteration, no graph chunk
        seen = []

        def cb(i, count, u, vx, vy, vz, _user):
            seen.append(int(i))
            return 0

        prm = pkg.default_params(width=w, height=h, depth=d, iteration_count=its,
                                 geometry=geometry, iteration_kernel=kernel,
                                 paint_iteration_interval=paint, callback_on_device=1)
        u, vx, vy, vz = (torch.empty_like(ft) for _ in range(4))
        cfun = pkg.CALLBACK(cb)
        with pkg.Context(prm) as ctx:
            ctx.run_dev(ft.data_ptr(), u.data_ptr(), vx.data_ptr(), vy.data_ptr(),
                        vz.data_ptr() if geometry == pkg.GEOMETRY_3D else None,
                        callback=cfun if paint else None)
            torch.cuda.synchronize()
        outs.append([t.cpu().numpy() for t in (u, vx, vy)])
        if paint:
            assert seen == list(range(1, its))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
