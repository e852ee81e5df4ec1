"""Generates tests/golden/*.npz from the reference's own kernels.

Each fixture holds seeded inputs and the outputs of the reference's CUDA sources
(source/modules/tgv_deshade, tgv_cuda, cuda_image_operations) compiled for the
CPU by oracle/ref_cpu/build_ref_cpu.py and run in the build container, where the
reference tree is available.  A machine without that tree never runs this script;
tests there read the committed .npz files.

    python oracle/ref_cpu/build_ref_cpu.py && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ambient_image_processor_gb300.phantoms import (  # noqa: E402
    rectangles_ellipses_2d, tissue_phantom_3d)

OUT = os.path.dirname(os.path.abspath(__file__))

# (name, shape (D,H,W), seed, lambda, alpha0, alpha1, iterations)
DESHADE_3D = [
    ("deshade3d", (8, 12, 16), 11, 1.0, 2.0, 1.0, 60),
    ("deshade3d_odd", (9, 13, 17), 12, 0.7, 1.5, 0.8, 45),
    ("deshade3d_d1", (1, 24, 32), 13, 1.0, 2.0, 1.0, 50),
    ("deshade3d_h1", (5, 1, 7), 14, 1.0, 2.0, 1.0, 30),
    ("deshade3d_w1", (6, 9, 1), 15, 1.0, 2.0, 1.0, 30),
    ("deshade3d_tiny", (2, 2, 2), 16, 1.0, 2.0, 1.0, 10),
]
DESHADE_2D = [
    ("deshade2d", (28, 40), 21, 1.0, 2.0, 1.0, 60),
    ("deshade2d_odd", (19, 23), 22, 0.5, 3.0, 1.5, 40),
]
DENOISE = [  # (name, data term, shape, seed, lambda, alpha0, alpha1, iterations)
    ("denoise_l1", 0, (7, 11, 13), 31, 0.9, 1.7, 1.1, 50),
    ("denoise_l2", 1, (7, 11, 13), 32, 0.9, 1.7, 1.1, 50),
    ("denoise_l2_d1", 1, (1, 16, 20), 33, 0.9, 1.7, 1.1, 50),
]
DCT_SHAPES = [(10, 12, 16), (1, 18, 24), (5, 7, 1), (1, 1, 9), (3, 1, 1), (4, 4, 4)]
PROCESS = [("process3d", (8, 12, 16), 41, 1.0, 2.0, 1.0, 40),
           ("process3d_d1", (1, 20, 24), 42, 1.0, 2.0, 1.0, 40)]
# masked deshade: (name, shape, seed, lambda, alpha0, alpha1, iterations, add_background_back)
MASKED = [("masked3d", (8, 12, 16), 61, 1.0, 2.0, 1.0, 40, 0),
          ("masked3d_odd", (7, 11, 13), 62, 0.8, 1.5, 0.9, 35, 1),
          ("masked2d", (1, 20, 24), 63, 1.0, 2.0, 1.0, 40, 0),
          ("masked2d_back", (1, 17, 21), 64, 1.0, 2.0, 1.0, 30, 1)]


# convergence metrics: (name, shape, seed, lambda, alpha0, alpha1, iterations, interval, masked)
CONVERGENCE = [("convergence3d", (6, 10, 12), 71, 1.0, 2.0, 1.0, 14, 1, False),
               ("convergence3d_mask", (5, 9, 11), 72, 1.0, 1.5, 0.8, 16, 2, True),
               ("convergence3d_d1", (1, 16, 20), 73, 1.0, 2.0, 1.0, 12, 1, False)]


def domain_mask(shape, seed):
    """An off-centre ellipsoid that reaches two faces of the volume, mostly 1 inside,
    a few voxels of 2 (inside, and weighting the outputs), a rim of 0.5 (outside the
    TGV domain, still weighting the outputs), 0 elsewhere."""
    rng = np.random.default_rng(seed)
    d, h, w = shape
    z, y, x = np.meshgrid(np.linspace(-1, 1, d) if d > 1 else np.zeros(1),
                          np.linspace(-1, 1, h), np.linspace(-1, 1, w), indexing="ij")
    r2 = ((x - 0.35) / 0.9) ** 2 + ((y + 0.3) / 0.8) ** 2 + (z / 1.1) ** 2
    m = np.where(r2 < 1.0, 1.0, np.where(r2 < 1.3, 0.5, 0.0))
    inside = np.flatnonzero(m == 1.0)
    m.flat[rng.choice(inside, max(1, inside.size // 20), replace=False)] = 2.0
    return m.astype(np.float32)


def empties(f, k):
    return [np.empty_like(f) for _ in range(k)]


def main() -> int:
    R = oracle.ref()
    cases = {}
    for name, shape, seed, lam, a0, a1, it in DESHADE_3D:
        f = tissue_phantom_3d(*shape, seed=seed)
        d, h, w = shape
        u, vx, vy, vz = empties(f, 4)
        R.ref_tgv2_l1_deshade_f32(f, w, h, d, lam, a0, a1, it, u, vx, vy, vz)
        cases[name] = dict(f=f, u=u, v_x=vx, v_y=vy, v_z=vz,
                           params=np.array([lam, a0, a1, it], np.float64))
    for name, shape, seed, lam, a0, a1, it in DESHADE_2D:
        f = rectangles_ellipses_2d(*shape, seed=seed)
        h, w = shape
        u, vx, vy = empties(f, 3)
        R.ref_tgv2_l1_deshade_2d_f32(f, w, h, lam, a0, a1, it, u, vx, vy)
        cases[name] = dict(f=f, u=u, v_x=vx, v_y=vy, params=np.array([lam, a0, a1, it], np.float64))
    for name, dt, shape, seed, lam, a0, a1, it in DENOISE:
        f = tissue_phantom_3d(*shape, seed=seed)
        d, h, w = shape
        (u,) = empties(f, 1)
        R.ref_tgv2_denoise_f32(dt, f, w, h, d, lam, a0, a1, it, u)
        cases[name] = dict(f=f, u=u, data_term=np.array(dt), params=np.array([lam, a0, a1, it]))
    rng = np.random.default_rng(51)
    for shape in DCT_SHAPES:
        d, h, w = shape
        tag = "x".join(str(s) for s in shape)
        for dtype, suf in ((np.float32, "f32"), (np.float64, "f64")):
            x = rng.standard_normal(shape).astype(dtype)
            vx, vy, vz = (rng.standard_normal(shape).astype(dtype) for _ in range(3))
            c = dict(x=x, v_x=vx, v_y=vy, v_z=vz)
            for op in ("cosine_transform", "inverse_cosine_transform", "solve_poisson"):
                out = np.empty_like(x)
                getattr(R, f"ref_{op}_{suf}")(x, w, h, d, out)
                c[op] = out
            out = np.empty_like(x)
            getattr(R, f"ref_divergence_{suf}")(vx, vy, vz, w, h, d, out)
            c["divergence"] = out
            out = np.empty_like(x)
            getattr(R, f"ref_integrate_poisson_dct_{suf}")(vx, vy, vz, w, h, d, out)
            c["integrate"] = out
            cases[f"dct_{tag}_{suf}"] = c
    for name, shape, seed, lam, a0, a1, it in PROCESS:
        f = tissue_phantom_3d(*shape, seed=seed)
        d, h, w = shape
        u, l, r = empties(f, 3)
        R.ref_process_tgv2_l1_f32(f, w, h, d, lam, a0, a1, it, 1, u, l, r)
        cases[name] = dict(f=f, denoised=u, shading=l, deshaded=r,
                           params=np.array([lam, a0, a1, it], np.float64))
    for name, shape, seed, lam, a0, a1, it, back in MASKED:
        f = tissue_phantom_3d(*shape, seed=seed)
        mask = domain_mask(shape, seed)
        d, h, w = shape
        u, vx, vy, vz = empties(f, 4)
        R.ref_tgv2_l1_deshade_masked_f32(f, mask, w, h, d, lam, a0, a1, it, u, vx, vy, vz)
        du, dl, dr = empties(f, 3)
        R.ref_process_tgv2_l1_masked_f32(f, mask, w, h, d, lam, a0, a1, it, 1, back, du, dl, dr)
        cases[name] = dict(f=f, mask=mask, u=u, v_x=vx, v_y=vy, v_z=vz, denoised=du,
                           shading=dl, deshaded=dr, add_background_back=np.array(back),
                           params=np.array([lam, a0, a1, it], np.float64))
    for name, shape, seed, lam, a0, a1, it, interval, masked in CONVERGENCE:
        f = tissue_phantom_3d(*shape, seed=seed)
        d, h, w = shape
        mask = domain_mask(shape, seed) if masked else None
        cap = it
        ncc, tv, mt = np.zeros(cap, np.float32), np.zeros(cap, np.float32), np.zeros(2, np.float32)
        k = R.ref_convergence_test_f32(f, None if mask is None else mask.ctypes.data_as(
            ctypes.c_void_p), w, h, d, lam, a0, a1, it, interval, ncc, tv, cap, mt)
        c = dict(f=f, ncc=ncc[:k], time_tv=tv[:k], metric_tv=mt,
                 params=np.array([lam, a0, a1, it, interval], np.float64))
        if mask is not None:
            c["mask"] = mask
        cases[name] = c
    written = 0
    for name, c in cases.items():
        path = os.path.join(OUT, name + ".npz")
        if os.path.exists(path):  # rewrite only fixtures whose arrays changed
            with np.load(path) as old:
                if set(old.files) == set(c) and all(np.array_equal(old[k], c[k]) for k in c):
                    continue
        np.savez_compressed(path, **c)
        written += 1
    print(f"{written} of {len(cases)} fixtures written to {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
