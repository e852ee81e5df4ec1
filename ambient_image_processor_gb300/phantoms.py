"""Seeded synthetic inputs for the TGV-DCT deshade workloads.

The reference ships no images (its evaluation data lives outside its repository),
so every workload runs on generated phantoms with fixed seeds:

* ``rectangles_ellipses_2d`` — piecewise-constant 2-D image: axis-aligned
  rectangles and ellipses with region values U[0, 1] plus Gaussian noise.
* ``tissue_phantom_3d`` — 5 tissue classes {0.2, 0.4, 0.6, 0.8, 1.0} painted by
  random ellipsoids, optionally multiplied by a smooth bias ``exp(b)`` (a random
  cubic polynomial plus Gaussian bumps, scaled so that ``|b| <= 0.3``) and with
  Rician-like noise.
* ``cosine_modes_rhs`` — a Poisson right-hand side made of random low-frequency
  cosine modes plus white noise, mean removed.

Arrays are float32 in (depth, height, width) order (x fastest), matching the
reference's voxel layout ``z*W*H + y*W + x``.
"""
from __future__ import annotations

import numpy as np


def rectangles_ellipses_2d(height=512, width=512, n_rect=12, n_ell=8, noise=0.05, seed=1):
    rng = np.random.default_rng(seed)
    img = np.zeros((height, width), np.float64)
    yy, xx = np.mgrid[0:height, 0:width].astype(np.float64)
    for _ in range(n_rect):
        x0, x1 = np.sort(rng.integers(0, width, 2))
        y0, y1 = np.sort(rng.integers(0, height, 2))
        img[y0:y1 + 1, x0:x1 + 1] = rng.uniform(0.0, 1.0)
    for _ in range(n_ell):
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        ax, ay = rng.uniform(0.05, 0.3) * width, rng.uniform(0.05, 0.3) * height
        inside = ((xx - cx) / ax) ** 2 + ((yy - cy) / ay) ** 2 <= 1.0
        img[inside] = rng.uniform(0.0, 1.0)
    img += rng.normal(0.0, noise, img.shape)
    return img.astype(np.float32)


def _class_volume(depth, height, width, rng, n_ellipsoids):
    classes = np.array([0.2, 0.4, 0.6, 0.8, 1.0])
    vol = np.full((depth, height, width), classes[0], np.float64)
    z = np.arange(depth, dtype=np.float64)[:, None, None]
    y = np.arange(height, dtype=np.float64)[None, :, None]
    x = np.arange(width, dtype=np.float64)[None, None, :]
    for _ in range(n_ellipsoids):
        c = rng.uniform(0.15, 0.85, 3) * np.array([width, height, depth])
        a = rng.uniform(0.08, 0.35, 3) * np.array([width, height, depth])
        a = np.maximum(a, 1.0)
        inside = (((x - c[0]) / a[0]) ** 2 + ((y - c[1]) / a[1]) ** 2
                  + ((z - c[2]) / a[2]) ** 2) <= 1.0
        vol[inside] = classes[rng.integers(0, len(classes))]
    return vol


def smooth_bias(depth, height, width, rng, max_abs=0.3, n_bumps=3, bump_sigma=(20.0, 40.0)):
    """b(x, y, z): random cubic polynomial + Gaussian bumps, scaled to |b| <= max_abs."""
    z = np.linspace(-1.0, 1.0, depth)[:, None, None] if depth > 1 else np.zeros((1, 1, 1))
    y = np.linspace(-1.0, 1.0, height)[None, :, None]
    x = np.linspace(-1.0, 1.0, width)[None, None, :]
    b = np.zeros((depth, height, width), np.float64)
    for i in range(4):
        for j in range(4 - i):
            for k in range(4 - i - j):
                b = b + rng.normal() * (x ** i) * (y ** j) * (z ** k)
    zi = np.arange(depth, dtype=np.float64)[:, None, None]
    yi = np.arange(height, dtype=np.float64)[None, :, None]
    xi = np.arange(width, dtype=np.float64)[None, None, :]
    scale = np.abs(b).max() or 1.0
    b = b / scale
    for _ in range(n_bumps):
        c = rng.uniform(0.0, 1.0, 3) * np.array([width, height, depth])
        s = rng.uniform(*bump_sigma)
        amp = rng.uniform(-1.0, 1.0)
        b = b + amp * np.exp(-(((xi - c[0]) ** 2 + (yi - c[1]) ** 2 + (zi - c[2]) ** 2)
                               / (2.0 * s * s)))
    b = b * (max_abs / max(np.abs(b).max(), 1e-12))
    return b


def tissue_phantom_3d(depth=128, height=128, width=128, *, bias=True, noise=0.02, rician=True,
                      n_ellipsoids=24, seed=2, return_parts=False):
    """5-class ellipsoid phantom, times exp(b), plus Rician-like (or Gaussian) noise."""
    rng = np.random.default_rng(seed)
    clean = _class_volume(depth, height, width, rng, n_ellipsoids)
    b = smooth_bias(depth, height, width, rng) if bias else np.zeros_like(clean)
    img = clean * np.exp(b)
    if noise > 0:
        n1 = rng.normal(0.0, noise, img.shape)
        if rician:
            n2 = rng.normal(0.0, noise, img.shape)
            img = np.sqrt((img + n1) ** 2 + n2 ** 2)
        else:
            img = img + n1
    img = img.astype(np.float32)
    if return_parts:
        return img, clean.astype(np.float32), b.astype(np.float32)
    return img


def cosine_modes_rhs(depth=256, height=256, width=256, n_modes=64, max_freq=8, noise=1e-3,
                     seed=3):
    """Sum of random low-frequency DCT-II cosine modes + white noise, mean removed."""
    rng = np.random.default_rng(seed)
    rhs = np.zeros((depth, height, width), np.float64)
    z = np.arange(depth, dtype=np.float64)[:, None, None]
    y = np.arange(height, dtype=np.float64)[None, :, None]
    x = np.arange(width, dtype=np.float64)[None, None, :]
    for _ in range(n_modes):
        kx, ky, kz = rng.integers(0, max_freq + 1, 3)
        a = rng.normal()
        rhs += a * (np.cos(np.pi * (x + 0.5) * kx / width)
                    * np.cos(np.pi * (y + 0.5) * ky / height)
                    * np.cos(np.pi * (z + 0.5) * kz / depth))
    rhs += rng.normal(0.0, noise, rhs.shape)
    rhs -= rhs.mean()
    return rhs.astype(np.float32)
