"""The oracle's cubic B-spline resize (ResizeProcessor with BSpline3 through ITK in the
reference; ITK is not here, so these are the properties of the published algorithm the
restatement must have) and the down-sampled deshade's host logic."""
import numpy as np
import pytest

import oracle


def test_factor_extents_follow_the_float_ceil():
    # ResizeProcessor.cpp:38-45: ceil(n * factor) in float, at least 1
    assert oracle.resize_factor_shape((192, 256, 256), 0.5) == (96, 128, 128)
    assert oracle.resize_factor_shape((1, 100, 75), 0.37) == (1, 37, 28)
    assert oracle.resize_factor_shape((3, 3, 3), 0.01) == (1, 1, 1)
    assert oracle.resize_factor_shape((10, 10, 10), 0.3) == (3, 3, 3)


def test_downsampling_by_half_samples_the_knots():
    """Output i of a factor-1/2 resize sits at input index 2i, where the cubic
    B-spline interpolant equals the data (up to the FP64 prefilter's rounding)."""
    x = np.random.default_rng(0).standard_normal((16, 24, 32)).astype(np.float32)
    y = oracle.resize_bspline3(x, oracle.resize_factor_shape(x.shape, 0.5))
    assert np.abs(y - x[::2, ::2, ::2]).max() < 1e-6


def test_constant_images_stay_exactly_constant():
    c = np.ones((10, 12, 14), np.float32)
    for shape in ((7, 9, 11), (20, 25, 30), (1, 3, 40)):
        assert np.all(oracle.resize_bspline3(c, shape) == 1.0)


def test_linear_ramp_is_reproduced_away_from_the_mirror_boundary():
    """Cubic B-splines reproduce linear functions; the mirror extension bends them
    within a few samples of an edge only.  Upsampling 64 -> 150 puts sample i at
    i / (float)(152 / 64) (two extra samples, then the first 150 kept)."""
    r = (0.5 * np.arange(64) + 3).astype(np.float32)[None, None, :].repeat(3, 0).repeat(3, 1)
    u = oracle.resize_bspline3(r, (3, 3, 150))
    pos = np.arange(150) / np.float64(np.float32(np.float32(152) / np.float32(64)))
    assert np.abs(u[1, 1, 40:110] - (0.5 * pos[40:110] + 3)).max() < 2e-6


def test_short_lines_use_the_closed_mirror_start():
    """Lines of at most 18 samples start the causal recursion from the closed mirror
    sum; the knots are still reproduced."""
    x = np.random.default_rng(1).standard_normal((6, 10, 18)).astype(np.float32)
    y = oracle.resize_bspline3(x, (3, 5, 9))
    assert np.abs(y - x[::2, ::2, ::2]).max() < 1e-6


def test_two_d_images_stay_two_d():
    x = np.random.default_rng(2).standard_normal((37, 50)).astype(np.float32)
    y = oracle.resize_bspline3(x, (1, 19, 25))
    assert y.shape == (19, 25)


def test_downsampled_deshade_at_factor_one_is_the_plain_processor():
    """A factor of 1 skips both resizes, so the masked variant reduces to the masked
    processor followed by the full-resolution tail."""
    from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
    f = tissue_phantom_3d(6, 10, 12, seed=3)
    mask = np.ones_like(f)
    mask[:, :2, :] = 0
    u, l, r, _ = oracle.process_tgvk_l1_downsampled(f, 1.0, 1.0, 2, [1.0, 2.0], 20, mask=mask,
                                                    add_background_back=True)
    ou, ol, orr = oracle.process_tgv2_l1_masked(f * mask, mask, 1.0, 2.0, 1.0, 20,
                                                add_background_back=True, dtype=np.float32)
    assert np.array_equal(u, ou)
    assert np.array_equal(l, ol * mask)
    with pytest.raises(ValueError):
        oracle.process_tgvk_l1_downsampled(f, 0.5, 1.0, 3, [1.0, 2.0, 3.0], 5)


# ---- pin against an independent implementation of the same cubic B-spline -------
# scipy.ndimage implements Unser's recursive prefilter (one pole z = sqrt(3) - 2) and
# the cubic B-spline evaluation with a whole-sample-symmetric ("mirror") extension,
# the boundary ITK's BSplineDecompositionImageFilter and BSplineInterpolateImageFunction
# use.  The two differ only in summation order and in the causal start (ITK truncates
# the mirror sum after ceil(log 1e-10 / log |z|) = 18 terms on longer lines; scipy sums
# it in full), about 1e-11 of the line's scale in FP64.  The oracle then rounds once
# to float32.  Tolerance: 2^-23 of the value (that rounding, twice over) plus 1e-9.

def _scipy_resize(x, shape):
    """ResizeProcessor's sample geometry (ResizeProcessor.cpp:55-90: size factor
    out_grid / n in float, origin 0, two extra samples per axis when any axis grows,
    the first `shape` samples kept) evaluated with scipy.ndimage."""
    ndimage = pytest.importorskip("scipy.ndimage")
    x64 = np.asarray(x, np.float64)
    if x64.ndim == 2:
        x64 = x64[None]
    d, h, w = x64.shape
    D, H, W = shape
    up = W > w or H > h or D > d
    axes = []
    for n, out in ((d, D), (h, H), (w, W)):
        grid = out + 2 if up else out
        size_factor = np.float32(grid) / np.float32(n)  # float division, as the reference
        spacing = 1.0 / np.float64(size_factor)
        axes.append(np.arange(out, dtype=np.float64) * spacing)
    coords = np.stack(np.meshgrid(*axes, indexing="ij"))
    # a single-sample axis stays at its one sample (ITK's mirror index is 0 there)
    keep = [n > 1 for n in (d, h, w)]
    x_in = x64.reshape([n for n, k in zip((d, h, w), keep) if k])
    c = coords[[i for i, k in enumerate(keep) if k]]
    y = ndimage.map_coordinates(x_in, c, order=3, mode="mirror", prefilter=True)
    return y.reshape(D, H, W)


@pytest.mark.parametrize("src,dst", [
    ((16, 24, 32), (8, 12, 16)),      # factor 0.5
    ((20, 30, 33), (12, 18, 20)),     # factor 0.6, odd extents
    ((9, 11, 40), (19, 23, 85)),      # upsampling (two extra samples, then cropped)
    ((12, 12, 12), (29, 29, 29)),     # upsampling by 2.4
    ((2, 3, 4), (1, 2, 2)),           # lines of 2-4 samples (closed mirror start)
    ((3, 5, 17), (7, 11, 41)),        # short lines upsampled
    ((1, 19, 37), (1, 10, 19)),       # a single plane
])
def test_resize_matches_scipy_cubic_bspline(src, dst):
    x = np.random.default_rng(sum(src) + sum(dst)).standard_normal(src).astype(np.float32)
    y = oracle.resize_bspline3(x, dst).reshape(dst)
    s = _scipy_resize(x, dst)
    assert np.all(np.abs(y - s) <= 2.0 ** -23 * np.abs(s) + 1e-9), float(np.abs(y - s).max())


def test_resize_matches_scipy_at_the_down_sampled_deshade_geometry():
    """The down-sampled deshade's round trip at factor 0.5 on the 256x256x192
    workload's proportions, scaled to 64x64x48: down to 32x32x24, then back up."""
    x = np.random.default_rng(9).standard_normal((48, 64, 64)).astype(np.float32)
    down_shape = oracle.resize_factor_shape(x.shape, 0.5)
    y = oracle.resize_bspline3(x, down_shape)
    s = _scipy_resize(x, down_shape)
    assert np.all(np.abs(y - s) <= 2.0 ** -23 * np.abs(s) + 1e-9)
    back = oracle.resize_bspline3(y, x.shape)
    sb = _scipy_resize(y, x.shape)
    assert np.all(np.abs(back - sb) <= 2.0 ** -23 * np.abs(sb) + 1e-9)
