"""The CPU oracle against the reference's own kernels (golden fixtures) and against
independent identities of the math.  CPU only."""
import platform

import numpy as np
import pytest

import oracle
from conftest import load_golden, rel_l2

EXACT = platform.machine() in ("x86_64", "AMD64")


def same(a, b):
    """Bit-exact where the fixtures were made (x86_64), else within float rounding."""
    if EXACT:
        return np.array_equal(a, b)
    return rel_l2(a, b) < 1e-6


@pytest.mark.parametrize("name", ["deshade3d", "deshade3d_odd", "deshade3d_d1", "deshade3d_h1",
                                  "deshade3d_w1", "deshade3d_tiny"])
def test_deshade3d_matches_reference(name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, vx, vy, vz = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), dtype=np.float32)
    for got, ref in ((u, g["u"]), (vx, g["v_x"]), (vy, g["v_y"]), (vz, g["v_z"])):
        assert same(got, ref)


@pytest.mark.parametrize("name", ["deshade2d", "deshade2d_odd"])
def test_deshade2d_matches_reference(name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, vx, vy, _ = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), two_d=True, dtype=np.float32)
    assert same(u, g["u"]) and same(vx, g["v_x"]) and same(vy, g["v_y"])


@pytest.mark.parametrize("name", ["denoise_l1", "denoise_l2", "denoise_l2_d1"])
def test_denoise_matches_reference(name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, *_ = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), data_term=int(g["data_term"]),
                                dtype=np.float32)
    assert same(u, g["u"])


DCT_CASES = ["10x12x16", "1x18x24", "5x7x1", "1x1x9", "3x1x1", "4x4x4"]


@pytest.mark.parametrize("suf", ["f32", "f64"])
@pytest.mark.parametrize("tag", DCT_CASES)
def test_dct_ops_match_reference(tag, suf):
    g = load_golden(f"dct_{tag}_{suf}")
    x = g["x"]
    assert same(oracle.cosine_transform(x), g["cosine_transform"])
    assert same(oracle.inverse_cosine_transform(x), g["inverse_cosine_transform"])
    assert same(oracle.solve_poisson(x), g["solve_poisson"])
    assert same(oracle.divergence(g["v_x"], g["v_y"], g["v_z"]), g["divergence"])
    assert same(oracle.integrate_poisson_dct(g["v_x"], g["v_y"], g["v_z"]), g["integrate"])


@pytest.mark.parametrize("name", ["process3d", "process3d_d1"])
def test_process_matches_reference(name):
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, l, r = oracle.process_tgv2_l1(g["f"], lam, a0, a1, int(it), dtype=np.float32)
    assert same(u, g["denoised"]) and same(l, g["shading"]) and same(r, g["deshaded"])


# ---- identities that do not depend on the reference -----------------------------------

MASKED = ["masked3d", "masked3d_odd", "masked2d", "masked2d_back"]


@pytest.mark.parametrize("name", MASKED)
def test_masked_deshade_matches_reference(name):
    """tgv_deshade_masked/: the loop over voxels with mask >= 1 (2-D operators when
    depth == 1) and the masked processor's epilogue."""
    g = load_golden(name)
    lam, a0, a1, it = g["params"]
    u, vx, vy, vz = oracle.tgv2_deshade_masked(g["f"], g["mask"], lam, a0, a1, int(it),
                                               dtype=np.float32)
    for got, ref in ((u, g["u"]), (vx, g["v_x"]), (vy, g["v_y"]), (vz, g["v_z"])):
        assert same(got, ref)
    du, dl, dr = oracle.process_tgv2_l1_masked(
        g["f"], g["mask"], lam, a0, a1, int(it),
        add_background_back=bool(g["add_background_back"]), dtype=np.float32)
    assert same(du, g["denoised"]) and same(dl, g["shading"]) and same(dr, g["deshaded"])


def test_masked_loop_freezes_the_outside():
    """Outside the domain nothing moves: u stays f, v stays 0."""
    g = load_golden("masked3d")
    lam, a0, a1, it = g["params"]
    u, vx, vy, vz = oracle.tgv2_deshade_masked(g["f"], g["mask"], lam, a0, a1, int(it))
    out = g["mask"] < 1
    assert np.array_equal(u[out], g["f"][out].astype(np.float64))
    for v in (vx, vy, vz):
        assert not np.any(v[out])
    assert np.any(u[~out] != g["f"][~out])


def test_full_mask_is_the_unmasked_loop():
    g = load_golden("deshade3d")
    lam, a0, a1, it = g["params"]
    ones = np.ones_like(g["f"])
    a = oracle.tgv2_deshade_masked(g["f"], ones, lam, a0, a1, int(it), dtype=np.float32)
    b = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), dtype=np.float32)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("name", ["convergence3d", "convergence3d_mask", "convergence3d_d1"])
def test_convergence_metrics_match_reference(name):
    """processTGV2L1DeshadeCuda_convergenceTest(+Metric): NCC and time-TV of l between
    checks, and their total variation over the history."""
    g = load_golden(name)
    lam, a0, a1, it, interval = g["params"]
    ncc, tv, mt = oracle.convergence_test(g["f"], lam, a0, a1, int(it), int(interval),
                                          mask=g.get("mask"), dtype=np.float32)
    assert same(ncc, g["ncc"]) and same(tv, g["time_tv"]) and same(mt, g["metric_tv"])


def test_forward_dct_is_scipy_dctn():
    scipy_fft = pytest.importorskip("scipy.fft")
    rng = np.random.default_rng(0)
    x = rng.standard_normal((6, 7, 9))
    # unnormalised DCT-II has a factor 2 per axis; the reference's x8 makes the 3-D
    # transform equal to scipy's, and twice scipy's in 2-D
    np.testing.assert_allclose(oracle.cosine_transform(x), scipy_fft.dctn(x, type=2),
                               rtol=1e-12, atol=1e-12)
    x2 = rng.standard_normal((7, 9))
    np.testing.assert_allclose(oracle.cosine_transform(x2), 2 * scipy_fft.dctn(x2, type=2),
                               rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("shape", [(6, 7, 9), (8, 5), (1, 4, 3)])
def test_dct_round_trip_is_identity(shape):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape)
    if len(shape) == 3 and shape[0] == 1:
        x = x[0]
    y = oracle.inverse_cosine_transform(oracle.cosine_transform(x))
    np.testing.assert_allclose(y, x, rtol=1e-12, atol=1e-12)


def neumann_laplacian(l):
    """-Laplacian with mirrored (Neumann) boundaries, the operator the DCT diagonalises."""
    out = np.zeros_like(l)
    for ax in range(l.ndim):
        if l.shape[ax] == 1:
            continue
        pad = [(1, 1) if a == ax else (0, 0) for a in range(l.ndim)]
        e = np.pad(l, pad, mode="edge")
        sl_m = [slice(None)] * l.ndim
        sl_p = [slice(None)] * l.ndim
        sl_m[ax] = slice(0, -2)
        sl_p[ax] = slice(2, None)
        out += 2 * l - e[tuple(sl_m)] - e[tuple(sl_p)]
    return out


@pytest.mark.parametrize("shape", [(5, 6, 7), (9, 11), (4, 1, 6)])
def test_poisson_solution_satisfies_neumann_poisson(shape):
    rng = np.random.default_rng(2)
    v = [rng.standard_normal(shape) for _ in range(3)]
    if len(shape) == 2:
        v = [a.reshape(1, *shape)[0] for a in v]
    rhs = oracle.divergence(*v)
    l = oracle.integrate_poisson_dct(*v)
    assert abs(l.mean()) < 1e-12
    if len(shape) == 2 or shape[0] == 1:
        # depth-1 volumes use the 2-D operators (4 - ... eigenvalues)
        lap = neumann_laplacian(l.reshape(shape[-2:]) if l.ndim == 3 else l).reshape(l.shape)
    else:
        lap = neumann_laplacian(l)
    np.testing.assert_allclose(lap, rhs - rhs.mean(), rtol=1e-9, atol=1e-9)


def test_float_oracle_close_to_fp64_oracle():
    g = load_golden("deshade3d")
    lam, a0, a1, it = g["params"]
    u32 = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), dtype=np.float32)
    u64 = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), dtype=np.float64)
    for a, b in zip(u32, u64):
        assert rel_l2(a, b) < 1e-5


def test_callback_free_loop_is_deterministic():
    g = load_golden("deshade3d_odd")
    lam, a0, a1, it = g["params"]
    a = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), dtype=np.float32)
    b = oracle.tgv2_deshade(g["f"], lam, a0, a1, int(it), dtype=np.float32)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
